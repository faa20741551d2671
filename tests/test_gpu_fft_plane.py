"""GPU parity of the FFT pass variants through chi0 and the FLEX loop,
against the FP64 oracle: the plane pass (PYRPA_GB_FFT_PLANE=1: x and y of
each (x, y) plane in one kernel), the long pass (PYRPA_GB_FFT_LONG=1: a
four-step axis in one kernel), autotuned plans (PYRPA_GB_FFT_TUNE=1) and the
TMA-staged strided passes.  TMA staging is on by default for FP32 (8-byte)
elements; PYRPA_GB_FFT_TMA=1 turns it on for 16-byte (FP64, double-float)
elements too, and the tests here cover both.  Mesh shapes here are used by
no other test, so their FFT plans are built while the switch is on; it is
cleared right after, so that plans made later take the default passes.
"""
import os

import numpy as np
import pytest

import _models as M
from oracle import api as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F():
    from pyrpa_gb300 import build, flibs
    if not build.LIB.exists():
        build.build()
    flibs.load_library()
    flibs.set_verbose(0)
    return flibs


def _model(F, Norb, Nx, Ny, Nz, Nw, seed):
    rvec, ham_r = M.random_hoppings(Norb, seed, dim=3 if Nz > 1 else 2, bandwidth=4.0)
    klist, kmap, invk = O.gen_irr_k_TRS(Nx, Ny, Nz)
    hamk = O.gen_ham(klist, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    temp, mu = 0.1, 0.05
    Gk = O.gen_Green0(eig, uni, mu, temp, Nw)
    olist = F.get_chi_orb_list(Norb)[0]
    _, site = O.get_chi_orb_list(Norb)
    S, C = O.gen_SCmatrix(np.asarray(olist), site, 0.6, 0.1)
    return dict(kmap=kmap, invk=invk, hamk=hamk, eig=eig, uni=uni, Gk=Gk, olist=olist, S=S, C=C, temp=temp, mu=mu)


def _close(a, b, rtol, atol):
    scale = max(np.abs(b).max(), 1e-300)
    err = np.abs(a - b).max()
    assert err <= rtol * scale + atol, f"max |diff| {err:.3e} vs scale {scale:.3e}"


# (Norb, Nx, Ny, Nz, Nw, FP32 run): shapes unique to this file
CASES = [(2, 6, 10, 1, 9, False), (1, 12, 12, 1, 7, False), (2, 10, 6, 2, 6, False), (2, 6, 10, 1, 11, True)]


@pytest.mark.parametrize("Norb,Nx,Ny,Nz,Nw,fp32", CASES)
def test_plane_pass_matches_oracle(F, Norb, Nx, Ny, Nz, Nw, fp32):
    _check(F, "PYRPA_GB_FFT_PLANE", Norb, Nx, Ny, Nz, Nw, fp32)


# (Norb, Nx, Ny, Nz, Nw, FP32 run): Nw = 48 gives a 96-point axis with the splits 4x24 ... 24x4
TUNED = [(1, 12, 10, 1, 48, False), (2, 10, 12, 1, 48, True)]


@pytest.mark.parametrize("Norb,Nx,Ny,Nz,Nw,fp32", TUNED)
def test_tuned_plan_matches_oracle(F, Norb, Nx, Ny, Nz, Nw, fp32):
    _check(F, "PYRPA_GB_FFT_TUNE", Norb, Nx, Ny, Nz, Nw, fp32)


# (Norb, Nx, Ny, Nz, Nw, FP32 run): long axes 256 = 16 x 16, 1024 = 16 x 64, 4096 = 64 x 64
LONG = [(2, 6, 10, 1, 128, False), (1, 10, 6, 1, 512, False), (1, 6, 10, 1, 2048, False),
        (2, 10, 6, 1, 128, True)]


@pytest.mark.parametrize("Norb,Nx,Ny,Nz,Nw,fp32", LONG)
def test_long_pass_matches_oracle(F, Norb, Nx, Ny, Nz, Nw, fp32):
    _check(F, "PYRPA_GB_FFT_LONG", Norb, Nx, Ny, Nz, Nw, fp32)


# (Norb, Nx, Ny, Nz, Nw, FP32 run): strides that are multiples of 32 lines:
# the Matsubara four-step passes of 4096 = 64 x 64 and 1024 = 32 x 32 points,
# a 512-point axis in FP32, and the z pass of an 8 x 4 x 8 mesh
TMA = [(1, 8, 8, 1, 2048, False), (2, 4, 8, 1, 512, False), (1, 16, 16, 1, 256, True), (1, 8, 4, 8, 64, False)]


@pytest.mark.parametrize("Norb,Nx,Ny,Nz,Nw,fp32", TMA)
def test_tma_pass_matches_oracle(F, Norb, Nx, Ny, Nz, Nw, fp32):
    _check(F, "PYRPA_GB_FFT_TMA", Norb, Nx, Ny, Nz, Nw, fp32)


def _check(F, switch, Norb, Nx, Ny, Nz, Nw, fp32):
    m = _model(F, Norb, Nx, Ny, Nz, Nw, seed=Nx + Ny + Nw)
    F.set_precision(32 if fp32 else 64)
    os.environ[switch] = "1"
    try:
        chi, st = F.get_chi0(m["S"], m["C"], m["Gk"], m["olist"], m["kmap"], m["invk"], m["temp"], Nx, Ny, Nz)
        sig, mu = F.mkself(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["mu"],
                           0.5 * Norb, m["temp"], Nw, Nx, Ny, Nz, False, False, scf_loop=3, eps=1e-12, pp=0.5)
    finally:
        os.environ.pop(switch, None)
        F.set_precision(64)
    chio, sto = O.get_chi0(m["S"], m["C"], m["Gk"], m["olist"], m["kmap"], m["invk"], m["temp"], Nx, Ny, Nz)
    sigo, muo = O.mkself(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["mu"],
                         0.5 * Norb, m["temp"], Nw, Nx, Ny, Nz, scf_loop=3, eps=1e-12, pp=0.5)
    rtol, atol = (2e-5, 1e-6) if fp32 else (1e-9, 2e-9)
    _close(chi, chio, rtol, atol)
    assert abs(st - sto) <= rtol * max(1.0, abs(sto)) + atol
    _close(sig, sigo, 1e-4 if fp32 else rtol, atol)
    assert abs(mu - muo) <= (1e-4 if fp32 else 1e-9)
