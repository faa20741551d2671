"""Failure paths of the FLEX entry points, on the GPU through the C ABI.

The reference stops the process on most of these (fself.f90:761-780,
fUJ.f90:353-356) or runs on with NaN; the engine reports an error instead
(pyrpa_gb_last_error, RuntimeError / ValueError in Python) and stays usable
for the next call.  Every failure here is made on the host: a file on
another mesh, a damaged record, a NaN in the seed, an exactly singular
(I - chi0 S).  None faults or hangs the GPU.

* sigma.bin written on another mesh: refused, as ck_sigma_meta refuses it.
* a truncated (temp, Nw, Norb, Nk) record: skipped, as the reference's read
  with iostat skips it; the seed is used.
* NaN in the Sigma seed (sigma.bin or the fused call's seed): refused before
  the loop starts, instead of a loop that runs to its cap on NaN residuals.
* scf_loop too small: the unconverged Sigma of the last iteration is
  returned, as in the reference, equal to the oracle's.
* a singular (I - chi0 S): "zgesv failed", where the reference stops.
* bare Stoner factor >= 1 with sw_rescale: chi0 is clamped to
  (1 - 1e-4) / Stoner (fself.f90:371-380), iteration for iteration as the
  oracle does.
"""
import os

import numpy as np
import pytest

from oracle import api as O
import _models as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F():
    from pyrpa_gb300 import build, flibs
    if not build.LIB.exists():
        build.build()
    flibs.load_library()
    flibs.set_verbose(0)
    flibs.set_precision(64)
    return flibs


def _model(U=1.0, N=4, Nw=16, temp=0.1, t2=0.5):
    rvec, ham_r = M.square_hoppings(1.0, t2)
    klist, kmap, invk = O.gen_irr_k_TRS(N, N, 1)
    hamk = O.gen_ham(klist, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    olist, site = O.get_chi_orb_list(1)
    olist = np.asfortranarray(olist)
    S, C = O.gen_SCmatrix(olist, site, U, 0.0)
    return dict(klist=klist, kmap=kmap, invk=invk, hamk=hamk, eig=eig, uni=uni, olist=olist, S=S, C=C, N=N, Nw=Nw,
                temp=temp)


def _args(m, fill=0.4, Nw=None, sw_out=False, sw_in=False):
    return (m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], 0.0, fill, m["temp"],
            Nw or m["Nw"], m["N"], m["N"], 1, sw_out, sw_in)


def _still_usable(F, m):
    sg, mu = F.mkself(*_args(m), eps=1e-6, pp=0.5)
    assert np.isfinite(sg).all() and np.isfinite(mu)
    assert F.last_error() == ""


def test_sigma_bin_on_another_mesh_is_refused(F, tmp_path):
    m = _model()
    old = os.getcwd()
    os.chdir(tmp_path)
    try:
        F.mkself(*_args(m, sw_out=True), eps=1e-6, pp=0.5)
        with pytest.raises(RuntimeError, match="different mesh"):
            F.mkself(*_args(m, Nw=32, sw_in=True), eps=1e-6, pp=0.5)
        assert "different mesh" in F.last_error()
        _still_usable(F, m)
    finally:
        os.chdir(old)


def test_truncated_footer_is_skipped(F, tmp_path):
    m = _model()
    old = os.getcwd()
    os.chdir(tmp_path)
    try:
        F.mkself(*_args(m, sw_out=True), eps=1e-6, pp=0.5)
        intact = (tmp_path / "sigma.bin").read_bytes()
        sg_a, mu_a = F.mkself(*_args(m, sw_in=True), eps=1e-6, pp=0.5)
        (tmp_path / "sigma.bin").write_bytes(intact[:-10])
        sg_b, mu_b = F.mkself(*_args(m, sw_in=True), eps=1e-6, pp=0.5)
        assert np.array_equal(sg_a, sg_b) and mu_a == mu_b
    finally:
        os.chdir(old)


def test_nan_in_the_seed_is_refused(F, tmp_path):
    m = _model()
    old = os.getcwd()
    os.chdir(tmp_path)
    try:
        F.mkself(*_args(m, sw_out=True), eps=1e-6, pp=0.5)
        raw = bytearray((tmp_path / "sigma.bin").read_bytes())
        raw[4 + 8 + 4 + 4 + 8 + 4 + 4: 4 + 8 + 4 + 4 + 8 + 4 + 4 + 8] = np.array([np.nan]).tobytes()
        (tmp_path / "sigma.bin").write_bytes(bytes(raw))
        with pytest.raises(ValueError, match="NaN"):
            F.mkself(*_args(m, sw_in=True), eps=1e-6, pp=0.5)
    finally:
        os.chdir(old)
    seed = np.zeros((1, 1, m["Nw"], len(m["klist"])), dtype=np.complex128)
    seed[0, 0, 3, 2] = np.nan
    init = F.get_initial_gap(m["klist"], 1, 0)
    with pytest.raises(ValueError, match="NaN"):
        F.flex_eliash(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], init,
                      np.ones(1), 0.0, 0.4, m["temp"], m["Nw"], m["N"], m["N"], 1, 0, sigma_seed=seed)
    _still_usable(F, m)


def test_iteration_cap_returns_the_unconverged_sigma(F):
    m = _model()
    kw = dict(eps=1e-12, pp=0.5, scf_loop=3)
    sg, mu = F.mkself(*_args(m), **kw)
    st = F.last_stats()
    sgo, muo, r = O.mkself(*_args(m), **kw, full=True)
    assert st["iterations"] == r.iterations == 3 and st["esterr"] > 1e-12
    assert abs(mu - muo) < 1e-9
    assert np.abs(sg - sgo).max() <= 1e-9 * np.abs(sgo).max() + 2e-9


def test_singular_vertex_is_reported(F):
    m = _model(U=2.0)
    S, C = m["S"], m["C"]
    chi = 0.05 * np.ones((1, 1, 4, 3), dtype=np.complex128)
    chi[0, 0, 0, 0] = 1.0 / S[0, 0]  # I - chi0 S = 0 exactly
    with pytest.raises(RuntimeError, match="zgesv failed"):
        F.get_Vsigma_nosoc_flex(chi, S, C)
    _still_usable(F, m)


def test_stoner_above_one_is_clamped_like_the_oracle(F):
    m = _model(U=2.0, N=8, Nw=32, temp=0.05, t2=1.0)
    for loops in (1, 4):
        kw = dict(eps=1e-8, pp=0.5, scf_loop=loops, sw_rescale=True)
        sg, mu = F.mkself(*_args(m, fill=0.5), **kw)
        st = F.last_stats()
        sgo, muo, r = O.mkself(*_args(m, fill=0.5), **kw, full=True)
        if loops == 1:
            assert st["stoner"] >= 1.0 and r.history[0]["stoner"] >= 1.0
            assert abs(st["stoner"] - r.history[0]["stoner"]) <= 1e-9 * r.history[0]["stoner"]
        assert abs(mu - muo) < 1e-9
        # the clamp leaves I - chi0 S a margin of 1e-4, which amplifies the
        # rounding difference of the two chi0 by up to 1e4 in the first
        # vertex; three further DIIS steps carry it (measured 1.3e-7)
        rtol = 1e-9 if loops == 1 else 1e-6
        assert np.abs(sg - sgo).max() <= rtol * np.abs(sgo).max() + 2e-9
