"""GPU parity of the CUDA engine against the FP64 oracle, through the C ABI.

Every call goes through ``pyrpa_gb300.flibs`` (ctypes -> libfmod.so), the
way pyrpa's own wrappers call the library, and is compared with the same
call on the oracle facade.  Tolerances: FP64 path 1e-9 relative to the array
maximum plus 2e-9 absolute (the reference zeroes real/imaginary parts below
1e-9, so values at that threshold may legitimately flip); FP32 bulk path
2e-5 relative.  The reference's own known-answer tests are re-run on the GPU
path as well (tail-corrected chi0 against the exact Lindhard bubble, zero
interaction limits, closed forms).
"""
import os

import numpy as np
import pytest

from oracle import api as O
import _models as M

pytestmark = pytest.mark.gpu

RTOL64, ATOL64 = 1e-9, 2e-9


@pytest.fixture(scope="module")
def F():
    from pyrpa_gb300 import build, flibs
    if not build.LIB.exists():
        build.build()
    flibs.load_library()
    flibs.set_verbose(0)
    flibs.set_precision(64)
    return flibs


def close(a, b, rtol=RTOL64, atol=ATOL64):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    scale = max(np.abs(b).max(), 1e-300)
    err = np.abs(a - b).max()
    assert err <= rtol * scale + atol, f"max |diff| {err:.3e} vs scale {scale:.3e}"
    return err / scale


def build_model(Norb, Nx, Ny, Nz, Nw, temp, mu, seed=0, complex_hop=False, U=0.0, J=0.0, api=None):
    api = api or O
    if Norb == 1 and seed == 0:
        rvec, ham_r = M.square_hoppings(1.0, 0.5)
    elif Norb == 2 and seed == 0:
        rvec, ham_r = M.two_orbital_hoppings()
    else:
        rvec, ham_r = M.random_hoppings(Norb, seed, complex_hop=complex_hop, dim=3 if Nz > 1 else 2,
                                        bandwidth=4.0)
    klist, kmap, invk = O.gen_irr_k_TRS(Nx, Ny, Nz)
    hamk = O.gen_ham(klist, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    Gk = O.gen_Green0(eig, uni, mu, temp, Nw)
    olist, site = O.get_chi_orb_list(Norb)
    from pyrpa_gb300 import flibs
    olist = flibs.get_chi_orb_list(Norb)[0]
    S, C = O.gen_SCmatrix(np.asarray(olist), site, U, J)
    return dict(Norb=Norb, Nx=Nx, Ny=Ny, Nz=Nz, Nw=Nw, temp=temp, mu=mu, rvec=rvec, ham_r=ham_r, klist=klist,
                kmap=kmap, invk=invk, hamk=hamk, eig=eig, uni=uni, Gk=Gk, olist=olist, site=site, S=S, C=C)


MODELS = {
    "1orb-8x8": dict(Norb=1, Nx=8, Ny=8, Nz=1, Nw=32, temp=0.05, mu=0.2, U=1.0),
    "2orb-4x4": dict(Norb=2, Nx=4, Ny=4, Nz=1, Nw=16, temp=0.1, mu=0.0, U=0.8, J=0.1),
    "3orb-cplx-4x6": dict(Norb=3, Nx=4, Ny=6, Nz=1, Nw=8, temp=0.1, mu=0.1, seed=3, complex_hop=True, U=0.6, J=0.1),
    "2orb-3d-4x4x4": dict(Norb=2, Nx=4, Ny=4, Nz=4, Nw=4, temp=0.2, mu=0.0, seed=5, U=0.5, J=0.05),
    "1orb-odd-5x5": dict(Norb=1, Nx=5, Ny=5, Nz=1, Nw=3, temp=0.1, mu=0.1, seed=7, U=0.5),
    "1orb-radix5-6x6": dict(Norb=1, Nx=6, Ny=6, Nz=1, Nw=5, temp=0.1, mu=0.1, seed=9, U=0.5),
}


@pytest.fixture(scope="module", params=list(MODELS))
def model(request):
    return build_model(**MODELS[request.param])


# ----------------------------------------------------------- band structure
def test_ham_eig_green(F, model):
    m = model
    hk = F.gen_ham(m["klist"], m["ham_r"], m["rvec"])
    close(hk, m["hamk"], 1e-13, 1e-14)
    eig, uni = F.get_eig(m["hamk"])
    close(eig, m["eig"], 1e-12, 1e-13)
    # eigenvector phases are solver conventions; G0 is invariant
    G = F.gen_Green0(eig, uni, m["mu"], m["temp"], m["Nw"])
    close(G, m["Gk"], 1e-11, 1e-13)
    f = F.get_ffermi(m["eig"], m["mu"], m["temp"])
    close(f, O.get_ffermi(m["eig"], m["mu"], m["temp"]), 1e-14, 1e-15)


def test_dyson(F, model):
    m = model
    rng = np.random.default_rng(1)
    sig = 0.1 * (rng.standard_normal(m["Gk"].shape) + 1j * rng.standard_normal(m["Gk"].shape))
    close(F.gen_green(sig, m["hamk"], m["mu"], m["temp"]), O.gen_green(sig, m["hamk"], m["mu"], m["temp"]),
          1e-12, 1e-14)


# --------------------------------------------------------------------- chi0
def test_chi0_conv(F, model):
    m = model
    args = (m["S"], m["C"], m["Gk"], m["olist"], m["kmap"], m["invk"], m["temp"], m["Nx"], m["Ny"], m["Nz"])
    chi, st = F.get_chi0(*args)
    chi_o, st_o = O.get_chi0(*args)
    close(chi, chi_o)
    assert abs(st - st_o) <= 1e-9 * max(1.0, abs(st_o))
    conv = F.get_chi0_conv(m["Gk"], m["kmap"], m["invk"], m["olist"], m["temp"], m["Nx"], m["Ny"], m["Nz"])
    close(conv, chi_o)


def test_chi0_tail(F, model):
    m = model
    args = (m["S"], m["C"], m["Gk"], m["eig"], m["uni"], m["olist"], m["kmap"], m["invk"], m["mu"], m["temp"],
            m["Nx"], m["Ny"], m["Nz"])
    chi, st = F.get_chi0_tail(*args)
    chi_o, st_o = O.get_chi0_tail(*args)
    close(chi, chi_o)
    assert abs(st - st_o) <= 1e-9 * max(1.0, abs(st_o))


def test_chi0_interacting_green(F, model):
    """chi0 of a non-trivial G (random self-energy), conv and tail."""
    m = model
    rng = np.random.default_rng(2)
    sig = 0.05 * (rng.standard_normal(m["Gk"].shape) - 1j * np.abs(rng.standard_normal(m["Gk"].shape)))
    G = O.gen_green(sig, m["hamk"], m["mu"], m["temp"])
    a = (m["S"], m["C"], G, m["olist"], m["kmap"], m["invk"], m["temp"], m["Nx"], m["Ny"], m["Nz"])
    close(F.get_chi0(*a)[0], O.get_chi0(*a)[0])
    t = (m["S"], m["C"], G, m["eig"], m["uni"], m["olist"], m["kmap"], m["invk"], m["mu"], m["temp"], m["Nx"],
         m["Ny"], m["Nz"])
    close(F.get_chi0_tail(*t)[0], O.get_chi0_tail(*t)[0])


# ---------------------------------------------------------------- vertices
def test_rpa_and_vertices(F, model):
    m = model
    chi, _ = O.get_chi0(m["S"], m["C"], m["Gk"], m["olist"], m["kmap"], m["invk"], m["temp"], m["Nx"], m["Ny"],
                        m["Nz"])
    s, c = F.get_chis_chic(chi, m["S"], m["C"])
    so, co = O.get_chis_chic(chi, m["S"], m["C"])
    close(s, so, 1e-11, 1e-14)
    close(c, co, 1e-11, 1e-14)
    for sw in (True, False):
        close(F.get_eig_or_tr_chi(s, m["invk"], sw), O.get_eig_or_tr_chi(so, m["invk"], sw), 1e-10, 1e-13)
    v = F.get_Vsigma_nosoc_flex(chi.copy(), m["S"], m["C"])
    close(v, O.get_Vsigma_nosoc_flex(chi.copy(), m["S"], m["C"]), 1e-11, 1e-14)
    slices = np.ascontiguousarray(np.transpose(chi[:, :, 0, :], (2, 0, 1)))
    close(F.get_chis(slices, m["S"]), O.get_chis(slices, m["S"]), 1e-11, 1e-14)


def test_reference_closed_forms(F):
    """test_rpa_flex.py:119-141 and 174-181 on the GPU path."""
    chi0 = np.array([[[0.20 + 0.10j]], [[0.05 + 0.02j]]])
    chis = F.get_chis(chi0, np.array([[1.2]]))
    assert np.allclose(chis[:, 0, 0], chi0[:, 0, 0] / (1.0 - 1.2 * chi0[:, 0, 0]))
    chi = np.zeros((2, 2, 1, 3), dtype=np.complex128)
    chi[:, :, 0, 0] = [[0.10, 0.02j], [-0.02j, 0.20]]
    chi[:, :, 0, 1] = [[0.05, 0.01], [0.03, 0.04]]
    z = np.zeros((2, 2))
    s, c = F.get_chis_chic(chi, z, z)
    assert np.allclose(s, chi[:, :, 0, :]) and np.allclose(c, chi[:, :, 0, :])
    v = F.get_Vsigma_nosoc_flex(np.ones((3, 2, 1, 1), dtype=np.complex128) * (0.2 + 0.1j), np.zeros((1, 1)),
                                np.zeros((1, 1)))
    assert v.shape == (3, 2, 1, 1) and np.allclose(v, 0.0)


def test_lindhard_orders_on_gpu(F):
    """test_rpa_flex.py:308-354 on the GPU path: sharp cutoff ~1/Nw, tail
    ~1/Nw^2, tail exact at q=0, nu=0."""
    m = build_model(1, 8, 8, 1, 32, 0.04, 0.3)
    ml = [0, 1, 2, 3]
    epsf = M.full_grid_dispersion_1orb(m["ham_r"], m["rvec"], 8, 8)
    ex = M.exact_chi0_1orb(epsf, m["klist"], ml, 0.04, 0.3)
    errs = {}
    for Nw in (32, 128):
        G = M.two_pole_green(m["eig"], 0.04, 0.3, Nw)
        co, _ = F.get_chi0(m["S"], m["C"], G, m["olist"], m["kmap"], m["invk"], 0.04, 8, 8, 1)
        cn, _ = F.get_chi0_tail(m["S"], m["C"], G, m["eig"], m["uni"], m["olist"], m["kmap"], m["invk"], 0.3,
                                0.04, 8, 8, 1)
        errs[Nw] = (max(np.abs(co[0, 0, q] - ex[:, j]).max() for j, q in enumerate(ml)),
                    max(np.abs(cn[0, 0, q] - ex[:, j]).max() for j, q in enumerate(ml)))
        if Nw == 32:
            assert abs(cn[0, 0, 0, 0] - ex[0, 0]) < 1e-10
    assert 2.5 < errs[32][0] / errs[128][0] < 7.0
    assert errs[32][1] / errs[128][1] > 9.0
    assert errs[128][1] < 0.35 * errs[128][0]


# -------------------------------------------------------------------- FLEX
@pytest.mark.parametrize("name,tail", [("1orb", False), ("1orb", True), ("2orb", False), ("2orb", True),
                                       ("3orb", True)])
def test_mkself_matches_oracle(F, name, tail):
    if name == "1orb":
        m = build_model(1, 4, 4, 1, 16, 0.1, 0.0, U=1.0)
        fill = 0.4
    elif name == "2orb":
        m = build_model(2, 4, 4, 1, 16, 0.1, 0.0, U=0.8, J=0.1)
        fill = 0.9
    else:
        m = build_model(3, 4, 4, 1, 8, 0.1, 0.0, seed=11, U=0.8, J=0.1)
        fill = 1.4
    args = (m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["mu"], fill,
            m["temp"], m["Nw"], m["Nx"], m["Ny"], m["Nz"], False, False)
    kw = dict(eps=1e-8, pp=0.5, sw_rescale=True, sw_tail=tail)
    sg, mu = F.mkself(*args, **kw)
    sgo, muo, r = O.mkself(*args, **kw, full=True)
    st = F.last_stats()
    assert st["iterations"] == r.iterations
    assert abs(mu - muo) < 1e-8
    close(sg, sgo, 1e-7, 1e-9)


def test_mkself_sw_tail_smoke(F):
    """test_rpa_flex.py:357-372 on the GPU path."""
    m = build_model(1, 4, 4, 1, 16, 0.1, 0.0, U=1.0)
    args = (m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], 0.0, 0.8, 0.1, 16,
            4, 4, 1, False, False)
    sg1, _ = F.mkself(*args, sw_tail=False)
    sg2, _ = F.mkself(*args, sw_tail=True)
    assert np.isfinite(sg2).all()
    smax = np.abs(sg1).max()
    assert smax > 0 and np.abs(sg1 - sg2).max() < 0.6 * smax


def test_sigma_bin_roundtrip(F, tmp_path):
    """sigma.bin written by sw_out is a gfortran sequential file with the
    metadata footer (fself.f90:742-759) and seeds sw_in."""
    m = build_model(1, 4, 4, 1, 16, 0.1, 0.0, U=1.0)
    args = (m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], 0.0, 0.8, 0.1, 16,
            4, 4, 1)
    old = os.getcwd()
    os.chdir(tmp_path)
    try:
        sg, mu = F.mkself(*args, True, False, eps=1e-6)
        from scipy.io import FortranFile
        with FortranFile("sigma.bin", "r") as f:
            mu_f = f.read_record(np.float64)[0]
            f.read_record(np.float64)
            s = f.read_record(np.complex128).reshape((-1, 16, 1, 1), order="F")
            meta = f.read_record(np.float64)
        assert np.allclose(meta, [0.1, 16, 1, len(m["klist"])])
        assert np.isfinite(mu_f)
        close(s.reshape(-1, order="F"), sg.T.reshape(-1, order="F"), 1e-12, 1e-14)
        sg2, mu2 = F.mkself(*args, False, True, eps=1e-6)
        assert F.last_stats()["iterations"] <= 2
        close(sg2, sg, 1e-5, 1e-7)
    finally:
        os.chdir(old)


# -------------------------------------------------------------- Eliashberg
def test_eliashberg_building_blocks(F, model):
    m = model
    rng = np.random.default_rng(4)
    d = rng.standard_normal(m["Gk"].shape) + 1j * rng.standard_normal(m["Gk"].shape)
    close(F.gen_Fk(m["Gk"], d, m["invk"]), O.mkfk_trs_nsoc(m["Gk"], d), 1e-12, 1e-14)
    for gs in (0, 1, -1):
        init = F.get_initial_gap(m["klist"], m["Norb"], gs)
        close(F.get_initial_delta(init, m["uni"], m["kmap"], m["invk"], m["Nw"], gs),
              O.get_initial_delta(init, m["uni"], m["invk"], m["Nw"], gs), 1e-12, 1e-14)
    plist = np.ones(m["Norb"])
    got = F.conv_delta_orb_to_band(d, m["uni"], m["invk"], plist, 1)
    want = O.conv_delta_orb_to_band(d, m["uni"], m["invk"], plist, 1)
    close(got, want, 1e-12, 1e-14)


# The reference's default 10-step two-pass Arnoldi can stop short of
# convergence: for the d-wave case below a 1e-14 perturbation of G moves its
# lambda by 4e-4 in the FP64 oracle itself, while at 20 steps lambda is stable
# to 1e-10 and equals the power-method value.  Parity is therefore checked at
# Krylov sizes where the oracle's answer is rounding-stable.
@pytest.mark.parametrize("name,gap_sym,arnoldi_m", [("1orb", 1, 20), ("1orb", 0, 10), ("2orb", 0, 6),
                                                    ("1orb", 1, 0)])
def test_lin_eliash_matches_oracle(F, name, gap_sym, arnoldi_m):
    if name == "1orb":
        m = build_model(1, 8, 8, 1, 16, 0.05, 0.0, U=1.6)
    else:
        m = build_model(2, 4, 4, 1, 16, 0.1, 0.0, U=0.8, J=0.1)
    chi, _ = O.get_chi0(m["S"], m["C"], m["Gk"], m["olist"], m["kmap"], m["invk"], m["temp"], m["Nx"], m["Ny"],
                        m["Nz"])
    init = F.get_initial_gap(m["klist"], m["Norb"], gap_sym)
    plist = np.ones(m["Norb"])
    a = dict(eps=1e-6, itemax=200, arnoldi_m=arnoldi_m)
    c1, c2 = chi.copy(), chi.copy()
    gap, lam = F.linearized_eliashberg(c1, m["Gk"], m["uni"], init, m["S"], m["C"], m["olist"], plist, m["kmap"],
                                       m["invk"], m["Nx"], m["Ny"], m["Nz"], m["temp"], gap_sym, **a)
    gapo, lamo = O.linearized_eliashberg(c2, m["Gk"], m["uni"], init, m["S"], m["C"], m["olist"], plist, m["kmap"],
                                         m["invk"], m["Nx"], m["Ny"], m["Nz"], m["temp"], gap_sym, **a)
    assert abs(lam - lamo) <= 1e-8 * max(1.0, abs(lamo)), (lam, lamo)
    # chi is overwritten with V_Delta, as in the reference
    from oracle import flex_oracle as FO
    vd = FO.vdelta_nsoc_flex(chi.T, m["S"].T, m["C"].T, gap_sym >= 0).T
    close(c1, vd, 1e-11, 1e-14)
    ph = np.vdot(gapo.ravel(), gap.ravel())
    ph = ph / abs(ph) if abs(ph) > 0 else 1.0
    close(gap, gapo * ph, 1e-6 if arnoldi_m else 1e-5, 1e-9)


@pytest.mark.parametrize("name,gap_sym", [("1orb", 1), ("2orb", 0)])
def test_lin_eliash_ritz_values_match_oracle(F, name, gap_sym):
    """The leading Ritz values of the final Arnoldi pass (pyrpa_gb_last_ritz):
    pass 2 with the shift undone, or pass 1 on its early exit.  The first is
    lambda.  The others are compared where the oracle itself is stable: its
    Ritz values under a 1e-13 relative perturbation of G move by less than
    1e-7 (unconverged ones move by up to 4e-2 here).  An s-wave start on the
    one-orbital model is left out: the leading d-wave mode enters that Krylov
    space only through rounding noise, so whether it shows up in 20 steps
    depends on the machine."""
    if name == "1orb":
        m = build_model(1, 8, 8, 1, 16, 0.05, 0.0, U=1.6)
    else:
        m = build_model(2, 4, 4, 1, 16, 0.1, 0.0, U=0.8, J=0.1)
    chi, _ = O.get_chi0(m["S"], m["C"], m["Gk"], m["olist"], m["kmap"], m["invk"], m["temp"], m["Nx"], m["Ny"],
                        m["Nz"])
    init = F.get_initial_gap(m["klist"], m["Norb"], gap_sym)
    plist = np.ones(m["Norb"])
    a = dict(eps=1e-6, itemax=200, arnoldi_m=20)
    F.linearized_eliashberg(chi.copy(), m["Gk"], m["uni"], init, m["S"], m["C"], m["olist"], plist, m["kmap"],
                            m["invk"], m["Nx"], m["Ny"], m["Nz"], m["temp"], gap_sym, **a)
    got = F.last_ritz(4)

    def oracle_ritz(G):
        _, lam, r = O.linearized_eliashberg(chi.copy(), G, m["uni"], init, m["S"], m["C"], m["olist"], plist,
                                            m["kmap"], m["invk"], m["Nx"], m["Ny"], m["Nz"], m["temp"], gap_sym,
                                            full=True, **a)
        if r.ritz2 is None:
            return lam, np.sort(r.ritz1.real)[::-1]
        return lam, np.sort(r.ritz2.real + r.ritz1.real.min())[::-1]

    lamo, ref = oracle_ritz(m["Gk"])
    rng = np.random.default_rng(0)
    _, ref_p = oracle_ritz(m["Gk"] * (1 + 1e-13 * rng.standard_normal(m["Gk"].shape)))
    n = min(4, len(ref))
    assert len(got) == n
    assert abs(got[0] - lamo) < 1e-8 * max(1.0, abs(lamo))
    stable = np.abs(ref[:n] - ref_p[:n]) < 1e-7
    assert stable.sum() >= 2
    # a stable value is one the oracle keeps to 1e-7 under the perturbation;
    # the engine's own rounding (FFT order, GPU sums) is such a perturbation,
    # so stable values agree to that threshold (the second Ritz value of the
    # two-orbital case moves by up to 1e-8 under 1e-13 relative changes of G)
    assert np.allclose(got[stable], ref[:n][stable], rtol=1e-6, atol=1e-7), (got, ref[:n], ref_p[:n])
    assert np.all(np.diff(got) <= 0)


def test_lin_eliash_zero_interaction(F):
    """test_rpa_flex.py:187-205 on the GPU path."""
    m = build_model(1, 2, 2, 1, 4, 0.1, 0.0)
    chi, _ = F.get_chi0(m["S"], m["C"], m["Gk"], m["olist"], m["kmap"], m["invk"], 0.1, 2, 2, 1)
    init = F.get_initial_gap(m["klist"], 1, 0)
    gap, lam = F.linearized_eliashberg(chi, m["Gk"], m["uni"], init, m["S"], m["C"], m["olist"], np.ones(1),
                                       m["kmap"], m["invk"], 2, 2, 1, 0.1, 0, itemax=3, arnoldi_m=2)
    assert gap.shape == (1, 1, 4, len(m["klist"]))
    assert np.isfinite(lam) and abs(lam) < 1e-12 and np.isfinite(gap).all()


# ------------------------------------------------------------ FP32 bulk path
def test_fp32_bulk_path(F):
    m = build_model(2, 8, 8, 1, 32, 0.1, 0.0, U=0.8, J=0.1)
    F.set_precision(32)
    try:
        a = (m["S"], m["C"], m["Gk"], m["eig"], m["uni"], m["olist"], m["kmap"], m["invk"], m["mu"], m["temp"], 8,
             8, 1)
        chi32, st32 = F.get_chi0_tail(*a)
        args = (m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["mu"], 0.9,
                m["temp"], m["Nw"], 8, 8, 1, False, False)
        sg32, mu32 = F.mkself(*args, eps=1e-6, pp=0.5, sw_tail=True, sw_rescale=True)
    finally:
        F.set_precision(64)
    chi64, st64 = F.get_chi0_tail(*a)
    close(chi32, chi64, 2e-5, 1e-8)
    assert abs(st32 - st64) < 1e-5
    sg64, mu64 = F.mkself(*args, eps=1e-6, pp=0.5, sw_tail=True, sw_rescale=True)
    close(sg32, sg64, 1e-4, 1e-7)
    assert abs(mu32 - mu64) < 1e-5


# ---------------------------------------------- register vertex, 16 and 25 pairs
@pytest.mark.parametrize("Norb", [4, 5])
@pytest.mark.parametrize("mode", ["fp64", "fp32", "fp32-reg", "df"])
def test_vertex_large_orbital_counts(F, Norb, mode):
    """V_sigma and V_Delta for Nchi = 16 and 25 (the register kernels with the
    shared-memory accumulator in FP64) against the oracle."""
    m = build_model(Norb, 2, 2, 1, 2, 0.2, 0.0, seed=11, U=1.0, J=0.15)
    rng = np.random.default_rng(Norb)
    Nchi, Nk = Norb * Norb, len(m["klist"])
    # the wrapper reads len(chi) x len(chi[0]) matrices (its Nk and Nw), so the
    # V_sigma input is (Nchi, Nchi, Nchi, Nchi): Nchi^2 matrices
    cs = (Nchi, Nchi, Nchi, Nchi)
    chis = 0.05 * (rng.standard_normal(cs) + 1j * rng.standard_normal(cs))
    chi = 0.05 * (rng.standard_normal((Nchi, Nchi, 2, Nk)) + 1j * rng.standard_normal((Nchi, Nchi, 2, Nk)))
    prec, tol = {"fp64": (64, (1e-11, 1e-14)), "df": (48, (1e-11, 1e-14))}.get(mode, (32, (2e-5, 1e-8)))
    old = os.environ.get("PYRPA_GB_VERTEX")
    F.set_precision(prec)
    try:
        if mode == "fp32-reg":
            os.environ["PYRPA_GB_VERTEX"] = "reg"
        v = F.get_Vsigma_nosoc_flex(chis.copy(), m["S"], m["C"])
    finally:
        F.set_precision(64)
        if old is None:
            os.environ.pop("PYRPA_GB_VERTEX", None)
        else:
            os.environ["PYRPA_GB_VERTEX"] = old
    close(v, O.get_Vsigma_nosoc_flex(chis.copy(), m["S"], m["C"]), *tol)
    if mode != "fp64":
        return
    from oracle import flex_oracle as FO
    init = F.get_initial_gap(m["klist"], Norb, 0)
    for gap_sym in (0, -1):
        c1 = chi.copy()
        F.linearized_eliashberg(c1, m["Gk"], m["uni"], init, m["S"], m["C"], m["olist"], np.ones(Norb), m["kmap"],
                                m["invk"], 2, 2, 1, m["temp"], gap_sym, eps=1e-6, itemax=2, arnoldi_m=2)
        vd = FO.vdelta_nsoc_flex(chi.T, m["S"].T, m["C"].T, gap_sym >= 0).T
        close(c1, vd, 1e-11, 1e-14)


@pytest.mark.parametrize("Norb", [1, 2, 3])
def test_double_float_vertex_small_orbital_counts(F, Norb):
    """The double-float V_sigma solve (precision 48 at get_vsigma) for Nchi = 1, 4, 9."""
    m = build_model(Norb, 2, 2, 1, 2, 0.2, 0.0, seed=11, U=1.0, J=0.15)
    rng = np.random.default_rng(Norb)
    Nchi = Norb * Norb
    cs = (Nchi, Nchi, Nchi, Nchi)
    chis = 0.05 * (rng.standard_normal(cs) + 1j * rng.standard_normal(cs))
    F.set_precision(48)
    try:
        v = F.get_Vsigma_nosoc_flex(chis.copy(), m["S"], m["C"])
    finally:
        F.set_precision(64)
    close(v, O.get_Vsigma_nosoc_flex(chis.copy(), m["S"], m["C"]), 1e-11, 1e-14)


# ------------------------------------------------------ mixed FP32/FP64 schedule
def test_mixed_schedule_matches_fp64(F):
    """FP32 bulk until the FP32 floor, then FP64 to eps: the converged Sigma and
    mu equal the all-FP64 solve's to the convergence tolerance."""
    m = build_model(2, 8, 8, 1, 32, 0.1, 0.0, U=0.8, J=0.1)
    args = (m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["mu"], 0.9,
            m["temp"], m["Nw"], 8, 8, 1, False, False)
    F.set_precision(F.MIXED)
    try:
        sgm, mum = F.mkself(*args, eps=1e-8, pp=0.5, sw_tail=True, sw_rescale=True)
        st = F.last_stats()
    finally:
        F.set_precision(64)
    assert 0 < st["iterations_fp32"] < st["iterations"], st
    assert st["esterr"] < 1e-8
    sg64, mu64 = F.mkself(*args, eps=1e-8, pp=0.5, sw_tail=True, sw_rescale=True)
    close(sgm, sg64, 1e-6, 1e-9)
    assert abs(mum - mu64) < 1e-8


# ------------------------------------------------------ coarse-mesh warm start
@pytest.mark.parametrize("dims,Nw", [((8, 8, 1), 32), ((4, 4, 4), 8)])
def test_warm_start_reaches_the_cold_fixed_point(F, dims, Nw):
    """The fused solve from a coarse-mesh seed converges to the same Sigma,
    mu and lambda as the cold start (FP64 bulk, eps 1e-8)."""
    Nx, Ny, Nz = dims
    m = build_model(2, Nx, Ny, Nz, Nw, 0.1, 0.0, seed=21 if Nz > 1 else 0, U=0.8, J=0.1)
    init = F.get_initial_gap(m["klist"], 2, 0)
    kw = dict(eps=1e-8, scf_loop=200, sw_tail=True, sw_rescale=True, arnoldi_m=20)
    args = (m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], init, np.ones(2),
            m["mu"], 0.9, m["temp"], Nw, Nx, Ny, Nz, 0)
    cold = F.flex_eliash(*args, **kw)
    st_cold = F.last_stats()
    warm = F.flex_eliash(*args, coarse=(2, 2), **kw)
    st_warm = F.last_stats()
    assert st_warm["iterations_coarse"] > 0 and st_cold["iterations_coarse"] == 0
    assert st_warm["iterations"] <= st_cold["iterations"], (st_warm, st_cold)
    close(warm["sigmak"], cold["sigmak"], 1e-6, 1e-9)
    assert abs(warm["mu"] - cold["mu"]) < 1e-8
    assert abs(warm["lam"] - cold["lam"]) <= 1e-6 * max(1.0, abs(cold["lam"]))


# ------------------------------------------------ double-float convolutions
def test_double_float_chi0_matches_oracle(F, model):
    """Precision 48: the chi0 FFT convolutions in double-float arithmetic on
    the FP32 pipe meet the FP64 tolerances against the oracle (random
    self-energy, conv and tail)."""
    m = model
    rng = np.random.default_rng(3)
    sig = 0.05 * (rng.standard_normal(m["Gk"].shape) - 1j * np.abs(rng.standard_normal(m["Gk"].shape)))
    G = O.gen_green(sig, m["hamk"], m["mu"], m["temp"])
    a = (m["S"], m["C"], G, m["olist"], m["kmap"], m["invk"], m["temp"], m["Nx"], m["Ny"], m["Nz"])
    t = (m["S"], m["C"], G, m["eig"], m["uni"], m["olist"], m["kmap"], m["invk"], m["mu"], m["temp"], m["Nx"],
         m["Ny"], m["Nz"])
    F.set_precision(48)
    try:
        conv, st = F.get_chi0(*a)
        tail, st_t = F.get_chi0_tail(*t)
    finally:
        F.set_precision(64)
    conv_o, st_o = O.get_chi0(*a)
    close(conv, conv_o)
    assert abs(st - st_o) <= 1e-9 * max(1.0, abs(st_o))
    close(tail, O.get_chi0_tail(*t)[0])


@pytest.mark.parametrize("tail", [False, True])
def test_double_float_mkself_matches_oracle(F, tail):
    """Precision 48 FLEX loop (double-float chi0 and Sigma, FP64 vertex) against
    the oracle's FP64 loop, same iteration count."""
    m = build_model(2, 4, 4, 1, 16, 0.1, 0.0, U=0.8, J=0.1)
    args = (m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["mu"], 0.9,
            m["temp"], m["Nw"], m["Nx"], m["Ny"], m["Nz"], False, False)
    kw = dict(eps=1e-8, pp=0.5, sw_rescale=True, sw_tail=tail)
    F.set_precision(48)
    try:
        sg, mu = F.mkself(*args, **kw)
        st = F.last_stats()
    finally:
        F.set_precision(64)
    sgo, muo, r = O.mkself(*args, **kw, full=True)
    assert st["iterations"] == r.iterations
    assert abs(mu - muo) < 1e-8
    close(sg, sgo, 1e-7, 1e-9)


# ------------------------------------------------------ sigma.bin regrid seed
def _regrid_golden():
    from pathlib import Path
    return np.load(Path(__file__).resolve().parent / "golden" / "regrid_sigma_golden.npz")


@pytest.mark.parametrize("case", range(4))
def test_regrid_sigma_matches_reference_output(F, case):
    """pyrpa_gb_regrid_sigma against the output of the reference's own
    plibs.regrid_sigma_bin (golden vectors), 1e-12 of the maximum."""
    g = _regrid_golden()
    sig, ref, par = g[f"case{case}_in"], g[f"case{case}_out"], g[f"case{case}_par"]
    T_old, T_new, Nw_new, ws = par
    out = F.regrid_sigma(sig.T, T_old, T_new, int(Nw_new), ws).T
    close(out, ref, 1e-12, 1e-15)


def test_regrid_sigma_bin_file_round_trip(F, tmp_path):
    """pyrpa_gb300.seed.regrid_sigma_bin reads and writes sigma.bin as the
    reference does (records, footer of the new mesh)."""
    from scipy.io import FortranFile
    from pyrpa_gb300 import seed
    g = _regrid_golden()
    sig, ref, par = g["case0_in"], g["case0_out"], g["case0_par"]
    Nk, Nw_old, No, _ = sig.shape
    path = tmp_path / "sigma.bin"
    with FortranFile(str(path), "w") as f:
        f.write_record(np.array([0.1]))
        f.write_record(np.array([0.12]))
        f.write_record(np.ascontiguousarray(sig.ravel(order="F")))
        f.write_record(np.array([par[0], float(Nw_old), float(No), float(Nk)]))
    assert seed.regrid_sigma_bin(temp_new=par[1], Nw_new=int(par[2]), path=str(path)) == (Nk, int(par[2]))
    with FortranFile(str(path), "r") as f:
        mu, mu_old = f.read_record(np.float64), f.read_record(np.float64)
        flat = f.read_record(np.complex128)
        meta = f.read_record(np.float64)
    assert mu[0] == 0.1 and mu_old[0] == 0.12
    assert np.allclose(meta, [par[1], par[2], No, Nk])
    close(flat.reshape((Nk, int(par[2]), No, No), order="F"), ref, 1e-12, 1e-15)
    with pytest.raises(ValueError):
        seed.regrid_sigma_bin(temp_old=0.5, temp_new=par[1], path=str(path))


# ------------------------------------------------------ Wannier R-space output
@pytest.mark.parametrize("case", range(3))
def test_wannier_output_matches_reference_files(F, case, tmp_path):
    """pyrpa_gb300.wannier against the files the reference's own
    output_self_wannier / output_gap_wannier wrote (golden vectors)."""
    from pathlib import Path
    from pyrpa_gb300 import wannier
    g = np.load(Path(__file__).resolve().parent / "golden" / "wannier_golden.npz")
    Nx, Ny, Nz, Nw, Ncut, tol, is_self = g[f"case{case}_par"]
    Nx, Ny, Nz, Nw, Ncut = int(Nx), int(Ny), int(Nz), int(Nw), int(Ncut)
    data = g[f"case{case}_data"]
    klist, kmap, invk = F.gen_irr_k_TRS(Nx, Ny, Nz)
    fname = str(tmp_path / "w")
    if is_self:
        wannier.output_self_wannier(data, 0.25, kmap, invk, Nx, Ny, Nz, Nw, 0.02, N_cut=Ncut, zero_tol=tol, fname=fname)
        key = "sigma"
    else:
        wannier.output_gap_wannier(data, kmap, invk, Nx, Ny, Nz, Nw, 0.02, N_cut=Ncut, zero_tol=tol, fname=fname)
        key = "gap"
    z = np.load(fname + ".npz")
    assert np.array_equal(z["rvec"], g[f"case{case}_npz_rvec"])
    close(z[key], g[f"case{case}_npz_{key}"], 1e-12, 1e-15)
    assert np.allclose(z["iw"], g[f"case{case}_npz_iw"], rtol=1e-15, atol=0)
    got = (tmp_path / "w.dat").read_text().splitlines()
    ref = str(g[f"case{case}_dat"]).splitlines()
    assert got[:2] == ref[:2] and len(got) == len(ref)
    for a, b in zip(got[2:], ref[2:]):
        assert a[:23] == b[:23]  # Rx Ry Rz (%4d), io jo (%3d), iw (%5d)
        assert np.allclose([float(a[23:39]), float(a[39:])], [float(b[23:39]), float(b[39:])], rtol=2e-8, atol=1e-20)
