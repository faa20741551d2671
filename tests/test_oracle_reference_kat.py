"""The FP64 oracle against the reference suite's own known-answer tests.

Each test restates one assertion of pyrpa's ``tests/test_rpa_flex.py`` or
``tests/test_tools.py`` (cited per test) and applies it to the oracle, which
pins the oracle to the reference's documented behaviour before it is used to
judge the CUDA engine.  CPU only.
"""
import numpy as np
import pytest

from oracle import api as O
import _models as M


def tiny_model(Nx=2, Ny=2, Nz=1, Nw=4, temp=0.1, tx=1.0, ty=0.5):
    rvec, ham_r = M.square_hoppings(tx, ty)
    klist, kmap, invk = O.gen_irr_k_TRS(Nx, Ny, Nz)
    hamk = O.gen_ham(klist, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    Gk = O.gen_Green0(eig, uni, 0.0, temp, Nw)
    olist, site = O.get_chi_orb_list(1)
    Smat, Cmat = O.gen_SCmatrix(olist, site, 0.0, 0.0)
    return dict(Nx=Nx, Ny=Ny, Nz=Nz, Nw=Nw, temp=temp, rvec=rvec, ham_r=ham_r, klist=klist,
                kmap=kmap, invk=invk, hamk=hamk, eig=eig, uni=uni, Gk=Gk, olist=olist,
                site=site, Smat=Smat, Cmat=Cmat, plist=np.array([1.0]))


def test_irreducible_k_counts_and_maps():
    """gen_irr_k_TRS: Nk formula (_hamiltonian.py:367-378) and a consistent TRS map."""
    for dims in [(2, 2, 1), (4, 4, 1), (8, 6, 1), (5, 5, 1), (6, 5, 1), (4, 4, 4), (6, 6, 3), (3, 3, 3)]:
        klist, kmap, invk = O.gen_irr_k_TRS(*dims)
        Nx, Ny, Nz = dims
        Nk = len(klist)
        from oracle.flex_oracle import irr_k_count
        assert Nk == irr_k_count(*dims)
        grid = np.round(klist * np.array(dims)).astype(int)
        for g in range(Nx * Ny * Nz):
            c = kmap[g]
            irr = grid[invk[g, 0] - 1]
            if invk[g, 1] == 0:
                assert (c == irr).all()
            else:
                assert (c == (-irr) % np.array(dims)).all()
        # every irreducible point has exactly one direct full-grid image
        direct = np.bincount(invk[invk[:, 1] == 0, 0] - 1, minlength=Nk)
        assert (direct == 1).all()


def test_uniform_sc_matrix_two_orbital_reference_values():
    """test_rpa_flex.py:70-88: U=1, J=0.2 two-orbital S and C."""
    olist, site = O.get_chi_orb_list(2)
    S, C = O.gen_SCmatrix(olist, site, 1.0, 0.2)
    es = np.array([[1.0, 0, 0, 0.2], [0, 0.6, 0.2, 0], [0, 0.2, 0.6, 0], [0.2, 0, 0, 1.0]])
    ec = np.array([[1.0, 0, 0, 1.0], [0, -0.2, 0.2, 0], [0, 0.2, -0.2, 0], [1.0, 0, 0, 1.0]])
    assert np.allclose(S, es) and np.allclose(C, ec)


def test_orbital_dependent_vertices_reference_values():
    """test_rpa_flex.py:91-113."""
    olist, site = O.get_chi_orb_list(2)
    S, C = O.gen_SCmatrix_orb(olist, site, np.full((2, 2), 1.0), np.full((2, 2), 0.2))
    es = np.array([[1.0, 0, 0, 0.2], [0, 1.0, 0.2, 0], [0, 0.2, 1.0, 0], [0.2, 0, 0, 1.0]])
    ec = np.array([[1.0, 0, 0, 1.8], [0, -0.6, 0.2, 0], [0, 0.2, -0.6, 0], [1.8, 0, 0, 1.0]])
    assert np.allclose(S, es) and np.allclose(C, ec)


def test_scalar_rpa_chis_matches_closed_form():
    """test_rpa_flex.py:119-127."""
    chi0 = np.array([[[0.20 + 0.10j]], [[0.05 + 0.02j]]])
    U = 1.2
    chis = O.get_chis(chi0, np.array([[U]]))
    assert np.allclose(chis[:, 0, 0], chi0[:, 0, 0] / (1.0 - U * chi0[:, 0, 0]))


def test_chis_chic_reduce_to_bare_chi_when_vertices_are_zero():
    """test_rpa_flex.py:130-141."""
    chi = np.zeros((2, 2, 1, 3), dtype=np.complex128)
    chi[:, :, 0, 0] = [[0.10, 0.02j], [-0.02j, 0.20]]
    chi[:, :, 0, 1] = [[0.05, 0.01], [0.03, 0.04]]
    z = np.zeros((2, 2))
    chis, chic = O.get_chis_chic(chi, z, z)
    assert chis.shape == (2, 2, 3)
    assert np.allclose(chis, chi[:, :, 0, :]) and np.allclose(chic, chi[:, :, 0, :])


def test_green0_noninteracting_inverse_for_one_orbital():
    """test_rpa_flex.py:147-154."""
    st = tiny_model(Nw=5, temp=0.07)
    wn = (2 * np.arange(5) + 1) * np.pi * 0.07
    assert np.allclose(st["Gk"][0, 0], 1.0 / (1j * wn[:, None] - st["eig"][:, 0][None, :]))


def test_chi0_convolution_matches_get_chi0_without_interaction():
    """test_rpa_flex.py:157-171."""
    st = tiny_model()
    chi, stoner = O.get_chi0(st["Smat"], st["Cmat"], st["Gk"], st["olist"], st["kmap"],
                             st["invk"], st["temp"], 2, 2, 1)
    conv = O.get_chi0_conv(st["Gk"], st["kmap"], st["invk"], st["olist"], st["temp"], 2, 2, 1)
    assert chi.shape == (1, 1, 4, len(st["klist"]))
    assert abs(stoner) < 1e-12 and np.allclose(chi, conv)


def test_flex_vertex_zero_interaction_returns_zero():
    """test_rpa_flex.py:174-181."""
    chi = np.ones((3, 2, 1, 1), dtype=np.complex128) * (0.2 + 0.1j)
    z = np.zeros((1, 1))
    v = O.get_Vsigma_nosoc_flex(chi, z, z)
    assert v.shape == chi.shape and np.allclose(v, 0.0)


def test_linearized_eliashberg_zero_interaction_has_zero_lambda_and_finite_gap():
    """test_rpa_flex.py:187-205."""
    st = tiny_model()
    chi, _ = O.get_chi0(st["Smat"], st["Cmat"], st["Gk"], st["olist"], st["kmap"], st["invk"],
                        st["temp"], 2, 2, 1)
    init = O.get_initial_gap(st["klist"], 1, 0)
    gap, lam = O.linearized_eliashberg(chi, st["Gk"], st["uni"], init, st["Smat"], st["Cmat"],
                                       st["olist"], st["plist"], st["kmap"], st["invk"], 2, 2, 1,
                                       st["temp"], 0, itemax=3, arnoldi_m=2)
    assert gap.shape == (1, 1, 4, len(st["klist"]))
    assert np.isfinite(lam) and abs(lam) < 1e-12 and np.isfinite(gap).all()


def lindhard_setup(Nx=8, Ny=8, temp=0.04, mu=0.3):
    rvec, ham_r = M.square_hoppings(1.0, 0.5)
    klist, kmap, invk = O.gen_irr_k_TRS(Nx, Ny, 1)
    hamk = O.gen_ham(klist, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    olist, site = O.get_chi_orb_list(1)
    S, C = O.gen_SCmatrix(olist, site, 1.0, 0.0)
    epsf = M.full_grid_dispersion_1orb(ham_r, rvec, Nx, Ny)
    return dict(Nx=Nx, Ny=Ny, temp=temp, mu=mu, klist=klist, kmap=kmap, invk=invk, eig=eig,
                uni=uni, olist=olist, S=S, C=C, epsf=epsf)


def test_chi0_tail_matches_lindhard_and_converges_second_order():
    """test_rpa_flex.py:308-333: sharp cutoff ~1/Nw, tail-corrected ~1/Nw^2."""
    st = lindhard_setup()
    ml = [0, 1, 2, 3]
    ex = M.exact_chi0_1orb(st["epsf"], st["klist"], ml, st["temp"], st["mu"])
    errs = {}
    for Nw in (32, 128):
        G = M.two_pole_green(st["eig"], st["temp"], st["mu"], Nw)
        co, _ = O.get_chi0(st["S"], st["C"], G, st["olist"], st["kmap"], st["invk"], st["temp"], 8, 8, 1)
        cn, _ = O.get_chi0_tail(st["S"], st["C"], G, st["eig"], st["uni"], st["olist"], st["kmap"],
                                st["invk"], st["mu"], st["temp"], 8, 8, 1)
        eo = max(np.abs(co[0, 0, m] - ex[:, j]).max() for j, m in enumerate(ml))
        en = max(np.abs(cn[0, 0, m] - ex[:, j]).max() for j, m in enumerate(ml))
        errs[Nw] = (eo, en)
    assert 2.5 < errs[32][0] / errs[128][0] < 7.0
    assert errs[32][1] / errs[128][1] > 9.0
    assert errs[128][1] < 0.35 * errs[128][0]


def test_chi0_tail_exact_at_q0_and_reduces_to_conv_api():
    """test_rpa_flex.py:336-354."""
    st = lindhard_setup()
    G = M.two_pole_green(st["eig"], st["temp"], st["mu"], 32)
    cn, _ = O.get_chi0_tail(st["S"], st["C"], G, st["eig"], st["uni"], st["olist"], st["kmap"],
                            st["invk"], st["mu"], st["temp"], 8, 8, 1)
    co, _ = O.get_chi0(st["S"], st["C"], G, st["olist"], st["kmap"], st["invk"], st["temp"], 8, 8, 1)
    cv = O.get_chi0_conv(G, st["kmap"], st["invk"], st["olist"], st["temp"], 8, 8, 1)
    ex0 = M.exact_chi0_1orb(st["epsf"], st["klist"][:1], [0], st["temp"], st["mu"])[0, 0]
    assert abs(cn[0, 0, 0, 0] - ex0) < 1e-10
    assert np.allclose(co, cv, atol=1e-12)


def test_exact_chi0_q0_sum_rule_and_tail_kernel():
    """test_tools.py:110-136."""
    st = lindhard_setup()
    ml = [0, 1, 2]
    ex = M.exact_chi0_1orb(st["epsf"], st["klist"], ml, st["temp"], st["mu"])
    f = M.fermi(st["epsf"], st["temp"], st["mu"])
    assert abs(ex[0, 0] - (f * (1 - f)).sum() / st["temp"] / f.size) < 1e-12
    G = M.two_pole_green(st["eig"], st["temp"], st["mu"], 256)
    chi, _ = O.get_chi0_tail(st["S"], st["C"], G, st["eig"], st["uni"], st["olist"], st["kmap"],
                             st["invk"], st["mu"], st["temp"], 8, 8, 1)
    err = max(np.abs(chi[0, 0, m] - ex[:, j]).max() for j, m in enumerate(ml))
    assert err < 5e-3 * np.abs(ex).max()


def test_exact_chi0_two_pole_against_sharp_cutoff_extrapolation():
    """test_tools.py:139-158: sharp cutoff converges with order ~1."""
    st = lindhard_setup()
    ml = [0, 1]
    ex = M.exact_chi0_1orb(st["epsf"], st["klist"], ml, st["temp"], st["mu"], a=0.5, delta=0.2)
    nws, errs = [64, 128, 256], []
    for Nw in nws:
        G = M.two_pole_green(st["eig"], st["temp"], st["mu"], Nw, a=0.5, delta=0.2)
        chi, _ = O.get_chi0(st["S"], st["C"], G, st["olist"], st["kmap"], st["invk"], st["temp"], 8, 8, 1)
        errs.append(max(np.abs(chi[0, 0, m] - ex[:, j]).max() for j, m in enumerate(ml)))
    assert 0.8 < M.fit_power_order(nws, errs) < 1.3


def test_two_orbital_bands_and_static_chi_psd():
    """test_tools.py:66-79 and 184-199."""
    rvec, ham_r = M.two_orbital_hoppings()
    klist, kmap, invk = O.gen_irr_k_TRS(4, 4, 1)
    hamk = O.gen_ham(klist, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    for ik, k in enumerate(klist):
        cx, cy = np.cos(2 * np.pi * k[0]), np.cos(2 * np.pi * k[1])
        e1, e2 = -2 * (cx + cy), -2 * 0.5 * (cx + cy) + 0.4
        rt = np.sqrt(0.25 * (e1 - e2) ** 2 + 0.04)
        assert np.abs(np.sort(eig[ik]) - [0.5 * (e1 + e2) - rt, 0.5 * (e1 + e2) + rt]).max() < 1e-10
    G = O.gen_Green0(eig, uni, 0.0, 0.1, 64)
    olist, site = O.get_chi_orb_list(2)
    S, C = O.gen_SCmatrix(olist, site, 0.5, 0.1)
    chi0, stoner = O.get_chi0(S, C, G, olist, kmap, invk, 0.1, 4, 4, 1)
    chis, chic = O.get_chis_chic(chi0, S, C)
    assert 0.0 < stoner < 1.0
    for chi in (chis, chic):
        st = np.transpose(chi, (2, 0, 1))
        assert np.abs(st - np.conj(np.swapaxes(st, 1, 2))).max() < 1e-8
        assert np.linalg.eigvalsh(st).min() > -1e-10


def test_mkself_sw_tail_smoke():
    """test_rpa_flex.py:357-372."""
    st = tiny_model(Nx=4, Ny=4, Nw=16, temp=0.1)
    S, C = O.gen_SCmatrix(st["olist"], st["site"], 1.0, 0.0)
    args = (S, C, st["kmap"], st["invk"], st["olist"], st["hamk"], st["eig"], st["uni"], 0.0,
            0.8, 0.1, 16, 4, 4, 1, False, False)
    sg1, mu1 = O.mkself(*args, sw_tail=False)
    sg2, mu2 = O.mkself(*args, sw_tail=True)
    assert np.isfinite(sg2).all()
    smax = np.abs(sg1).max()
    assert smax > 0 and np.abs(sg1 - sg2).max() < 0.6 * smax


def test_nonlinear_eliashberg_zero_seed_and_zero_interaction_stays_zero():
    """test_rpa_flex.py:208-224: the nonlinear FLEX-Eliashberg loop keeps the
    trivial zero-gap solution at S = C = 0."""
    rvec, ham_r = M.square_hoppings(1.0, 0.5)
    klist, kmap, invk = O.gen_irr_k_TRS(2, 2, 1)
    hamk = O.gen_ham(klist, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    Nw, temp = 3, 0.1
    Gk = O.gen_Green0(eig, uni, 0.0, temp, Nw)
    olist, site = O.get_chi_orb_list(1)
    S, C = O.gen_SCmatrix(np.asarray(olist), site, 0.0, 0.0)
    delta0 = np.zeros((1, 1, Nw, len(klist)), dtype=np.complex128)
    delta, sigmak = O.nonlinear_eliashberg(delta0, Gk.copy(), hamk, S, C, olist, np.ones(1), kmap, invk, 0.0, temp,
                                           0, 2, 2, 1, sw_sigma=False, sw_Vconst=True, eps=1e-6, itemax=2, m_diis=1,
                                           gap_min=0.0, sw_amp_newton=False)
    assert delta.shape == delta0.shape and sigmak.shape == delta0.shape
    assert np.allclose(delta, 0.0) and np.allclose(sigmak, 0.0)


def test_nonlinear_eliashberg_oracle_runs_all_branches():
    """Finite, Hermitian-structured output on a 2-orbital model for the
    amplitude-secant and DIIS paths, with and without the FLEX self-energy."""
    rvec, ham_r = M.two_orbital_hoppings()
    klist, kmap, invk = O.gen_irr_k_TRS(4, 4, 1)
    hamk = O.gen_ham(klist, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    Nw, temp = 8, 0.1
    olist, site = O.get_chi_orb_list(2)
    S, C = O.gen_SCmatrix(np.asarray(olist), site, 1.2, 0.2)
    init = O.get_initial_gap(klist, 2, 0)
    d0 = 0.05 * O.get_initial_delta(init, uni, invk, Nw, 0)
    for kw in (dict(sw_amp_newton=True, sw_sigma=False), dict(sw_amp_newton=False, sw_sigma=True, m_diis=3)):
        Gk = O.gen_Green0(eig, uni, 0.0, temp, Nw)
        delta, sigmak, r = O.nonlinear_eliashberg(d0, Gk, hamk, S, C, olist, np.ones(2), kmap, invk, 0.0, temp, 0,
                                                  4, 4, 1, eps=1e-12, itemax=4, gap_min=0.0, full=True, **kw)
        assert np.isfinite(delta).all() and np.isfinite(sigmak).all() and np.isfinite(Gk).all()
        assert r.iterations == 4
        assert np.allclose(delta[0, 1], np.conj(delta[1, 0]))  # Hermitian in the orbital pair
