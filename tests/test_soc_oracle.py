"""CPU checks of the spin-orbit oracle (oracle/soc_oracle.py).

The reference's test suite has no spin-orbit case, so these pin what can be
pinned without it: the spin-orbit bubble of a spin-degenerate model equals the
(pinned) non-SOC bubble block by block, the onsite vertex has the Kanamori
values the reference's comments give, and the solver paths agree with each
other.
"""
import numpy as np
import pytest

from oracle import api as O
from oracle import soc_oracle as SO
import _models as M


def soc_setup(alpha, Nx=6, Ny=6, Nw=8, temp=0.1, mu=0.1, U=1.5, J=0.0, n=1):
    base = M.square_hoppings(1.0, 1.0, -0.25) if n == 1 else M.two_orbital_hoppings()
    rvec, H, slist, invs = M.spin_orbit_hoppings(*base, alpha=alpha)
    klist, kmap, invk = O.gen_irr_k_TRS(Nx, Ny, 1)
    hamk = O.gen_ham(klist, H, rvec)
    eig, uni = O.get_eig(hamk)
    olist, site = O.get_chi_orb_list(2 * n)
    olist = np.asfortranarray(olist)
    V = O.gen_Vmatrix(olist, slist, site, invs, U, J)
    G = O.gen_Green0(eig, uni, mu, temp, Nw)
    return dict(rvec=rvec, H=H, slist=slist, invs=invs, klist=klist, kmap=kmap, invk=invk, hamk=hamk, eig=eig,
                uni=uni, olist=olist, site=site, V=V, G=G, Nx=Nx, Ny=Ny, Nw=Nw, temp=temp, mu=mu)


def test_rashba_model_keeps_the_time_reversal_the_reference_assumes():
    m = soc_setup(0.4)
    Nx, Ny = m["Nx"], m["Ny"]
    kk = np.array([[x / Nx, y / Ny, 0.0] for x in range(Nx) for y in range(Ny)])
    Hp, Hm = O.gen_ham(kk, m["H"], m["rvec"]), O.gen_ham(-kk, m["H"], m["rvec"])
    inv = m["invs"] - 1
    ss = np.outer(m["slist"], m["slist"])
    # numpy element [a,b] of the wrapper layout is the Fortran (b,a) = H_ba
    rhs = ss[None] * np.swapaxes(Hp[:, inv][:, :, inv], 1, 2)
    assert np.abs(Hm - rhs).max() < 1e-14


def test_vmat_soc_single_orbital_values():
    """fUJ.f90:130-175 for one orbital: (uu,dd) = U, (ud,ud) = -U, rest 0."""
    m = soc_setup(0.0, U=1.7)
    V = m["V"].T  # Fortran view V(j,i)
    ol = [tuple(r) for r in np.asarray(m["olist"])]
    idx = {p: i for i, p in enumerate(ol)}
    uu, dd, ud, du = idx[(1, 1)], idx[(2, 2)], idx[(1, 2)], idx[(2, 1)]
    assert V[uu, dd] == V[dd, uu] == 1.7
    assert V[ud, ud] == V[du, du] == -1.7
    assert V[uu, uu] == V[dd, dd] == 0.0
    assert np.abs(V).sum() == pytest.approx(4 * 1.7)


def test_vmat_soc_orbital_dependent_matches_uniform():
    olist, site = O.get_chi_orb_list(4)
    olist = np.asfortranarray(olist)
    _, _, slist, invs = M.spin_orbit_hoppings(*M.two_orbital_hoppings())
    U, J = 1.3, 0.2
    Umat = np.full((4, 4), U - 2 * J)
    Jmat = np.full((4, 4), J)
    for a in range(4):
        Umat[a, a] = U
    a = O.gen_Vmatrix(olist, slist, site, invs, U, J)
    b = O.gen_Vmatrix_orb(olist, slist, site, invs, Umat, Jmat)
    assert np.array_equal(a, b)
    assert np.array_equal(a, a.T)


def test_soc_bubble_reduces_to_the_non_soc_bubble():
    m = soc_setup(0.0)
    chi, sg, sg2, invschi = O.get_chi0_soc(m["V"], m["G"], m["olist"], m["slist"], m["kmap"], m["invk"], m["invs"],
                                          m["temp"], m["Nx"], m["Ny"], 1)
    h1 = O.gen_ham(m["klist"], m["H"][:, :1, :1], m["rvec"])
    e1, u1 = O.get_eig(h1)
    G1 = O.gen_Green0(e1, u1, m["mu"], m["temp"], m["Nw"])
    ol1 = np.asfortranarray(O.get_chi_orb_list(1)[0])
    c1 = O.get_chi0_conv(G1, m["kmap"], m["invk"], ol1, m["temp"], m["Nx"], m["Ny"], 1)
    ol = [tuple(r) for r in np.asarray(m["olist"])]
    idx = {p: i for i, p in enumerate(ol)}
    for a, b in (((1, 1), (1, 1)), ((2, 2), (2, 2)), ((1, 2), (1, 2)), ((2, 1), (2, 1))):
        assert np.abs(chi[idx[a], idx[b]] - c1[0, 0]).max() < 1e-15
    for a, b in (((1, 1), (2, 2)), ((1, 2), (2, 1)), ((1, 1), (1, 2))):
        assert np.abs(chi[idx[a], idx[b]]).max() == 0.0
    for p, i in idx.items():
        assert ol[invschi[i] - 1] == (3 - p[0], 3 - p[1])  # both spins flipped


def test_soc_bubble_exchange_partner_sign():
    """chi_(m2,l2) = sgnsig2 conj chi_(m,l) for every irreducible pair of a
    Rashba model (fchi0withsoc.f90:106)."""
    m = soc_setup(0.4)
    chi, sg, sg2, invschi = O.get_chi0_soc(m["V"], m["G"], m["olist"], m["slist"], m["kmap"], m["invk"], m["invs"],
                                          m["temp"], m["Nx"], m["Ny"], 1)
    cm, irr = SO.get_chi_map_soc(np.asarray(m["olist"]), m["invs"])
    X = chi.T
    for (l, mm) in irr:
        m2, l2 = cm[mm, l]
        assert np.array_equal(X[:, :, m2, l2], sg2.T[mm, l] * np.conj(X[:, :, mm, l]))


@pytest.mark.parametrize("gap_sym", [1, -1])
def test_soc_arnoldi_and_power_method_agree(gap_sym):
    """The leading eigenvalue from the two-pass Arnoldi and from the shifted
    power method.  The triplet operator of this Rashba model has a complex
    pair 0.596 +- 0.003i at the top, which a 30-vector Krylov space misses
    (it reports 0.570); 60 vectors resolve it."""
    m = soc_setup(0.3, U=2.2, temp=0.08)
    chi, sg, sg2, invschi = O.get_chi0_soc(m["V"], m["G"], m["olist"], m["slist"], m["kmap"], m["invk"], m["invs"],
                                          m["temp"], m["Nx"], m["Ny"], 1)
    init = O.get_initial_gap(m["klist"], 2, gap_sym)
    args = (m["G"], m["uni"], init, m["V"], sg, sg2, np.ones(2), m["slist"], m["olist"], m["kmap"], m["invk"],
            m["invs"], invschi, m["Nx"], m["Ny"], 1, m["temp"], gap_sym)
    _, lam_a, ra = O.linearized_eliashberg_soc(chi.copy(), *args, eps=1e-10, arnoldi_m=60, full=True)
    _, lam_p, rp = O.linearized_eliashberg_soc(chi.copy(), *args, eps=1e-9, itemax=3000, arnoldi_m=0, full=True)
    assert abs(lam_a - lam_p) < 1e-6 * max(1.0, abs(lam_a)), (lam_a, lam_p)


def test_library_vmat_soc_matches_oracle():
    """get_vmat_soc / get_vmat_soc_orb are host code in the library: no GPU needed."""
    from pyrpa_gb300 import build, flibs
    if not build.LIB.exists():
        build.build()
    flibs.load_library()
    olist, site = O.get_chi_orb_list(4)
    olist = np.asfortranarray(olist)
    _, _, slist, invs = M.spin_orbit_hoppings(*M.two_orbital_hoppings())
    a = flibs.gen_Vmatrix(olist, slist, site, invs, 1.3, 0.2)
    assert np.array_equal(a, O.gen_Vmatrix(olist, slist, site, invs, 1.3, 0.2))
    rng = np.random.default_rng(0)
    Um = rng.uniform(0.5, 1.5, (4, 4))
    Jm = rng.uniform(0.0, 0.3, (4, 4))
    b = flibs.gen_Vmatrix_orb(olist, slist, site, invs, Um, Jm)
    assert np.array_equal(b, O.gen_Vmatrix_orb(olist, slist, site, invs, Um, Jm))
