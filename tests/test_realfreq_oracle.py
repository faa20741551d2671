"""CPU checks of the real-frequency / Pade oracle (oracle/realfreq_oracle.py).

The reference's test suite does not cover these routines; what pins the
restatement here: k+q lookups against integer mesh arithmetic, the Lindhard
sum of a one-orbital model written out term by term, the static q -> 0
limit, and the exactness of Pade continuation for rational data (the
continued fraction through 2n+1 points of an n-pole function is that function).
"""
import numpy as np
import pytest

from oracle import api as O
import _models as M


def full_mesh(Nx, Ny):
    return np.array([[x / Nx, y / Ny, 0.0] for x in range(Nx) for y in range(Ny)])


def test_qshift_is_the_mesh_translation():
    Nx, Ny = 8, 6
    kl = full_mesh(Nx, Ny)
    for qx, qy in ((0, 0), (1, 0), (3, 5), (7, 2)):
        qs = O.get_qshift(kl, np.array([qx / Nx, qy / Ny, 0.0]))
        iq = O.get_iqshift(kl, np.array([qx / Nx, qy / Ny, 0.0]))
        for i in range(Nx * Ny):
            x, y = divmod(i, Ny)
            assert qs[i] - 1 == ((x + qx) % Nx) * Ny + (y + qy) % Ny
            assert iq[i] - 1 == ((qx - x) % Nx) * Ny + (qy - y) % Ny


def one_band(Nx=8, Ny=8, mu=0.2, temp=0.05):
    rvec, ham_r = M.square_hoppings(1.0, 1.0, -0.25)
    kl = full_mesh(Nx, Ny)
    hamk = O.gen_ham(kl, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    f = O.get_ffermi(eig, mu, temp)
    return kl, eig, uni, f


def test_lindhard_one_band_term_by_term():
    kl, eig, uni, f = one_band()
    olist = np.asfortranarray(O.get_chi_orb_list(1)[0])
    q = np.array([3 / 8, 1 / 8, 0.0])
    qs = O.get_qshift(kl, q)
    w = np.array([0.3, -0.7, 1.5])
    chi = O.get_chi_irr(uni, eig, f, qs, olist, w, 0.05, 0.05)
    e, fk = eig[:, 0], f[:, 0]
    for n, ww in enumerate(w):
        df = fk[qs - 1] - fk
        # terms with |f(k+q) - f(k)| <= eps = 1e-3 idelta are skipped (fchi.f90:138-144)
        ref = np.mean(np.where(np.abs(df) > 0.05e-3, df / (ww + e - e[qs - 1] + 0.05j), 0.0))
        assert abs(chi[n, 0, 0] - ref) < 1e-14
        phi = O.get_phi_irr(uni, eig, f, O.get_iqshift(kl, q), olist, w, 0.05, 0.2, 0.05)
        iq = O.get_iqshift(kl, q) - 1
        refp = np.mean(-(1 - fk[iq] - fk) / (ww - e - e[iq] + 0.4 + 0.05j))
        assert abs(phi[n, 0, 0] - refp) < 1e-14


def test_static_bubble_uses_the_derivative_limit():
    """At w = 0 and q = 0 every term takes the f(1-f)/T branch."""
    kl, eig, uni, f = one_band()
    olist = np.asfortranarray(O.get_chi_orb_list(1)[0])
    qs = O.get_qshift(kl, np.zeros(3))
    chi = O.get_chi_irr(uni, eig, f, qs, olist, np.array([0.0]), 0.01, 0.05)
    assert abs(chi[0, 0, 0] - np.mean(f[:, 0] * (1 - f[:, 0]) / 0.05)) < 1e-14


def test_chis_qmap_one_band_rpa():
    kl, eig, uni, f = one_band(Nx=4, Ny=4)
    olist, site = O.get_chi_orb_list(1)
    olist = np.asfortranarray(olist)
    S, C = O.gen_SCmatrix(olist, site, 1.1, 0.0)
    trs, tr0 = O.chis_qmap(uni, eig, f, kl, S, olist, 4, 4, 0.05, 0.2, 0.02)
    assert np.allclose(trs, tr0 / (1 - 1.1 * tr0), rtol=1e-13)


def test_pade_is_exact_for_rational_data():
    rng = np.random.default_rng(1)
    poles = rng.uniform(-1, 1, 4) - 0.05j
    res = rng.uniform(0.1, 1.0, 4)
    f = lambda z: np.sum(res[None, :] / (z[:, None] - poles[None, :]), axis=1)
    iw = 1j * np.pi * 0.05 * (2 * np.arange(12) + 1)
    w = np.linspace(-1.5, 1.5, 31) + 0.01j
    a = O.get_a(f(iw), iw)
    Q, P = O.get_QP(a, iw, w)
    # exact in exact arithmetic; the recursion loses about 1e-8 next to a pole
    assert np.abs(P / Q - f(w)).max() < 1e-6 * np.abs(f(w)).max()


def test_pade_with_trace_reproduces_the_green_function():
    rvec, ham_r = M.two_orbital_hoppings()
    kl = full_mesh(4, 4)
    hamk = O.gen_ham(kl, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    temp, mu = 0.05, 0.1
    G = O.gen_Green0(eig, uni, mu, temp, 16)                 # [a, b, iw, k]
    iw = 1j * np.pi * temp * (2 * np.arange(16) + 1)
    w = np.linspace(-2, 2, 21) + 0.02j
    out = O.pade_with_trace(G, iw, w)                         # [k, w]
    exact = np.sum(1.0 / (w[None, :, None] + mu - eig[:, None, :]), axis=2)
    assert np.abs(out - exact).max() < 1e-8 * np.abs(exact).max()


@pytest.fixture(scope="module")
def lib():
    from pyrpa_gb300 import build, flibs
    if not build.LIB.exists():
        build.build()
    flibs.load_library()
    return flibs


def test_library_host_entries_match_oracle(lib):
    """get_qshift_/get_iqshift_, get_tr_chi/get_tr_phi, get_a_/get_qp_ are host
    code in the library."""
    F = lib
    rng = np.random.default_rng(7)
    kl = full_mesh(6, 5)
    for q in (np.zeros(3), np.array([2 / 6, 3 / 5, 0.0]), np.array([0.5, 0.1, 0.0])):  # the last misses the mesh
        assert np.array_equal(F.get_qshift(kl, q), O.get_qshift(kl, q))
        assert np.array_equal(F.get_iqshift(kl, q), O.get_iqshift(kl, q))
    olist = np.asfortranarray(O.get_chi_orb_list(4)[0])
    n = len(olist)
    chis = rng.standard_normal((5, n, n)) + 1j * rng.standard_normal((5, n, n))
    chi0 = rng.standard_normal((5, n, n)) + 1j * rng.standard_normal((5, n, n))
    for a, b in zip(F.get_tr_chi(chis, chi0, olist), O.get_tr_chi(chis, chi0, olist)):
        assert np.abs(a - b).max() < 1e-13
    for a, b in zip(F.get_tr_phi(chis, olist), O.get_tr_phi(chis, olist)):
        assert np.abs(a - b).max() < 1e-13
    iw = 1j * np.pi * 0.05 * (2 * np.arange(10) + 1)
    # more poles than half the points: the continued fraction does not
    # terminate (a terminated one continues with 0/0 noise after 2n+1 terms)
    poles = rng.uniform(-1, 1, 8)
    data = np.sum(rng.uniform(0.1, 1, 8)[None, :] / (iw[:, None] - poles[None, :]), axis=1)
    a1, a2 = F.get_a(data, iw), O.get_a(data, iw)
    # the recursion amplifies rounding: a 1e-15 relative change of the data
    # moves the last of these coefficients by 1e-7 relative
    assert (np.abs(a1 - a2) / np.abs(a2)).max() < 1e-5
    w = np.linspace(-1, 1, 9) + 0.01j
    for x, y in zip(F.get_QP(a2, iw, w), O.get_QP(a2, iw, w)):
        assert np.abs(x - y).max() < 1e-12 * np.abs(y).max()
