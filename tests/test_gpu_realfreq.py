"""GPU parity of the real-frequency maps and the Pade trace (fchi.f90:95-318,
fphi.f90:89-305, fpade.f90:77-129) against the oracle, through the C ABI."""
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
    return flibs


def close(a, b, rtol, atol=1e-300):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    scale = max(np.abs(b).max(), 1e-300)
    err = np.abs(a - b).max()
    assert err <= rtol * scale + atol, f"max |diff| {err:.3e} vs scale {scale:.3e}"


def band_model(Norb, Nx, Ny, mu=0.1, temp=0.05, seed=0):
    if Norb == 1:
        rvec, ham_r = M.square_hoppings(1.0, 1.0, -0.25)
    elif Norb == 2:
        rvec, ham_r = M.two_orbital_hoppings()
    else:
        rvec, ham_r = M.random_hoppings(Norb, seed, complex_hop=True, bandwidth=4.0)
    kl = np.array([[x / Nx, y / Ny, 0.0] for x in range(Nx) for y in range(Ny)])
    hamk = O.gen_ham(kl, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    f = O.get_ffermi(eig, mu, temp)
    olist, site = O.get_chi_orb_list(Norb)
    return dict(kl=kl, eig=eig, uni=uni, f=f, olist=np.asfortranarray(olist), site=site, mu=mu, temp=temp,
                Nx=Nx, Ny=Ny, Norb=Norb)


@pytest.mark.parametrize("Norb", [1, 2, 3])
def test_chi_and_phi_irr(F, Norb):
    m = band_model(Norb, 8, 6)
    q = np.array([3 / 8, 2 / 6, 0.0])
    w = np.array([0.0, 0.25, -0.6, 1.3])
    qs = O.get_qshift(m["kl"], q)
    a = F.get_chi_irr(m["uni"], m["eig"], m["f"], qs, m["olist"], w, 0.02, m["temp"])
    b = O.get_chi_irr(m["uni"], m["eig"], m["f"], qs, m["olist"], w, 0.02, m["temp"])
    close(a, b, 1e-11, 1e-14)
    qq = np.zeros(3)  # q = 0, w = 0: the derivative branch
    a = F.get_chi_irr(m["uni"], m["eig"], m["f"], O.get_qshift(m["kl"], qq), m["olist"], w[:1], 0.02, m["temp"])
    b = O.get_chi_irr(m["uni"], m["eig"], m["f"], O.get_qshift(m["kl"], qq), m["olist"], w[:1], 0.02, m["temp"])
    close(a, b, 1e-11, 1e-14)
    iq = O.get_iqshift(m["kl"], q)
    a = F.get_phi_irr(m["uni"], m["eig"], m["f"], iq, m["olist"], w, 0.02, m["mu"], m["temp"])
    b = O.get_phi_irr(m["uni"], m["eig"], m["f"], iq, m["olist"], w, 0.02, m["mu"], m["temp"])
    close(a, b, 1e-11, 1e-14)


@pytest.mark.parametrize("Norb", [1, 2, 3])
def test_chis_qmap(F, Norb):
    m = band_model(Norb, 6, 6)
    S, C = O.gen_SCmatrix(m["olist"], m["site"], 0.8, 0.1)
    a = F.chis_qmap(m["uni"], m["eig"], m["f"], m["kl"], S, m["olist"], 4, 3, m["temp"], 0.2, 0.02)
    b = O.chis_qmap(m["uni"], m["eig"], m["f"], m["kl"], S, m["olist"], 4, 3, m["temp"], 0.2, 0.02)
    for x, y in zip(a, b):
        close(x, y, 1e-10, 1e-14)


@pytest.mark.parametrize("sw_omega", [True, False])
def test_phi_qmap(F, sw_omega):
    m = band_model(2, 6, 6)
    a = F.phi_qmap(m["uni"], m["eig"], m["f"], m["kl"], m["olist"], 3, 4, m["mu"], m["temp"], 0.2, 0.02, sw_omega)
    b = O.phi_qmap(m["uni"], m["eig"], m["f"], m["kl"], m["olist"], 3, 4, m["mu"], m["temp"], 0.2, 0.02, sw_omega)
    close(a, b, 1e-10, 1e-14)


def test_pade_with_trace(F):
    """Four-pole data on six Matsubara points (the continued fraction does not
    terminate).  The oracle's own spread under a 1e-15 relative perturbation of
    this data is 3e-11; the tolerance is 100x that."""
    rng = np.random.default_rng(5)
    Nk, No, Niw = 7, 2, 6
    iw = 1j * np.pi * 0.05 * (2 * np.arange(Niw) + 1)
    A = np.zeros((No, No, Niw, Nk), dtype=np.complex128)
    for k in range(Nk):
        for o in range(No):
            p = rng.uniform(-1, 1, 4)
            r = rng.uniform(0.1, 1, 4)
            A[o, o, :, k] = np.sum(r[None, :] / (iw[:, None] - p[None, :]), axis=1)
    w = np.linspace(-1.5, 1.5, 25) + 0.05j
    a = F.pade_with_trace(A, iw, w)
    b = O.pade_with_trace(A, iw, w)
    close(a, b, 3e-9)
