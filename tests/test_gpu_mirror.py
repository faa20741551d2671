"""The Python mirror's optional arguments that call GPU entry points:
gen_ham with overlap blocks returns (hamk, Ovlk) like the reference
(libs/flibs/_hamiltonian.py:134-157), and get_eig(sw=False) returns the
eigenvalues alone (:181-185)."""

import numpy as np
import pytest

import _models as M

pytestmark = pytest.mark.gpu


def test_gen_ham_overlap_and_eigenvalues_only():
    from pyrpa_gb300 import build, flibs as F
    if not build.LIB.exists():
        build.build()
    F.load_library()
    rvec, ham_r = M.random_hoppings(2, 3)
    klist, _, _ = F.gen_irr_k_TRS(4, 4, 1)
    ovl = np.zeros_like(ham_r)
    ovl[np.all(rvec == 0, axis=1)] = np.eye(2)
    hamk, ovlk = F.gen_ham(klist, ham_r, rvec, Ovl_r=ovl)
    assert np.array_equal(hamk, F.gen_ham(klist, ham_r, rvec))
    assert np.allclose(ovlk, np.eye(2)[None])
    eig, uni = F.get_eig(hamk)
    assert np.array_equal(F.get_eig(hamk, sw=False), eig)


def test_green_from_eigenpairs_matches_oracle():
    """gen_green_from_eig (fself.f90:85-129, then getinv_) equals G from H(k)
    and Sigma: U (iw + mu - E) U^dagger - Sigma is (iw + mu) - H - Sigma."""
    from oracle import api as O
    from pyrpa_gb300 import build, flibs as F
    if not build.LIB.exists():
        build.build()
    F.load_library()
    F.set_precision(64)
    rvec, ham_r = M.random_hoppings(3, 7, bandwidth=4.0)
    klist, _, _ = O.gen_irr_k_TRS(6, 6, 1)
    hamk = O.gen_ham(klist, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    rng = np.random.default_rng(3)
    Nw, mu, temp = 16, 0.1, 0.05
    sig = 0.1 * (rng.normal(size=(3, 3, Nw, len(klist))) + 1j * rng.normal(size=(3, 3, Nw, len(klist))))
    got = F.gen_green_from_eig(sig, eig, uni, mu, temp)
    ref = O.gen_green(sig, hamk, mu, temp)
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max() + 2e-9


def test_green_inverse_from_eigenpairs_with_non_unitary_vectors():
    """gen_green_inv_from_eig takes the eigenvectors as given: with a U that is
    not unitary the i w + mu term carries U U^dagger, as in fself.f90:85-129,
    not the identity."""
    from oracle import api as O
    from pyrpa_gb300 import build, flibs as F
    if not build.LIB.exists():
        build.build()
    F.load_library()
    rng = np.random.default_rng(5)
    rvec, ham_r = M.random_hoppings(3, 2, bandwidth=4.0)
    klist, _, _ = O.gen_irr_k_TRS(4, 4, 1)
    eig, uni = O.get_eig(O.gen_ham(klist, ham_r, rvec))
    uni = uni + 0.05 * (rng.normal(size=uni.shape) + 1j * rng.normal(size=uni.shape))
    Nw, mu, temp = 8, -0.2, 0.1
    sig = 0.1 * (rng.normal(size=(3, 3, Nw, len(klist))) + 1j * rng.normal(size=(3, 3, Nw, len(klist))))
    got = np.zeros_like(sig)
    F._call("gen_green_inv_from_eig", got, sig, np.ascontiguousarray(uni), np.ascontiguousarray(eig), F.dbl(mu),
            F.dbl(temp), F.i64(len(klist)), F.i64(Nw), F.i64(3))
    ref = O.gen_green_inv_from_eig(sig, eig, uni, mu, temp)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def _overlap_model(seed, singular):
    """Three orbitals with an overlap S(k) = 1 + overlap hoppings (Hermitian,
    positive definite), or with the first two basis functions identical
    (an exactly singular S, whose null direction get_eig_mlo drops)."""
    rng = np.random.default_rng(seed)
    from oracle import api as O
    rvec, ham_r = M.random_hoppings(3, seed, bandwidth=4.0)
    klist, _, _ = O.gen_irr_k_TRS(6, 6, 1)
    hamk = O.gen_ham(klist, ham_r, rvec)
    if singular:
        # basis functions 1 and 2 are the same function: S = P P^T, H -> P H P^T
        P = np.array([[1.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
        Sk = np.tile((P @ P.T).astype(np.complex128), (len(klist), 1, 1))
        hamk = np.einsum("ij,kjl,ml->kim", P, hamk, P).astype(np.complex128)
    else:
        A = 0.1 * (rng.normal(size=hamk.shape) + 1j * rng.normal(size=hamk.shape))
        Sk = np.eye(3)[None] + 0.5 * (A + np.conj(np.swapaxes(A, 1, 2)))
    return klist, np.ascontiguousarray(hamk), np.ascontiguousarray(Sk)


@pytest.mark.parametrize("singular", [False, True])
def test_get_eig_mlo_matches_oracle(singular):
    """get_eig_mlo (fmod.f90:250-310) against the oracle's canonical
    orthogonalization: eigenvalues to 1e-12, and the Green function
    sum_n U_mn conj(U_ln) / (i w - e_n), which does not depend on the
    eigenvector phases, to 1e-11.  With an exactly singular overlap the
    dropped direction shows as an eigenvalue 0 with a zero eigenvector."""
    from oracle import api as O
    from pyrpa_gb300 import build, flibs as F
    if not build.LIB.exists():
        build.build()
    F.load_library()
    klist, hamk, Sk = _overlap_model(3, singular)
    eig, uni = F.get_eig(hamk, Ovlk=Sk)
    eo, uo = O.get_eig_mlo(hamk, Sk)
    assert np.abs(eig - eo).max() <= 1e-12 * np.abs(eo).max()
    if singular:
        assert np.all(np.abs(eig).min(axis=1) < 1e-12)
    Gg = F.gen_Green0(eig, uni, 0.1, 0.05, 8)
    Go = O.gen_Green0(eo, uo, 0.1, 0.05, 8)
    assert np.abs(Gg - Go).max() <= 1e-11 * np.abs(Go).max()
