"""GPU parity on a model of two sites (4 orbitals as [2, 2], Nchi = 8 pairs
within the sites): chi0 and three FLEX iterations through the C ABI against
the FP64 oracle, at the FP64 tolerances of the other parity tests.
"""

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
    flibs.set_precision(64)
    return flibs


def _close(a, b, rtol=1e-9, atol=2e-9):
    scale = max(np.abs(b).max(), 1e-300)
    err = np.abs(a - b).max()
    assert err <= rtol * scale + atol, f"max |diff| {err:.3e} vs scale {scale:.3e}"


@pytest.mark.parametrize("prof", [[2, 2], [1, 3]])
def test_two_site_chi0_and_flex_match_oracle(F, prof):
    Nx, Ny, Nw, temp, mu = 6, 6, 8, 0.1, 0.0
    rvec, ham_r = M.random_hoppings(4, 21, bandwidth=4.0)
    klist, kmap, invk = O.gen_irr_k_TRS(Nx, Ny, 1)
    hamk = O.gen_ham(klist, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    Gk = O.gen_Green0(eig, uni, mu, temp, Nw)
    olist, site = F.get_chi_orb_list(4, prof)
    S, C = F.gen_SCmatrix(olist, site, 0.8, 0.1)
    chi, st = F.get_chi0(S, C, Gk, olist, kmap, invk, temp, Nx, Ny, 1)
    chio, sto = O.get_chi0(S, C, Gk, np.asarray(olist), kmap, invk, temp, Nx, Ny, 1)
    _close(chi, chio)
    assert abs(st - sto) <= 1e-9 * max(1.0, abs(sto))
    sig, mu1 = F.mkself(S, C, kmap, invk, olist, hamk, eig, uni, mu, 2.0, temp, Nw, Nx, Ny, 1, False, False,
                        scf_loop=3, eps=1e-12, pp=0.5)
    sigo, muo = O.mkself(S, C, kmap, invk, np.asarray(olist), hamk, eig, uni, mu, 2.0, temp, Nw, Nx, Ny, 1,
                         scf_loop=3, eps=1e-12, pp=0.5)
    _close(sig, sigo)
    assert abs(mu1 - muo) <= 1e-9
