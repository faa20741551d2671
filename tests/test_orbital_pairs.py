"""Orbital-pair lists against the reference's own get_chi_orb_list (golden
vectors from tests/golden/make_orbital_pairs_golden.py), on CPU: one and
several sites, Fortran memory order at the library boundary, and the
refused profile."""
import ctypes
from pathlib import Path

import numpy as np
import pytest

from oracle import flex_oracle as FO
from pyrpa_gb300 import flibs as F

GOLD = np.load(Path(__file__).parent / "golden" / "orbital_pairs_golden.npz")
NCASES = len([k for k in GOLD.files if k.endswith("_olist")])


@pytest.mark.parametrize("c", range(NCASES))
def test_pairs_and_sites_match_reference(c):
    Norb, prof = int(GOLD[f"case{c}_norb"]), list(GOLD[f"case{c}_prof"])
    for ol, site in (F.get_chi_orb_list(Norb, prof), FO.get_chi_orb_list(Norb, prof)):
        assert np.array_equal(ol, GOLD[f"case{c}_olist"])
        assert np.array_equal(site, GOLD[f"case{c}_site"])
    ol, _ = F.get_chi_orb_list(Norb, prof)
    # what ctypes hands the library: the Fortran olist(Nchi,2), column by column
    raw = np.ctypeslib.as_array(ol.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), (ol.size,))
    assert np.array_equal(raw, np.concatenate([ol[:, 0], ol[:, 1]]))


def test_profile_that_does_not_add_up_is_refused():
    assert bool(GOLD["refuses_bad_profile"])
    with pytest.raises(SystemExit):
        F.get_chi_orb_list(6, [3, 2])
    with pytest.raises(SystemExit):
        FO.get_chi_orb_list(6, [3, 2])


@pytest.mark.parametrize("Norb,prof", [(4, [2, 2]), (5, [2, 1, 2]), (6, [3, 3])])
def test_kanamori_matrices_of_several_sites_match_oracle(Norb, prof):
    from pyrpa_gb300 import build
    if not build.LIB.exists():
        pytest.skip("libfmod.so is not built")
    from oracle import api as O
    F.load_library()
    ol, site = F.get_chi_orb_list(Norb, prof)
    for x, y in zip(F.gen_SCmatrix(ol, site, 1.3, 0.25), O.gen_SCmatrix(np.asarray(ol), site, 1.3, 0.25)):
        assert np.array_equal(x, y)
    S, C = F.gen_SCmatrix(ol, site, 1.3, 0.25)
    # no interaction between pairs of different sites
    same = site[:, None] == site[None, :]
    assert np.all(S[~same] == 0) and np.all(C[~same] == 0)
