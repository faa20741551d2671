"""The drop-in claim checked with the reference's own binding code: pyrpa's
ctypes layer (libs/flibs of a pyrpa checkout) is imported with its loader
pointed at this engine's libfmod.so.  Every submodule sets argtypes on all
71 symbols at import, so a missing symbol fails the import.  The host-side
entry points (irreducible mesh, k weights, Kanamori matrices, parity list)
then run through the reference's wrappers and must give what this package's
mirror gives.  No GPU is needed; the test is skipped without a checkout
(PYRPA_REFERENCE names its root)."""
import ctypes
import importlib
import os
import sys
from pathlib import Path

import numpy as np
import pytest

import _models as M

REF = Path(os.environ.get("PYRPA_REFERENCE", "/root/reference"))


@pytest.fixture(scope="module")
def ref_flibs():
    if not (REF / "libs" / "flibs" / "_loader.py").exists():
        pytest.skip("no pyrpa checkout to bind")
    from pyrpa_gb300 import build
    if not build.LIB.exists():
        build.build()
    original = np.ctypeslib.load_library

    def load(name, path):
        # the reference's loader asks for libfmod.so next to libs/; hand it ours
        return ctypes.CDLL(str(build.LIB)) if name == "libfmod.so" else original(name, path)

    saved = {m: sys.modules.pop(m) for m in list(sys.modules) if m == "libs" or m.startswith("libs.")}
    np.ctypeslib.load_library = load
    sys.path.insert(0, str(REF))
    try:
        mod = importlib.import_module("libs.flibs")
    finally:
        np.ctypeslib.load_library = original
        sys.path.remove(str(REF))
    yield mod
    for m in [m for m in list(sys.modules) if m == "libs" or m.startswith("libs.")]:
        del sys.modules[m]
    sys.modules.update(saved)


def test_reference_wrappers_bind_every_symbol(ref_flibs):
    from pyrpa_gb300 import build
    lib = importlib.import_module("libs.flibs._loader")._lib
    assert Path(lib._name).resolve() == build.LIB.resolve()
    for name in ("mkself", "lin_eliash", "get_chi0", "get_chi0_tail", "get_vsigma_flex_nosoc_", "get_chis_chic",
                 "gen_green0_", "mkfk_trs_nsoc_", "remap_delta_", "conv_delta_orb_to_band"):
        assert getattr(lib, name).argtypes, name  # argtypes were set by the reference's submodules


def test_reference_wrappers_compute_host_entry_points(ref_flibs):
    from pyrpa_gb300 import flibs as F
    for dims in [(4, 4, 1), (8, 6, 1), (5, 5, 1), (4, 4, 4), (6, 6, 3)]:
        for x, y in zip(ref_flibs.gen_irr_k_TRS(*dims), F.gen_irr_k_TRS(*dims)):
            assert np.array_equal(x, y)
        klist, kmap, invk = F.gen_irr_k_TRS(*dims)
        assert np.array_equal(ref_flibs.gen_kpoint_weight(invk, len(klist)), F.gen_kpoint_weight(invk, len(klist)))
    for Norb in (1, 3, 5):
        olist, site = F.get_chi_orb_list(Norb)
        for x, y in zip(ref_flibs.gen_SCmatrix(olist, site, 1.1, 0.2), F.gen_SCmatrix(olist, site, 1.1, 0.2)):
            assert np.array_equal(x, y)
        rvec, ham_r = M.random_hoppings(Norb, Norb)
        assert np.array_equal(ref_flibs.get_plist(rvec, ham_r), F.get_plist(rvec, ham_r))


def test_reference_soc_wrappers_against_the_library(ref_flibs):
    """The reference's spin-orbit wrappers bind to this library; the host-side
    vertex matches this package's mirror.  lin_eliash_soc's argtypes in the
    reference list 27 entries for the 28 Fortran arguments (prt is missing),
    which the C ABI follows (28); its own call therefore fails in ctypes."""
    from pyrpa_gb300 import flibs as F
    lib = importlib.import_module("libs.flibs._loader")._lib
    olist, site = F.get_chi_orb_list(4)
    _, _, slist, invs = M.spin_orbit_hoppings(*M.two_orbital_hoppings())
    a = ref_flibs.gen_Vmatrix(olist, slist, site, invs, 1.3, 0.2)
    assert np.array_equal(a, F.gen_Vmatrix(olist, slist, site, invs, 1.3, 0.2))
    assert len(lib.lin_eliash_soc.argtypes) == 27
    for name in ("mkself_soc", "get_chi0_soc", "get_chis_chic_soc", "mkfk_trs_soc_", "conv_delta_orb_to_band_soc"):
        assert len(getattr(lib, name).argtypes) == len(F._SIGNATURES[name]), name


@pytest.mark.parametrize("Norb,prof", [(1, [1]), (3, [1]), (5, [1]), (4, [2, 2]), (5, [2, 1, 2])])
def test_chi_map_matches_reference_port(ref_flibs, Norb, prof):
    """The exchange-symmetry index map that get_chi0_conv_ takes, against the
    reference's own Python port of fchi.f90 get_chi_map
    (libs/flibs/_susceptibility.py:206-242)."""
    from oracle import flex_oracle as FO
    from pyrpa_gb300 import flibs as F
    ref_port = importlib.import_module("libs.flibs._susceptibility")._get_chi_map
    olist, _ = F.get_chi_orb_list(Norb, prof)
    cmap_ref, irr_ref = ref_port(np.asarray(olist))
    cmap, irr = F.chi_map_arrays(olist)
    assert np.array_equal(cmap, cmap_ref) and np.array_equal(irr, irr_ref)
    # the oracle's 0-based form: chi_map[m1, l1] = (m2, l2), irr = [(l1, m1)]
    omap, oirr = FO.get_chi_map(np.asarray(olist))
    n = len(olist)
    for l1 in range(n):
        for m1 in range(n):
            assert tuple(omap[m1, l1]) == (cmap_ref[0, l1, m1] - 1, cmap_ref[1, l1, m1] - 1)
    assert [(l + 1, m + 1) for (l, m) in oirr] == list(zip(irr_ref[0][:len(oirr)], irr_ref[1][:len(oirr)]))
