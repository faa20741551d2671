"""CPU tests of the C ABI surface of libfmod.so.

* every function declared in include/fmod.h and every symbol pyrpa's ctypes
  wrappers bind (libs/flibs/*.py, 71 names) is exported;
* the host-side setup routines (k-mesh reduction, Kanamori vertices, k
  weights, orbital parities) agree exactly with the oracle;
* no compute entry point is called here (no GPU in this environment).
"""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import api as O
from oracle import flex_oracle as FO
import _models as M

ROOT = Path(__file__).resolve().parents[1]

REFERENCE_SYMBOLS = """calc_kn calc_lij calc_lij_wl calc_sigma_hall calc_tau_epa calc_tdf chiq_map
conv_delta_orb_to_band conv_delta_orb_to_band_soc eliashberg gen_dos gen_green0_ gen_green_inv_
gen_green_inv_from_eig gen_ham gen_imp_ham gen_tr_greenw_0 generate_irr_kpoint_inv get_a_
get_band_to_orb_delta get_chi0 get_chi0_conv_ get_chi0_soc get_chi0_tail get_chi_irr get_chi_irr_sc
get_chis get_chis_chic get_chis_chic_soc get_dft_imp_ham get_eig get_eig_mlo get_eig_or_tr_chi
get_ffermi get_imass0 get_imassk get_initial_delta_ get_iqshift_ get_kweight get_parity_prop
get_phi_irr get_qp_ get_qshift_ get_scmat get_scmat_orb get_spectrum_spaghetti get_tau get_tr_chi
get_tr_phi get_veloc get_vlm0 get_vmat_soc get_vmat_soc_orb get_vnm get_vsigma_flex_nosoc_ getinv_
lin_eliash lin_eliash_soc matrix_riccati_batch matrix_riccati_chords mkbdghamk mkfk_trs_nsoc_
mkfk_trs_soc_ mkself mkself_soc openmp_params pade_with_trace phiq_map remap_delta_ riccati_chords
solve_cpa_array""".split()


@pytest.fixture(scope="module")
def lib():
    from pyrpa_gb300 import build, flibs
    path = build.LIB if build.LIB.exists() else build.build()
    return flibs.load_library(path)


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True).stdout
    return {l.split()[-1] for l in out.splitlines() if " T " in l}


def header_functions():
    text = (ROOT / "include" / "fmod.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\bvoid\s+(\w+)\s*\(", text))


def test_reference_symbol_set_is_exported(lib):
    from pyrpa_gb300 import build
    names = exported(build.LIB)
    assert len(REFERENCE_SYMBOLS) == 71
    missing = [s for s in REFERENCE_SYMBOLS if s not in names]
    assert not missing, missing


def test_header_declarations_are_exported(lib):
    from pyrpa_gb300 import build
    names = exported(build.LIB)
    decl = header_functions()
    assert len(decl) >= 30
    assert decl <= names, sorted(decl - names)
    for d in decl:
        assert hasattr(lib, d)


def header_arity():
    text = (ROOT / "include" / "fmod.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for name, params in re.findall(r"\bvoid\s+(\w+)\s*\(([^)]*)\)", text):
        params = params.strip()
        out[name] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_signatures_match_header_arity():
    """Every argtypes list the wrappers bind has as many entries as the
    declaration in include/fmod.h has parameters."""
    from pyrpa_gb300 import flibs
    arity = header_arity()
    checked = 0
    for name, types in flibs._SIGNATURES.items():
        if name in arity:
            assert len(types) == arity[name], (name, len(types), arity[name])
            checked += 1
    assert checked >= 25


def test_irreducible_k_mesh_matches_oracle(lib):
    from pyrpa_gb300 import flibs as F
    for dims in [(2, 2, 1), (4, 4, 1), (8, 6, 1), (5, 5, 1), (6, 5, 1), (4, 4, 4), (6, 6, 3), (3, 3, 3),
                 (24, 24, 24), (64, 64, 1)]:
        a = F.gen_irr_k_TRS(*dims)
        b = O.gen_irr_k_TRS(*dims)
        for x, y in zip(a, b):
            assert np.array_equal(x, y) if x.dtype.kind == "i" else np.allclose(x, y, rtol=0, atol=1e-15)
        w = F.gen_kpoint_weight(a[2], len(a[0]))
        assert np.array_equal(w, O.gen_kpoint_weight(b[2], len(b[0])))


def test_kanamori_vertices_match_oracle_and_reference_values(lib):
    from pyrpa_gb300 import flibs as F
    olist, site = F.get_chi_orb_list(2)
    S, C = F.gen_SCmatrix(olist, site, 1.0, 0.2)
    es = np.array([[1.0, 0, 0, 0.2], [0, 0.6, 0.2, 0], [0, 0.2, 0.6, 0], [0.2, 0, 0, 1.0]])
    ec = np.array([[1.0, 0, 0, 1.0], [0, -0.2, 0.2, 0], [0, 0.2, -0.2, 0], [1.0, 0, 0, 1.0]])
    assert np.allclose(S, es) and np.allclose(C, ec)
    S2, C2 = F.gen_SCmatrix_orb(olist, site, np.full((2, 2), 1.0), np.full((2, 2), 0.2))
    assert np.allclose(S2, [[1.0, 0, 0, 0.2], [0, 1.0, 0.2, 0], [0, 0.2, 1.0, 0], [0.2, 0, 0, 1.0]])
    assert np.allclose(C2, [[1.0, 0, 0, 1.8], [0, -0.6, 0.2, 0], [0, 0.2, -0.6, 0], [1.8, 0, 0, 1.0]])
    for Norb in (1, 3, 5):
        ol, st = F.get_chi_orb_list(Norb)
        rng = np.random.default_rng(Norb)
        Um = rng.uniform(0.5, 2.0, (Norb, Norb)); Um = Um + Um.T
        Jm = rng.uniform(0.0, 0.3, (Norb, Norb)); Jm = Jm + Jm.T
        for got, want in ((F.gen_SCmatrix(ol, st, 1.3, 0.21), O.gen_SCmatrix(np.asarray(ol), st, 1.3, 0.21)),
                          (F.gen_SCmatrix_orb(ol, st, Um, Jm), O.gen_SCmatrix_orb(np.asarray(ol), st, Um, Jm))):
            assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


def test_parity_list_matches_oracle(lib):
    from pyrpa_gb300 import flibs as F
    for Norb, seed in ((1, 0), (3, 1), (5, 2)):
        rvec, ham_r = M.random_hoppings(Norb, seed)
        assert np.array_equal(F.get_plist(rvec, ham_r), O.get_plist(rvec, ham_r))


def test_compute_entry_fails_loudly_without_gpu(lib):
    """A compute entry point either runs on a visible GPU or raises; it never
    falls back to a CPU computation."""
    from pyrpa_gb300 import flibs as F
    eig = np.zeros((2, 1))
    uni = np.ones((2, 1, 1), dtype=np.complex128)
    try:
        G = F.gen_Green0(eig, uni, 0.0, 0.1, 4)
    except RuntimeError as e:
        assert "no CUDA device" in str(e)
    else:
        assert np.isfinite(G).all()


def test_non_orthogonal_basis_runs_on_the_gpu(lib):
    """get_eig with an overlap (the reference's get_eig_mlo path,
    libs/flibs/_hamiltonian.py:176-179) binds the six-argument routine; without
    a GPU it fails loudly instead of falling back to the CPU."""
    from pyrpa_gb300 import flibs as F
    hamk = np.tile(np.eye(2, dtype=np.complex128), (3, 1, 1))
    try:
        eig, uni = F.get_eig(hamk, Ovlk=hamk)
    except RuntimeError as e:
        assert "CUDA device" in str(e)
    else:
        assert np.allclose(eig, 1.0)
