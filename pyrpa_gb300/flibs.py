"""Python host side of the GB300 FLEX/RPA engine.

The functions mirror the pyrpa ctypes wrappers of the hot path
(``libs/flibs/_hamiltonian.py``, ``_green.py``, ``_interaction.py``,
``_susceptibility.py``, ``_selfenergy.py``, ``_eliashberg.py``): same names,
argument order, array shapes and return values.  They bind the in-tree
``libfmod.so`` built from ``csrc/`` (``pyrpa_gb300.build``).  There is no CPU
implementation behind them: if the library is missing or no GPU is visible,
the call raises.

Where the reference library stops the process on a LAPACK failure, these
functions raise ``RuntimeError`` with the library's message.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, byref, c_bool, c_char, c_double, c_int64
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libfmod.so"

_c128 = np.ctypeslib.ndpointer(dtype=np.complex128)
_f64 = np.ctypeslib.ndpointer(dtype=np.float64)
_i64 = np.ctypeslib.ndpointer(dtype=np.int64)
_i32 = np.ctypeslib.ndpointer(dtype=np.int32)
_f32 = np.ctypeslib.ndpointer(dtype=np.float32)
_vp = ctypes.c_void_p
_pi = POINTER(c_int64)
_pd = POINTER(c_double)
_pb = POINTER(c_bool)

# argument types of every bound symbol, in the order of the reference wrappers
_SIGNATURES = {
    "openmp_params": [_pi, _pb],
    "generate_irr_kpoint_inv": [_f64, _i64, _i64, _pi, _pi, _pi, _pi],
    "get_kweight": [_f64, _i64, _pi, _pi],
    "gen_ham": [_c128, _f64, _c128, _f64, _pi, _pi, _pi],
    "get_eig": [_f64, _c128, _c128, _pi, _pi],
    "get_eig_mlo": [_f64, _c128, _c128, _c128, _pi, _pi],
    "get_ffermi": [_f64, _f64, _pd, _pd, _pi, _pi],
    "get_parity_prop": [_f64, _f64, _c128, _pi, _pi],
    "get_scmat": [_f64, _f64, _i64, _i64, _pd, _pd, _pi],
    "get_scmat_orb": [_f64, _f64, _i64, _i64, _f64, _f64, _pi, _pi],
    "gen_green0_": [_c128, _f64, _c128, _pd, _pd, _pi, _pi, _pi],
    "gen_green_inv_": [_c128, _c128, _c128, _pd, _pd, _pi, _pi, _pi],
    "getinv_": [_c128, _pi, _pi, _pi],
    "get_chi0_conv_": [_c128, _c128, _i64, _i64, _i32, _i32, _i64, _pd] + [_pi] * 8,
    "get_chi0": [_c128, _f64, _f64, _c128, _i64, _i64, _i64, _pd] + [_pi] * 8 + [_pd],
    "get_chi0_tail": [_c128, _f64, _f64, _c128, _f64, _c128, _i64, _i64, _i64, _pd, _pd] + [_pi] * 8 + [_pd],
    "get_chis": [_c128, _c128, _f64, _pi, _pi],
    "get_chis_chic": [_c128, _c128, _c128, _f64, _f64, _pi, _pi, _pi],
    "get_eig_or_tr_chi": [_c128, _c128, _i64, _pi, _pi, _pi, _pb],
    "get_vsigma_flex_nosoc_": [_c128, _f64, _f64, _pi, _pi, _pi],
    "mkself": [_c128, _pd, _f64, _f64, _i64, _i64, _i64, _c128, _f64, _c128, _pd, _pd, _pd, _pi, _pd, _pd]
    + [_pi] * 9 + [_pb, _pb, _pi, _pb, _pb, _pd],
    "lin_eliash": [_c128, _c128, _c128, _c128, _f64, _f64, _f64, _i64, _f64, _i64, _i64, _pd, _pd]
    + [_pi] * 11 + [_pd],
    "eliashberg": [_c128, _c128, _c128, _c128, _f64, _f64, _i64, _f64, _i64, _i64, _pd, _pd, _pd]
    + [_pi] * 10 + [_pb, _pb, _pi, _pd, _pb],
    "pyrpa_gb_chi0sc": [_c128, _c128, _c128, _c128, _f64, _f64, _i64, _f64, _i64, _i64, _pd] + [_pi] * 10,
    "pyrpa_gb_sc_dyson": [_c128, _c128, _c128, _c128, _pi, _pi, _pi],
    "mkfk_trs_nsoc_": [_c128, _c128, _c128, _pi, _pi, _pi],
    "get_vmat_soc": [_f64, _i64, _i64, _i64, _i64, _pd, _pd, _pi, _pi],
    "get_qshift_": [_f64, _f64, _i64, _pi],
    "get_iqshift_": [_f64, _f64, _i64, _pi],
    "get_chi_irr": [_c128, _c128, _f64, _f64, _i64, _i64, _f64, _pi, _pi, _pi, _pi, _pd, _pd, _pd],
    "get_phi_irr": [_c128, _c128, _f64, _f64, _i64, _i64, _f64, _pi, _pi, _pi, _pi, _pd, _pd, _pd, _pd],
    "chiq_map": [_c128, _c128, _c128, _f64, _f64, _f64, _f64, _i64, _pd, _pd, _pd, _pd] + [_pi] * 5,
    "phiq_map": [_c128, _c128, _f64, _f64, _f64, _i64, _pd, _pd, _pd, _pd, _pd] + [_pi] * 5 + [_pb],
    "get_tr_chi": [_c128, _c128, _c128, _c128, _c128, _i64, _pi, _pi, _pi],
    "get_tr_phi": [_c128, _c128, _c128, _i64, _pi, _pi, _pi],
    "get_a_": [_c128, _c128, _c128, _pi],
    "get_qp_": [_c128, _c128, _c128, _c128, _c128, _pi, _pi],
    "pade_with_trace": [_c128, _c128, _c128, _c128, _pi, _pi, _pi, _pi],
    "get_vmat_soc_orb": [_f64, _i64, _i64, _i64, _i64, _f64, _f64, _pi, _pi],
    "mkself_soc": [_c128, _pd, _f64, _i64, _i64, _i64, _i64, _i64, _c128, _f64, _c128, _pd, _pd, _pd, _pi, _pd, _pd]
    + [_pi] * 9 + [_pb, _pb, _pi, _pb, _pd],
    "get_chi0_soc": [_c128, _f64, _f64, _i64, _f64, _c128, _i64, _i64, _i64, _i64, _i64, _pd] + [_pi] * 8,
    "get_chis_chic_soc": [_c128, _c128, _c128, _c128, _f64, _i64, _i64, _i64, _i64] + [_pi] * 4,
    "lin_eliash_soc": [_c128, _c128, _c128, _c128, _f64, _f64, _f64, _f64, _f64, _i64, _i64, _i64, _i64, _i64,
                       _i64, _pd, _pd] + [_pi] * 11,
    "mkfk_trs_soc_": [_c128, _c128, _c128, _f64, _i64, _i64, _i64] + [_pi] * 5,
    "conv_delta_orb_to_band_soc": [_c128, _c128, _c128, _i64, _i64, _i64] + [_pi] * 4,
    "get_initial_delta_": [_c128, _f64, _c128, _i64, _i64, _pi, _pi, _pi, _pi, _pi],
    "remap_delta_": [_c128, _c128, _f64, _i64, _pi, _pi, _pi, _pi, _pi],
    "conv_delta_orb_to_band": [_c128, _c128, _c128, _f64, _i64, _pi, _pi, _pi, _pi, _pi],
    "pyrpa_gb_flex_eliash": [_c128, _pd, _c128, _pd, _pd, _f64, _f64, _f64, _i64, _i64, _i64, _c128, _f64, _c128,
                             _f64, _f64, ctypes.c_void_p, _pd, _pd, _pd, _pd, _pd, _pi, _pd, _pd] + [_pi] * 10
    + [_pb, _pb, _pi, _pi, _pi, _pd, _i64],
    "pyrpa_gb_regrid_sigma": [_c128, _c128, _pi, _pi, _pi, _pi, _pd, _pd, _pd],
    "pyrpa_gb_regrid_sigma_file": [ctypes.c_char_p, ctypes.c_char_p, _pd, _pd, _pi, _pi, _pi, _pd, _pi, _pi],
    "pyrpa_gb_wannier_r": [_c128, _c128, _i64, _i64, _pi, _pi, _pi, _pi, _pi, _pi, _pi],
    "pyrpa_gb_fft_candidates": [_pi, _pi, _i64, _pi, _pi],
    "gen_green_inv_from_eig": [_c128, _c128, _c128, _f64, _pd, _pd, _pi, _pi, _pi],
    "pyrpa_gb_sigma_interp": [_c128, _c128, _i64, _i64, _pi, _pi, _pi, _pi, _pi, _i64, _i64, _pi, _pi, _pi, _pi, _pi,
                              _pi, _pd],
    "pyrpa_gb_lws_create": [_pi],
    "pyrpa_gb_lws_destroy": [_pi],
    "pyrpa_gb_lws_set_params": [_pi, _f32, _pi],
    "pyrpa_gb_lws_get_params": [_pi, _f32, _pi],
    "pyrpa_gb_lws_add_samples": [_pi, _c128, _c128, _c128, _f64, _i64, _pi, _pi, _pi, _pi, _pi, _f64],
    "pyrpa_gb_lws_clear_samples": [_pi],
    "pyrpa_gb_lws_num_samples": [_pi, _pi],
    "pyrpa_gb_lws_features": [_f32, _vp, _c128, _vp, _c128, _f64, _i64, _pi, _pi, _pi, _pi, _pi, _f64],
    "pyrpa_gb_lws_forward": [_pi, _f32, _pi, _f32],
    "pyrpa_gb_lws_loss_grad": [_pi, _pd, _f32],
    "pyrpa_gb_lws_step": [_pi, _pd, _pd, _pd, _pd, _pd],
    "pyrpa_gb_lws_train": [_pi, _pi, _pi, _pd, _pd, _pd, _pd, _pi, _f64],
    "pyrpa_gb_lws_apply": [_pi, _c128, _c128, _f64, _pi, _pi, _pi, _pi, _f64],
    "pyrpa_gb_set_precision": [_pi],
    "pyrpa_gb_last_ritz": [_f64, _pi, _pi],
    "pyrpa_gb_get_precision": [_pi],
    "pyrpa_gb_set_verbose": [_pi],
    "pyrpa_gb_set_arnoldi_tol": [_pd],
    "pyrpa_gb_set_thread_stream": [_pi],
    "pyrpa_gb_last_error": [POINTER(c_char), _pi, _pi],
    "pyrpa_gb_clear_error": [],
    "pyrpa_gb_kernel_launches": [_pi],
    "pyrpa_gb_last_stats": [_f64],
    "pyrpa_gb_device_info": [_pi, _pi],
    "pyrpa_gb_fft_profile": [_pi],
    "pyrpa_gb_fft_stats": [_f64],
}

_lib = None


def load_library(path: str | Path | None = None):
    """Load libfmod.so (once) and set the argument types of its symbols."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with `python -m pyrpa_gb300.build` "
                          "(needs nvcc); there is no CPU implementation of this path")
    lib = ctypes.CDLL(str(p))
    for name, args in _SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = None
    _lib = lib
    return lib


def i64(v):
    return byref(c_int64(int(v)))


def _real_gap(init_delta):
    """The band-basis initial gap as float64.  The Fortran dummy is real
    (feliash.f90:38, 653) and the reference binds it as a float64 ndpointer,
    which rejects a complex array (the p+ip gap of get_initial_gap)."""
    a = np.asarray(init_delta)
    if np.iscomplexobj(a):
        raise TypeError("init_delta must be real (float64): the library takes a real band-basis gap")
    return np.ascontiguousarray(a, dtype=np.float64)


def dbl(v):
    return byref(c_double(float(v)))


def last_error() -> str:
    """Message of the last failure recorded by the library ('' if none)."""
    lib = load_library()
    code = c_int64(0)
    buf = ctypes.create_string_buffer(2048)
    lib.pyrpa_gb_last_error(buf, i64(len(buf)), byref(code))
    return buf.value.decode(errors="replace") if code.value else ""


def _call(name, *args):
    """Calls one entry point; a recorded failure becomes ValueError when the
    library flags the input (error code 2), RuntimeError otherwise."""
    lib = load_library()
    lib.pyrpa_gb_clear_error()
    getattr(lib, name)(*args)
    code = c_int64(0)
    buf = ctypes.create_string_buffer(2048)
    lib.pyrpa_gb_last_error(buf, i64(len(buf)), byref(code))
    if code.value:
        raise (ValueError if code.value == 2 else RuntimeError)(buf.value.decode(errors="replace"))


# ------------------------------------------------------------------ control
MIXED = 3264


def set_precision(bits: int) -> None:
    """64: FP64 everywhere (the reference's arithmetic); 48: double-float chi0
    and Sigma convolutions, FP64 elsewhere; 32: complex FP32 FFTs,
    contractions and vertex solves, FP64 for G, Sigma, mu, DIIS and lambda;
    3264 (MIXED): the FLEX loop runs FP32 bulk to the FP32 rounding floor,
    then double-float chi0 and Sigma with an FP32 vertex, then double-float
    judging iterations; the fused solve's Eliashberg stage is double-float.
    Other entry points run as in 32."""
    load_library().pyrpa_gb_set_precision(i64(bits))


def get_precision() -> int:
    v = c_int64(0)
    load_library().pyrpa_gb_get_precision(byref(v))
    return v.value


def set_verbose(level: int) -> None:
    load_library().pyrpa_gb_set_verbose(i64(level))


def kernel_launches() -> int:
    v = c_int64(0)
    load_library().pyrpa_gb_kernel_launches(byref(v))
    return v.value


def last_stats() -> dict:
    out = np.zeros(20)
    load_library().pyrpa_gb_last_stats(out)
    keys = ["iterations", "esterr", "stoner", "mu", "lambda", "applies", "t_chi0_ms", "t_vertex_ms",
            "t_sigma_ms", "t_diis_ms", "t_mu_ms", "t_dyson_ms", "t_apply_ms", "iterations_fp32",
            "iterations_coarse", "t_warm_ms", "t_stoner_ms", "iterations_fp64_fp32vertex", "ritz_residual",
            "arnoldi_cycles"]
    return dict(zip(keys, out[: len(keys)].tolist()))


def last_ritz(n: int = 4):
    """Largest real parts of the last Arnoldi pass's Ritz values (the first is
    lambda); fewer than n when the Krylov space was smaller."""
    out = np.zeros(max(1, n))
    count = c_int64(0)
    load_library().pyrpa_gb_last_ritz(out, i64(n), byref(count))
    return out[: min(n, count.value)].copy()


def set_arnoldi_tol(tol: float) -> None:
    """0: lin_eliash runs the reference's fixed arnoldi_m steps per pass; tol > 0
    restarts the pass that gives lambda until the Ritz residual over |lambda|
    is below tol (last_stats()["ritz_residual"], ["arnoldi_cycles"])."""
    _call("pyrpa_gb_set_arnoldi_tol", dbl(tol))


def set_thread_stream(on: bool) -> None:
    """Gives the calling thread its own engine context (CUDA stream, error
    flags, last error and statistics; settings copied from the process
    context) so that solves from several threads overlap on the GPU; False
    hands it back."""
    _call("pyrpa_gb_set_thread_stream", i64(1 if on else 0))


def fft_profile(on: bool) -> None:
    """Bracket every FFT pass launch with CUDA events (see fft_stats)."""
    load_library().pyrpa_gb_fft_profile(i64(1 if on else 0))


def fft_stats() -> dict:
    """Launches, summed device milliseconds and algorithmic bytes of the FFT
    passes since the last call (requires fft_profile(True))."""
    out = np.zeros(3)
    load_library().pyrpa_gb_fft_stats(out)
    return dict(launches=int(out[0]), ms=float(out[1]), bytes=float(out[2]))


def omp_params():
    n, c = c_int64(0), c_bool(False)
    _call("openmp_params", byref(n), byref(c))
    return n.value, c.value


# -------------------------------------------------- k mesh and band structure
def irr_k_count(Nx: int, Ny: int, Nz: int) -> int:
    """Irreducible TRS k count (libs/flibs/_hamiltonian.py:367-378)."""
    N = Nx * Ny * Nz
    if N % 2 == 0:
        if Nz % 2 == 0:
            if Nx % 2 == 0 and Ny % 2 == 0:
                return N // 2 + 4
            return N // 2 + 2 if (Nx % 2 == 0 or Ny % 2 == 0) else N // 2 + 1
        return N // 2 + 2 if (Nx % 2 == 0 and Ny % 2 == 0) else N // 2 + 1
    return (N + 1) // 2


def gen_irr_k_TRS(Nx: int, Ny: int, Nz: int):
    """(klist[Nk,3], kmap[Nkall,3], invk[Nkall,3]) (libs/flibs/_hamiltonian.py:356-382)."""
    Nk, Nkall = irr_k_count(Nx, Ny, Nz), Nx * Ny * Nz
    klist = np.zeros((Nk, 3))
    kmap = np.zeros((Nkall, 3), dtype=np.int64)
    invk = np.zeros((Nkall, 3), dtype=np.int64)
    _call("generate_irr_kpoint_inv", klist, kmap, invk, i64(Nk), i64(Nx), i64(Ny), i64(Nz))
    return klist, kmap, invk


def gen_kpoint_weight(invk, Nk: int):
    w = np.zeros(Nk)
    _call("get_kweight", w, invk, i64(Nk), i64(len(invk)))
    return w


def gen_ham(klist, ham_r, rvec, Ovl_r=None):
    """k-space Hamiltonian [Nk,Norb,Norb], and with overlap blocks Ovl_r also
    the k-space overlap, (hamk, Ovlk) (libs/flibs/_hamiltonian.py:134-157)."""
    Nk, Nr, Norb = len(klist), len(rvec), ham_r.shape[1]

    def transform(blocks):
        out = np.zeros((Nk, Norb, Norb), dtype=np.complex128)
        _call("gen_ham", out, np.ascontiguousarray(klist, dtype=np.float64),
              np.ascontiguousarray(blocks, dtype=np.complex128), np.ascontiguousarray(rvec, dtype=np.float64),
              i64(Nk), i64(Nr), i64(Norb))
        return out

    hamk = transform(ham_r)
    return hamk if Ovl_r is None else (hamk, transform(Ovl_r))


def get_eig(hamk, Ovlk=None, sw: bool = True):
    """(eig[Nk,Norb] ascending, uni[Nk,Norb,Norb]), or eig alone when sw is
    False (libs/flibs/_hamiltonian.py:160-185).  With an overlap Ovlk the
    generalized problem goes through get_eig_mlo (canonical orthogonalization,
    fmod.f90:250-310)."""
    Nk, Norb = len(hamk), hamk.shape[1]
    eig = np.zeros((Nk, Norb))
    uni = np.zeros((Nk, Norb, Norb), dtype=np.complex128)
    if Ovlk is None:
        _call("get_eig", eig, uni, np.ascontiguousarray(hamk), i64(Nk), i64(Norb))
    else:
        _call("get_eig_mlo", eig, uni, np.ascontiguousarray(hamk), np.ascontiguousarray(Ovlk, dtype=np.complex128),
              i64(Nk), i64(Norb))
    return (eig, uni) if sw else eig


def get_ffermi(eig, mu: float, temp: float):
    f = np.zeros_like(eig, dtype=np.float64)
    _call("get_ffermi", f, np.ascontiguousarray(eig, dtype=np.float64), dbl(mu), dbl(temp),
          i64(len(eig)), i64(eig.shape[1]))
    return f


def get_plist(rvec, ham_r):
    """Orbital parities from H(R) vs H(-R) (libs/flibs/_hamiltonian.py:411-423)."""
    Norb = ham_r.shape[1]
    P = np.zeros((Norb, Norb))
    _call("get_parity_prop", P, np.ascontiguousarray(rvec, dtype=np.float64),
          np.ascontiguousarray(ham_r, dtype=np.complex128), i64(Norb), i64(len(rvec)))
    return np.sign(P[0, :])


# --------------------------------------------------------------- vertices
def get_chi_orb_list(Norb: int, site_prof=(1,)):
    """Orbital-pair list and site labels as plibs.get_chi_orb_list returns
    them (libs/plibs/_response.py:382-413).  One site: all Norb^2 pairs, pair
    l = (l % Norb + 1, l // Norb + 1), site 1.  Several sites (orbital counts
    in site_prof): the pairs within each site, labelled by the site's first
    orbital.  The array's memory is the Fortran olist(Nchi,2) in both cases.
    (The reference's several-site list is C-ordered, and the library would
    read that memory as other pairs.)  A profile that does not add up to Norb
    ends the program, as in the reference."""
    prof = [int(x) for x in site_prof]
    if len(prof) == 1:
        t = np.arange(Norb) + 1
        o1, o2 = np.meshgrid(t, t)
        return np.array([o1.flatten(), o2.flatten()]).T, np.ones(Norb * Norb, dtype=np.int64)
    if Norb != sum(prof):
        print("site_prof doesn't correspond to Hamiltonian")
        raise SystemExit
    cols, site, n0 = [], [], 1
    for ns in prof:
        t = np.arange(ns) + n0
        o1, o2 = np.meshgrid(t, t)
        cols.append(np.array([o1.flatten(), o2.flatten()]))
        site += [n0] * (ns * ns)
        n0 += ns
    return np.concatenate(cols, axis=1).T, np.array(site, dtype=np.int64)


def gen_SCmatrix(olist, site, U: float, J: float):
    Nchi = len(olist)
    S, C = np.zeros((Nchi, Nchi)), np.zeros((Nchi, Nchi))
    _call("get_scmat", S, C, olist, np.asarray(site, dtype=np.int64), dbl(U), dbl(J), i64(Nchi))
    return S, C


def gen_SCmatrix_orb(olist, site, Umat, Jmat):
    Nchi, Norb = len(olist), len(Umat)
    S, C = np.zeros((Nchi, Nchi)), np.zeros((Nchi, Nchi))
    _call("get_scmat_orb", S, C, olist, np.asarray(site, dtype=np.int64), np.ascontiguousarray(Umat, dtype=np.float64),
          np.ascontiguousarray(Jmat, dtype=np.float64), i64(Nchi), i64(Norb))
    return S, C


# ----------------------------------------------------------------- Green
def gen_Green0(eig, uni, mu: float, temp: float, Nw: int):
    Nk, Norb = eig.shape
    Gk = np.zeros((Norb, Norb, Nw, Nk), dtype=np.complex128)
    _call("gen_green0_", Gk, np.ascontiguousarray(eig), np.ascontiguousarray(uni), dbl(mu), dbl(temp),
          i64(Nk), i64(Nw), i64(Norb))
    return Gk


def gen_green_from_eig(selfen, eig, uni, mu: float, temp: float):
    """Interacting G [Norb,Norb,Nw,Nk] from the band energies and eigenvectors
    (libs/flibs/_green.py:119-139: gen_green_inv_from_eig, then getinv_)."""
    Nk, Norb, Nw = len(eig), eig.shape[1], selfen.shape[2]
    Gk = np.zeros((Norb, Norb, Nw, Nk), dtype=np.complex128)
    _call("gen_green_inv_from_eig", Gk, np.ascontiguousarray(selfen), np.ascontiguousarray(uni),
          np.ascontiguousarray(eig, dtype=np.float64), dbl(mu), dbl(temp), i64(Nk), i64(Nw), i64(Norb))
    _call("getinv_", Gk, i64(Nk), i64(Nw), i64(Norb))
    return Gk


def gen_green(selfen, hamk, mu: float, temp: float):
    Nk, Norb, Nw = len(hamk), hamk.shape[1], selfen.shape[2]
    Gk = np.zeros((Norb, Norb, Nw, Nk), dtype=np.complex128)
    _call("gen_green_inv_", Gk, np.ascontiguousarray(selfen), np.ascontiguousarray(hamk), dbl(mu), dbl(temp),
          i64(Nk), i64(Nw), i64(Norb))
    _call("getinv_", Gk, i64(Nk), i64(Nw), i64(Norb))
    return Gk


# ---------------------------------------------------------- susceptibility
def chi_map_arrays(olist):
    """(chi_map, irr_chi) int32, 1-based, memory = Fortran chi_map(Nchi,Nchi,2) and
    irr_chi(Nchi(Nchi+1)/2,2); exchange symmetry chi_1234 = chi*_4321 (fchi.f90:421-481)."""
    ol = np.asarray(olist, dtype=np.int64)
    n = len(ol)
    cmap = np.zeros((2, n, n), dtype=np.int32)
    is_irr = np.zeros((n, n), dtype=bool)
    for l1 in range(n):
        for m1 in range(n):
            want = (ol[l1, 0], ol[l1, 1], ol[m1, 0], ol[m1, 1])
            hit = next(((l2, m2) for l2 in range(n) for m2 in range(n)
                        if (ol[m2, 1], ol[m2, 0], ol[l2, 1], ol[l2, 0]) == want), None)
            if hit is None:
                continue
            l2, m2 = hit
            cmap[0, l1, m1], cmap[1, l1, m1] = m2 + 1, l2 + 1
            if not is_irr[l2, m2]:
                is_irr[l1, m1] = True
    irr = np.zeros((2, n * (n + 1) // 2), dtype=np.int32)
    for it, (l1, m1) in enumerate((l, m) for l in range(n) for m in range(n) if is_irr[l, m]):
        irr[0, it], irr[1, it] = l1 + 1, m1 + 1
    return cmap, irr


def _dims(Gk):
    Norb = len(Gk)
    return Norb, Gk.shape[2], Gk.shape[3]


def get_chi0_conv(Gk, kmap, invk, olist, temp: float, Nx: int, Ny: int, Nz: int):
    Norb, Nw, Nk = _dims(Gk)
    Nchi = len(olist)
    chi = np.zeros((Nchi, Nchi, Nw, Nk), dtype=np.complex128)
    cmap, irr = chi_map_arrays(olist)
    _call("get_chi0_conv_", chi, np.ascontiguousarray(Gk), kmap, invk, irr, cmap, olist, dbl(temp), i64(Nx),
          i64(Ny), i64(Nz), i64(Nw), i64(Nk), i64(len(kmap)), i64(Norb), i64(Nchi))
    return chi


def get_chi0(Smat, Cmat, Gk, olist, kmap, invk, temp: float, Nx: int, Ny: int, Nz: int):
    """(chi0 [Nchi,Nchi,Nw,Nk], Stoner factor) (libs/flibs/_susceptibility.py:425-455)."""
    Norb, Nw, Nk = _dims(Gk)
    Nchi = len(olist)
    chi = np.zeros((Nchi, Nchi, Nw, Nk), dtype=np.complex128)
    st = c_double(0.0)
    _call("get_chi0", chi, Smat, Cmat, np.ascontiguousarray(Gk), kmap, invk, olist, dbl(temp), i64(Nx), i64(Ny),
          i64(Nz), i64(Nw), i64(Nk), i64(len(kmap)), i64(Norb), i64(Nchi), byref(st))
    return chi, st.value


def get_chi0_tail(Smat, Cmat, Gk, eig, uni, olist, kmap, invk, mu: float, temp: float, Nx: int, Ny: int, Nz: int):
    """Tail-corrected chi0 (libs/flibs/_susceptibility.py:457-490)."""
    Norb, Nw, Nk = _dims(Gk)
    Nchi = len(olist)
    chi = np.zeros((Nchi, Nchi, Nw, Nk), dtype=np.complex128)
    st = c_double(0.0)
    _call("get_chi0_tail", chi, Smat, Cmat, np.ascontiguousarray(Gk), np.ascontiguousarray(eig),
          np.ascontiguousarray(uni), kmap, invk, olist, dbl(mu), dbl(temp), i64(Nx), i64(Ny), i64(Nz), i64(Nw),
          i64(Nk), i64(len(kmap)), i64(Norb), i64(Nchi), byref(st))
    return chi, st.value


def get_chis(chi0, Smat):
    Nchi, Nw = len(Smat), len(chi0)
    chis = np.zeros((Nw, Nchi, Nchi), dtype=np.complex128)
    _call("get_chis", chis, np.ascontiguousarray(chi0), Smat, i64(Nchi), i64(Nw))
    return chis


def get_chis_chic(chi, Smat, Cmat):
    Nk, Nw, Nchi = chi.shape[3], chi.shape[2], len(Smat)
    chis = np.zeros((Nchi, Nchi, Nk), dtype=np.complex128)
    chic = np.zeros((Nchi, Nchi, Nk), dtype=np.complex128)
    _call("get_chis_chic", chis, chic, np.ascontiguousarray(chi), Smat, Cmat, i64(Nk), i64(Nw), i64(Nchi))
    return chis, chic


def get_eig_or_tr_chi(chi, invk, sw_eig: bool):
    Nkall, Nk, Nchi = len(invk), chi.shape[-1], chi.shape[0]
    out = np.zeros(Nkall, dtype=np.complex128)
    _call("get_eig_or_tr_chi", out, np.ascontiguousarray(chi), invk, i64(Nkall), i64(Nk), i64(Nchi),
          byref(c_bool(bool(sw_eig))))
    return out


def eig_or_tr_chi_noalloc(out_ptr: int, chi_ptr: int, invk_ptr: int, Nkall: int, Nk: int, Nchi: int,
                          sw_eig: bool, stream: int = 0) -> None:
    """get_eig_or_tr_chi on device buffers (integer device addresses), enqueued
    on `stream` without allocating device memory; Nk <= 65536.  One call at a
    time per device: overlapping calls share the entry's fixed scratch."""
    lib = load_library()
    f = lib.pyrpa_gb_eig_or_tr_chi_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_int64, c_int64, c_int64, ctypes.c_int32,
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    lib.pyrpa_gb_clear_error()
    rc = f(out_ptr, chi_ptr, invk_ptr, Nkall, Nk, Nchi, 1 if sw_eig else 0, stream or None)
    if rc != 0:
        raise RuntimeError(last_error())


def regrid_sigma(sigmak, temp_old: float, temp_new: float, Nw_new: int, w_scale: float = 1.0):
    """sigmak [Norb, Norb, Nw_old, Nk] (the wrappers' layout) onto Nw_new
    frequencies at temp_new, as plibs.regrid_sigma_bin does to sigma.bin."""
    sigmak = np.ascontiguousarray(sigmak, dtype=np.complex128)
    Norb, _, Nw_old, Nk = sigmak.shape
    out = np.zeros((Norb, Norb, Nw_new, Nk), dtype=np.complex128)
    _call("pyrpa_gb_regrid_sigma", out, sigmak, i64(Nk), i64(Nw_old), i64(Nw_new), i64(Norb), dbl(temp_old),
          dbl(temp_new), dbl(w_scale))
    return out


def regrid_sigma_file(path: str, out_path: str, temp_old, temp_new: float, Norb, Nw_old, Nw_new,
                      w_scale: float = 1.0):
    """Reads a sigma.bin seed, moves it onto Nw_new frequencies at temp_new and
    writes it to out_path, all inside the library (record parsing, checks
    against the file's (temp, Nw, Norb, Nk) record, the GPU regrid, the new
    file).  None means "take it from the file" (temp_old, Norb, Nw_old) or
    "keep Nw_old" (Nw_new).  Returns (Nk, Nw_new); ValueError for a file or
    argument the caller has to fix."""
    nk, nw = c_int64(-1), c_int64(-1)
    _call("pyrpa_gb_regrid_sigma_file", os.fsencode(path), os.fsencode(out_path),
          dbl(np.nan if temp_old is None else temp_old), dbl(np.nan if temp_new is None else temp_new),
          i64(0 if Norb is None else Norb), i64(0 if Nw_old is None else Nw_old),
          i64(0 if Nw_new is None else Nw_new), dbl(w_scale), byref(nk), byref(nw))
    return int(nk.value), int(nw.value)


def fft_candidates(n: int, elem_bytes: int):
    """(L1, lines) settings the FFT autotuner may try for an axis of length n
    (PYRPA_GB_FFT_TUNE=1); (0, 0) is the heuristic.  Needs no GPU."""
    out = np.zeros(2 * 64, dtype=np.int64)
    count = c_int64(0)
    _call("pyrpa_gb_fft_candidates", i64(n), i64(elem_bytes), out, i64(64), byref(count))
    return [tuple(int(v) for v in out[2 * i: 2 * i + 2]) for i in range(min(64, count.value))]


def sigma_interp(sigmak_c, kmap_c, invk_c, Nx_c: int, Ny_c: int, Nz_c: int, kmap_f, invk_f, Nx_f: int,
                 Ny_f: int, Nz_f: int, Nk_f: int, Nw_f: int, temp: float):
    """Sigma of a coarse solve [Norb, Norb, Nw_c, Nk_c] (the wrappers' layout)
    on a finer irreducible mesh: Fourier interpolation over k (each coarse
    axis length divides the fine one; Sigma(-k) = Sigma(k)^T fills the coarse
    grid) and c0 + c1/(i w) through two interior coarse frequencies beyond
    the coarse Matsubara set.  Returns [Norb, Norb, Nw_f, Nk_f].  This is the
    seed step of the coarse-mesh warm start; the reference has none."""
    sigmak_c = np.ascontiguousarray(sigmak_c, dtype=np.complex128)
    Norb, _, Nw_c, Nk_c = sigmak_c.shape
    out = np.zeros((Norb, Norb, Nw_f, Nk_f), dtype=np.complex128)
    _call("pyrpa_gb_sigma_interp", out, sigmak_c, np.ascontiguousarray(kmap_c, dtype=np.int64),
          np.ascontiguousarray(invk_c, dtype=np.int64), i64(Nx_c), i64(Ny_c), i64(Nz_c), i64(Nk_c), i64(Nw_c),
          np.ascontiguousarray(kmap_f, dtype=np.int64), np.ascontiguousarray(invk_f, dtype=np.int64), i64(Nx_f),
          i64(Ny_f), i64(Nz_f), i64(Nk_f), i64(Nw_f), i64(Norb), dbl(temp))
    return out


def wannier_r(data, kmap, invk, Nx: int, Ny: int, Nz: int, N_cut: int):
    """data [Norb, Norb, Nw, Nk_irr or Nkall] -> inverse k-FFT for the first
    N_cut frequencies, [Norb, Norb, N_cut, Nx, Ny, Nz] (conj at -k when data
    are on the irreducible points)."""
    data = np.ascontiguousarray(data, dtype=np.complex128)
    Norb, _, Nw, Nkd = data.shape
    ncut = min(N_cut, Nw)
    out = np.zeros((Norb, Norb, ncut, Nz, Ny, Nx), dtype=np.complex128)
    _call("pyrpa_gb_wannier_r", out, data, np.ascontiguousarray(kmap, dtype=np.int64),
          np.ascontiguousarray(invk, dtype=np.int64), i64(Nx), i64(Ny), i64(Nz), i64(Nkd), i64(Nw), i64(Norb),
          i64(N_cut))
    return np.ascontiguousarray(out.transpose(0, 1, 2, 5, 4, 3))


def get_Vsigma_nosoc_flex(chi, Smat, Cmat):
    """V_sigma in place; like the reference wrapper it passes Nk=len(chi),
    Nw=len(chi[0]) (libs/flibs/_selfenergy.py:60-73)."""
    Nk, Nw, Nchi = len(chi), len(chi[0]), len(Smat)
    if Nk * Nw * Nchi * Nchi > np.asarray(chi).size:
        # the reference library would read past the end of the buffer here
        raise ValueError(f"chi holds {np.asarray(chi).size} elements, the call reads Nk*Nw*Nchi^2 = "
                         f"{Nk * Nw * Nchi * Nchi} (Nk=len(chi), Nw=len(chi[0]) as in the reference wrapper)")
    _call("get_vsigma_flex_nosoc_", chi, Smat, Cmat, i64(Nk), i64(Nw), i64(Nchi))
    return chi.copy()


# --------------------------------------------------------------- FLEX loop
def mkself(Smat, Cmat, kmap, invk, olist, hamk, eig, uni, mu: float, fill: float, temp: float, Nw: int,
           Nx: int, Ny: int, Nz: int, sw_out: bool, sw_in: bool, sub_sigma: int = 1, scf_loop: int = 300,
           eps: float = 1.0e-4, pp: float = 0.3, m_diis: int = 5, sw_rescale: bool = False,
           sw_tail: bool = False, sigma_scale: float = 1.0):
    """FLEX self-consistency (libs/flibs/_selfenergy.py:76-127): (sigmak [Norb,Norb,Nw,Nk], mu)."""
    Nkall, Nk, Nchi = len(kmap), len(hamk), len(Smat)
    Norb = hamk.shape[1]
    mu_self = c_double()
    sigmak = np.zeros((Norb, Norb, Nw, Nk), dtype=np.complex128)
    _call("mkself", sigmak, byref(mu_self), Smat, Cmat, kmap, invk, olist, np.ascontiguousarray(hamk),
          np.ascontiguousarray(eig), np.ascontiguousarray(uni), dbl(mu), dbl(fill), dbl(temp), i64(scf_loop),
          dbl(pp), dbl(eps), i64(Nkall), i64(Nk), i64(Nw), i64(Norb), i64(Nchi), i64(Nx), i64(Ny), i64(Nz),
          i64(sub_sigma), byref(c_bool(sw_out)), byref(c_bool(sw_in)), i64(m_diis), byref(c_bool(sw_rescale)),
          byref(c_bool(sw_tail)), dbl(sigma_scale))
    return sigmak, mu_self.value


# -------------------------------------------------------------- Eliashberg
def linearized_eliashberg(chi, Gk, uni, init_delta, Smat, Cmat, olist, plist, kmap, invk, Nx: int, Ny: int,
                          Nz: int, temp: float, gap_sym: int, eps: float = 1.0e-5, itemax: int = 300,
                          arnoldi_m: int = 10):
    """Leading eigenvalue and gap (libs/flibs/_eliashberg.py:145-181); chi is
    overwritten with the pairing vertex, as in the reference."""
    Norb, Nchi = len(Gk), len(Smat)
    Nkall, Nk, Nw = len(kmap), Gk.shape[3], Gk.shape[2]
    delta = np.zeros((Norb, Norb, Nw, Nk), dtype=np.complex128)
    lam = c_double(0.0)
    _call("lin_eliash", delta, chi, np.ascontiguousarray(Gk), np.ascontiguousarray(uni),
          _real_gap(init_delta), Smat, Cmat, olist,
          np.ascontiguousarray(plist, dtype=np.float64), kmap, invk, dbl(temp), dbl(eps), i64(Nkall), i64(Nk),
          i64(Nw), i64(Nchi), i64(Norb), i64(Nx), i64(Ny), i64(Nz), i64(itemax), i64(gap_sym), i64(arnoldi_m),
          byref(lam))
    return delta, lam.value


def nonlinear_eliashberg(delta_init, Gk, hamk, Smat, Cmat, olist, plist, kmap, invk, mu: float, temp: float,
                         gap_sym: int, Nx: int, Ny: int, Nz: int, sw_sigma: bool = False, sw_Vconst: bool = False,
                         eps: float = 1.0e-4, itemax: int = 100, m_diis: int = 5, gap_min: float = 1.0e-2,
                         sw_amp_newton: bool = True):
    """Nonlinear FLEX-Eliashberg loop (libs/flibs/_eliashberg.py:225-300).
    Like the reference, a C-contiguous complex128 delta_init is updated in
    place and Gk is overwritten with the last self-consistent G; returns
    (delta, sigmak), sigmak zero unless sw_sigma."""
    if delta_init.dtype != np.complex128 or not delta_init.flags['C_CONTIGUOUS']:
        delta = np.ascontiguousarray(delta_init, dtype=np.complex128)
    else:
        delta = delta_init
    if Gk.dtype != np.complex128 or not Gk.flags['C_CONTIGUOUS']:
        raise ValueError("Gk must be a C-contiguous complex128 array: it is overwritten with the final G")
    Norb, _, Nw, Nk = delta.shape
    Nkall, Nchi = len(kmap), len(Smat)
    if Gk.shape != delta.shape or len(hamk) != Nk or Nkall != Nx * Ny * Nz:
        raise ValueError("delta_init, Gk, hamk and the k-mesh sizes disagree")
    sigmak = np.zeros((Norb, Norb, Nw, Nk), dtype=np.complex128)
    _call("eliashberg", delta, sigmak, Gk, np.ascontiguousarray(hamk), Smat, Cmat, olist,
          np.ascontiguousarray(plist, dtype=np.float64), kmap, invk, dbl(mu), dbl(temp), dbl(eps), i64(Nkall),
          i64(Nk), i64(Nw), i64(Nchi), i64(Norb), i64(Nx), i64(Ny), i64(Nz), i64(itemax), i64(gap_sym),
          byref(c_bool(bool(sw_sigma))), byref(c_bool(bool(sw_Vconst))), i64(m_diis), dbl(gap_min),
          byref(c_bool(bool(sw_amp_newton))))
    return delta, sigmak


def get_chi0sc(Gk, Fk, Smat, Cmat, olist, plist, kmap, invk, Nx: int, Ny: int, Nz: int, temp: float, gap_sym: int,
               vertex: bool = False):
    """chi0_S, chi0_C = chi^GG +- chi^FF of the nonlinear loop (ffeliash.f90:454-489),
    or with vertex=True its V_sigma, V_Delta (ffeliash.f90:379-452); (Nchi,Nchi,Nw,Nk)."""
    Norb, Nchi = len(Gk), len(Smat)
    Nk, Nw = Gk.shape[3], Gk.shape[2]
    xs = np.zeros((Nchi, Nchi, Nw, Nk), dtype=np.complex128)
    xc = np.zeros_like(xs)
    _call("pyrpa_gb_chi0sc", xs, xc, np.ascontiguousarray(Gk), np.ascontiguousarray(Fk), Smat, Cmat, olist,
          np.ascontiguousarray(plist, dtype=np.float64), kmap, invk, dbl(temp), i64(len(kmap)), i64(Nk), i64(Nw),
          i64(Nchi), i64(Norb), i64(Nx), i64(Ny), i64(Nz), i64(gap_sym), i64(1 if vertex else 0))
    return xs, xc


def sc_dyson(G0, Fk, delta):
    """One SC Dyson step of the nonlinear loop (ffeliash.f90:316-377):
    G = G0 (1 + delta Fk^+), then F = -G0 delta G^+; returns (G, F)."""
    Norb, Nw, Nk = len(G0), G0.shape[2], G0.shape[3]
    G = np.zeros_like(G0)
    F = np.array(Fk, dtype=np.complex128, order="C", copy=True)
    _call("pyrpa_gb_sc_dyson", G, F, np.ascontiguousarray(G0), np.ascontiguousarray(delta), i64(Nk), i64(Nw),
          i64(Norb))
    return G, F


def gen_Fk(Gk, delta, invk):
    """F = -G Delta G^dagger (libs/flibs/_eliashberg.py:343-355)."""
    Nk, Nw, Norb = Gk.shape[3], delta.shape[2], len(delta)
    Fk = np.zeros((Norb, Norb, Nw, Nk), dtype=np.complex128)
    _call("mkfk_trs_nsoc_", Fk, np.ascontiguousarray(Gk), np.ascontiguousarray(delta), i64(Nk), i64(Nw), i64(Norb))
    return Fk


def get_initial_delta(init_delta, uni, kmap, invk, Nw: int, gap_sym: int):
    Norb, Nk = init_delta.shape
    delta = np.zeros((Norb, Norb, Nw, Nk), dtype=np.complex128)
    _call("get_initial_delta_", delta, _real_gap(init_delta),
          np.ascontiguousarray(uni), kmap, invk, i64(len(kmap)), i64(Nk), i64(Nw), i64(Norb), i64(gap_sym))
    return delta


def remap_gap(delta0, plist, invk, gap_sym: int):
    Nkall, Nk, Norb = len(invk), delta0.shape[-1], len(plist)
    Nw = delta0.shape[2]
    delta = np.zeros((Norb, Norb, Nw, Nkall), dtype=np.complex128)
    _call("remap_delta_", delta, np.ascontiguousarray(delta0), np.ascontiguousarray(plist, dtype=np.float64), invk,
          i64(Nkall), i64(Nk), i64(Nw), i64(Norb), i64(gap_sym))
    return delta


def conv_delta_orb_to_band(delta, uni, invk, plist, gap_sym: int):
    Nkall, Nk, Nw, Norb = len(invk), len(uni), delta.shape[2], len(delta)
    deltab = np.zeros((Norb, Norb, Nkall), dtype=np.complex128)
    _call("conv_delta_orb_to_band", deltab, np.ascontiguousarray(delta), np.ascontiguousarray(uni),
          np.ascontiguousarray(plist, dtype=np.float64), invk, i64(Norb), i64(Nkall), i64(Nk), i64(Nw), i64(gap_sym))
    return deltab


def get_initial_gap(klist, Norb: int, gap_sym: int):
    """Band-basis initial gap [Norb, Nk] (libs/plibs/_response.py:415-462):
    s, dx2-y2, s+-, dxy, dxz, dyz for gap_sym 0..5, px, py, p+ip (complex)
    for -1, -2, -3; other values raise IndexError, as in the reference."""
    A = 2 * np.pi
    kx, ky, kz = klist[:, 0], klist[:, 1], klist[:, 2]
    rows = {0: np.ones(len(klist)), 1: np.cos(A * kx) - np.cos(A * ky), 2: 2 * np.cos(A * kx) * np.cos(A * ky),
            3: 2 * np.sin(A * kx) * np.sin(A * ky), 4: 2 * np.sin(A * kx) * np.sin(A * kz),
            5: 2 * np.sin(A * ky) * np.sin(A * kz), -1: 2 * np.sin(A * kx), -2: 2 * np.sin(A * ky),
            -3: 2 * np.sin(A * kx) + 2j * np.sin(A * ky)}
    if gap_sym not in rows:
        # the reference looks the symmetry's label up in a list and fails there
        raise IndexError(f"gap_sym {gap_sym} outside -3..5 (s, dx2-y2, s+-, dxy, dxz, dyz, px, py, p+ip)")
    return np.tile(rows[gap_sym], (Norb, 1))


# ------------------------------------------------ fused FLEX + Eliashberg
def flex_eliash(Smat, Cmat, kmap, invk, olist, hamk, eig, uni, init_delta, plist, mu: float, fill: float,
                temp: float, Nw: int, Nx: int, Ny: int, Nz: int, gap_sym: int, sub_sigma: int = 1,
                scf_loop: int = 300, eps: float = 1.0e-4, pp: float = 0.5, m_diis: int = 5,
                sw_rescale: bool = True, sw_tail: bool = False, arnoldi_m: int = 10, itemax: int = 300,
                eps_eliash: float = 1.0e-5, sigma_seed=None, seed_mu: float = 0.0, seed_mu_old: float = 0.0,
                coarse=(1, 1)):
    """mkself -> gen_green -> get_chi0(_tail) -> linearized_eliashberg in one
    device-resident call (libs/plibs/_calc.py:370-405 with sw_self=True).

    Returns a dict with sigmak [Norb,Norb,Nw,Nk], mu, gap, lambda, stoner and
    the H2D / device / D2H milliseconds of the call.  ``sigma_seed`` (same
    layout as sigmak) starts the loop from a given self-energy.  ``coarse`` =
    (k divisor, frequency divisor) other than (1, 1) first solves the model on
    the k mesh and Matsubara set divided by them (FP32 bulk, down to the FP32
    rounding floor) and starts the fine loop from its interpolated Sigma."""
    Nkall, Nk, Nchi = len(kmap), len(hamk), len(Smat)
    Norb = hamk.shape[1]
    sigmak = np.zeros((Norb, Norb, Nw, Nk), dtype=np.complex128)
    gap = np.zeros((Norb, Norb, Nw, Nk), dtype=np.complex128)
    mu_o, lam, st = c_double(), c_double(), c_double()
    times = np.zeros(3)
    seed_ptr = None
    if sigma_seed is not None:
        sigma_seed = np.ascontiguousarray(sigma_seed, dtype=np.complex128)
        assert sigma_seed.shape == sigmak.shape
        seed_ptr = sigma_seed.ctypes.data_as(ctypes.c_void_p)
    _call("pyrpa_gb_flex_eliash", sigmak, byref(mu_o), gap, byref(lam), byref(st), times, Smat, Cmat, kmap, invk,
          olist, np.ascontiguousarray(hamk), np.ascontiguousarray(eig), np.ascontiguousarray(uni),
          _real_gap(init_delta), np.ascontiguousarray(plist, dtype=np.float64),
          seed_ptr, dbl(seed_mu), dbl(seed_mu_old), dbl(mu), dbl(fill), dbl(temp), i64(scf_loop), dbl(pp), dbl(eps),
          i64(Nkall), i64(Nk), i64(Nw), i64(Norb), i64(Nchi), i64(Nx), i64(Ny), i64(Nz), i64(sub_sigma),
          i64(m_diis), byref(c_bool(sw_rescale)), byref(c_bool(sw_tail)), i64(gap_sym), i64(arnoldi_m),
          i64(itemax), dbl(eps_eliash), np.asarray(coarse, dtype=np.int64))
    return dict(sigmak=sigmak, mu=mu_o.value, gap=gap, lam=lam.value, stoner=st.value,
                h2d_ms=times[0], compute_ms=times[1], d2h_ms=times[2])


# ------------------------------------------------------------- spin-orbit
# Mirrors of the reference's spin-orbit wrappers (libs/flibs/_interaction.py:
# gen_Vmatrix(_orb); _susceptibility.py: get_chi0_soc, get_chis_chic_soc;
# _selfenergy.py: mkself_soc; _eliashberg.py: linearized_eliashberg_soc,
# conv_delta_orb_to_band_soc, gen_Fk_soc), same arguments and layouts.
def gen_Vmatrix(olist, slist, site, invs, U: float, J: float):
    Nchi, Norb = len(olist), len(slist)
    Vmat = np.zeros((Nchi, Nchi), dtype=np.float64)
    _call("get_vmat_soc", Vmat, olist, np.asarray(slist, dtype=np.int64), np.asarray(site, dtype=np.int64),
          np.asarray(invs, dtype=np.int64), dbl(U), dbl(J), i64(Nchi), i64(Norb))
    return Vmat


def gen_Vmatrix_orb(olist, slist, site, invs, Umat, Jmat):
    Nchi, Norb = len(olist), len(Umat)
    Vmat = np.zeros((Nchi, Nchi), dtype=np.float64)
    _call("get_vmat_soc_orb", Vmat, olist, np.asarray(slist, dtype=np.int64), np.asarray(site, dtype=np.int64),
          np.asarray(invs, dtype=np.int64), np.ascontiguousarray(Umat, dtype=np.float64),
          np.ascontiguousarray(Jmat, dtype=np.float64), i64(Nchi), i64(Norb))
    return Vmat


def get_chi0_soc(Vmat, Gk, olist, slist, kmap, invk, invs, temp: float, Nx: int, Ny: int, Nz: int):
    """(chi, sgnsig, sgnsig2, invschi) (libs/flibs/_susceptibility.py:496-528)."""
    Norb, Nchi = len(slist), len(olist)
    Nkall, Nk, Nw = len(kmap), Gk.shape[3], Gk.shape[2]
    chi = np.zeros((Nchi, Nchi, Nw, Nk), dtype=np.complex128)
    sgnsig = np.zeros((Norb, Norb), dtype=np.float64)
    sgnsig2 = np.zeros((Nchi, Nchi), dtype=np.float64)
    invschi = np.zeros(Nchi, dtype=np.int64)
    _call("get_chi0_soc", chi, sgnsig, sgnsig2, invschi, np.ascontiguousarray(Vmat, dtype=np.float64),
          np.ascontiguousarray(Gk), kmap, invk, np.asarray(invs, dtype=np.int64), olist,
          np.asarray(slist, dtype=np.int64), dbl(temp), i64(Nx), i64(Ny), i64(Nz), i64(Nw), i64(Nk), i64(Nkall),
          i64(Nchi), i64(Norb))
    return chi, sgnsig, sgnsig2, invschi


def get_chis_chic_soc(chi, Vmat, olist, slist, invs):
    """(chic, chiszz, chispm) (libs/flibs/_susceptibility.py:530-566)."""
    slist = np.asarray(slist, dtype=np.int64)
    invs = np.asarray(invs, dtype=np.int64)
    Norb, Nchi = len(slist), len(olist)
    Nk, Nw = chi.shape[3], chi.shape[2]
    orbs = np.where(slist == 1)[0]
    o1, o2 = np.meshgrid(orbs, orbs)
    orb_chi = np.array([o1.flatten(), o2.flatten()]).T
    orb_list = np.zeros(Nchi, dtype=np.int64)
    for i, ol in enumerate(np.asarray(olist)):
        a = (ol[0] if slist[ol[0] - 1] == 1 else invs[ol[0] - 1]) - 1
        b = (ol[1] if slist[ol[1] - 1] == 1 else invs[ol[1] - 1]) - 1
        for j, ob in enumerate(orb_chi):
            if a == ob[0] and b == ob[1]:
                orb_list[i] = j + 1
                break
    n4 = Nchi // 4
    chic = np.zeros((n4, n4, Nk), dtype=np.complex128)
    chiszz = np.zeros_like(chic)
    chispm = np.zeros_like(chic)
    _call("get_chis_chic_soc", chic, chiszz, chispm, np.ascontiguousarray(chi),
          np.ascontiguousarray(Vmat, dtype=np.float64), orb_list, olist, slist, invs, i64(Nk), i64(Nw), i64(Nchi),
          i64(Norb))
    return chic, chiszz, chispm


def mkself_soc(Vmat, kmap, invk, invs, olist, slist, hamk, eig, uni, mu: float, fill: float, temp: float, Nw: int,
               Nx: int, Ny: int, Nz: int, sw_out: bool, sw_in: bool, sub_sigma: int = 1, scf_loop: int = 300,
               eps: float = 1.0e-4, pp: float = 0.3, m_diis: int = 5, sw_rescale: bool = False,
               sigma_scale: float = 1.0):
    """FLEX with spin-orbit coupling (libs/flibs/_selfenergy.py:129-175)."""
    Nkall, Nk, Nchi = len(kmap), len(hamk), len(Vmat)
    Norb = hamk.shape[1]
    mu_self = c_double(0.0)
    sigmak = np.zeros((Norb, Norb, Nw, Nk), dtype=np.complex128)
    _call("mkself_soc", sigmak, byref(mu_self), np.ascontiguousarray(Vmat, dtype=np.float64), kmap, invk,
          np.asarray(invs, dtype=np.int64), olist, np.asarray(slist, dtype=np.int64), np.ascontiguousarray(hamk),
          np.ascontiguousarray(eig), np.ascontiguousarray(uni), dbl(mu), dbl(fill), dbl(temp), i64(scf_loop),
          dbl(pp), dbl(eps), i64(Nkall), i64(Nk), i64(Nw), i64(Norb), i64(Nchi), i64(Nx), i64(Ny), i64(Nz),
          i64(sub_sigma), byref(c_bool(bool(sw_out))), byref(c_bool(bool(sw_in))), i64(m_diis),
          byref(c_bool(bool(sw_rescale))), dbl(sigma_scale))
    return sigmak, mu_self.value


def linearized_eliashberg_soc(chi, Gk, uni, init_delta, Vmat, sgnsig, sgnsig2, plist, slist, olist, kmap, invk,
                              invs, invschi, Nx: int, Ny: int, Nz: int, temp: float, gap_sym: int, eps: float = 1.0e-4,
                              itemax: int = 300, arnoldi_m: int = 10):
    """Gap on the full mesh (libs/flibs/_eliashberg.py:183-222); chi is
    overwritten with V_Delta.  The reference's argtypes list for this call has
    27 entries for the 28 Fortran arguments (prt is missing), so its own wrapper
    raises TypeError; this one passes the Fortran signature.  lambda is in
    last_stats()["lambda"]."""
    Norb, Nchi = len(slist), len(Vmat)
    Nkall, Nk, Nw = len(kmap), Gk.shape[3], Gk.shape[2]
    delta = np.zeros((Norb, Norb, Nw, Nkall), dtype=np.complex128)
    _call("lin_eliash_soc", delta, chi, np.ascontiguousarray(Gk), np.ascontiguousarray(uni),
          _real_gap(init_delta), np.ascontiguousarray(Vmat, dtype=np.float64),
          np.ascontiguousarray(sgnsig, dtype=np.float64), np.ascontiguousarray(sgnsig2, dtype=np.float64),
          np.ascontiguousarray(plist, dtype=np.float64), olist, np.asarray(slist, dtype=np.int64), kmap, invk,
          np.asarray(invs, dtype=np.int64), np.asarray(invschi, dtype=np.int64), dbl(temp), dbl(eps), i64(Nkall),
          i64(Nk), i64(Nw), i64(Nchi), i64(Norb), i64(Nx), i64(Ny), i64(Nz), i64(itemax), i64(gap_sym),
          i64(arnoldi_m))
    return delta


def conv_delta_orb_to_band_soc(delta, uni, invk, invs, slist):
    Nkall, Nk, Nw, Norb = len(invk), len(uni), delta.shape[2], len(delta)
    deltab = np.zeros((Norb, Norb, Nkall), dtype=np.complex128)
    _call("conv_delta_orb_to_band_soc", deltab, np.ascontiguousarray(delta), np.ascontiguousarray(uni), invk,
          np.asarray(invs, dtype=np.int64), np.asarray(slist, dtype=np.int64), i64(Norb), i64(Nkall), i64(Nk),
          i64(Nw))
    return deltab


def gen_Fk_soc(Gk, delta, invk, invs, slist, gap_sym: int):
    Nkall, Nk, Nw, Norb = len(invk), Gk.shape[3], delta.shape[2], len(delta)
    Fk = np.zeros((Norb, Norb, Nw, Nkall), dtype=np.complex128)
    slist = np.asarray(slist, dtype=np.int64)
    sgnsig = np.outer(slist, slist).astype(np.float64)
    _call("mkfk_trs_soc_", Fk, np.ascontiguousarray(Gk), np.ascontiguousarray(delta), sgnsig, slist, invk,
          np.asarray(invs, dtype=np.int64), i64(Nkall), i64(Nk), i64(Nw), i64(Norb), i64(gap_sym))
    return Fk


# ------------------------------------------------------- real-frequency maps
# Mirrors of libs/flibs/_hamiltonian.py (get_qshift, get_iqshift),
# _susceptibility.py (get_chi_irr, chis_qmap, get_tr_chi, get_phi_irr,
# phi_qmap, get_tr_phi) and _green.py (get_a, get_QP, pade_with_trace).
def get_qshift(klist, qpoint):
    Nk = len(klist)
    qshift = np.zeros(Nk, dtype=np.int64)
    _call("get_qshift_", np.ascontiguousarray(qpoint, dtype=np.float64), np.ascontiguousarray(klist, dtype=np.float64),
          qshift, i64(Nk))
    return qshift


def get_iqshift(klist, qpoint):
    Nk = len(klist)
    qshift = np.zeros(Nk, dtype=np.int64)
    _call("get_iqshift_", np.ascontiguousarray(qpoint, dtype=np.float64),
          np.ascontiguousarray(klist, dtype=np.float64), qshift, i64(Nk))
    return qshift


def get_chi_irr(uni, eig, ffermi, qshift, olist, wlist, idelta: float, temp: float):
    """chi0(q, w) [Nw, Nchi, Nchi] (libs/flibs/_susceptibility.py:271-293)."""
    Nk, Nw = len(eig), len(wlist)
    Norb, Nchi = eig.shape[1], len(olist)
    chi = np.zeros((Nw, Nchi, Nchi), dtype=np.complex128)
    _call("get_chi_irr", chi, np.ascontiguousarray(uni), np.ascontiguousarray(eig), np.ascontiguousarray(ffermi),
          np.ascontiguousarray(qshift, dtype=np.int64), olist, np.ascontiguousarray(wlist, dtype=np.float64),
          i64(Nchi), i64(Norb), i64(Nk), i64(Nw), dbl(idelta), dbl(idelta * 1e-3), dbl(temp))
    return chi


def chis_qmap(uni, eig, ffermi, klist, Smat, olist, Nx: int, Ny: int, temp: float, ecut: float, idelta: float):
    """(chis, chi) maps [Nx, Ny] (libs/flibs/_susceptibility.py:295-324)."""
    Nk = len(eig)
    Norb, Nchi = eig.shape[1], len(olist)
    chi = np.zeros((Nx, Ny), dtype=np.complex128)
    chis = np.zeros((Nx, Ny), dtype=np.complex128)
    _call("chiq_map", chis, chi, np.ascontiguousarray(uni), np.ascontiguousarray(eig), np.ascontiguousarray(ffermi),
          np.ascontiguousarray(klist, dtype=np.float64), np.ascontiguousarray(Smat, dtype=np.float64), olist,
          dbl(temp), dbl(ecut), dbl(idelta), dbl(idelta * 1e-3), i64(Nx), i64(Ny), i64(Nk), i64(Norb), i64(Nchi))
    return chis, chi


def get_tr_chi(chis, chi0, olist):
    Nchi, Nw, Norb = len(olist), len(chi0), int(np.asarray(olist).max())
    trchis = np.zeros(Nw, dtype=np.complex128)
    trchi0 = np.zeros(Nw, dtype=np.complex128)
    chis_orb = np.zeros((Nw, Norb + 2), dtype=np.complex128)
    _call("get_tr_chi", trchis, trchi0, chis_orb, np.ascontiguousarray(chis), np.ascontiguousarray(chi0), olist,
          i64(Nw), i64(Nchi), i64(Norb))
    return trchis, trchi0, chis_orb


def get_phi_irr(uni, eig, ffermi, qshift, olist, wlist, idelta: float, mu: float, temp: float):
    Nk, Nw = len(eig), len(wlist)
    Norb, Nchi = eig.shape[1], len(olist)
    phi = np.zeros((Nw, Nchi, Nchi), dtype=np.complex128)
    _call("get_phi_irr", phi, np.ascontiguousarray(uni), np.ascontiguousarray(eig), np.ascontiguousarray(ffermi),
          np.ascontiguousarray(qshift, dtype=np.int64), olist, np.ascontiguousarray(wlist, dtype=np.float64),
          i64(Nchi), i64(Norb), i64(Nk), i64(Nw), dbl(idelta), dbl(idelta * 1e-3), dbl(mu), dbl(temp))
    return phi


def phi_qmap(uni, eig, ffermi, klist, olist, Nx: int, Ny: int, mu: float, temp: float, ecut: float, idelta: float,
             sw_omega: bool):
    Nk = len(eig)
    Norb, Nchi = eig.shape[1], len(olist)
    phi = np.zeros((Nx, Ny), dtype=np.complex128)
    _call("phiq_map", phi, np.ascontiguousarray(uni), np.ascontiguousarray(eig), np.ascontiguousarray(ffermi),
          np.ascontiguousarray(klist, dtype=np.float64), olist, dbl(mu), dbl(temp), dbl(ecut), dbl(idelta),
          dbl(idelta * 1e-3), i64(Nx), i64(Ny), i64(Nk), i64(Norb), i64(Nchi), byref(c_bool(bool(sw_omega))))
    return phi


def get_tr_phi(phi, olist):
    Nchi, Nw, Norb = len(olist), len(phi), int(np.asarray(olist).max())
    trphi = np.zeros(Nw, dtype=np.complex128)
    phi_orb = np.zeros((Nw, Norb + 2), dtype=np.complex128)
    _call("get_tr_phi", trphi, phi_orb, np.ascontiguousarray(phi), olist, i64(Nw), i64(Nchi), i64(Norb))
    return trphi, phi_orb


def get_a(inp_data, xlist):
    Np = len(inp_data)
    a = np.zeros(Np, dtype=np.complex128)
    _call("get_a_", a, np.ascontiguousarray(xlist, dtype=np.complex128),
          np.ascontiguousarray(inp_data, dtype=np.complex128), i64(Np))
    return a


def get_QP(a, xlist, wlist):
    """(Q, P), in the reference wrapper's return order (libs/flibs/_green.py:190-204)."""
    Nw, Np = len(wlist), len(a)
    Q = np.zeros(Nw, dtype=np.complex128)
    P = np.zeros(Nw, dtype=np.complex128)
    _call("get_qp_", P, Q, np.ascontiguousarray(a, dtype=np.complex128),
          np.ascontiguousarray(xlist, dtype=np.complex128), np.ascontiguousarray(wlist, dtype=np.complex128),
          i64(Nw), i64(Np))
    return Q, P


def pade_with_trace(A, iwlist, wlist):
    """[Nk, Nw] (libs/flibs/_green.py:206-220)."""
    Nk, Nw, Niw = A.shape[3], len(wlist), len(iwlist)
    Norb = A.shape[0]
    B = np.zeros((Nk, Nw), dtype=np.complex128)
    _call("pade_with_trace", np.ascontiguousarray(A), B, np.ascontiguousarray(iwlist, dtype=np.complex128),
          np.ascontiguousarray(wlist, dtype=np.complex128), i64(Nk), i64(Niw), i64(Nw), i64(Norb))
    return B
