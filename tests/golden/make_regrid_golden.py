"""Generates regrid_sigma_golden.npz from the reference's own
plibs.regrid_sigma_bin (libs/plibs/_calc.py:52-182).

Run in a container that holds a pyrpa checkout (PYRPA_REFERENCE, default the
path below); the checkout is not needed afterwards.  plibs imports libs.flibs,
whose loader is pointed at this engine's libfmod.so (regrid_sigma_bin itself
calls no library function).  The self-energies are synthetic and causal:
Sigma(k, iw) = sum_p R_p(k) / (iw - e_p(k)) + Sigma_inf(k) with Hermitian
positive residues, so Sigma(-iw) = Sigma(iw)^H and Im Sigma_ll(iw > 0) < 0.

    python tests/golden/make_regrid_golden.py
"""
import ctypes
import os
import shutil
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REF = Path(os.environ.get("PYRPA_REFERENCE", "/root/reference"))


def synthetic_sigma(rng, Nk, Nw, No, temp):
    w = (2.0 * np.arange(Nw) + 1.0) * np.pi * temp
    sig = np.zeros((Nk, Nw, No, No), dtype=np.complex128)
    for k in range(Nk):
        X = rng.standard_normal((No, No)) + 1j * rng.standard_normal((No, No))
        sig[k] += 0.1 * (X + X.conj().T)[None]
        for _ in range(2):
            Y = rng.standard_normal((No, No)) + 1j * rng.standard_normal((No, No))
            R = 0.2 * Y @ Y.conj().T
            e = rng.uniform(-1.5, 1.5)
            sig[k] += R[None] / (1j * w - e)[:, None, None]
    return sig


def main():
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(REF))
    from pyrpa_gb300 import build
    if not build.LIB.exists():
        build.build()
    original = np.ctypeslib.load_library
    np.ctypeslib.load_library = lambda n, p: ctypes.CDLL(str(build.LIB)) if n == "libfmod.so" else original(n, p)
    from libs.plibs import regrid_sigma_bin
    from scipy.io import FortranFile
    np.ctypeslib.load_library = original

    rng = np.random.default_rng(2026)
    cases = [  # (Nk, Nw_old, Norb, T_old, T_new, Nw_new, w_scale)
        (6, 16, 2, 0.02, 0.01, 40, None),    # cooling: new points beyond the kept cutoff use the tail
        (6, 16, 2, 0.02, 0.01, 40, 2.0),     # index-map-like compression
        (5, 24, 3, 0.01, 0.03, 10, None),    # heating onto fewer frequencies
        (4, 12, 1, 0.05, 0.05, 30, None),    # same T, more frequencies
    ]
    work = HERE / "_work_regrid"
    work.mkdir(exist_ok=True)
    out = {}
    try:
        for c, (Nk, Nw_old, No, T_old, T_new, Nw_new, ws) in enumerate(cases):
            sig = synthetic_sigma(rng, Nk, Nw_old, No, T_old)
            path = work / "sigma.bin"
            with FortranFile(str(path), "w") as f:
                f.write_record(np.array([0.1]))
                f.write_record(np.array([0.12]))
                f.write_record(np.ascontiguousarray(sig.ravel(order="F")))
                f.write_record(np.array([T_old, float(Nw_old), float(No), float(Nk)]))
            regrid_sigma_bin(temp_new=T_new, Nw_new=Nw_new, w_scale=ws, path=str(path), out_path=str(path))
            with FortranFile(str(path), "r") as f:
                f.read_record(np.float64)
                f.read_record(np.float64)
                flat = f.read_record(np.complex128)
            new = flat.reshape((Nk, Nw_new, No, No), order="F")
            out[f"case{c}_in"] = sig
            out[f"case{c}_out"] = new
            out[f"case{c}_par"] = np.array([T_old, T_new, float(Nw_new), 1.0 if ws is None else ws])
    finally:
        shutil.rmtree(work, ignore_errors=True)
    np.savez_compressed(HERE / "regrid_sigma_golden.npz", **out)
    print("wrote", HERE / "regrid_sigma_golden.npz", len(cases), "cases")


if __name__ == "__main__":
    main()
