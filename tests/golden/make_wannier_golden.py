"""Generates wannier_golden.npz from the reference's own
plibs.output_self_wannier / output_gap_wannier (libs/plibs/_wannier_io.py:
145-216): for each case the input, the arrays of fname.npz and the text of
fname.dat.  Run in a container with a pyrpa checkout (PYRPA_REFERENCE);
plibs imports libs.flibs, whose loader is pointed at this engine's
libfmod.so (the writers call no library function).

    python tests/golden/make_wannier_golden.py
"""
import contextlib
import ctypes
import io
import os
import shutil
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REF = Path(os.environ.get("PYRPA_REFERENCE", "/root/reference"))


def main():
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(REF))
    from pyrpa_gb300 import build, flibs
    if not build.LIB.exists():
        build.build()
    original = np.ctypeslib.load_library
    np.ctypeslib.load_library = lambda n, p: ctypes.CDLL(str(build.LIB)) if n == "libfmod.so" else original(n, p)
    from libs.plibs import output_self_wannier, output_gap_wannier
    np.ctypeslib.load_library = original
    rng = np.random.default_rng(77)
    cases = [  # (kind, Nx, Ny, Nz, Nw, Norb, N_cut, zero_tol, full_bz)
        ("self", 4, 4, 1, 8, 2, 6, 1e-5, False),
        ("gap", 4, 4, 2, 6, 1, 4, 1e-3, False),
        ("gap", 4, 2, 1, 5, 2, 8, 1e-5, True),
    ]
    work = HERE / "_work_wannier"
    work.mkdir(exist_ok=True)
    out = {}
    cwd = os.getcwd()
    try:
        os.chdir(work)
        for c, (kind, Nx, Ny, Nz, Nw, No, Ncut, tol, full) in enumerate(cases):
            klist, kmap, invk = flibs.gen_irr_k_TRS(Nx, Ny, Nz)
            Nk = Nx * Ny * Nz if full else len(klist)
            data = rng.standard_normal((No, No, Nw, Nk)) + 1j * rng.standard_normal((No, No, Nw, Nk))
            data *= np.exp(-np.arange(Nw) / 3.0)[None, None, :, None]
            with contextlib.redirect_stdout(io.StringIO()):
                if kind == "self":
                    output_self_wannier(data, 0.25, kmap, invk, Nx, Ny, Nz, Nw, 0.02, N_cut=Ncut, zero_tol=tol,
                                        fname="w")
                else:
                    output_gap_wannier(data, kmap, invk, Nx, Ny, Nz, Nw, 0.02, N_cut=Ncut, zero_tol=tol, fname="w")
            z = np.load("w.npz")
            out[f"case{c}_data"] = data
            out[f"case{c}_par"] = np.array([Nx, Ny, Nz, Nw, Ncut, tol, 1.0 if kind == "self" else 0.0])
            for key in z.files:
                out[f"case{c}_npz_{key}"] = z[key]
            out[f"case{c}_dat"] = np.array(Path("w.dat").read_text())
    finally:
        os.chdir(cwd)
        shutil.rmtree(work, ignore_errors=True)
    np.savez_compressed(HERE / "wannier_golden.npz", **out)
    print("wrote", HERE / "wannier_golden.npz", len(cases), "cases")


if __name__ == "__main__":
    main()
