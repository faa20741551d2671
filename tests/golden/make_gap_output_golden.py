"""Generates gap_output_golden.npz from the reference's own
plibs.output_gap_function (libs/plibs/_calc.py:311-336): the gap_ij.dat texts
it writes for a full-mesh spin-orbit gap given in the band basis (soc=True,
sw_orb=True, the branch that calls no library function), on a 2-D and a 3-D
mesh.

Run in a container that holds a pyrpa checkout (PYRPA_REFERENCE, default the
path below); the checkout is not needed afterwards.  plibs imports
libs.flibs, whose loader is pointed at this engine's libfmod.so.

    python tests/golden/make_gap_output_golden.py
"""
import contextlib
import ctypes
import io
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REF = Path(os.environ.get("PYRPA_REFERENCE", "/root/reference"))


def main():
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(REF))
    from pyrpa_gb300 import build
    from pyrpa_gb300 import flibs as F
    if not build.LIB.exists():
        build.build()
    original = np.ctypeslib.load_library
    np.ctypeslib.load_library = lambda n, p: ctypes.CDLL(str(build.LIB)) if n == "libfmod.so" else original(n, p)
    from libs.plibs import output_gap_function
    np.ctypeslib.load_library = original
    rng = np.random.default_rng(11)
    out = {}
    for c, (Nx, Ny, Nz, No) in enumerate([(4, 3, 1, 2), (3, 3, 2, 2)]):
        klist, kmap, invk = F.gen_irr_k_TRS(Nx, Ny, Nz)
        Nkall = len(kmap)
        gap = rng.normal(size=(No, No, 2, Nkall)) + 1j * rng.normal(size=(No, No, 2, Nkall))
        with tempfile.TemporaryDirectory() as d:
            old = os.getcwd()
            os.chdir(d)
            try:
                with contextlib.redirect_stdout(io.StringIO()):
                    ret = output_gap_function(invk, kmap, gap, None, None, 0, Nx, soc=True, sw_orb=True)
                texts = {f"gap_{a + 1}{b + 1}.dat": Path(f"gap_{a + 1}{b + 1}.dat").read_text()
                         for a in range(No) for b in range(No)}
            finally:
                os.chdir(old)
        out[f"case{c}_dims"] = np.array([Nx, Ny, Nz])
        out[f"case{c}_gap"] = gap
        out[f"case{c}_ret"] = np.array(ret)
        for name, t in texts.items():
            out[f"case{c}_{name}"] = np.array(t)
    np.savez_compressed(HERE / "gap_output_golden.npz", **out)
    print("wrote", HERE / "gap_output_golden.npz")


if __name__ == "__main__":
    main()
