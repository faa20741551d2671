"""Generates initial_gap_golden.npz from the reference's own
plibs.get_initial_gap (libs/plibs/_response.py:415-462): the band-basis form
factors of every pairing symmetry it knows (gap_sym -3..5) on a 3-D k list,
and the gap_sym values it rejects.

Run in a container that holds a pyrpa checkout (PYRPA_REFERENCE, default the
path below); the checkout is not needed afterwards.  plibs imports
libs.flibs, whose loader is pointed at this engine's libfmod.so
(get_initial_gap itself calls no library function).

    python tests/golden/make_initial_gap_golden.py
"""
import contextlib
import ctypes
import io
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REF = Path(os.environ.get("PYRPA_REFERENCE", "/root/reference"))


def main():
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(REF))
    from pyrpa_gb300 import build
    if not build.LIB.exists():
        build.build()
    original = np.ctypeslib.load_library
    np.ctypeslib.load_library = lambda n, p: ctypes.CDLL(str(build.LIB)) if n == "libfmod.so" else original(n, p)
    from libs.plibs import get_initial_gap
    np.ctypeslib.load_library = original

    rng = np.random.default_rng(7)
    klist = rng.uniform(0.0, 1.0, (37, 3))
    out = {"klist": klist}
    for gs in range(-3, 6):
        with contextlib.redirect_stdout(io.StringIO()):
            out[f"gap_{gs}"] = get_initial_gap(klist, 3, gs)
    rejected = []
    for gs in (-4, 6, 9):
        try:
            with contextlib.redirect_stdout(io.StringIO()):
                get_initial_gap(klist, 3, gs)
        except IndexError:
            rejected.append(gs)
    out["rejected"] = np.array(rejected, dtype=np.int64)
    np.savez_compressed(HERE / "initial_gap_golden.npz", **out)
    print("wrote", HERE / "initial_gap_golden.npz", "rejected", rejected)


if __name__ == "__main__":
    main()
