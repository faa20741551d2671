"""Generates orbital_pairs_golden.npz from the reference's own
plibs.get_chi_orb_list (libs/plibs/_response.py:382-413): orbital-pair lists
and site labels for one and several sites, and the profile it refuses.

Run in a container that holds a pyrpa checkout (PYRPA_REFERENCE, default the
path below); the checkout is not needed afterwards.  plibs imports
libs.flibs, whose loader is pointed at this engine's libfmod.so.

    python tests/golden/make_orbital_pairs_golden.py
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

CASES = [(1, [1]), (2, [1]), (5, [1]), (8, [1]), (2, [1, 1]), (6, [3, 3]), (5, [2, 1, 2]), (8, [4, 4]),
         (7, [5, 2])]


def main():
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(REF))
    from pyrpa_gb300 import build
    if not build.LIB.exists():
        build.build()
    original = np.ctypeslib.load_library
    np.ctypeslib.load_library = lambda n, p: ctypes.CDLL(str(build.LIB)) if n == "libfmod.so" else original(n, p)
    from libs.plibs import get_chi_orb_list
    np.ctypeslib.load_library = original
    out = {}
    for c, (Norb, prof) in enumerate(CASES):
        ol, site = get_chi_orb_list(Norb, np.array(prof))
        out[f"case{c}_norb"] = np.array(Norb)
        out[f"case{c}_prof"] = np.array(prof)
        out[f"case{c}_olist"] = np.array(ol)
        out[f"case{c}_site"] = np.array(site)
    refused = False
    try:
        with contextlib.redirect_stdout(io.StringIO()):
            get_chi_orb_list(6, np.array([3, 2]))
    except SystemExit:
        refused = True
    out["refuses_bad_profile"] = np.array(refused)
    np.savez_compressed(HERE / "orbital_pairs_golden.npz", **out)
    print("wrote", HERE / "orbital_pairs_golden.npz", len(CASES), "cases; bad profile refused:", refused)


if __name__ == "__main__":
    main()
