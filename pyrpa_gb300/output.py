"""Gap-function text output of the linearized Eliashberg step.

``output_gap_function`` has the signature, files and text format of
plibs.output_gap_function (libs/plibs/_calc.py:311-336), which a pyrpa script
calls after the Eliashberg solve.  The gap is first brought to the band basis
on the full k mesh through this engine's conversions (conv_delta_orb_to_band
or remap_gap, and their spin-orbit forms).  Then every band pair (i, j) is
written to gap_ij.dat in the working directory.  There is one line per k
point of the kz = 0 plane in the mesh's full-list order ("kx ky Re Im"), and
a blank line after each kx = Nx - 1.
"""
from __future__ import annotations

import numpy as np

from . import flibs


def _band_gap(invk, gap, uni, plist, gap_sym, soc, invs, slist, sw_orb):
    if sw_orb:
        return gap[:, :, 0, :] if soc else flibs.remap_gap(gap[:, :, 0, :], plist, invk, gap_sym)
    if soc:
        return flibs.conv_delta_orb_to_band_soc(gap, uni, invk, invs, slist)
    return flibs.conv_delta_orb_to_band(gap, uni, invk, plist, gap_sym)


def output_gap_function(invk, kmap, gap, uni, plist, gap_sym, Nx: int, soc=False, invs=None, slist=None,
                        sw_orb=False):
    """Write gap_ij.dat for every band pair; returns 0 (a file that cannot be
    written is reported and skipped)."""
    gapb = _band_gap(invk, gap, uni, plist, gap_sym, soc, invs, slist, sw_orb)
    print("output gap function")
    kmap = np.asarray(kmap)
    plane = [(i, int(km[0]), int(km[1])) for i, km in enumerate(kmap) if km[2] == 0]
    n = len(gapb)
    for a in range(n):
        for b in range(n):
            name = f"gap_{a + 1}{b + 1}.dat"
            try:
                with open(name, "w") as f:
                    for i, kx, ky in plane:
                        v = gapb[a, b, i]
                        f.write(f"{kx:3} {ky:3} {v.real:15.8e} {v.imag:15.8e}\n")
                        if kx == Nx - 1:
                            f.write("\n")
            except IOError as e:
                print(f"output_gap_function: {name} not written ({e})", flush=True)
                continue
    return 0
