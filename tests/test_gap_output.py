"""Gap-function text output (pyrpa_gb300/output.py) against the files the
reference's own output_gap_function writes (golden texts from
tests/golden/make_gap_output_golden.py), on CPU: the spin-orbit band-basis
branch, which needs no library call."""
import contextlib
import io
import os
from pathlib import Path

import numpy as np
import pytest

from pyrpa_gb300 import flibs as F
from pyrpa_gb300.output import output_gap_function

GOLD = np.load(Path(__file__).parent / "golden" / "gap_output_golden.npz")


@pytest.mark.parametrize("c", [0, 1])
def test_gap_files_match_reference(c, tmp_path):
    Nx, Ny, Nz = (int(x) for x in GOLD[f"case{c}_dims"])
    _, kmap, invk = F.gen_irr_k_TRS(Nx, Ny, Nz)
    gap = GOLD[f"case{c}_gap"]
    old = os.getcwd()
    os.chdir(tmp_path)
    try:
        with contextlib.redirect_stdout(io.StringIO()) as out:
            ret = output_gap_function(invk, kmap, gap, None, None, 0, Nx, soc=True, sw_orb=True)
        assert ret == int(GOLD[f"case{c}_ret"]) == 0
        assert out.getvalue() == "output gap function\n"
        names = sorted(k.split("_", 1)[1] for k in GOLD.files if k.startswith(f"case{c}_gap_") and k.endswith(".dat"))
        assert names
        for name in names:
            assert Path(name).read_text() == str(GOLD[f"case{c}_{name}"]), name
    finally:
        os.chdir(old)
