"""The oracle's restatement of plibs.regrid_sigma_bin against golden vectors
that the reference function itself produced (tests/golden/make_regrid_golden.py)."""
from pathlib import Path

import numpy as np
import pytest

from oracle import flex_oracle as FO

GOLDEN = Path(__file__).resolve().parent / "golden" / "regrid_sigma_golden.npz"


@pytest.mark.parametrize("case", range(4))
def test_regrid_restatement_matches_reference_output(case):
    g = np.load(GOLDEN)
    sig, ref, par = g[f"case{case}_in"], g[f"case{case}_out"], g[f"case{case}_par"]
    T_old, T_new, Nw_new, ws = par
    out = FO.regrid_sigma(sig, T_old, T_new, int(Nw_new), ws)
    assert out.shape == ref.shape
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max(), np.abs(out - ref).max()
