"""Band-basis initial gaps against the reference's own get_initial_gap
(golden vectors from tests/golden/make_initial_gap_golden.py), on CPU, and
the real-gap check at the library boundary."""
from pathlib import Path

import numpy as np
import pytest

from oracle import api as O
from pyrpa_gb300 import flibs as F

GOLD = np.load(Path(__file__).parent / "golden" / "initial_gap_golden.npz")


@pytest.mark.parametrize("gap_sym", list(range(-3, 6)))
def test_initial_gap_matches_reference(gap_sym):
    ref = GOLD[f"gap_{gap_sym}"]
    for got in (F.get_initial_gap(GOLD["klist"], 3, gap_sym), O.get_initial_gap(GOLD["klist"], 3, gap_sym)):
        assert got.shape == ref.shape and np.iscomplexobj(got) == np.iscomplexobj(ref)
        assert np.allclose(got, ref, rtol=0, atol=1e-15)


def test_unknown_symmetries_are_rejected_like_the_reference():
    assert list(GOLD["rejected"]) == [-4, 6, 9]
    for gs in GOLD["rejected"]:
        with pytest.raises(IndexError):
            F.get_initial_gap(GOLD["klist"], 3, int(gs))


def test_complex_gap_is_refused_at_the_boundary():
    """The Fortran gap is real; the reference's float64 ndpointer refuses the
    complex p+ip gap, and so do these wrappers, before any library call."""
    init = F.get_initial_gap(GOLD["klist"], 3, -3)
    uni = np.tile(np.eye(3, dtype=np.complex128), (37, 1, 1))
    kmap = np.zeros((37, 3), dtype=np.int64)
    invk = np.ones((37, 3), dtype=np.int64)
    with pytest.raises(TypeError, match="real"):
        F.get_initial_delta(init, uni, kmap, invk, 4, -3)
