"""Host side of the parameter sweep (pyrpa_gb300/sweep.py), on CPU: the
instances follow the sweep's ranges and are reproducible."""
import numpy as np

from oracle import flex_oracle as FO
from pyrpa_gb300 import sweep as S


def test_draw_ranges_and_reproducibility():
    a = S.draw(256, seed=3)
    assert a == S.draw(256, seed=3)
    assert a != S.draw(256, seed=4)
    assert [x.index for x in a] == list(range(256))
    assert {x.Norb for x in a} == set(S.ORBITALS)
    assert {x.N for x in a} == set(S.MESHES)
    assert {x.Nw for x in a} == set(S.MATSUBARA)
    for x in a:
        assert 0.5 <= x.u_frac <= 0.95
        assert 0.005 <= x.temp <= 0.05
        assert 0.7 <= x.n_per_orb <= 1.0
        assert np.isclose(x.fill, 0.5 * x.n_per_orb * x.Norb)
    # log-uniform temperature: about half of the draws below the geometric mean
    below = np.mean([x.temp < np.sqrt(0.005 * 0.05) for x in a])
    assert 0.35 < below < 0.65


def test_irr_count_matches_oracle():
    for N in (16, 32, 64, 128, 5, 7):
        assert S.irr_count(N) == FO.irr_k_count(N, N, 1)


def test_device_bytes_grow_with_size():
    base = S.Instance(0, 1, 16, 256, 1, 0.7, 0.01, 0.8)
    big = S.Instance(1, 3, 128, 4096, 1, 0.7, 0.01, 0.8)
    assert 0 < S.device_bytes(base) < S.device_bytes(big)
    # the largest instance fits one GB300's HBM in complex128
    assert S.device_bytes(big, 16) < 200e9
