"""Host side of the learned warm start (pyrpa_gb300/warmstart.py), on CPU:
the parameter initialisation and descriptors follow the oracle's definition,
pair sampling stays on the mesh, and the C ABI refuses to run without a GPU."""
import numpy as np
import pytest

from oracle import warmstart_oracle as W
from pyrpa_gb300 import warmstart as L


def test_layout_and_init_match_oracle():
    assert L.NPARAM == W.NPARAM == 5378
    assert L.SHAPES == W.SHAPES
    for seed in (0, 3):
        assert np.array_equal(L.init_params(seed), W.init_params(seed))


def test_descriptors_match_oracle():
    rng = np.random.default_rng(1)
    eig = rng.normal(size=(10, 3))
    sig = rng.normal(size=(3, 3, 8, 10)) + 1j * rng.normal(size=(3, 3, 8, 10))
    a = L.descriptors(1.2, 0.2, 0.01, 1.5, 3, 0.97, 0.33, eig, sig)
    b = W.descriptors(1.2, 0.2, 0.01, 1.5, 3, 0.97, 0.33, eig, sig.T)
    assert np.array_equal(a, b)


def test_pairs():
    assert np.array_equal(L.all_pairs(5, 3), W.all_pairs(5, 3))
    p = L.sample_pairs(7, 11, 20, seed=2)
    assert p.shape == (20, 2)
    flat = p[:, 0] + 7 * p[:, 1]
    assert np.all(np.diff(flat) > 0)
    assert p[:, 0].min() >= 0 and p[:, 0].max() < 7 and p[:, 1].min() >= 0 and p[:, 1].max() < 11
    assert np.array_equal(L.sample_pairs(3, 4, 100), L.all_pairs(3, 4))


def test_network_needs_a_gpu():
    from pyrpa_gb300 import build, flibs
    if not build.LIB.exists():
        pytest.skip("libfmod.so is not built")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    flibs.load_library()
    with pytest.raises(RuntimeError, match="no CUDA device"):
        L.LearnedWarmStart()
