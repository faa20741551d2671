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


def test_orchestration_with_oracle_backed_library(monkeypatch):
    """coarse_solution -> interpolated_seed -> add_training_solution ->
    learned_seed on a small 2-orbital model, with the library's GPU entry
    points replaced by their oracle restatements: the coarse model is the same
    model on the divided mesh, the seed is the oracle's interpolation of the
    coarse solve, and the learned seed is that seed plus the network's
    correction."""
    from oracle import api as O
    from oracle import flex_oracle as FO
    from pyrpa_gb300 import flibs as F
    from pyrpa_gb300 import models
    from pyrpa_gb300 import build
    if not build.LIB.exists():
        pytest.skip("libfmod.so is not built")
    F.load_library()
    stats = {}

    def mkself(S, C, kmap, invk, olist, hamk, eig, uni, mu, fill, temp, Nw, Nx, Ny, Nz, sw_out, sw_in, **kw):
        sig, mu2, r = O.mkself(S, C, kmap, invk, np.asarray(olist), hamk, eig, uni, mu, fill, temp, Nw, Nx, Ny, Nz,
                               full=True, **kw)
        stats.update(stoner=r.stoner, iterations=r.iterations)
        return sig, mu2

    def sigma_interp(sc, kmap_c, invk_c, Nx_c, Ny_c, Nz_c, kmap_f, invk_f, Nx_f, Ny_f, Nz_f, Nk_f, Nw_f, temp):
        gc = FO.KGrid(kmap_c, invk_c, Nx_c, Ny_c, Nz_c)
        gf = FO.KGrid(kmap_f, invk_f, Nx_f, Ny_f, Nz_f)
        return W.sigma_interp(np.asarray(sc).T, gc, gf, Nw_f, temp).T

    monkeypatch.setattr(F, "gen_ham", lambda k, h, r, Ovl_r=None: O.gen_ham(k, h, r))
    monkeypatch.setattr(F, "get_eig", lambda h, Ovlk=None, sw=True: O.get_eig(h))
    monkeypatch.setattr(F, "mkself", mkself)
    monkeypatch.setattr(F, "last_stats", lambda: dict(stats))
    monkeypatch.setattr(F, "sigma_interp", sigma_interp)

    class Net:
        def __init__(self):
            self.theta = W.init_params(0)
            self.rows = 0

        def add_samples(self, s, f, uni, eig, Nw_c, desc, pairs):
            self.rows += len(pairs) * s.shape[0] ** 2
            self.last = (Nw_c, desc, pairs)

        @property
        def num_rows(self):
            return self.rows

        def apply(self, s, uni, eig, Nw_c, desc):
            U = np.swapaxes(uni, 1, 2)
            kn = W.all_pairs(s.shape[3], s.shape[2])
            y, _ = W.forward(self.theta, W.features(s.T, U, eig, Nw_c, desc, kn))
            return W.apply_correction(s.T, U, desc, y).T

    m = models.prepare("c2", Norb=2, Nx=8, Ny=8, Nz=1, Nw=16, temp=0.1, fill=1.0, U=0.8, J=0.8 / 6, seed=5,
                       bandwidth=4.0)
    coarse = L.coarse_solution(m, 2, 2, eps=1e-8)
    assert coarse["model"]["cfg"]["Nx"] == 4 and coarse["model"]["cfg"]["Nw"] == 8
    assert coarse["sigmak"].shape == (2, 2, 8, len(coarse["model"]["klist"]))
    seed = L.interpolated_seed(m, coarse)
    assert seed.shape == (2, 2, 16, len(m["klist"]))
    net = Net()
    rows = L.add_training_solution(net, m, coarse, seed + 0.01, max_pairs=50, seed=3)
    assert rows == 50 * 4 and net.last[0] == 8 and len(net.last[2]) == 50
    learned, mu_seed = L.learned_seed(net, m, coarse)
    assert mu_seed == coarse["mu"]
    desc = L.seed_descriptors(m, coarse, seed)
    assert np.allclose(learned, net.apply(seed, m["uni"], m["eig"], 8, desc))
    assert not np.allclose(learned, seed)
