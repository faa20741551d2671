"""GPU parity of the coarse-mesh interpolation and of the learned warm start
(csrc/lws.cu through the C ABI) against oracle/warmstart_oracle.py.

Tolerances: the interpolation runs in FP32 on the device (1e-6 of the array
maximum).  Features are bf16 on both sides, computed from FP64 sums in a
different order, so they agree to one bf16 step.  Forward passes accumulate
in FP32 in another order than numpy, so an activation can round to the
neighbouring bf16 value in rare rows.  With 128 stored activations a row and
a float-rounding-sized chance (about 2^-16 x a few) for each to sit on a
bf16 rounding boundary, about 0.1-0.3% of the rows differ by one bf16 step:
all rows agree to 5e-3 and 99.5% of them to 2e-5.  The whole-set gradient agrees to 5e-3 relative (norm).  One
Adam step from the device's own gradient repeats the oracle's float32
operations one by one.
"""

import numpy as np
import pytest

from oracle import flex_oracle as FO
from oracle import warmstart_oracle as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F():
    from pyrpa_gb300 import build, flibs
    if not build.LIB.exists():
        build.build()
    flibs.load_library()
    flibs.set_verbose(0)
    flibs.set_precision(64)
    return flibs


@pytest.fixture(scope="module")
def L(F):
    from pyrpa_gb300 import warmstart
    return warmstart


def _random_solution(seed, Nk, Nw, No):
    rng = np.random.default_rng(seed)
    H = rng.normal(size=(Nk, No, No)) + 1j * rng.normal(size=(Nk, No, No))
    H = H + np.conj(np.swapaxes(H, 1, 2))
    eig, vec = np.linalg.eigh(H)              # vec[k, a, m]: band m in column m
    uni = np.ascontiguousarray(np.swapaxes(vec, 1, 2))   # wrappers' layout uni[k, m, a]
    seed_s = 0.3 * (rng.normal(size=(No, No, Nw, Nk)) + 1j * rng.normal(size=(No, No, Nw, Nk)))
    fine = seed_s + 0.05 * (rng.normal(size=seed_s.shape) + 1j * rng.normal(size=seed_s.shape))
    return eig, uni, seed_s, fine


def _oracle_rows(seed_s, fine, uni, eig, Nw_c, desc, pairs):
    U = np.swapaxes(uni, 1, 2)
    x = W.features(seed_s.T, U, eig, Nw_c, desc, pairs)
    t = W.targets(seed_s.T, fine.T, U, desc, pairs) if fine is not None else None
    return x, t


@pytest.mark.parametrize("Nc,Nf,Nw_c,Nw_f,No", [(4, 8, 8, 16, 1), (8, 16, 8, 12, 2), (6, 12, 4, 4, 3)])
def test_sigma_interp_matches_oracle(F, Nc, Nf, Nw_c, Nw_f, No):
    rng = np.random.default_rng(Nc + No)
    kc, kmap_c, invk_c = F.gen_irr_k_TRS(Nc, Nc, 1)
    kf, kmap_f, invk_f = F.gen_irr_k_TRS(Nf, Nf, 1)
    sc = rng.normal(size=(No, No, Nw_c, len(kc))) + 1j * rng.normal(size=(No, No, Nw_c, len(kc)))
    got = F.sigma_interp(sc, kmap_c, invk_c, Nc, Nc, 1, kmap_f, invk_f, Nf, Nf, 1, len(kf), Nw_f, 0.05)
    gc = FO.KGrid(kmap_c, invk_c, Nc, Nc, 1)
    gf = FO.KGrid(kmap_f, invk_f, Nf, Nf, 1)
    ref = W.sigma_interp(sc.T, gc, gf, Nw_f, 0.05).T
    assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("No", [1, 2, 5])
def test_features_and_targets_match_oracle(L, No):
    Nk, Nw, Nw_c = 9, 12, 6
    eig, uni, s, f = _random_solution(No, Nk, Nw, No)
    desc = L.descriptors(1.2, 0.2, 0.01, 0.5 * No, No, 0.93, 0.1, eig, s)
    pairs = L.sample_pairs(Nk, Nw, 40, seed=No)
    x, t = L.features(s, uni, eig, Nw_c, desc, pairs, sigma_fine=f)
    xo, to = _oracle_rows(s, f, uni, eig, Nw_c, desc, pairs)
    xo = W.bf16(xo)
    step = np.maximum(np.abs(xo), 1e-30) * 2.0 ** -7
    assert np.all(np.abs(x - xo) <= step), np.abs(x - xo).max()
    assert np.mean(x == xo) > 0.999
    assert np.allclose(t, to, rtol=1e-6, atol=1e-7)


def test_forward_matches_oracle(L):
    rng = np.random.default_rng(4)
    theta = W.init_params(5)
    theta[W.NPARAM - 130:] *= 10.0
    net = L.LearnedWarmStart(params=theta)
    x = rng.normal(size=(20000, W.NF)).astype(np.float32)
    y = net.forward(x)
    yo, _ = W.forward(theta, x)
    d = np.abs(y - yo).max(axis=1)
    assert d.max() < 5e-3
    assert np.mean(d < 2e-5) > 0.995


def _loaded_net(L, No=2, seed=7, params_seed=2):
    Nk, Nw, Nw_c = 11, 16, 8
    eig, uni, s, f = _random_solution(seed, Nk, Nw, No)
    desc = L.descriptors(1.0, 0.15, 0.02, 1.0, No, 0.9, 0.0, eig, s)
    pairs = L.all_pairs(Nk, Nw)
    theta = W.init_params(params_seed)
    theta[W.NPARAM - 130:] *= 10.0
    net = L.LearnedWarmStart(params=theta)
    net.add_samples(s, f, uni, eig, Nw_c, desc, pairs)
    x, t = L.features(s, uni, eig, Nw_c, desc, pairs, sigma_fine=f)
    return net, theta, x, t, (s, f, uni, eig, Nw_c, desc)


def test_loss_and_gradient_match_oracle(L):
    net, theta, x, t, _ = _loaded_net(L)
    assert net.num_rows == len(x)
    loss, g = net.loss_grad()
    lo, go = W.loss_and_grad(theta, x, t)
    assert abs(loss - lo) <= 1e-4 * lo
    assert np.linalg.norm(g - go) <= 5e-3 * np.linalg.norm(go)


def test_adam_step_repeats_oracle(L):
    net, theta, x, t, _ = _loaded_net(L, seed=8)
    _, g = net.loss_grad()
    net.step(1e-3)
    want, _, _ = W.adam_step(theta, g, np.zeros_like(theta), np.zeros_like(theta), 1, 1e-3)
    assert np.allclose(net.params, want, rtol=2e-7, atol=0)


def test_apply_matches_oracle(L):
    net, theta, _, _, (s, f, uni, eig, Nw_c, desc) = _loaded_net(L, No=3, seed=9)
    got = net.apply(s, uni, eig, Nw_c, desc)
    pairs = L.all_pairs(s.shape[3], s.shape[2])
    x, _ = _oracle_rows(s, None, uni, eig, Nw_c, desc, pairs)
    y, _ = W.forward(theta, x)
    ref = W.apply_correction(s.T, np.swapaxes(uni, 1, 2), desc, y).T
    corr = np.abs(ref - s).max()
    assert corr > 0
    assert np.abs(got - ref).max() <= 5e-3 * corr


def test_training_reduces_loss(L):
    net, _, _, _, _ = _loaded_net(L, seed=10)
    l0, _ = net.loss_grad()
    losses = net.train(300, batch=1024, lr=3e-3, seed=1)
    assert np.all(np.isfinite(losses))
    l1, _ = net.loss_grad()
    assert l1 < 0.5 * l0


def test_learned_seed_converges_to_cold_fixed_point(F, L):
    """A network trained on one model seeds another; the fine loop from that
    seed reaches the cold start's Sigma and mu."""
    from pyrpa_gb300 import models
    kw = dict(Nx=16, Ny=16, Nz=1, Nw=64, temp=0.05, U=1.0, J=1.0 / 6, fill=1.0, Norb=2, seed=11, bandwidth=4.0)
    net = L.LearnedWarmStart(seed=0)
    for s in (11, 12):
        m = models.prepare("c2", **dict(kw, seed=s))
        c = m["cfg"]
        fine, _ = F.mkself(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["mu"],
                           c["fill"], c["temp"], c["Nw"], c["Nx"], c["Ny"], c["Nz"], False, False, eps=1e-8,
                           pp=0.5, sw_rescale=True)
        L.add_training_solution(net, m, L.coarse_solution(m, 2, 2), fine)
    net.train(400, batch=4096, lr=3e-3, seed=0)
    m = models.prepare("c2", **dict(kw, seed=13))
    c = m["cfg"]
    coarse = L.coarse_solution(m, 2, 2)
    seed_sig, mu_seed = L.learned_seed(net, m, coarse)
    cold = F.flex_eliash(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["init"],
                         m["plist"], m["mu"], c["fill"], c["temp"], c["Nw"], c["Nx"], c["Ny"], c["Nz"], 0, eps=1e-8)
    warm = F.flex_eliash(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["init"],
                         m["plist"], m["mu"], c["fill"], c["temp"], c["Nw"], c["Nx"], c["Ny"], c["Nz"], 0, eps=1e-8,
                         sigma_seed=seed_sig, seed_mu=mu_seed, seed_mu_old=mu_seed)
    scale = np.abs(cold["sigmak"]).max()
    assert np.abs(warm["sigmak"] - cold["sigmak"]).max() <= 1e-6 * scale
    assert abs(warm["mu"] - cold["mu"]) <= 1e-7
