"""CPU checks of the warm-start oracle (oracle/warmstart_oracle.py): the
coarse-mesh interpolation is exact on band-limited input, the band-basis
features and corrections round-trip, bf16 rounding ties to even, and the
network's analytic gradients agree with finite differences."""
import numpy as np
import pytest

from oracle import flex_oracle as FO
from oracle import warmstart_oracle as W


def _grid(N, Nz=1):
    klist, kmap, invk = FO.generate_irr_kpoint_inv(N, N, Nz)
    return klist, FO.KGrid(kmap, invk, N, N, Nz)


def _bandlimited(klist, Nw, No, R, A, fw):
    """Sigma(k, n) = fw[n] * sum_R A_R exp(2 pi i k.R), Fortran view."""
    ph = np.exp(2j * np.pi * klist @ np.asarray(R, dtype=np.float64).T)  # [Nk, nR]
    S = np.einsum("kr,rab->kab", ph, A)
    return fw[None, :, None, None] * S[:, None]


def _trs_coeffs(rng, No, Rmax, nyq=None):
    """A_{-R} = A_R^T, so that Sigma(-k) = Sigma(k)^T; Nyquist terms symmetric."""
    R, A = [], []
    for rx in range(-Rmax, Rmax + 1):
        for ry in range(-Rmax, Rmax + 1):
            if (rx, ry) < (0, 0):
                continue
            M = rng.normal(size=(No, No)) + 1j * rng.normal(size=(No, No))
            if (rx, ry) == (0, 0):
                R.append((0, 0, 0))
                A.append(M + M.T)
                continue
            R += [(rx, ry, 0), (-rx, -ry, 0)]
            A += [M, M.T]
    if nyq is not None:  # the Nyquist plane as a cosine: half at +nyq, half at -nyq
        M = rng.normal(size=(No, No)) + 1j * rng.normal(size=(No, No))
        R += [(nyq, 0, 0), (-nyq, 0, 0)]
        A += [0.5 * (M + M.T), 0.5 * (M + M.T)]
    return R, np.array(A)


@pytest.mark.parametrize("Nc,Nf,No", [(4, 8, 1), (8, 16, 2), (6, 12, 3), (4, 12, 2)])
def test_interp_exact_on_bandlimited_sigma(Nc, Nf, No):
    rng = np.random.default_rng(Nc * 10 + No)
    Rmax = (Nc - 1) // 2 if Nc % 2 else Nc // 2 - 1
    R, A = _trs_coeffs(rng, No, Rmax, nyq=Nc // 2 if Nc % 2 == 0 else None)
    temp, Nw_c = 0.1, 8
    fw = rng.normal(size=Nw_c) + 1j * rng.normal(size=Nw_c)
    kc, gc = _grid(Nc)
    kf, gf = _grid(Nf)
    sc = _bandlimited(kc, Nw_c, No, R, A, fw)
    ref = _bandlimited(kf, Nw_c, No, R, A, fw)
    got = W.sigma_interp(sc, gc, gf, Nw_c, temp)
    assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max()


def test_interp_tail_exact_for_c0_plus_c1_over_iw():
    rng = np.random.default_rng(3)
    temp, Nw_c, Nw_f, No = 0.05, 16, 48, 2
    kc, gc = _grid(4)
    kf, gf = _grid(4)
    Nk = len(kc)
    c0 = rng.normal(size=(Nk, No, No)) + 1j * rng.normal(size=(Nk, No, No))
    c1 = rng.normal(size=(Nk, No, No)) + 1j * rng.normal(size=(Nk, No, No))
    # the same k on both meshes: make Sigma(-k) = Sigma(k)^T hold on the irreducible set by construction
    iw = lambda n: 1j * (2 * np.arange(n) + 1) * np.pi * temp
    sig = lambda n: c0[:, None] + c1[:, None] / iw(n)[None, :, None, None]
    got = W.sigma_interp(sig(Nw_c), gc, gf, Nw_f, temp)
    ref = sig(Nw_f)
    assert np.abs(got - ref).max() < 1e-11 * np.abs(ref).max()


def test_tail_points():
    assert W.tail_points(64) == (48, 62)
    assert W.tail_points(4) == (3, 2)
    assert W.tail_points(2) == (1, 1)


def test_bf16_ties_to_even():
    x = np.array([1.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8, 1 + 2 ** -8 + 2 ** -20, -(1 + 3 * 2 ** -8), 3.0e-39,
                  65504.0, 0.0], dtype=np.float32)
    want = np.array([1.0, 1.0, 1 + 2 ** -6, 1 + 2 ** -7, -(1 + 2 ** -6), None, 65536.0, 0.0], dtype=object)
    got = W.bf16(x)
    for g, w, xi in zip(got, want, x):
        if w is None:  # subnormal: rounding keeps the top 16 bits' neighbourhood
            assert abs(g - xi) <= 2 ** -133
        else:
            assert g == np.float32(w), (xi, g, w)
    # every result is representable in bf16 (low 16 bits clear)
    assert np.all((W.bf16(np.random.default_rng(0).normal(size=1000).astype(np.float32)).view(np.uint32)
                   & 0xFFFF) == 0)


def _model_arrays(seed, Nk, Nw, No):
    rng = np.random.default_rng(seed)
    H = rng.normal(size=(Nk, No, No)) + 1j * rng.normal(size=(Nk, No, No))
    H = H + np.conj(np.swapaxes(H, 1, 2))
    eig, U = np.linalg.eigh(H)
    sig = 0.3 * (rng.normal(size=(Nk, Nw, No, No)) + 1j * rng.normal(size=(Nk, Nw, No, No)))
    return eig, U, sig


def test_features_targets_correction_round_trip():
    Nk, Nw, No, Nw_c = 7, 12, 3, 6
    eig, U, seed = _model_arrays(1, Nk, Nw, No)
    fine = seed + 0.05 * _model_arrays(2, Nk, Nw, No)[2]
    desc = W.descriptors(1.2, 0.2, 0.01, 1.5, No, 0.9, 0.1, eig, seed)
    kn = W.all_pairs(Nk, Nw)
    x = W.features(seed, U, eig, Nw_c, desc, kn)
    t = W.targets(seed, fine, U, desc, kn)
    assert x.shape == (Nk * Nw * No * No, W.NF) and t.shape == (Nk * Nw * No * No, 2)
    xr = x.reshape(Nw, Nk, No, No, W.NF)
    assert np.array_equal(xr[..., 6], np.broadcast_to(np.eye(No), (Nw, Nk, No, No)))
    assert np.all(xr[:Nw_c, ..., 5] == 0) and np.all(xr[Nw_c:, ..., 5] == 1)
    assert np.allclose(xr[..., 0] + 1j * xr[..., 1],
                       np.transpose(W.to_band(seed, U), (1, 0, 2, 3)) / desc[7], atol=1e-6)
    back = W.apply_correction(seed, U, desc, t)
    assert np.abs(back - fine).max() < 1e-6 * np.abs(fine).max()


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    theta = W.init_params(7).astype(np.float64)
    theta[W.NPARAM - 130:] *= 10.0  # a non-trivial output layer
    x = rng.normal(size=(40, W.NF))
    t = rng.normal(size=(40, 2))
    L, g = W.loss_and_grad(theta, x, t, round_bf16=False, dtype=np.float64)
    idx = rng.choice(W.NPARAM, 60, replace=False)
    h = 1e-6
    for i in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        fd = (W.loss_and_grad(tp, x, t, False, np.float64)[0] - W.loss_and_grad(tm, x, t, False, np.float64)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_gradient_close_to_exact():
    rng = np.random.default_rng(6)
    theta = W.init_params(3)
    x = rng.normal(size=(256, W.NF)).astype(np.float32)
    t = rng.normal(size=(256, 2)).astype(np.float32)
    _, g32 = W.loss_and_grad(theta, x, t)
    _, g64 = W.loss_and_grad(theta.astype(np.float64), x.astype(np.float64), t.astype(np.float64), False,
                             np.float64)
    assert np.linalg.norm(g32 - g64) < 2e-2 * np.linalg.norm(g64)


def test_adam_first_step_is_signed_lr():
    theta = np.ones(5, dtype=np.float32)
    g = np.array([1.0, -2.0, 0.5, -1e-3, 3.0], dtype=np.float32)
    z = np.zeros(5, dtype=np.float32)
    th, m, v = W.adam_step(theta, g, z, z, 1, 1e-2)
    assert np.allclose(th, 1 - 1e-2 * np.sign(g), rtol=0, atol=1e-6)
    assert np.allclose(m, 0.1 * g) and np.allclose(v, 0.001 * g * g)


def test_training_reduces_loss():
    rng = np.random.default_rng(8)
    x = rng.normal(size=(2048, W.NF)).astype(np.float32)
    t = np.stack([np.tanh(x[:, 0] - 0.5 * x[:, 2]), 0.3 * x[:, 1] * x[:, 4]], axis=1).astype(np.float32)
    theta = W.init_params(1)
    m = np.zeros_like(theta)
    v = np.zeros_like(theta)
    L0 = W.loss_and_grad(theta, x, t)[0]
    for step in range(1, 301):
        _, g = W.loss_and_grad(theta, x, t)
        theta, m, v = W.adam_step(theta, g, m, v, step, 3e-3)
    assert W.loss_and_grad(theta, x, t)[0] < 0.1 * L0
