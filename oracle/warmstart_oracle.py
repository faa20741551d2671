"""CPU restatement of the coarse-mesh seed and of the learned warm-start
corrector that refines it.

TEST INFRASTRUCTURE: this module is the checker for the GPU engine, not part
of the product.  Only tests, the smoke check and the CPU-baseline leg of the
benchmark import it.

The reference has no warm start of this kind: a pyrpa user seeds the FLEX
loop by hand through sigma.bin (fself.f90:742-780) after regridding it with
plibs.regrid_sigma_bin (libs/plibs/_calc.py:52-182), whose c0 + c1/(i w)
tail this module's frequency extension follows.  Parity is therefore
unpinned by the reference's tests: the interpolation is pinned by exact
cases (band-limited Sigma on the coarse mesh is reproduced to rounding), the
network by finite-difference gradients.

Arrays are in the Fortran view: Sigma [k, n, a, b] = sigma(k, n, a, b),
U [k, a, m] = uni(a, m, k) (orbital a, band m), eig [k, m].

Network (one row per fine irreducible k, Matsubara index n and band pair
(i, j)): 16 features -> 64 -> 64 -> 2 with tanh, FP32 weights, activations
rounded to bf16 where they are stored, FP32 gradients, Adam.  Parameters are
one flat float32 vector: W1 [64, 16], b1 [64], W2 [64, 64], b2 [64],
W3 [2, 64], b3 [2], each row-major.
"""
from __future__ import annotations

import numpy as np

from oracle.flex_oracle import KGrid

NF, NH, NO = 16, 64, 2
SHAPES = (("W1", (NH, NF)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NO, NH)), ("b3", (NO,)))
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


# --------------------------------------------------------------------------- #
#  coarse-mesh seed: Fourier interpolation in k, c0 + c1/(i w) beyond the
#  coarse Matsubara set
# --------------------------------------------------------------------------- #
def _pad_axis(a, axis, nf):
    """Zero-pad the Fourier components of one axis from nc to nf points; an
    even nc's Nyquist component is split in half between +nc/2 and -nc/2."""
    nc = a.shape[axis]
    if nc == nf:
        return a
    shp = list(a.shape)
    shp[axis] = nf
    out = np.zeros(shp, dtype=a.dtype)

    def at(i):
        s = [slice(None)] * a.ndim
        s[axis] = i
        return tuple(s)

    for r in range(-(nc // 2), (nc - 1) // 2 + 1):
        if nc % 2 == 0 and abs(r) == nc // 2:
            out[at(r % nf)] += 0.5 * a[at(r % nc)]
            out[at((-r) % nf)] += 0.5 * a[at(r % nc)]
        else:
            out[at(r % nf)] += a[at(r % nc)]
    return out


def tail_points(Nw_c):
    """The two coarse frequencies (0-based) the c0 + c1/(i w) tail goes through."""
    n2 = Nw_c - 2 if Nw_c >= 4 else Nw_c - 1
    n1 = (3 * Nw_c) // 4 if Nw_c >= 4 else n2
    return n1, n2


def sigma_interp(sig_c, grid_c: KGrid, grid_f: KGrid, Nw_f, temp):
    """Sigma on the fine irreducible mesh from the coarse solution.

    Sigma(-k) = Sigma(k)^T fills the coarse grid; the spatial transform is
    zero-padded to the fine grid and transformed back; frequencies beyond
    the coarse set follow c0 + c1/(i w) through two interior coarse
    frequencies (3/4 of the set and the last but one)."""
    Nk_c, Nw_c, No, _ = sig_c.shape
    full = np.zeros((grid_c.Nx, grid_c.Ny, grid_c.Nz, Nw_c, No, No), dtype=np.complex128)
    d = grid_c.flag == 0
    full[grid_c.gx[d], grid_c.gy[d], grid_c.gz[d]] = sig_c[grid_c.ki[d]]
    full[grid_c.gx[~d], grid_c.gy[~d], grid_c.gz[~d]] = np.swapaxes(sig_c[grid_c.ki[~d]], -1, -2)
    R = np.fft.fftn(full, axes=(0, 1, 2))
    for ax, nf in enumerate((grid_f.Nx, grid_f.Ny, grid_f.Nz)):
        R = _pad_axis(R, ax, nf)
    scale = (grid_f.Nx * grid_f.Ny * grid_f.Nz) / (grid_c.Nx * grid_c.Ny * grid_c.Nz)
    ff = np.fft.ifftn(R, axes=(0, 1, 2)) * scale
    Nk_f = int(grid_f.ki.max()) + 1
    out = np.zeros((Nk_f, Nw_f, No, No), dtype=np.complex128)
    dd = grid_f.direct
    out[grid_f.ki[dd], :Nw_c] = ff[grid_f.gx[dd], grid_f.gy[dd], grid_f.gz[dd]]
    if Nw_f > Nw_c:
        n1, n2 = tail_points(Nw_c)
        z = lambda n: -1j / ((2 * n + 1) * np.pi * temp)
        s1, s2 = out[:, n1], out[:, n2]
        if n1 == n2:
            out[:, Nw_c:] = s2[:, None]
        else:
            c1 = (s1 - s2) / (z(n1) - z(n2))
            c0 = s1 - c1 * z(n1)
            n = np.arange(Nw_c, Nw_f)
            out[:, Nw_c:] = c0[:, None] + c1[:, None] * z(n)[None, :, None, None]
    return out


# --------------------------------------------------------------------------- #
#  features and targets
# --------------------------------------------------------------------------- #
def descriptors(U, J, temp, fill, Norb, stoner_c, mu_c, eig, sig_seed):
    """Per-solution scalars [U, J, T, fill, stoner, mu_c, W, s_scale, Norb]:
    W the band width of eig, s_scale = max |Sigma_seed| (floored at 1e-12)."""
    W = float(eig.max() - eig.min())
    s = max(float(np.abs(sig_seed).max()), 1e-12)
    return np.array([U, J, temp, fill, stoner_c, mu_c, W, s, Norb], dtype=np.float64)


def to_band(sig, U):
    """Sigma_b(k, n) = U(k)^dagger Sigma(k, n) U(k)."""
    return np.einsum("kai,knab,kbj->knij", np.conj(U), sig, U)


def from_band(sig_b, U):
    return np.einsum("kai,knij,kbj->knab", U, sig_b, np.conj(U))


def features(sig_seed, U, eig, Nw_c, desc, kn):
    """Rows [len(kn) * No * No, 16] float32 for the (k, n) pairs kn [P, 2]
    (0-based), row order (pair, i, j) with j fastest:
      0, 1   Re, Im Sigma_b(k, n)_ij / s_scale
      2, 3   (eps_i(k) - mu_c) / W, (eps_j(k) - mu_c) / W
      4      w_n / w_c, w_c = (2 Nw_c - 1) pi T the last coarse frequency
      5      1 beyond the coarse set, else 0
      6      1 on the diagonal (i == j), else 0
      7-10   U / W, J / W, 100 T / W, fill / Norb
      11     Stoner factor of the coarse solve
      12     W / (W + w_n)
      13, 14 Re, Im Sigma_b(k, 0)_ij / s_scale
      15     0"""
    Uh, Jh, T, fill, stoner, mu_c, W, s, Norb = desc
    No = sig_seed.shape[2]
    k, n = kn[:, 0], kn[:, 1]
    Sb = np.einsum("pai,pab,pbj->pij", np.conj(U[k]), sig_seed[k, n], U[k])
    S0 = np.einsum("pai,pab,pbj->pij", np.conj(U[k]), sig_seed[k, 0], U[k])
    wn = (2 * n + 1) * np.pi * T
    wc = (2 * Nw_c - 1) * np.pi * T
    P = len(kn)
    f = np.zeros((P, No, No, NF), dtype=np.float64)
    f[..., 0] = Sb.real / s
    f[..., 1] = Sb.imag / s
    f[..., 2] = ((eig[k] - mu_c) / W)[:, :, None]
    f[..., 3] = ((eig[k] - mu_c) / W)[:, None, :]
    f[..., 4] = (wn / wc)[:, None, None]
    f[..., 5] = (n >= Nw_c).astype(np.float64)[:, None, None]
    f[..., 6] = np.eye(No)[None]
    f[..., 7] = Uh / W
    f[..., 8] = Jh / W
    f[..., 9] = 100.0 * T / W
    f[..., 10] = fill / Norb
    f[..., 11] = stoner
    f[..., 12] = (W / (W + wn))[:, None, None]
    f[..., 13] = S0.real / s
    f[..., 14] = S0.imag / s
    return f.reshape(P * No * No, NF).astype(np.float32)


def targets(sig_seed, sig_fine, U, desc, kn):
    """Rows [len(kn) * No * No, 2]: Re, Im (Sigma_fine - Sigma_seed)_b / s_scale."""
    s = desc[7]
    k, n = kn[:, 0], kn[:, 1]
    D = np.einsum("pai,pab,pbj->pij", np.conj(U[k]), sig_fine[k, n] - sig_seed[k, n], U[k]) / s
    No = sig_seed.shape[2]
    return np.stack([D.real, D.imag], axis=-1).reshape(len(kn) * No * No, 2).astype(np.float32)


def apply_correction(sig_seed, U, desc, y):
    """Sigma_seed + U (s_scale (y0 + i y1)) U^dagger for every (k, n); y rows
    in the order of features() over all pairs (k fastest, then n)."""
    Nk, Nw, No, _ = sig_seed.shape
    s = desc[7]
    yb = (y[:, 0].astype(np.float64) + 1j * y[:, 1].astype(np.float64)).reshape(Nw, Nk, No, No)
    yb = np.transpose(yb, (1, 0, 2, 3)) * s
    return sig_seed + from_band(yb, U)


def all_pairs(Nk, Nw):
    """Every (k, n) pair, k fastest (the Fortran order of the per-(k, n) arrays)."""
    n, k = np.meshgrid(np.arange(Nw), np.arange(Nk), indexing="ij")
    return np.stack([k.ravel(), n.ravel()], axis=1).astype(np.int64)


# --------------------------------------------------------------------------- #
#  the network
# --------------------------------------------------------------------------- #
def bf16(x):
    """Round float32 to the nearest bfloat16 (ties to even), as float32."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((b >> 16) & np.uint32(1)) + np.uint32(0x7FFF)
    return ((b + r) & np.uint32(0xFFFF0000)).view(np.float32)


def unpack(theta):
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = theta[o:o + n].reshape(shp)
        o += n
    return out


def init_params(seed):
    """Glorot-uniform weights, zero biases, from numpy's PCG64 with `seed`;
    W3 is scaled by 0.1 so that the untrained correction is small."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shp in SHAPES:
        if name.startswith("W"):
            lim = np.sqrt(6.0 / (shp[0] + shp[1]))
            w = rng.uniform(-lim, lim, shp)
            if name == "W3":
                w *= 0.1
            parts.append(w.ravel())
        else:
            parts.append(np.zeros(shp).ravel())
    return np.concatenate(parts).astype(np.float32)


def forward(theta, x, round_bf16=True, dtype=np.float32):
    """y, (x_b, h1, h2): inputs and tanh activations as stored (bf16-rounded
    when round_bf16), layers accumulated in `dtype`."""
    p = {k: v.astype(dtype) for k, v in unpack(theta).items()}
    if round_bf16:
        def store(a):
            return bf16(a.astype(np.float32)).astype(dtype)
    else:
        def store(a):
            return a.astype(dtype)
    xb = store(x)
    h1 = store(np.tanh(xb @ p["W1"].T + p["b1"]))
    h2 = store(np.tanh(h1 @ p["W2"].T + p["b2"]))
    y = h2 @ p["W3"].T + p["b3"]
    return y, (xb, h1, h2)


def loss_and_grad(theta, x, t, round_bf16=True, dtype=np.float32):
    """L = (1/M) sum_rows sum_outputs (y - t)^2 and dL/dtheta (flat).  The
    tanh derivative uses the stored activation: 1 - h^2."""
    M = x.shape[0]
    p = {k: v.astype(dtype) for k, v in unpack(theta).items()}
    y, (xb, h1, h2) = forward(theta, x, round_bf16, dtype)
    d = y - t.astype(dtype)
    L = float(np.sum(d.astype(np.float64) ** 2) / M)
    dy = (2.0 / M) * d
    g = {"W3": dy.T @ h2, "b3": dy.sum(0)}
    dz2 = (dy @ p["W3"]) * (1 - h2 * h2)
    g["W2"], g["b2"] = dz2.T @ h1, dz2.sum(0)
    dz1 = (dz2 @ p["W2"]) * (1 - h1 * h1)
    g["W1"], g["b1"] = dz1.T @ xb, dz1.sum(0)
    return L, np.concatenate([g[name].ravel() for name, _ in SHAPES]).astype(dtype)


def adam_step(theta, g, m, v, t, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update in float32 (Kingma and Ba 2015, bias-corrected);
    returns new (theta, m, v).  t counts steps from 1."""
    f = np.float32
    m = f(beta1) * m + f(1 - beta1) * g
    v = f(beta2) * v + f(1 - beta2) * g * g
    mh = m / f(1 - beta1 ** t)
    vh = v / f(1 - beta2 ** t)
    theta = theta - f(lr) * mh / (np.sqrt(vh) + f(eps))
    return theta.astype(np.float32), m.astype(np.float32), v.astype(np.float32)
