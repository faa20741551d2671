"""Index model of the FFT plane pass (csrc/fft.cu, fft_plane_kernel), on CPU.

The plane pass transforms the x and y axes of one (x, y) plane in shared
memory: rows of the plane sit at stride nx + 1 (one element of padding), the
x lines are transformed with element stride 1 and line stride nx + 1, the y
lines with element stride nx + 1 and line stride 1, by the same Stockham
stage as the other passes (Govindaraju et al., SC08), ping-ponging between
two buffers.  This test restates that index arithmetic line by line in numpy
and checks it against numpy's 2-D FFT, so that the kernel's addressing is
verified before it runs on a GPU."""
import numpy as np
import pytest

PREF = (8, 4, 2, 3, 5, 7, 11, 13)


def factor_line(L):
    """Radix list of csrc/fft.cu factor_line: 8, 4, 2, 3, 5, 7, 11, 13 greedily."""
    out, n = [], L
    for r in PREF:
        while n % r == 0 and n > 1:
            out.append(r)
            n //= r
    assert n == 1
    return out


def line_table(L):
    t = np.arange(L)
    return np.exp(-2j * np.pi * t / L)


def twid(tab, t, sign):
    w = tab[t]
    return w if sign < 0 else np.conj(w)


def dft(v, sign):
    R = len(v)
    k = np.arange(R)
    return np.exp(sign * 2j * np.pi * np.outer(k, k) / R) @ v


def stage2(inp, out, L, Ns, nl, es, ls, sign, tab, rad):
    """One Stockham stage over nl lines: line b starts at b * ls, element j of
    a line sits at j * es (the kernel's stage with element and line strides)."""
    nbf = L // rad
    tstride = L // (Ns * rad)
    for idx in range(nl * nbf):
        b, j = divmod(idx, nbf)
        jj = j % Ns
        v = np.empty(rad, dtype=complex)
        for r in range(rad):
            v[r] = inp[b * ls + (j + r * nbf) * es]
            if r > 0 and jj > 0:
                v[r] *= twid(tab, r * jj * tstride, sign)
        v = dft(v, sign)
        idxD = (j // Ns) * Ns * rad + jj
        for r in range(rad):
            out[b * ls + (idxD + r * Ns) * es] = v[r]


def plane_pass(plane, sign):
    """plane [ny, nx] (x fastest, as stored) -> its 2-D DFT, by the kernel's steps."""
    ny, nx = plane.shape
    sx = nx + 1
    buf = [np.zeros(ny * sx, dtype=complex), np.zeros(ny * sx, dtype=complex)]
    for e in range(nx * ny):
        y, x = divmod(e, nx)
        buf[0][y * sx + x] = plane.ravel()[e]
    cur = 0
    Ns = 1
    for rad in factor_line(nx):
        stage2(buf[cur], buf[1 - cur], nx, Ns, ny, 1, sx, sign, line_table(nx), rad)
        cur = 1 - cur
        Ns *= rad
    Ns = 1
    for rad in factor_line(ny):
        stage2(buf[cur], buf[1 - cur], ny, Ns, nx, sx, 1, sign, line_table(ny), rad)
        cur = 1 - cur
        Ns *= rad
    out = np.zeros(nx * ny, dtype=complex)
    for e in range(nx * ny):
        y, x = divmod(e, nx)
        out[e] = buf[cur][y * sx + x]
    return out.reshape(ny, nx)


@pytest.mark.parametrize("nx,ny", [(8, 8), (16, 4), (6, 10), (5, 7), (12, 13), (64, 2), (24, 18)])
@pytest.mark.parametrize("sign", [-1, 1])
def test_plane_pass_model_matches_fft2(nx, ny, sign):
    rng = np.random.default_rng(nx * 100 + ny)
    a = rng.normal(size=(ny, nx)) + 1j * rng.normal(size=(ny, nx))
    got = plane_pass(a, sign)
    ref = np.fft.fft2(a) if sign < 0 else np.fft.ifft2(a) * nx * ny
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_shared_memory_of_the_plane_pass():
    """Two padded buffers of ny (nx + 1) elements must fit the 227 KB a block
    can have: 64 x 64 planes in 8- and 16-byte elements."""
    for elem in (8, 16):
        assert 2 * 64 * 65 * elem <= 227 * 1024
