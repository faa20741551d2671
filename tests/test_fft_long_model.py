"""Index model of the single-pass long-axis FFT (csrc/fft.cu,
fft_long_kernel), on CPU.

A CTA holds nl adjacent lines of length M = L1 * L2 (L1, L2 in {4, 16, 64})
in shared memory, each as L1 rows of L2 elements padded to L2 + 1.  Element
n = L2 n1 + n2 of a line sits in row n1, column n2.  The forward transform
runs length-L1 DFTs down each column, multiplies by w_M^(n2 k1) and runs
length-L2 DFTs along each row, which leaves frequency k = k1 + L1 k2 in row
k1, column k2.  That is the digit-transposed order of the plan's two-pass
four-step split, so the position tables stay as they are.  The backward
transform undoes the steps in reverse.  Each length-G^2 DFT is done in place
by G threads.  Thread j holds the G values G i + j and runs a radix-G DFT
over i, multiplies by w_L^(j kA) and writes back the slots it read.  Then
thread kA reads the slots G kA + j, runs a radix-G DFT over j and writes
frequency kA + G kB.  This test restates that arithmetic line by line and
checks it against numpy's FFT, so the kernel's addressing is verified before
it runs on a GPU."""
import numpy as np
import pytest

SQRT = {4: 2, 16: 4, 64: 8}


def dft(v, sign):
    R = len(v)
    k = np.arange(R)
    return np.exp(sign * 2j * np.pi * np.outer(k, k) / R) @ v


def w(t, L, sign):
    return np.exp(sign * 2j * np.pi * t / L)


def group_dft(buf, slot, L, sign, tw_line=None, M=None):
    """In-place length-L DFT of the elements slot(0..L-1) of buf by G = sqrt(L)
    emulated threads; tw_line: multiply output k by w_M^(tw_line * k)."""
    G = SQRT[L]
    # stage 1: thread j reads G i + j, DFT over i, twiddle w_L^(j kA), writes back the same slots
    regs = []
    for j in range(G):
        v = np.array([buf[slot(G * i + j)] for i in range(G)])
        v = dft(v, sign)
        v = v * w(j * np.arange(G), L, sign)
        regs.append(v)
    for j in range(G):
        for kA in range(G):
            buf[slot(G * kA + j)] = regs[j][kA]
    # stage 2: thread kA reads G kA + j, DFT over j, writes output kA + G kB
    regs = []
    for kA in range(G):
        u = np.array([buf[slot(G * kA + j)] for j in range(G)])
        regs.append(dft(u, sign))
    for kA in range(G):
        for kB in range(G):
            k = kA + G * kB
            val = regs[kA][kB]
            if tw_line is not None:
                val = val * w(tw_line * k, M, sign)
            buf[slot(k)] = val


def long_pass(lines, L1, L2, sign):
    """lines [nl, M] as stored on the axis -> the kernel's result per line."""
    nl, M = lines.shape
    ls = L1 * (L2 + 1)
    phys = lambda b, r, c: b * ls + r * (L2 + 1) + c
    buf = np.zeros(nl * ls, dtype=complex)
    for b in range(nl):
        for p in range(M):
            buf[phys(b, p // L2, p % L2)] = lines[b, p]
    for b in range(nl):
        if sign < 0:
            for n2 in range(L2):      # columns: DFT over n1, twiddle w_M^(n2 k1)
                group_dft(buf, lambda i, b=b, n2=n2: phys(b, i, n2), L1, sign, tw_line=n2, M=M)
            for k1 in range(L1):      # rows: DFT over n2 -> k2
                group_dft(buf, lambda i, b=b, k1=k1: phys(b, k1, i), L2, sign)
        else:
            for k1 in range(L1):      # rows: DFT over k2 -> n2, twiddle w_M^(k1 n2)
                group_dft(buf, lambda i, b=b, k1=k1: phys(b, k1, i), L2, sign, tw_line=k1, M=M)
            for n2 in range(L2):      # columns: DFT over k1 -> n1
                group_dft(buf, lambda i, b=b, n2=n2: phys(b, i, n2), L1, sign)
    out = np.zeros_like(lines)
    for b in range(nl):
        for p in range(M):
            out[b, p] = buf[phys(b, p // L2, p % L2)]
    return out


def digit_pos(k, L1, L2):
    """Where the plan stores frequency k of a four-step axis: (k / L1) + L2 (k % L1)."""
    return k // L1 + L2 * (k % L1)


@pytest.mark.parametrize("L1,L2", [(4, 4), (16, 16), (16, 64), (64, 16), (4, 64), (64, 64)])
def test_forward_matches_fft_in_digit_transposed_order(L1, L2):
    M = L1 * L2
    rng = np.random.default_rng(M + L1)
    x = rng.normal(size=(2, M)) + 1j * rng.normal(size=(2, M))
    got = long_pass(x, L1, L2, -1)
    ref = np.fft.fft(x, axis=1)
    k = np.arange(M)
    assert np.allclose(got[:, digit_pos(k, L1, L2)], ref, rtol=1e-11, atol=1e-11 * np.abs(ref).max())


@pytest.mark.parametrize("L1,L2", [(4, 4), (16, 64), (64, 16), (64, 64)])
def test_backward_inverts_forward(L1, L2):
    M = L1 * L2
    rng = np.random.default_rng(M + L2)
    X = rng.normal(size=(3, M)) + 1j * rng.normal(size=(3, M))
    stored = np.zeros_like(X)
    k = np.arange(M)
    stored[:, digit_pos(k, L1, L2)] = X          # spectrum in the plan's storage order
    got = long_pass(stored, L1, L2, +1)
    ref = np.fft.ifft(X, axis=1) * M             # unnormalised backward, natural order
    assert np.allclose(got, ref, rtol=1e-11, atol=1e-11 * np.abs(ref).max())


def test_shared_memory_of_the_long_pass():
    """4 lines (8-byte elements) or 2 lines (16-byte elements) of 64 x 65 fit 227 KB."""
    assert 4 * 64 * 65 * 8 <= 227 * 1024 and 2 * 64 * 65 * 16 <= 227 * 1024
