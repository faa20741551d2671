"""Algorithm model of the vertex kernel's warp Gauss-Jordan inverse
(csrc/flex.cu, warp_inverse_rot), on CPU.

The kernel keeps one matrix row per lane and restructures the textbook
in-place Gauss-Jordan elimination so that a step is little more than its
multiply-adds: the column being eliminated always sits in register slot 0
(each step writes slot s into slot s - 1 and the new column into slot N-1),
pivot rows are not divided by their pivot (each row is scaled once, at the
end, by the reciprocal of its own pivot), the pivot is the candidate with
the largest |Re| + |Im| taken from a key of the magnitude's top 27 bits and
the row label, row interchanges relabel lanes, and column interchanges are
applied only to the output positions.  This test restates those steps for a
32-lane warp in numpy and checks the result against numpy's inverse, the
singular flag, and that the pivot sequence equals the textbook partial
pivoting on matrices without near-ties."""
import numpy as np
import pytest

LANES = 32


def pivot_key(mag, label):
    bits = np.array([mag], dtype=np.float32).view(np.uint32)[0]
    return (int(bits) & ~31) | (31 - label)


def inverse_rot(A):
    """Returns (inverse, ok, pivot labels) following warp_inverse_rot."""
    N = A.shape[0]
    a = np.zeros((LANES, N), complex)
    a[:N] = A
    a[N:] = A[0]  # lanes >= N hold copies of row 0, as in the kernel
    label = np.arange(LANES)
    scale = np.zeros(LANES, complex)
    piv, ok = [], True
    for k in range(N):
        ak = a[:, 0].copy()
        keys = [pivot_key(abs(ak[l].real) + abs(ak[l].imag), label[l]) if (l < N and label[l] >= k) else 0
                for l in range(LANES)]
        best = max(keys)
        plabel = 31 - (best & 31)
        if not np.array([best & ~31], dtype=np.uint32).view(np.float32)[0] > 0:
            ok = False
        is_piv = label == plabel
        new_label = label.copy()
        new_label[label == k] = plabel
        new_label[(label != k) & is_piv] = k
        label = new_label
        piv.append(plabel)
        prow = a[np.flatnonzero(is_piv)[0]].copy()
        ip = 1 / prow[0] if ok else 0
        scale[is_piv] = ip
        f = np.where(is_piv, 0, -(ak * ip))
        nxt = np.empty_like(a)
        nxt[:, :N - 1] = a[:, 1:] + f[:, None] * prow[None, 1:]
        nxt[:, N - 1] = np.where(is_piv, 1, f)
        a = nxt
    pos = []
    for c in range(N):
        cc = c
        for k in range(N - 1, -1, -1):
            if cc == k:
                cc = piv[k]
            elif cc == piv[k]:
                cc = k
        pos.append(cc)
    out = np.zeros((N, N), complex)
    for lane in range(N):
        for j in range(N):
            out[label[lane], pos[j]] = scale[lane] * a[lane, j]
    return out, ok, piv


def textbook_pivots(A):
    """Partial pivoting of the textbook Gauss-Jordan (largest |Re| + |Im|, first maximum)."""
    M = A.astype(complex).copy()
    N = M.shape[0]
    out = []  # the physical row swapped into place at each step
    for k in range(N):
        cand = [(abs(M[r, k].real) + abs(M[r, k].imag), r) for r in range(k, N)]
        m = max(v for v, _ in cand)
        r = next(r for v, r in cand if v == m)
        out.append(r)
        M[[k, r]] = M[[r, k]]
        M[k] /= M[k, k]
        for i in range(N):
            if i != k:
                M[i] -= M[i, k] * M[k]
    return out


@pytest.mark.parametrize("N", [1, 2, 4, 9, 16, 25])
@pytest.mark.parametrize("kind", ["random", "dominant", "permuted"])
def test_inverse_matches_numpy(N, kind):
    rng = np.random.default_rng(100 * N + len(kind))
    A = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    if kind == "dominant":
        A += 5 * np.eye(N)
    if kind == "permuted":
        A = A[rng.permutation(N)]
    X, ok, _ = inverse_rot(A)
    ref = np.linalg.inv(A)
    assert ok
    assert np.abs(X - ref).max() <= 1e-10 * np.abs(ref).max()


def test_pivots_follow_partial_pivoting():
    rng = np.random.default_rng(5)
    for _ in range(20):
        A = rng.standard_normal((9, 9)) + 1j * rng.standard_normal((9, 9))
        _, _, piv = inverse_rot(A)
        assert piv == textbook_pivots(A)


def test_singular_matrix_is_flagged():
    _, ok, _ = inverse_rot(np.ones((4, 4), complex))
    assert not ok
