"""Candidate settings of the FFT autotuner (PYRPA_GB_FFT_TUNE=1), on CPU:
the heuristic comes first, four-step splits have two-level kernels on both
lengths, and every setting's shared memory fits its kernel's launch."""
import numpy as np
import pytest

FAST = {(8, 8), (4, 8), (8, 4), (4, 4), (2, 8), (8, 2), (2, 4), (4, 2), (2, 2), (3, 8), (8, 3), (3, 4), (4, 3),
        (3, 3), (2, 3), (3, 2), (5, 5), (4, 5), (5, 4), (2, 5), (5, 2), (3, 5), (5, 3), (5, 8), (8, 5)}


def fast_pair(L):
    """The two-level kernel of length L (the closest pair), as the plan picks it."""
    best = None
    for a, b in FAST:
        if a * b == L and (best is None or abs(a - b) < abs(best[0] - best[1])):
            best = (a, b)
    return best


def fits(L, lines, elem):
    p = fast_pair(L)
    if p:
        return lines * p[0] * (p[1] + 1) * elem <= 48 * 1024
    return 2 * lines * L * elem <= 96 * 1024


@pytest.fixture(scope="module")
def F():
    from pyrpa_gb300 import build, flibs
    if not build.LIB.exists():
        build.build()
    flibs.load_library()
    return flibs


@pytest.mark.parametrize("n", [64, 32, 24, 4096, 2048, 1024, 512, 6, 7 * 64, 1])
@pytest.mark.parametrize("elem", [8, 16])
def test_candidates(F, n, elem):
    c = F.fft_candidates(n, elem)
    if n == 1:
        assert c == []
        return
    assert c[0] == (0, 0)
    assert len(set(c)) == len(c)
    for L1, lines in c[1:]:
        assert lines in (8, 16, 32, 64)
        if L1:
            assert n > 64 and n % L1 == 0 and n // L1 <= 64
            assert fast_pair(L1) and fast_pair(n // L1)
            assert fits(L1, lines, elem) and fits(n // L1, lines, elem)
        else:
            assert n <= 64 or fast_pair(n) is None
            assert fits(n, lines, elem)


def test_expected_sets(F):
    # 64: one pass, lines up to 64 in FP32; 64 lines of 16-byte elements exceed 48 KB
    assert F.fft_candidates(64, 8) == [(0, 0), (0, 8), (0, 16), (0, 32), (0, 64)]
    assert F.fft_candidates(64, 16) == [(0, 0), (0, 8), (0, 16), (0, 32)]
    # 4096 = 64 x 64 only; 2048 = 32 x 64 or 64 x 32
    assert {L1 for L1, _ in F.fft_candidates(4096, 8)[1:]} == {64}
    assert {L1 for L1, _ in F.fft_candidates(2048, 8)[1:]} == {32, 64}
    # 448 = 7 x 64 has no two-level split: only the heuristic
    assert F.fft_candidates(7 * 64, 8) == [(0, 0)]
