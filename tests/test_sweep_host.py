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


def test_run_records_failures_and_keeps_the_draw_order(monkeypatch):
    """run() solves the largest footprint first, records a failing instance
    instead of raising, and returns the results in draw order."""
    from pyrpa_gb300 import flibs
    calls = []

    def fake_solve(inst, eps=1e-4, scf_loop=300):
        calls.append(inst.index)
        if inst.index == 2:
            raise RuntimeError("singular G^-1 in the Dyson step")
        return dict(index=inst.index, iterations=3)

    monkeypatch.setattr(S, "solve", fake_solve)
    monkeypatch.setattr(flibs, "load_library", lambda *a, **k: None)
    monkeypatch.setattr(flibs, "set_verbose", lambda v: None)
    insts = S.draw(6, seed=1)
    res = S.run(insts)
    assert calls == [x.index for x in sorted(insts, key=S.device_bytes, reverse=True)]
    assert [r["index"] for r in res] == list(range(6))
    assert "error" in res[2] and "Dyson" in res[2]["error"]
    assert all("error" not in r for i, r in enumerate(res) if i != 2)


def test_run_packed_solves_each_instance_once_within_the_budget(monkeypatch):
    """run_packed() gives every worker thread its own context, solves each
    instance exactly once, keeps the estimated footprint in flight within the
    budget (an instance above it runs alone), records failures and returns
    the results in draw order."""
    import threading
    import time

    from pyrpa_gb300 import flibs
    lock = threading.Lock()
    seen, live, peaks, ctx_calls = [], [], [], []

    def fake_solve(inst, eps=1e-4, scf_loop=300):
        b = S.device_bytes(inst)
        with lock:
            seen.append(inst.index)
            live.append(b)
            peaks.append((sum(live), len(live), b))
        time.sleep(0.002)
        with lock:
            live.remove(b)
        if inst.index == 4:
            raise RuntimeError("zgesv failed in V_sigma")
        return dict(index=inst.index, iterations=5)

    monkeypatch.setattr(S, "solve", fake_solve)
    monkeypatch.setattr(flibs, "load_library", lambda *a, **k: None)
    monkeypatch.setattr(flibs, "set_verbose", lambda v: None)
    monkeypatch.setattr(flibs, "set_precision", lambda v: None)
    monkeypatch.setattr(flibs, "set_thread_stream", lambda on: ctx_calls.append(bool(on)))
    insts = S.draw(24, seed=2)
    budget = 2.0 * sorted(S.device_bytes(x) for x in insts)[len(insts) // 2]
    res = S.run_packed(insts, workers=4, precision=3264, budget_bytes=budget)
    assert sorted(seen) == list(range(24))
    assert [r["index"] for r in res] == list(range(24))
    assert "error" in res[4] and "zgesv" in res[4]["error"]
    for total, n, b in peaks:
        assert n == 1 or total <= budget * (1 + 1e-12)
    assert ctx_calls.count(True) == 4 and ctx_calls.count(False) == 4
    assert S.run_packed.peak_bytes <= max(budget, max(S.device_bytes(x) for x in insts))
