"""The bench's whole-solve traffic model (bench.solve_traffic), on CPU: it
reproduces the per-iteration and per-application bytes of the 5-orbital
64x64x2048 model quoted with the path's roofline plan (676 GB per FP32 FLEX
iteration, 1352 GB in complex128, 198 GB per FP32 Eliashberg application)."""
import importlib.util
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
spec = importlib.util.spec_from_file_location("bench", ROOT / "bench.py")
bench = importlib.util.module_from_spec(spec)
spec.loader.exec_module(bench)

C2 = dict(Norb=5, Nk=2050, Nkall=4096, Nw=2048)


def st(it, n32=0, nmid=0, applies=0):
    return {"iterations": it, "iterations_fp32": n32, "iterations_fp64_fp32vertex": nmid, "applies": applies}


def test_per_iteration_and_application_bytes():
    assert abs(bench.solve_traffic(**C2, stats=st(1), precision="32") / 1e9 - 676) < 1
    assert abs(bench.solve_traffic(**C2, stats=st(1), precision="64") / 1e9 - 1352) < 2
    assert abs(bench.solve_traffic(**C2, stats=st(0, applies=1), precision="32") / 1e9 - 198) < 1


def test_mixed_phases_add_up():
    one32 = bench.solve_traffic(**C2, stats=st(1), precision="32")
    one64 = bench.solve_traffic(**C2, stats=st(1), precision="64")
    mixed = bench.solve_traffic(**C2, stats=st(18, n32=11, nmid=6, applies=10), precision="mixed")
    # the middle phase: 16-byte chi0/Sigma with an 8-byte vertex
    mid = one64 - 8 * 2 * (2050 * 2048) * 625
    apply64 = bench.solve_traffic(**C2, stats=st(0, applies=1), precision="64")
    assert abs(mixed - (11 * one32 + 6 * mid + 1 * one64 + 10 * apply64)) < 1e3
