#!/usr/bin/env python
"""Time to a converged FLEX self-energy plus the linearized-Eliashberg
eigenvalue on one GB300, for the 5-orbital 64x64x2048 model (config c2).

One step = one full solve of the reference's calc_lin_eliashberg_eq path
(mkself to the residual eps -> G -> tail-corrected chi0 -> lin_eliash), run
through the engine's C ABI (pyrpa_gb_flex_eliash, host buffers in and out).
  value        device seconds of the solve with the inputs already in HBM
               (CUDA events on the library stream, between upload and download)
  e2e          wall seconds of the whole ABI call from host buffers, copies included
  roofline     the FFT passes (fft2_kernel<R, A, B>; every pass of the 64x64x4096
               transforms), the kernel that moves the most bytes, timed live per
               launch with CUDA events during the timed steps
  cpu_baseline the oracle's per-orbital-pair FFT convolution at full size on
               all host cores, extrapolated to one solve with this run's
               iteration and Eliashberg-application counts
Inputs are larger than L2 (every FFT array is >= 134 MB), so no L2 flush is
needed between steps.  `--impl reference` prints the CPU line only.
Under torchrun every rank solves its own copy of the model (replicas, no
collective on the data path); the reported time is the maximum over ranks.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
METRIC = "time-to-converged FLEX Σ+λ, 5-orb 64²×2048: FP32+warm-start vs plain FP64"
# FLEX iterations and Eliashberg operator applications of one c2 solve as
# measured by the GPU engine (FP32 bulk, eps 1e-4, DIIS 5, Arnoldi 10); the
# CPU-only reference arm extrapolates with them.
DEFAULT_COUNTS = {"c2": (30, 20), "c1": (30, 20), "c5": (30, 20)}


# ------------------------------------------------------ profiling cases
# Small launches of single engine kernels for ncu captures: each runs one ABI
# call on a synthetic input larger than L2 (129 MB) but a few hundred MB at
# most, so that a capture of one launch replays quickly.
#   vertex  get_vsigma_flex_nosoc_ on a 5-orbital chi0 (Nchi = 25), 130
#           irreducible q x 512 frequencies = 66,560 matrices
#   chi0    get_chi0_tail on a 5-orbital 16x16 mesh with 512 frequencies
#   flex    mkself, one FLEX iteration of the same model
#   fft     get_chi0 of a 1-orbital 64x64 mesh with 2048 frequencies: FFT
#           passes over 64x64x4096 arrays (134 MB in FP32)
def _profile_model(F, models, Norb=5, N=16, Nw=512, temp=0.02):
    rvec, ham_r = models.seeded_hoppings(Norb, 4, [(1, 0, 0), (1, 1, 0), (2, 0, 0)], dim=2, bandwidth=4.0)
    klist, kmap, invk = F.gen_irr_k_TRS(N, N, 1)
    hamk = F.gen_ham(klist, ham_r, rvec)
    eig, uni = F.get_eig(hamk)
    olist, site = F.get_chi_orb_list(Norb)
    S, C = F.gen_SCmatrix(olist, site, 1.2, 0.2)
    w = F.gen_kpoint_weight(invk, len(klist))
    mu = models.bare_mu(eig, w, 0.6 * Norb, temp)
    return dict(Norb=Norb, N=N, Nw=Nw, temp=temp, klist=klist, kmap=kmap, invk=invk, hamk=hamk, eig=eig, uni=uni,
                olist=olist, S=S, C=C, mu=mu)


def profile_case(case: str, precision: int, repeat: int) -> int:
    sys.path.insert(0, str(ROOT))
    from pyrpa_gb300 import flibs as F, models
    F.load_library()
    F.set_verbose(0)
    F.set_precision(precision)
    t0 = time.perf_counter()
    for _ in range(repeat):
        if case == "vertex":
            Nchi, Nk, Nw = 25, 130, 512
            rng = np.random.default_rng(0)
            chi = 0.05 * (rng.standard_normal((Nchi, Nchi, Nw, Nk)) + 1j * rng.standard_normal((Nchi, Nchi, Nw, Nk)))
            olist, site = F.get_chi_orb_list(5)
            S, C = F.gen_SCmatrix(olist, site, 1.2, 0.2)
            # the raw entry with explicit Nk, Nw (the Python wrapper reads
            # them off the array the way the reference wrapper does)
            F._call("get_vsigma_flex_nosoc_", chi, S, C, F.i64(Nk), F.i64(Nw), F.i64(Nchi))
        elif case == "chi0":
            m = _profile_model(F, models)
            Gk = F.gen_Green0(m["eig"], m["uni"], m["mu"], m["temp"], m["Nw"])
            F.get_chi0_tail(m["S"], m["C"], Gk, m["eig"], m["uni"], m["olist"], m["kmap"], m["invk"], m["mu"],
                            m["temp"], m["N"], m["N"], 1)
        elif case == "fft":
            m = _profile_model(F, models, Norb=1, N=64, Nw=2048, temp=0.01)
            Gk = F.gen_Green0(m["eig"], m["uni"], m["mu"], m["temp"], m["Nw"])
            F.get_chi0(m["S"], m["C"], Gk, m["olist"], m["kmap"], m["invk"], m["temp"], m["N"], m["N"], 1)
        else:
            m = _profile_model(F, models)
            F.mkself(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["mu"],
                     0.6 * m["Norb"], m["temp"], m["Nw"], m["N"], m["N"], 1, False, False, scf_loop=1, eps=1e-4,
                     pp=0.5, sw_tail=True, sw_rescale=True)
    print(f"{case}: {repeat} call(s) in {time.perf_counter() - t0:.3f} s", flush=True)
    return 0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--profile-case", choices=["vertex", "chi0", "flex", "fft"],
                   help="run one small profiling case instead of the benchmark")
    p.add_argument("--repeat", type=int, default=1, help="calls of the profiling case")
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--config", default="c2", choices=["c1", "c2", "c5"])
    p.add_argument("--precision", default="mixed", choices=["mixed", "32", "64"],
                   help="mixed: FP32 bulk to the FP32 rounding floor, then double-float bulk to eps")
    p.add_argument("--eps", type=float, default=1.0e-4)
    p.add_argument("--scf-loop", type=int, default=300)
    p.add_argument("--no-tail", action="store_true")
    p.add_argument("--coarse", default="2,2",
                   help="warm start: k-mesh and frequency divisors of the coarse solve ('1,1' = cold start)")
    p.add_argument("--cpu-pairs", type=int, default=0, help="orbital pairs in the CPU sample (0: one per core)")
    p.add_argument("--flex-iters", type=int, default=0)
    p.add_argument("--applies", type=int, default=0)
    p.add_argument("--with-fp64", action="store_true",
                   help="after the timed steps, solve once more in plain FP64 from G0 (the metric's denominator) "
                        "and report its time and the lambda, Sigma and mu differences")
    return p.parse_args()


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------- CPU baseline
def _cpu_pair_worker(args):
    """One reference orbital-pair convolution at full grid size with the
    oracle (pad G on the full grid, two forward 4-D FFTs, the G(r,t)G(-r,-t)
    product, one backward FFT, gather to the irreducible mesh) on random data:
    the unit of work of chi0_conv_acc / calc_sigma / mkdelta_nsoc."""
    Nx, Ny, Nz, Nw, reps, seed = args
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    sys.path.insert(0, str(ROOT))
    from oracle import flex_oracle as FO
    klist, kmap, invk = FO.generate_irr_kpoint_inv(Nx, Ny, Nz)
    grid = FO.KGrid(kmap, invk, Nx, Ny, Nz)
    rng = np.random.default_rng(seed)
    G = (rng.standard_normal((len(klist), Nw, 1, 1)) + 1j * rng.standard_normal((len(klist), Nw, 1, 1)))
    t0 = time.perf_counter()
    for _ in range(reps):
        A = np.fft.fftn(grid.pad_green(G, 0, 0))
        B = np.fft.fftn(grid.pad_green(G, 0, 0))
        tmp = np.fft.ifftn(-A * FO._reverse_all(B))
        grid.gather_irr(tmp, Nw)
    return time.perf_counter() - t0, reps


def cpu_pair_rate(cfg, npairs: int):
    """Pairs per second on all host cores (spawned workers, one pair each)."""
    cores = os.cpu_count() or 1
    npairs = npairs or cores
    work = [(cfg["Nx"], cfg["Ny"], cfg["Nz"], cfg["Nw"], 1, i) for i in range(npairs)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(processes=min(cores, npairs)) as pool:
        res = pool.map(_cpu_pair_worker, work)
    wall = time.perf_counter() - t0
    return npairs / wall, min(cores, npairs), npairs, wall


def pair_counts(cfg, tail: bool):
    Nchi = cfg["Norb"] ** 2
    nirr = Nchi * (Nchi + 1) // 2
    per_iter = (3 * nirr if tail else nirr) + Nchi * Nchi
    no = cfg["Norb"]
    per_apply = sum(1 for a in range(no) for c in range(no) for b in range(no) for d in range(no) if a >= b)
    final_chi0 = 3 * nirr if tail else nirr
    return per_iter, per_apply, final_chi0


def cpu_seconds(cfg, tail, iters, applies, rate):
    per_iter, per_apply, final_chi0 = pair_counts(cfg, tail)
    return (iters * per_iter + final_chi0 + applies * per_apply) / rate


# ------------------------------------------------------------------ main
def solve_traffic(Norb: int, Nk: int, Nkall: int, Nw: int, stats: dict, precision: str) -> float:
    """Algorithmic HBM bytes of one fine solve (the coarse warm start left
    out), with P = Nkall 2Nw, K = Nk Nw, Nchi = Norb^2 and an ideal 4-D FFT of
    two read-write sweeps:
      per FLEX iteration        B [4P (2 Norb^2 + Nchi(Nchi+1)/2 + Nchi^2) + P Nchi^2 + 16 K Norb^2]
                                + Bv 2 K Nchi^2
      per Eliashberg application  Be [8P Norb^2 + 2P Nchi^2 + 4K Norb^2]
    B, Bv and Be are the bytes of a complex chi0/Sigma, vertex and Eliashberg
    element in each phase: 8 for FP32, 16 for FP64 and double-float."""
    nchi = Norb * Norb
    P, K = Nkall * 2 * Nw, Nk * Nw

    def it_bytes(B, Bv):
        return (B * (4 * P * (2 * Norb ** 2 + nchi * (nchi + 1) // 2 + nchi ** 2) + P * nchi ** 2
                     + 16 * K * Norb ** 2) + Bv * 2 * K * nchi ** 2)

    n = int(stats["iterations"])
    if precision == "mixed":
        n32, nmid = int(stats["iterations_fp32"]), int(stats["iterations_fp64_fp32vertex"])
        flex = n32 * it_bytes(8, 8) + nmid * it_bytes(16, 8) + (n - n32 - nmid) * it_bytes(16, 16)
        be = 16
    elif precision == "32":
        flex, be = n * it_bytes(8, 8), 8
    else:
        flex, be = n * it_bytes(16, 16), 16
    return float(flex + int(stats["applies"]) * be * (8 * P * Norb ** 2 + 2 * P * nchi ** 2 + 4 * K * Norb ** 2))


def max_over_ranks(values, dist):
    """Replicas: every rank solved its own instance; the job's time is the
    slowest rank's (all-reduce MAX, then a barrier)."""
    import torch
    t = torch.tensor(values, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return [float(x) for x in t]


def main():
    a = parse()
    if a.profile_case:
        return profile_case(a.profile_case, {"mixed": 32, "32": 32, "64": 64}[a.precision], a.repeat)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    sys.path.insert(0, str(ROOT))
    from pyrpa_gb300 import models

    cfg = dict(models.CONFIGS[a.config])
    tail = not a.no_tail
    config = {"workload": f"{a.config}: {cfg['Norb']}-orbital {cfg['Nx']}x{cfg['Ny']}x{cfg['Nz']} k-mesh, "
                          f"{cfg['Nw']} Matsubara, FLEX+linearized Eliashberg",
              "Norb": cfg["Norb"], "k_mesh": [cfg["Nx"], cfg["Ny"], cfg["Nz"]], "Nw": cfg["Nw"],
              "U": cfg["U"], "J": cfg["J"], "T": cfg["temp"], "fill_per_spin": cfg["fill"], "eps": a.eps,
              "chi0": "tail-corrected" if tail else "sharp cutoff",
              "parallelism": f"replicas x{a.gpus}" if a.gpus > 1 else "single GPU",
              "l2": "inputs larger than L2 (FFT arrays >= 134 MB); no flush"}

    if a.impl == "reference":
        if rank != 0:
            return 0
        iters, applies = (a.flex_iters or DEFAULT_COUNTS[a.config][0]), (a.applies or DEFAULT_COUNTS[a.config][1])
        vals = []
        for i in range(a.warmup + a.steps):
            rate, cores, npairs, wall = cpu_pair_rate(cfg, a.cpu_pairs)
            if i >= a.warmup:
                vals.append(cpu_seconds(cfg, tail, iters, applies, rate))
        v = statistics.mean(vals)
        sample = (f"{npairs} full-size orbital-pair FFT convolutions per step on {cores} spawned numpy workers, "
                  f"extrapolated with {iters} FLEX iterations and {applies} Eliashberg applications")
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": 0, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "c128", "data": "synthetic seeded tight-binding model",
                "config": config,
                "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": "port", "sample": sample},
                "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0

    from pyrpa_gb300 import flibs as F

    F.load_library()
    F.set_verbose(0)
    F.set_precision({"mixed": F.MIXED, "32": 32, "64": 64}[a.precision])
    m = models.prepare(a.config)
    c = m["cfg"]
    coarse = tuple(int(x) for x in a.coarse.split(","))
    call = dict(mu=m["mu"], fill=c["fill"], temp=c["temp"], Nw=c["Nw"], Nx=c["Nx"], Ny=c["Ny"], Nz=c["Nz"],
                gap_sym=c["gap_sym"], eps=a.eps, scf_loop=a.scf_loop, sw_tail=tail, sw_rescale=True, coarse=coarse)
    config["warm_start"] = ("none (cold G0 start)" if coarse == (1, 1) else
                            f"coarse-mesh seed: {c['Nx'] // coarse[0]}x{c['Ny'] // coarse[0]} k mesh, "
                            f"{c['Nw'] // coarse[1]} frequencies, FP32 bulk (itself seeded one level further "
                            f"down), interpolated to the full mesh")

    def solve():
        return F.flex_eliash(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"],
                             m["init"], m["plist"], **call)

    for _ in range(a.warmup):
        solve()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        dist.barrier()
    F.fft_profile(True)
    F.fft_stats()
    k0 = F.kernel_launches()
    dev, wall, res = [], [], None
    with ClockSampler(local if world == 1 else 0) as clk:
        for _ in range(a.steps):
            t0 = time.perf_counter()
            res = solve()
            wall.append(time.perf_counter() - t0)
            dev.append(res["compute_ms"] / 1e3)
    F.fft_profile(False)
    fft = F.fft_stats()
    launches = F.kernel_launches() - k0
    stats = F.last_stats()
    value, e2e = max(dev), max(wall)
    if dist is not None:
        value, e2e = max_over_ranks([value, e2e], dist)
    if rank != 0:
        return 0
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = (fft["bytes"] / (fft["ms"] / 1e3) / 1e9) if fft["ms"] > 0 else None
    per_launch_bytes = fft["bytes"] / max(1, fft["launches"])
    # DRAM bytes per algorithmic byte of an FFT pass, from an ncu capture of
    # fft2_kernel<float,8,8> on one 64x64x4096 array (dram__bytes_read.sum +
    # dram__bytes_write.sum = 208.7 MB over 268.4 MB algorithmic, mean of 3
    # launches; the write total misses what is still in L2 at kernel end)
    traffic_per_byte = 208.7 / 268.4
    in_bytes = sum(x.nbytes for x in (m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"],
                                        m["uni"], m["init"], m["plist"]))
    out_bytes = res["sigmak"].nbytes + res["gap"].nbytes
    iters, applies = int(stats["iterations"]), int(stats["applies"])
    solve_bytes = solve_traffic(c["Norb"], len(m["klist"]), len(m["kmap"]), c["Nw"], stats, a.precision)
    solve_s = value - stats["t_warm_ms"] / 1e3
    rate, cores, npairs, cwall = cpu_pair_rate(c, a.cpu_pairs)
    cpu_v = cpu_seconds(c, tail, iters, applies, rate)
    config.update({"flex_iterations": iters, "eliashberg_applications": applies, "lambda": res["lam"],
                   "lambda_top4": [float(x) for x in F.last_ritz(4)],
                   "warm_start_iterations": int(stats["iterations_coarse"]),
                   "warm_start_ms": stats["t_warm_ms"],
                   "stoner": res["stoner"], "mu": res["mu"], "esterr": stats["esterr"],
                   "precision": {"mixed": f"FP32 bulk for {int(stats['iterations_fp32'])} iterations, double-float chi0 "
                                          f"and Sigma with FP32 vertex for {int(stats['iterations_fp64_fp32vertex'])}, "
                                          f"then double-float chi0, vertex and Sigma to eps; Eliashberg stage "
                                          f"double-float (chi0, V_Delta, contractions)",
                                 "32": "FP32 bulk", "64": "FP64"}[a.precision]})
    line = {
        "metric": METRIC, "value": value, "unit": "s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": {"mixed": "c64+c128", "32": "c64", "64": "c128"}[a.precision], "data": "synthetic seeded tight-binding model",
        "config": config,
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": int(in_bytes), "d2h_bytes_per_step": int(out_bytes)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "fft2_kernel (FFT passes)", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                     "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback",
                     "bytes_per_launch": per_launch_bytes, "launches": fft["launches"],
                     "avg_launch_ms": fft["ms"] / max(1, fft["launches"]),
                     "traffic": per_launch_bytes * traffic_per_byte,
                     "traffic_source": "ncu capture of one 64x64x4096 FP32 pass, scaled by bytes per launch"},
        "solve_roofline": {"bound": "hbm", "bytes": solve_bytes, "seconds": solve_s,
                           "achieved": solve_bytes / solve_s / 1e9 if solve_s > 0 else None, "peak": peak,
                           "unit": "GB/s", "frac": solve_bytes / solve_s / 1e9 / peak if solve_s > 0 else None,
                           "scope": "fine FLEX iterations and Eliashberg applications, algorithmic bytes with an "
                                    "ideal two-sweep 4-D FFT; the coarse warm start is left out of bytes and time"},
        "cpu_baseline": {"value": cpu_v, "unit": "s", "cores": cores, "kind": "port",
                         "sample": f"{npairs} full-size orbital-pair FFT convolutions (oracle, numpy) in {cwall:.1f} s "
                                   f"on {cores} spawned workers, extrapolated with this run's {iters} FLEX iterations "
                                   f"and {applies} Eliashberg applications (FFT-pair work only)"},
        "clocks": clk.summary(),
        "stages_ms": {k: v for k, v in stats.items() if k.startswith("t_")},
    }
    if a.with_fp64:
        line["plain_fp64"] = plain_fp64_comparison(F, solve_args=(m, call), res=res)
    print(json.dumps(line), flush=True)
    return 0


def plain_fp64_comparison(F, solve_args, res) -> dict:
    """The same model solved in plain FP64 from G0 (no warm start), to the same
    eps: its device seconds and how far the fast form's lambda, Sigma and mu
    sit from it."""
    m, call = solve_args
    F.set_precision(64)
    ref = F.flex_eliash(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"],
                        m["init"], m["plist"], **dict(call, coarse=(1, 1)))
    st = F.last_stats()
    return {"seconds": ref["compute_ms"] / 1e3, "flex_iterations": int(st["iterations"]), "lambda": ref["lam"],
            "lambda_rel_diff": abs(res["lam"] - ref["lam"]) / abs(ref["lam"]),
            "sigma_max_rel_diff": float(np.abs(res["sigmak"] - ref["sigmak"]).max() / np.abs(ref["sigmak"]).max()),
            "mu_diff": abs(res["mu"] - ref["mu"])}


if __name__ == "__main__":
    sys.exit(main())
