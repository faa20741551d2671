"""Parameter sweeps over many independent FLEX instances (config 3).

Instances have uneven sizes: 1 to 3 orbitals, square k meshes of 16 to 128
points per axis and 256 to 4096 Matsubara frequencies, with seeded hoppings
of the 5-orbital model's kind (shells (1,0), (1,1), (2,0), bandwidth 4 eV).
U is a fraction of the model's own Stoner U (uniform in [0.5, 0.95]), J = U/6,
T log-uniform in [0.005, 0.05] eV and the filling uniform in [0.7, 1.0]
electrons per orbital.

``run`` solves them one after another through the engine: the per-instance
loop.  ``run_packed`` solves them from several host threads at once, each
with its own engine context (its own CUDA stream), so that the kernels of
small instances, which fill only part of the GPU and are bound by launch
latency, overlap.  Instances are taken largest first, as long as the
estimated device footprint of those in flight stays within a budget.

    python -m pyrpa_gb300.sweep --count 256 --out sweep.json
    python -m pyrpa_gb300.sweep --count 256 --workers 4 --out packed.json
"""
from __future__ import annotations

import argparse
import json
import threading
import time
from dataclasses import asdict, dataclass

import numpy as np

ORBITALS = (1, 2, 3)
MESHES = (16, 32, 64, 128)
MATSUBARA = (256, 512, 1024, 4096)
J_OVER_U = 1.0 / 6.0
U_REF = 0.05  # reference U of the Stoner pass, small enough that chi0 S stays below 1


@dataclass(frozen=True)
class Instance:
    index: int
    Norb: int
    N: int            # k points per axis (N x N x 1)
    Nw: int           # Matsubara frequencies
    seed: int         # hopping seed
    u_frac: float     # U / U_Stoner
    temp: float       # eV
    n_per_orb: float  # electrons per orbital (both spins)

    @property
    def fill(self) -> float:
        """Electrons per spin, the reference's `fill`."""
        return 0.5 * self.n_per_orb * self.Norb


def draw(count: int = 256, seed: int = 0) -> list[Instance]:
    """`count` instances from numpy's PCG64 with `seed`."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        out.append(Instance(index=i, Norb=int(rng.choice(ORBITALS)), N=int(rng.choice(MESHES)),
                            Nw=int(rng.choice(MATSUBARA)), seed=int(rng.integers(1, 2 ** 31 - 1)),
                            u_frac=float(rng.uniform(0.5, 0.95)),
                            temp=float(np.exp(rng.uniform(np.log(0.005), np.log(0.05)))),
                            n_per_orb=float(rng.uniform(0.7, 1.0))))
    return out


def irr_count(N: int) -> int:
    """Irreducible k points of the time-reversal-reduced N x N mesh."""
    return N * N // 2 + 2 if N % 2 == 0 else (N * N + 1) // 2


def device_bytes(inst: Instance, elem: int = 16) -> int:
    """Rough HBM footprint of one FLEX solve: chi0 on the irreducible (q, nu)
    points, the padded G arrays of the convolutions and the DIIS history
    (m = 5) of Sigma, at `elem` bytes per complex value."""
    No, Nchi = inst.Norb, inst.Norb ** 2
    K = irr_count(inst.N) * inst.Nw
    P = inst.N * inst.N * 2 * inst.Nw
    return elem * (K * Nchi * Nchi + 2 * P * No * No + 2 * 5 * K * No * No + 4 * K * No * No)


def model(inst: Instance, U: float) -> dict:
    """Arrays of one instance at interaction U, through the engine's setup
    entry points (the layout of ``models.prepare``)."""
    from . import flibs as F
    from . import models
    rvec, ham_r = models.seeded_hoppings(inst.Norb, inst.seed, [(1, 0, 0), (1, 1, 0), (2, 0, 0)], dim=2,
                                         bandwidth=4.0)
    klist, kmap, invk = F.gen_irr_k_TRS(inst.N, inst.N, 1)
    hamk = F.gen_ham(klist, ham_r, rvec)
    eig, uni = F.get_eig(hamk)
    olist, site = F.get_chi_orb_list(inst.Norb)
    S, C = F.gen_SCmatrix(olist, site, U, J_OVER_U * U)
    w = F.gen_kpoint_weight(invk, len(klist))
    mu = models.bare_mu(eig, w, inst.fill, inst.temp)
    return dict(klist=klist, kmap=kmap, invk=invk, hamk=hamk, eig=eig, uni=uni, olist=olist, site=site, S=S, C=C,
                mu=mu)


def stoner_u(inst: Instance) -> float:
    """U at which the bare Stoner factor reaches 1: one FLEX iteration (whose
    chi0 is the bare one) at U_REF, U_Stoner = U_REF / Stoner(U_REF)."""
    from . import flibs as F
    m = model(inst, U_REF)
    F.mkself(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["mu"], inst.fill,
             inst.temp, inst.Nw, inst.N, inst.N, 1, False, False, scf_loop=1, eps=0.0)
    st = F.last_stats()["stoner"]
    if not st > 0:
        raise RuntimeError(f"instance {inst.index}: bare Stoner factor {st}")
    return U_REF / st


def solve(inst: Instance, eps: float = 1e-4, scf_loop: int = 300) -> dict:
    """One instance: its Stoner U, then the FLEX loop at u_frac * U_Stoner
    from G0 (DIIS m=5, mixing 0.5, rescale on).  Wall and device times in
    seconds, iterations, mu, final Stoner factor and residual."""
    from . import flibs as F
    t0 = time.perf_counter()
    U = inst.u_frac * stoner_u(inst)
    t1 = time.perf_counter()
    m = model(inst, U)
    t2 = time.perf_counter()
    sigma, mu = F.mkself(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["mu"],
                         inst.fill, inst.temp, inst.Nw, inst.N, inst.N, 1, False, False, eps=eps, pp=0.5,
                         scf_loop=scf_loop, sw_rescale=True)
    t3 = time.perf_counter()
    st = F.last_stats()
    dev_ms = sum(st[k] for k in ("t_chi0_ms", "t_vertex_ms", "t_sigma_ms", "t_diis_ms", "t_mu_ms", "t_dyson_ms",
                                 "t_stoner_ms"))
    return dict(asdict(inst), U=U, mu=mu, iterations=int(st["iterations"]), esterr=st["esterr"],
                stoner=st["stoner"], sigma_abs_sum=float(np.abs(sigma).sum()), t_stoner_u_s=t1 - t0,
                t_setup_s=t2 - t1, t_solve_s=t3 - t2, t_solve_device_s=dev_ms / 1e3)


def run(instances, eps: float = 1e-4, precision: int | None = None, log=None) -> list[dict]:
    """Solve the instances in order (largest device footprint first, so that
    the memory pool grows once); failures are recorded, not raised."""
    from . import flibs as F
    F.load_library()
    F.set_verbose(0)
    if precision is not None:
        F.set_precision(precision)
    out = []
    for inst in sorted(instances, key=device_bytes, reverse=True):
        try:
            r = solve(inst, eps)
        except RuntimeError as e:
            r = dict(asdict(inst), error=str(e))
        out.append(r)
        if log:
            log(r)
    return sorted(out, key=lambda r: r["index"])


def run_packed(instances, workers: int = 4, eps: float = 1e-4, precision: int | None = None,
               budget_bytes: float = 120e9, log=None) -> list[dict]:
    """Solve the instances from `workers` host threads, each on its own
    engine context, so that their kernels overlap on the GPU.  A thread takes
    the largest instance left whose estimated footprint (device_bytes) fits
    the budget beside those in flight; an instance above the budget runs
    when nothing else does.  Failures are recorded, not raised; the results
    come back in draw order and equal those of ``run``."""
    from . import flibs as F
    F.load_library()
    F.set_verbose(0)
    if precision is not None:
        F.set_precision(precision)  # the thread contexts copy the process settings
    pending = sorted(instances, key=device_bytes, reverse=True)
    cond = threading.Condition()
    state = dict(in_flight=0.0, running=0, peak=0.0)
    out, errors = [], []

    def take():
        with cond:
            while pending:
                for i, inst in enumerate(pending):
                    b = float(device_bytes(inst))
                    if state["running"] == 0 or state["in_flight"] + b <= budget_bytes:
                        pending.pop(i)
                        state["in_flight"] += b
                        state["running"] += 1
                        state["peak"] = max(state["peak"], state["in_flight"])
                        return inst, b
                cond.wait()
            return None, 0.0

    def worker():
        try:
            F.set_thread_stream(True)
            F.set_verbose(0)
        except RuntimeError as e:  # no context for this thread: the others carry on
            errors.append(str(e))
            return
        try:
            while True:
                inst, b = take()
                if inst is None:
                    return
                try:
                    r = solve(inst, eps)
                except Exception as e:  # recorded like run(); the thread goes on
                    r = dict(asdict(inst), error=str(e))
                with cond:
                    state["in_flight"] -= b
                    state["running"] -= 1
                    out.append(r)
                    if log:
                        log(r)
                    cond.notify_all()
        finally:
            F.set_thread_stream(False)

    threads = [threading.Thread(target=worker, name=f"sweep-{w}") for w in range(max(1, workers))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if pending:
        raise RuntimeError("no sweep thread could get an engine context: " + "; ".join(errors))
    run_packed.peak_bytes = state["peak"]
    return sorted(out, key=lambda r: r["index"])


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--count", type=int, default=256)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--eps", type=float, default=1e-4)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "32", "48", "64"])
    ap.add_argument("--workers", type=int, default=0,
                    help="host threads solving at once, each on its own stream (0: one after another)")
    ap.add_argument("--budget-gb", type=float, default=120.0,
                    help="estimated device footprint allowed in flight with --workers")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    prec = {"mixed": 3264, "32": 32, "48": 48, "64": 64}[a.precision]
    insts = draw(a.count, a.seed)
    log = lambda r: print(json.dumps(r), flush=True)  # noqa: E731
    t0 = time.perf_counter()
    if a.workers > 0:
        res = run_packed(insts, a.workers, a.eps, prec, a.budget_gb * 1e9, log=log)
    else:
        res = run(insts, a.eps, prec, log=log)
    wall = time.perf_counter() - t0
    ok = [r for r in res if "error" not in r]
    summary = dict(instances=len(res), solved=len(ok), wall_s=wall,
                   solve_s=sum(r["t_solve_s"] for r in ok), stoner_u_s=sum(r["t_stoner_u_s"] for r in ok),
                   iterations=sum(r["iterations"] for r in ok), precision=a.precision, eps=a.eps, seed=a.seed,
                   workers=a.workers)
    print(json.dumps(summary))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(dict(summary=summary, results=res), f)


if __name__ == "__main__":
    main()
