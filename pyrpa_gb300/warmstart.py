"""Learned warm start of the FLEX loop.

The coarse-mesh warm start solves a model on a k mesh and Matsubara set
divided by (kdiv, wdiv), interpolates that Sigma to the fine mesh
(``flibs.sigma_interp``: Fourier interpolation over k, c0 + c1/(i w) beyond
the coarse frequencies) and starts the fine loop from it.  ``LearnedWarmStart``
refines that seed with a small network before the fine loop runs; the loop
then iterates to its own residual as usual, so the result is the fine mesh's
fixed point whatever the seed.

The network sees one row per fine irreducible k, Matsubara index n and band
pair (i, j): 16 features of the seed in the band basis U^dagger Sigma U, the
band energies, w_n against the coarse cutoff and the model's descriptors,
and predicts the band-basis correction in units of max |Sigma_seed|
(16 -> 64 -> 64 -> 2, tanh; FP32 weights, bf16 inputs and activations, FP32
gradients, Adam).  Features, forward and backward passes, Adam and the
correction run in libfmod.so (csrc/lws.cu); this module draws the training
pairs, keeps a copy of the parameters and runs the solves.

The reference has no counterpart: a pyrpa user seeds mkself by hand through
sigma.bin (fself.f90:742-780) after plibs.regrid_sigma_bin.

    python -m pyrpa_gb300.warmstart --train 8 --test 4     # train and measure
"""
from __future__ import annotations

import ctypes
import time
from ctypes import byref, c_double, c_int64
from pathlib import Path

import numpy as np

from . import flibs as F
from .flibs import _call, dbl, i64

NF, NH, NO = 16, 64, 2
SHAPES = (("W1", (NH, NF)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NO, NH)), ("b3", (NO,)))
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)  # 5378


def init_params(seed: int = 0) -> np.ndarray:
    """Glorot-uniform weights (numpy PCG64 with `seed`), zero biases, the
    output layer scaled by 0.1 so that the untrained correction is small."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shp in SHAPES:
        if name.startswith("W"):
            lim = np.sqrt(6.0 / (shp[0] + shp[1]))
            w = rng.uniform(-lim, lim, shp) * (0.1 if name == "W3" else 1.0)
            parts.append(w.ravel())
        else:
            parts.append(np.zeros(int(np.prod(shp))))
    return np.concatenate(parts).astype(np.float32)


def descriptors(U: float, J: float, temp: float, fill: float, Norb: int, stoner_c: float, mu_c: float, eig,
                sigma_seed) -> np.ndarray:
    """desc[9] of the C ABI: U, J, T, electrons per spin, Stoner factor and mu
    of the coarse solve, band width W of the fine mesh, max |Sigma_seed|
    (floored at 1e-12) and Norb."""
    W = float(np.max(eig) - np.min(eig))
    s = max(float(np.abs(sigma_seed).max()), 1e-12)
    return np.array([U, J, temp, fill, stoner_c, mu_c, W, s, Norb], dtype=np.float64)


def all_pairs(Nk: int, Nw: int) -> np.ndarray:
    """Every (k, n) pair [Nk * Nw, 2], k fastest."""
    n, k = np.meshgrid(np.arange(Nw), np.arange(Nk), indexing="ij")
    return np.stack([k.ravel(), n.ravel()], axis=1).astype(np.int64)


def sample_pairs(Nk: int, Nw: int, count: int, seed: int = 0) -> np.ndarray:
    """`count` distinct (k, n) pairs drawn uniformly (all of them when count
    >= Nk * Nw), in increasing pair order."""
    total = Nk * Nw
    if count >= total:
        return all_pairs(Nk, Nw)
    p = np.sort(np.random.default_rng(seed).choice(total, size=count, replace=False))
    return np.stack([p % Nk, p // Nk], axis=1).astype(np.int64)


def _sig(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def features(sigma_seed, uni, eig, Nw_c: int, desc, pairs, sigma_fine=None):
    """Rows of the given (k, n) pairs: x [P * Norb^2, 16] (the bf16 features
    as float32) and, with sigma_fine, the targets t [P * Norb^2, 2].  Arrays in
    the wrappers' layouts: sigma [Norb, Norb, Nw, Nk], uni [Nk, Norb, Norb],
    eig [Nk, Norb]."""
    sigma_seed = _sig(sigma_seed)
    Norb, _, Nw, Nk = sigma_seed.shape
    pairs = np.ascontiguousarray(pairs, dtype=np.int64)
    P = len(pairs)
    x = np.zeros((P * Norb * Norb, NF), dtype=np.float32)
    t = np.zeros((P * Norb * Norb, 2), dtype=np.float32) if sigma_fine is not None else None
    sf = _sig(sigma_fine) if sigma_fine is not None else None
    _call("pyrpa_gb_lws_features", x, t.ctypes.data_as(ctypes.c_void_p) if t is not None else None, sigma_seed,
          sf.ctypes.data_as(ctypes.c_void_p) if sf is not None else None, np.ascontiguousarray(uni),
          np.ascontiguousarray(eig), pairs, i64(P), i64(Nk), i64(Nw), i64(Nw_c), i64(Norb),
          np.ascontiguousarray(desc, dtype=np.float64))
    return x, t


class LearnedWarmStart:
    """One network and its training rows, held in HBM by the library."""

    def __init__(self, params=None, seed: int = 0):
        h = c_int64(0)
        _call("pyrpa_gb_lws_create", byref(h))
        self.handle = h.value
        self.params = init_params(seed) if params is None else params

    def close(self) -> None:
        if getattr(self, "handle", 0):
            F.load_library().pyrpa_gb_lws_destroy(i64(self.handle))
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> np.ndarray:
        out = np.zeros(NPARAM, dtype=np.float32)
        _call("pyrpa_gb_lws_get_params", i64(self.handle), out, i64(NPARAM))
        return out

    @params.setter
    def params(self, theta) -> None:
        """Setting the parameters also resets the Adam moments."""
        theta = np.ascontiguousarray(theta, dtype=np.float32)
        if theta.shape != (NPARAM,):
            raise ValueError(f"expected {NPARAM} parameters, got {theta.shape}")
        _call("pyrpa_gb_lws_set_params", i64(self.handle), theta, i64(NPARAM))

    def save(self, path) -> None:
        np.savez(Path(path), params=self.params, shapes=np.array([NF, NH, NO]))

    @classmethod
    def load(cls, path) -> "LearnedWarmStart":
        with np.load(Path(path)) as f:
            if tuple(f["shapes"]) != (NF, NH, NO):
                raise ValueError("saved network has other layer sizes")
            return cls(params=f["params"])

    # --------------------------------------------------------- training set
    def add_samples(self, sigma_seed, sigma_fine, uni, eig, Nw_c: int, desc, pairs) -> None:
        sigma_seed = _sig(sigma_seed)
        Norb, _, Nw, Nk = sigma_seed.shape
        pairs = np.ascontiguousarray(pairs, dtype=np.int64)
        _call("pyrpa_gb_lws_add_samples", i64(self.handle), sigma_seed, _sig(sigma_fine), np.ascontiguousarray(uni),
              np.ascontiguousarray(eig), pairs, i64(len(pairs)), i64(Nk), i64(Nw), i64(Nw_c), i64(Norb),
              np.ascontiguousarray(desc, dtype=np.float64))

    def clear_samples(self) -> None:
        _call("pyrpa_gb_lws_clear_samples", i64(self.handle))

    @property
    def num_rows(self) -> int:
        n = c_int64(0)
        _call("pyrpa_gb_lws_num_samples", i64(self.handle), byref(n))
        return n.value

    # ------------------------------------------------------------ training
    def loss_grad(self):
        """(loss, grad): mean over the training rows of sum (y - t)^2."""
        loss = c_double(0.0)
        g = np.zeros(NPARAM, dtype=np.float32)
        _call("pyrpa_gb_lws_loss_grad", i64(self.handle), byref(loss), g)
        return loss.value, g

    def step(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> float:
        """One Adam step on the whole training set; the loss before it."""
        loss = c_double(0.0)
        _call("pyrpa_gb_lws_step", i64(self.handle), dbl(lr), dbl(beta1), dbl(beta2), dbl(eps), byref(loss))
        return loss.value

    def train(self, steps: int, batch: int = 8192, lr: float = 3e-3, beta1: float = 0.9, beta2: float = 0.999,
              eps: float = 1e-8, seed: int = 0) -> np.ndarray:
        """Adam on batches drawn with replacement; the loss of every batch."""
        out = np.zeros(max(1, steps))
        _call("pyrpa_gb_lws_train", i64(self.handle), i64(steps), i64(batch), dbl(lr), dbl(beta1), dbl(beta2),
              dbl(eps), i64(seed), out)
        return out[:steps]

    def forward(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros((len(x), NO), dtype=np.float32)
        _call("pyrpa_gb_lws_forward", i64(self.handle), x, i64(len(x)), y)
        return y

    # ------------------------------------------------------------ inference
    def apply(self, sigma_seed, uni, eig, Nw_c: int, desc) -> np.ndarray:
        """sigma_seed + U (max|sigma_seed| y) U^dagger at every (k, n)."""
        out = _sig(sigma_seed).copy()
        Norb, _, Nw, Nk = out.shape
        _call("pyrpa_gb_lws_apply", i64(self.handle), out, np.ascontiguousarray(uni), np.ascontiguousarray(eig),
              i64(Nk), i64(Nw), i64(Nw_c), i64(Norb), np.ascontiguousarray(desc, dtype=np.float64))
        return out


# ----------------------------------------------------------------- solves
def coarse_solution(m: dict, kdiv: int = 4, wdiv: int = 4, eps: float = 1e-6, scf_loop: int = 300) -> dict:
    """The model of ``models.prepare`` (dict m) solved on its k mesh and
    Matsubara set divided by (kdiv, wdiv): Sigma, mu and Stoner factor of the
    coarse FLEX loop, with the coarse mesh's maps."""
    from . import models
    cfg = m["cfg"]
    div = lambda n: n // kdiv if (kdiv > 1 and n % kdiv == 0 and n // kdiv >= 2) else n
    over = dict(cfg, Nx=div(cfg["Nx"]), Ny=div(cfg["Ny"]), Nz=div(cfg["Nz"]) if cfg["Nz"] > 1 else 1,
                Nw=max(1, cfg["Nw"] // max(1, wdiv)))
    mc = models.prepare(m["name"], **over)
    c = mc["cfg"]
    sig, mu = F.mkself(mc["S"], mc["C"], mc["kmap"], mc["invk"], mc["olist"], mc["hamk"], mc["eig"], mc["uni"],
                       mc["mu"], c["fill"], c["temp"], c["Nw"], c["Nx"], c["Ny"], c["Nz"], False, False, eps=eps,
                       pp=0.5, scf_loop=scf_loop, sw_rescale=True)
    st = F.last_stats()
    return dict(model=mc, sigmak=sig, mu=mu, stoner=st["stoner"], iterations=int(st["iterations"]))


def interpolated_seed(m: dict, coarse: dict) -> np.ndarray:
    """The coarse Sigma on m's fine mesh (wrappers' layout)."""
    c, mc = m["cfg"], coarse["model"]
    cc = mc["cfg"]
    return F.sigma_interp(coarse["sigmak"], mc["kmap"], mc["invk"], cc["Nx"], cc["Ny"], cc["Nz"], m["kmap"],
                          m["invk"], c["Nx"], c["Ny"], c["Nz"], len(m["klist"]), c["Nw"], c["temp"])


def seed_descriptors(m: dict, coarse: dict, sigma_seed) -> np.ndarray:
    c = m["cfg"]
    return descriptors(c["U"], c["J"], c["temp"], c["fill"], c["Norb"], coarse["stoner"], coarse["mu"], m["eig"],
                       sigma_seed)


def add_training_solution(net: LearnedWarmStart, m: dict, coarse: dict, sigma_fine, max_pairs: int | None = None,
                          seed: int = 0) -> int:
    """Rows of one solved model: its interpolated seed against its converged
    fine Sigma, on max_pairs (k, n) pairs drawn with `seed` (all pairs when
    None).  Returns the rows added."""
    s = interpolated_seed(m, coarse)
    desc = seed_descriptors(m, coarse, s)
    Nw, Nk = s.shape[2], s.shape[3]
    pairs = all_pairs(Nk, Nw) if max_pairs is None else sample_pairs(Nk, Nw, max_pairs, seed)
    before = net.num_rows
    net.add_samples(s, sigma_fine, m["uni"], m["eig"], coarse["model"]["cfg"]["Nw"], desc, pairs)
    return net.num_rows - before


def learned_seed(net: LearnedWarmStart, m: dict, coarse: dict):
    """(Sigma seed, mu seed) for m's fine loop: the interpolated coarse Sigma
    refined by the network, and the coarse mu."""
    s = interpolated_seed(m, coarse)
    desc = seed_descriptors(m, coarse, s)
    return net.apply(s, m["uni"], m["eig"], coarse["model"]["cfg"]["Nw"], desc), coarse["mu"]


# ---------------------------------------------------------- measurement
def family(count: int, seed: int = 0, Norb: int = 5, N: int = 64, Nw: int = 2048):
    """Models of the 5-orbital family on one mesh with the sweep's parameter
    ranges (U / U_Stoner, T, filling), as sweep.Instance records."""
    from . import sweep
    return [sweep.Instance(index=x.index, Norb=Norb, N=N, Nw=Nw, seed=x.seed, u_frac=x.u_frac, temp=x.temp,
                           n_per_orb=x.n_per_orb) for x in sweep.draw(count, seed)]


def _prepared(inst, U: float) -> dict:
    from . import models
    return models.prepare("c2", Norb=inst.Norb, Nx=inst.N, Ny=inst.N, Nz=1, Nw=inst.Nw, temp=inst.temp,
                          fill=inst.fill, U=U, J=U / 6.0, seed=inst.seed, bandwidth=4.0)


def _fused(m: dict, eps: float, sigma_seed=None, mu_seed: float = 0.0) -> dict:
    """The fused FLEX + Eliashberg solve of m from G0 or from a seed; FLEX
    iterations and the device seconds of the FLEX stages."""
    c = m["cfg"]
    t0 = time.perf_counter()
    r = F.flex_eliash(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["init"],
                      m["plist"], m["mu"], c["fill"], c["temp"], c["Nw"], c["Nx"], c["Ny"], c["Nz"], c["gap_sym"],
                      eps=eps, sigma_seed=sigma_seed, seed_mu=mu_seed, seed_mu_old=mu_seed)
    wall = time.perf_counter() - t0
    st = F.last_stats()
    flex_ms = sum(st[k] for k in ("t_chi0_ms", "t_vertex_ms", "t_sigma_ms", "t_diis_ms", "t_mu_ms", "t_dyson_ms",
                                  "t_stoner_ms"))
    return dict(sigmak=r["sigmak"], mu=r["mu"], lam=r["lam"], iterations=int(st["iterations"]),
                esterr=st["esterr"], flex_s=flex_ms / 1e3, wall_s=wall)


def main(argv=None):
    """Train the network on solved models of the family and time the fine
    loop of held-out models from the interpolated and the learned seed,
    beside the cold start."""
    import argparse
    import json

    from . import sweep
    ap = argparse.ArgumentParser(description="learned warm start: train and measure")
    ap.add_argument("--train", type=int, default=8)
    ap.add_argument("--test", type=int, default=4)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--mesh", type=int, default=64)
    ap.add_argument("--nw", type=int, default=2048)
    ap.add_argument("--kdiv", type=int, default=4)
    ap.add_argument("--wdiv", type=int, default=4)
    ap.add_argument("--eps", type=float, default=1e-6)
    ap.add_argument("--pairs", type=int, default=200000, help="(k, n) pairs per training model")
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "64"])
    ap.add_argument("--save", default=None)
    a = ap.parse_args(argv)
    F.load_library()
    F.set_verbose(0)
    F.set_precision(F.MIXED if a.precision == "mixed" else 64)
    insts = family(a.train + a.test, a.seed, N=a.mesh, Nw=a.nw)
    net = LearnedWarmStart(seed=a.seed)
    held = []
    for i, inst in enumerate(insts):
        U = inst.u_frac * sweep.stoner_u(inst)
        m = _prepared(inst, U)
        coarse = coarse_solution(m, a.kdiv, a.wdiv, eps=a.eps)
        cold = _fused(m, a.eps)
        rec = dict(index=inst.index, U=U, temp=inst.temp, fill=inst.fill, cold_iterations=cold["iterations"],
                   cold_flex_s=cold["flex_s"], coarse_iterations=coarse["iterations"])
        if i < a.train:
            rec["rows"] = add_training_solution(net, m, coarse, cold["sigmak"], a.pairs, seed=inst.index)
        else:
            held.append((inst, m, coarse, cold))
        print(json.dumps(rec), flush=True)
    t0 = time.perf_counter()
    losses = net.train(a.steps, a.batch, a.lr, seed=a.seed)
    print(json.dumps(dict(train_s=time.perf_counter() - t0, loss_first=float(losses[0]),
                          loss_last=float(np.mean(losses[-50:])))), flush=True)
    if a.save:
        net.save(a.save)
    for inst, m, coarse, cold in held:
        s_int = interpolated_seed(m, coarse)
        s_lrn, mu_c = learned_seed(net, m, coarse)
        ri = _fused(m, a.eps, s_int, mu_c)
        rl = _fused(m, a.eps, s_lrn, mu_c)
        nrm = np.linalg.norm(cold["sigmak"])
        print(json.dumps(dict(
            index=inst.index, seed_err_interp=float(np.linalg.norm(s_int - cold["sigmak"]) / nrm),
            seed_err_learned=float(np.linalg.norm(s_lrn - cold["sigmak"]) / nrm),
            iterations=dict(cold=cold["iterations"], interp=ri["iterations"], learned=rl["iterations"]),
            flex_s=dict(cold=cold["flex_s"], interp=ri["flex_s"], learned=rl["flex_s"]),
            coarse_iterations=coarse["iterations"],
            lambda_rel_diff=dict(interp=abs(ri["lam"] - cold["lam"]) / abs(cold["lam"]),
                                 learned=abs(rl["lam"] - cold["lam"]) / abs(cold["lam"])))), flush=True)


if __name__ == "__main__":
    main()
