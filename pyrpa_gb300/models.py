"""Seeded synthetic tight-binding models of the benchmark configurations.

No public dataset is involved: the workloads are model Hamiltonians.
  c1  one orbital, square lattice, t=1, t'=-0.25, n=0.85 (fill 0.425 per
      spin), T=0.02, U=3, 32x32, 1024 Matsubara frequencies;
  c2  five orbitals, real symmetric H(R)=H(-R) out to third neighbours
      (shells (1,0), (1,1), (2,0)), on-site levels U[-0.3,0.3] eV, hoppings
      N(0,0.3)*0.4^(shell-1) rescaled to a 4 eV bandwidth, 6 electrons per site
      (fill 3.0 per spin), U=1.2, J=U/6, T=0.01 eV, 64x64, 2048 frequencies;
  c5  three orbitals in 3D (t2g-like) out to second neighbours, bandwidth
      3 eV, fill 2.0 per spin, U=1.5, J=0.25, T=0.008 eV, 24^3, 1024 frequencies.
``prepare`` turns a configuration into the arrays the C ABI takes, through
the engine's own setup entry points.
"""
from __future__ import annotations

import itertools

import numpy as np

CONFIGS = {
    "c1": dict(Norb=1, Nx=32, Ny=32, Nz=1, Nw=1024, temp=0.02, fill=0.425, U=3.0, J=0.0, gap_sym=1),
    "c2": dict(Norb=5, Nx=64, Ny=64, Nz=1, Nw=2048, temp=0.01, fill=3.0, U=1.2, J=0.2, gap_sym=0, seed=4,
               bandwidth=4.0),
    "c5": dict(Norb=3, Nx=24, Ny=24, Nz=24, Nw=1024, temp=0.008, fill=2.0, U=1.5, J=0.25, gap_sym=0, seed=5,
               bandwidth=3.0),
}


def square_t_tprime(t: float = 1.0, tp: float = -0.25):
    """One orbital: nearest neighbours -t, next-nearest -t' (H = +0.25 for t'=-0.25)."""
    rv = [(0, 0, 0)] + [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0)] + [(1, 1, 0), (-1, -1, 0), (1, -1, 0), (-1, 1, 0)]
    hv = [0.0] + [-t] * 4 + [-tp] * 4
    return np.array(rv, dtype=np.float64), np.array(hv, dtype=np.complex128).reshape(-1, 1, 1)


def _shell_images(base, dim):
    out = set()
    perms = itertools.permutations(range(3)) if dim == 3 else [(0, 1, 2), (1, 0, 2)]
    for perm in perms:
        for signs in itertools.product((1, -1), repeat=3):
            v = tuple(int(base[perm[i]] * signs[i]) for i in range(3))
            if dim == 2 and v[2] != 0:
                continue
            out.add(v)
    return sorted(out)


def seeded_hoppings(Norb: int, seed: int, shells, dim: int = 2, sigma: float = 0.3, decay: float = 0.4,
                    onsite: float = 0.3, bandwidth: float | None = None):
    """Real symmetric H(R) = H(-R) (time reversal and inversion), Python layout
    ham_r[Nr, Norb, Norb]; shell s has amplitudes N(0, sigma) * decay**s."""
    rng = np.random.default_rng(seed)
    shell_of = {}
    for s, base in enumerate(shells):
        for v in _shell_images(base, dim):
            shell_of.setdefault(v, s)
    rlist = [(0, 0, 0)] + sorted(shell_of)
    H = np.zeros((len(rlist), Norb, Norb))
    idx = {r: i for i, r in enumerate(rlist)}
    H[0][np.diag_indices(Norb)] = rng.uniform(-onsite, onsite, Norb)
    done = set()
    for r in rlist[1:]:
        if r in done:
            continue
        A = rng.normal(0.0, sigma * decay ** shell_of[r], (Norb, Norb))
        A = 0.5 * (A + A.T)
        mr = tuple(-x for x in r)
        H[idx[r]] = A
        H[idx[mr]] = A
        done |= {r, mr}
    rvec = np.array(rlist, dtype=np.float64)
    if bandwidth is not None:
        g = np.arange(24) / 24
        ks = np.stack(np.meshgrid(g, g, g if dim == 3 else [0.0], indexing="ij"), -1).reshape(-1, 3)
        Hk = np.einsum("kr,rml->kml", np.cos(2 * np.pi * ks @ rvec.T), H)
        e = np.linalg.eigvalsh(Hk)
        H = H * (bandwidth / (e.max() - e.min()))
    return rvec, np.ascontiguousarray(np.transpose(H, (0, 2, 1))).astype(np.complex128)


def hoppings(cfg: dict):
    if cfg["Norb"] == 1:
        return square_t_tprime()
    if cfg["Nz"] > 1:
        return seeded_hoppings(cfg["Norb"], cfg["seed"], [(1, 0, 0), (1, 1, 0)], dim=3, bandwidth=cfg["bandwidth"])
    return seeded_hoppings(cfg["Norb"], cfg["seed"], [(1, 0, 0), (1, 1, 0), (2, 0, 0)], dim=2,
                           bandwidth=cfg["bandwidth"])


def bare_mu(eig, weight, fill: float, temp: float) -> float:
    """Chemical potential of the bare bands at `fill` electrons per spin
    (the reference's plibs.calc_mu solves the same equation with brentq)."""
    lo, hi = eig.min() - 1.0, eig.max() + 1.0
    tot = weight.sum()
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        n = (weight[:, None] * 0.5 * (1.0 - np.tanh(0.5 * (eig - mid) / temp))).sum() / tot
        lo, hi = (mid, hi) if n < fill else (lo, mid)
    return 0.5 * (lo + hi)


def prepare(name: str, **over) -> dict:
    """All arrays of one configuration, built with the engine's setup calls."""
    from . import flibs as F
    cfg = dict(CONFIGS[name])
    cfg.update(over)
    rvec, ham_r = hoppings(cfg)
    klist, kmap, invk = F.gen_irr_k_TRS(cfg["Nx"], cfg["Ny"], cfg["Nz"])
    hamk = F.gen_ham(klist, ham_r, rvec)
    eig, uni = F.get_eig(hamk)
    olist, site = F.get_chi_orb_list(cfg["Norb"])
    S, C = F.gen_SCmatrix(olist, site, cfg["U"], cfg["J"])
    w = F.gen_kpoint_weight(invk, len(klist))
    mu = bare_mu(eig, w, cfg["fill"], cfg["temp"])
    init = F.get_initial_gap(klist, cfg["Norb"], cfg["gap_sym"])
    plist = F.get_plist(rvec, ham_r)
    return dict(cfg=cfg, name=name, rvec=rvec, ham_r=ham_r, klist=klist, kmap=kmap, invk=invk, hamk=hamk, eig=eig,
                uni=uni, olist=olist, site=site, S=S, C=C, mu=mu, init=init, plist=plist)
