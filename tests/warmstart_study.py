"""CPU study of the warm start on the oracle: how much does a better seed
shorten the fine FLEX loop?  (Not collected by pytest; run it directly.)

    python tests/warmstart_study.py            # about 4 minutes on 8 cores
    python tests/warmstart_study.py --bound    # about 1 minute

Models: two orbitals, seeded hoppings out to the (2,0) shell (bandwidth 4),
U uniform in [0.8, 1.4], J = U/6, T log-uniform in [0.03, 0.06], electrons
per spin uniform in [0.7, 1.0]; fine mesh 16x16 with 128 Matsubara
frequencies, coarse 8x8 with 64.  Coarse and fine solves are the oracle's
FP64 FLEX loop (oracle/flex_oracle.py mkself, DIIS m=5, mixing 0.3,
eps 1e-8 coarse / 1e-10 fine).  The seed is oracle/warmstart_oracle.py's
interpolation; the network (same definition as csrc/lws.cu) is trained in
numpy on 12 models and evaluated on 4 held out.  Printed per held-out model:
the relative L2 error of the seed before and after the network, and the
fine-loop iterations to a residual of 1e-4 and 1e-6 from each seed (coarse
mu), from the learned seed with the exact fine mu, and from the learned seed
with mu re-solved on the fine mesh for it.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)


def _model(Norb, N, Nw, seed, U, J, temp):
    import _models as M
    from oracle import api as A
    from oracle import flex_oracle as O
    rvec, ham_r = M.random_hoppings(Norb, seed, bandwidth=4.0)
    klist, kmap, invk = A.gen_irr_k_TRS(N, N, 1)
    hamk = A.gen_ham(klist, ham_r, rvec)
    eig, uni = A.get_eig(hamk)
    olist, site = A.get_chi_orb_list(Norb)
    S, C = A.gen_SCmatrix(np.asarray(olist), site, U, J)
    return dict(kmap=kmap, invk=invk, hamk=hamk, eig=eig, uni=uni, olist=np.asarray(olist), S=S, C=C, N=N, Nw=Nw,
                temp=temp, grid=O.KGrid(kmap, invk, N, N, 1))


def _solve(m, fill, eps, sigma_in=None, mu0=0.0):
    from oracle import flex_oracle as O
    return O.mkself(m["S"].T, m["C"].T, m["kmap"], m["invk"], m["olist"], m["hamk"].transpose(0, 2, 1), m["eig"],
                    m["uni"].transpose(0, 2, 1), mu0, fill, m["temp"], 300, 0.3, eps, m["N"], m["N"], 1, m["Nw"],
                    sigma_in=sigma_in, mu_old_in=mu0 if sigma_in is not None else None, sw_rescale=True)


def _mu_for_seed(m, sig_F, fill, mu0):
    """mu at which the reference's filling n(mu) (fself.f90:662-687) with
    eig(H + Sigma_seed) equals `fill`, by bisection."""
    from oracle import flex_oracle as O
    temp, eig = m["temp"], m["eig"]
    H = m["hamk"].transpose(0, 2, 1)
    wl = O.matsubara(temp, sig_F.shape[1])
    eg = np.linalg.eigvals(H[:, None] + sig_F)

    def rn(mu):
        t = np.sum(0.5 * (1.0 - np.tanh(0.5 * (eig - mu) / temp)))
        z = mu + 1j * wl
        dg = np.sum((1.0 / (z[None, :, None] - eg) - 1.0 / (z[None, :, None] - eig[:, None, :])).real)
        return (t + 2 * temp * dg) / eig.shape[0]

    lo, hi = mu0 - 0.5, mu0 + 0.5
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        lo, hi = (mid, hi) if rn(mid) < fill else (lo, mid)
    return 0.5 * (lo + hi)


def _generate(job):
    from oracle import warmstart_oracle as W
    seed, U, temp, fill = job
    mf = _model(2, 16, 128, seed, U, U / 6, temp)
    mc = _model(2, 8, 64, seed, U, U / 6, temp)
    rc = _solve(mc, fill, 1e-8)
    rf = _solve(mf, fill, 1e-10)
    s = W.sigma_interp(rc.sigma, mc["grid"], mf["grid"], 128, temp)
    return dict(job=job, seed_sig=s, fine=rf.sigma, mu_c=rc.mu, mu_f=rf.mu, stoner_c=rc.stoner,
                U=mf["uni"].transpose(0, 2, 1), eig=mf["eig"])


def _rows(d):
    from oracle import warmstart_oracle as W
    seed, U, temp, fill = d["job"]
    desc = W.descriptors(U, U / 6, temp, fill, 2, d["stoner_c"], d["mu_c"], d["eig"], d["seed_sig"])
    kn = W.all_pairs(*d["seed_sig"].shape[:2])
    return desc, W.features(d["seed_sig"], d["U"], d["eig"], 64, desc, kn), \
        W.targets(d["seed_sig"], d["fine"], d["U"], desc, kn)


def _evaluate(args):
    from oracle import warmstart_oracle as W
    d, theta = args
    seed, U, temp, fill = d["job"]
    mf = _model(2, 16, 128, seed, U, U / 6, temp)
    desc, x, _ = _rows(d)
    y, _ = W.forward(theta, x)
    new = W.apply_correction(d["seed_sig"], d["U"], desc, y)
    nrm = np.linalg.norm(d["fine"])
    out = dict(seed=seed, err0=np.linalg.norm(d["seed_sig"] - d["fine"]) / nrm,
               err1=np.linalg.norm(new - d["fine"]) / nrm)
    for name, s in (("interp", d["seed_sig"]), ("learned", new)):
        out[name] = [_solve(mf, fill, e, sigma_in=s, mu0=d["mu_c"]).iterations for e in (1e-4, 1e-6)]
    out["learned_exact_mu"] = _solve(mf, fill, 1e-6, sigma_in=new, mu0=d["mu_f"]).iterations
    out["learned_resolved_mu"] = _solve(mf, fill, 1e-6, sigma_in=new,
                                        mu0=_mu_for_seed(mf, new, fill, d["mu_c"])).iterations
    return out


def main():
    from oracle import warmstart_oracle as W
    rng = np.random.default_rng(0)
    jobs = [(100 + s, rng.uniform(0.8, 1.4), float(np.exp(rng.uniform(np.log(0.03), np.log(0.06)))),
             rng.uniform(0.7, 1.0)) for s in range(16)]
    t0 = time.time()
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(8, os.cpu_count() or 1)) as pool:
        data = pool.map(_generate, jobs)
    print(f"16 coarse + fine oracle solves in {time.time() - t0:.0f} s")
    train, test = data[:12], data[12:]
    X = np.concatenate([_rows(d)[1] for d in train])
    T = np.concatenate([_rows(d)[2] for d in train])
    theta = W.init_params(0)
    m = np.zeros_like(theta)
    v = np.zeros_like(theta)
    brng = np.random.default_rng(1)
    for step in range(1, 1501):
        idx = brng.integers(0, len(X), 8192)
        _, g = W.loss_and_grad(theta, X[idx], T[idx])
        theta, m, v = W.adam_step(theta, g, m, v, step, 3e-3 if step < 900 else 1e-3)
    print(f"trained on {len(X)} rows of 12 models, 1500 Adam steps of 8192 rows")
    with ctx.Pool(4) as pool:
        res = pool.map(_evaluate, [(d, theta) for d in test])
    print("model  seed err -> learned | iterations to 1e-4 / 1e-6: interp seed | learned seed |"
          " learned + exact mu (1e-6) | learned + re-solved mu (1e-6)")
    for r in res:
        print(f"{r['seed']:5d}  {r['err0']:.3f} -> {r['err1']:.3f}   | {r['interp'][0]:2d} / {r['interp'][1]:2d}"
              f"       | {r['learned'][0]:2d} / {r['learned'][1]:2d}        | {r['learned_exact_mu']:2d}"
              f"                        | {r['learned_resolved_mu']:2d}")


def bound():
    """Seeds between the fine fixed point and the interpolated seed,
    Sigma_fine + alpha (Sigma_interp - Sigma_fine), started with the coarse
    or the exact fine mu: iterations of the fine loop to 1e-6 (one model:
    hopping seed 1, U = 1.2, T = 0.05, 1.0 electron per spin)."""
    from oracle import warmstart_oracle as W
    mf = _model(2, 16, 128, 1, 1.2, 0.2, 0.05)
    mc = _model(2, 8, 64, 1, 1.2, 0.2, 0.05)
    rc = _solve(mc, 1.0, 1e-8)
    rf = _solve(mf, 1.0, 1e-10)
    err = W.sigma_interp(rc.sigma, mc["grid"], mf["grid"], 128, 0.05) - rf.sigma
    print("alpha   coarse mu   exact mu   (iterations to 1e-6)")
    for alpha in (1.0, 0.1, 0.01, 0.0):
        s = rf.sigma + alpha * err
        its = [_solve(mf, 1.0, 1e-6, sigma_in=s, mu0=mu).iterations for mu in (rc.mu, rf.mu)]
        print(f"{alpha:5.2f}   {its[0]:9d}   {its[1]:8d}")


if __name__ == "__main__":
    bound() if "--bound" in sys.argv else main()
