"""Small, self-contained launches of single engine kernels for profiling.

Each case runs one ABI call on a synthetic input that is larger than L2
(129 MB) but a few hundred MB at most, so that a profiler capture of one
launch replays quickly:

  vertex   get_vsigma_flex_nosoc_ (FP64, as in the reference) on a 5-orbital
           chi0 (Nchi = 25), 130 irreducible q x 512 frequencies = 66,560
           matrices (666 MB c128)
  chi0     get_chi0_tail on a 5-orbital 16x16 mesh with 512 frequencies
  flex     mkself, one FLEX iteration, same model (the FP32 vertex, chi0 and
           Sigma kernels at --precision 32)
  fft      get_chi0 of a 1-orbital model on the 64x64 mesh with 2048
           frequencies: FFT passes over 64x64x4096 arrays (134 MB in FP32,
           larger than L2) as in the 5-orbital benchmark

Run as  python -m pyrpa_gb300.profile_cases <case> [--precision 32|64] [--repeat n]
"""
from __future__ import annotations

import argparse
import ctypes
import sys
import time

import numpy as np


def _model(Norb=5, N=16, Nw=512, temp=0.02):
    from . import flibs as F, models
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


def case_vertex(F, repeat):
    Nchi, Nk, Nw = 25, 130, 512
    rng = np.random.default_rng(0)
    chi = (0.05 * (rng.standard_normal((Nchi, Nchi, Nw, Nk)) + 1j * rng.standard_normal((Nchi, Nchi, Nw, Nk))))
    olist, site = F.get_chi_orb_list(5)
    S, C = F.gen_SCmatrix(olist, site, 1.2, 0.2)
    lib = F.load_library()
    i64 = ctypes.c_int64
    for _ in range(repeat):
        x = chi.copy()
        lib.get_vsigma_flex_nosoc_(x, S, C, ctypes.byref(i64(Nk)), ctypes.byref(i64(Nw)), ctypes.byref(i64(Nchi)))


def case_chi0(F, repeat):
    m = _model()
    Gk = F.gen_Green0(m["eig"], m["uni"], m["mu"], m["temp"], m["Nw"])
    for _ in range(repeat):
        F.get_chi0_tail(m["S"], m["C"], Gk, m["eig"], m["uni"], m["olist"], m["kmap"], m["invk"], m["mu"],
                        m["temp"], m["N"], m["N"], 1)


def case_fft(F, repeat):
    m = _model(Norb=1, N=64, Nw=2048, temp=0.01)
    Gk = F.gen_Green0(m["eig"], m["uni"], m["mu"], m["temp"], m["Nw"])
    for _ in range(repeat):
        F.get_chi0(m["S"], m["C"], Gk, m["olist"], m["kmap"], m["invk"], m["temp"], m["N"], m["N"], 1)


def case_flex(F, repeat):
    m = _model()
    for _ in range(repeat):
        F.mkself(m["S"], m["C"], m["kmap"], m["invk"], m["olist"], m["hamk"], m["eig"], m["uni"], m["mu"],
                 0.6 * m["Norb"], m["temp"], m["Nw"], m["N"], m["N"], 1, False, False, scf_loop=1, eps=1e-4,
                 pp=0.5, sw_tail=True, sw_rescale=True)


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("case", choices=["vertex", "chi0", "flex", "fft"])
    p.add_argument("--precision", type=int, default=32, choices=[32, 64])
    p.add_argument("--repeat", type=int, default=1)
    a = p.parse_args(argv)
    from . import flibs as F
    F.load_library()
    F.set_verbose(0)
    F.set_precision(a.precision)
    t0 = time.perf_counter()
    {"vertex": case_vertex, "chi0": case_chi0, "flex": case_flex, "fft": case_fft}[a.case](F, a.repeat)
    print(f"{a.case}: {a.repeat} call(s) in {time.perf_counter() - t0:.3f} s", flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
