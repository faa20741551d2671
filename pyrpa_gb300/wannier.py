"""Sigma(k, iw_n) and Delta(k, iw_n) in Wannier real space, as the reference's
output_self_wannier / output_gap_wannier write them (libs/plibs/_wannier_io.py:
145-216): the k -> R transform runs on the GPU (pyrpa_gb_wannier_r); the
zeroing below zero_tol * max, the choice of R vectors with a non-zero
component and the two output files (fname.npz and the text fname.dat, one
line 'Rx Ry Rz io jo iw Re Im' per value) follow the reference's format.
"""
from __future__ import annotations

import numpy as np

from . import flibs


def _nonzero_r(data_r, Nx, Ny, Nz, zero_tol):
    """Zero Re/Im parts below zero_tol * max|data|; keep the R points with a
    non-zero value (C order of the (x, y, z) grid), R centred on the origin."""
    tol = np.abs(data_r).max() * zero_tol
    data_r.real[np.abs(data_r.real) < tol] = 0.0
    data_r.imag[np.abs(data_r.imag) < tol] = 0.0
    keep = np.abs(data_r).max(axis=(0, 1, 2)) > 0
    ix, iy, iz = np.nonzero(keep)
    centre = lambda i, n: np.where(i <= n // 2, i, i - n)
    rvec = np.stack([centre(ix, Nx), centre(iy, Ny), centre(iz, Nz)], axis=1).astype(np.int64)
    return data_r[:, :, :, ix, iy, iz], rvec


def _write_dat(fname, data, rvec, label, mu=None, temp=None):
    Norb, _, Ncut, Nr = data.shape
    head = f"# {label}: Norb={Norb} N_iw={Ncut} Nr={Nr}"
    if mu is not None:
        head += f" mu={mu:.8f}"
    if temp is not None:
        head += f" temp={temp:.8e}"
    rows = []
    for r in range(Nr):
        rx, ry, rz = (int(v) for v in rvec[r])
        for n in range(Ncut):
            for i in range(Norb):
                for j in range(Norb):
                    v = data[i, j, n, r]
                    rows.append(f"{rx:4d}{ry:4d}{rz:4d}{i + 1:3d}{j + 1:3d}{n + 1:5d}{v.real:16.8e}{v.imag:16.8e}")
    with open(f"{fname}.dat", "w") as f:
        f.write(f"{head}\n{Norb} {Ncut} {Nr}\n")
        f.write("\n".join(rows) + "\n")


def _output(data, kmap, invk, Nx, Ny, Nz, temp, N_cut, zero_tol, fname, key, label, mu=None):
    data_r = flibs.wannier_r(data, kmap, invk, Nx, Ny, Nz, N_cut)
    out, rvec = _nonzero_r(data_r, Nx, Ny, Nz, zero_tol)
    if out.size == 0:
        print(f"{key}: no non-zero R-vectors found", flush=True)
        return
    iw = (2 * np.arange(out.shape[2]) + 1) * np.pi * temp
    extra = {"mu": mu} if mu is not None else {}
    np.savez(fname, **{key: out}, rvec=rvec, iw=iw, **extra, temp=temp)
    _write_dat(fname, out, rvec, label, mu=mu, temp=temp)


def output_self_wannier(sigmak, mu_self, kmap, invk, Nx, Ny, Nz, Nw, temp, N_cut=64, zero_tol=1e-5,
                        fname="self_en_wannier"):
    """sigmak [Norb, Norb, Nw, Nk_irr] -> fname.npz (sigma, rvec, iw, mu, temp) and fname.dat."""
    _output(sigmak, kmap, invk, Nx, Ny, Nz, temp, N_cut, zero_tol, fname, "sigma", "Self-energy", mu=mu_self)


def output_gap_wannier(gap, kmap, invk, Nx, Ny, Nz, Nw, temp, N_cut=64, zero_tol=1e-5, fname="gap_wannier"):
    """gap [Norb, Norb, Nw, Nk_irr or Nkall] -> fname.npz (gap, rvec, iw, temp) and fname.dat."""
    _output(gap, kmap, invk, Nx, Ny, Nz, temp, N_cut, zero_tol, fname, "gap", "Gap function")
