"""Self-energy seeds: the reference's sigma.bin regrid with the compute on the GPU.

``regrid_sigma_bin`` has the signature and the file semantics of
plibs.regrid_sigma_bin (libs/plibs/_calc.py:52-182): it reads the
gfortran-sequential sigma.bin that mkself writes (mu, mu_OLD, sigmak in
Fortran order and the (temp, Nw, Norb, Nk) footer), regrids Sigma along the
Matsubara axis and writes the file back with a footer for the new mesh.  The
regrid itself runs in libfmod.so (pyrpa_gb_regrid_sigma).
"""
from __future__ import annotations

import numpy as np

from . import flibs


def regrid_sigma_bin(temp_old: float | None = None, temp_new: float | None = None, Norb: int | None = None,
                     Nw_old: int | None = None, Nw_new: int | None = None, w_scale: float | None = None,
                     path: str = "sigma.bin", out_path: str | None = None):
    """Returns (Nk, Nw_new) like the reference; raises ValueError where it does."""
    from scipy.io import FortranFile
    if temp_new is None:
        raise ValueError("temp_new is required")
    w_scale = 1.0 if w_scale is None else w_scale
    with FortranFile(path, "r") as f:
        mu = f.read_record(np.float64)
        mu_old = f.read_record(np.float64)
        flat = f.read_record(np.complex128)
        try:
            meta = f.read_record(np.float64)
            if meta.size != 4:
                meta = None
        except Exception:
            meta = None
    if meta is not None:
        stored = {"temp_old": meta[0], "Nw_old": int(round(meta[1])), "Norb": int(round(meta[2]))}
        for name, given in (("temp_old", temp_old), ("Nw_old", Nw_old), ("Norb", Norb)):
            if given is not None and not np.isclose(given, stored[name], rtol=1e-8, atol=0.0):
                raise ValueError(f"{name}={given} contradicts the sigma.bin metadata footer ({stored[name]})")
        temp_old, Nw_old, Norb = stored["temp_old"], stored["Nw_old"], stored["Norb"]
    elif temp_old is None or Nw_old is None or Norb is None:
        raise ValueError("sigma.bin carries no metadata footer: temp_old, Norb and Nw_old must be given")
    Nw_new = Nw_old if Nw_new is None else Nw_new
    Nk, rem = divmod(flat.size, Nw_old * Norb * Norb)
    if rem:
        raise ValueError(f"sigma.bin size {flat.size} is not divisible by Nw_old*Norb^2 = {Nw_old * Norb * Norb}")
    if meta is not None and Nk != int(round(meta[3])):
        raise ValueError(f"inferred Nk={Nk} contradicts the metadata footer ({int(round(meta[3]))})")
    # Fortran (Nk, Nw, Norb, Norb) is the wrappers' [Norb, Norb, Nw, Nk] in C order
    sig = flat.reshape((Norb, Norb, Nw_old, Nk))
    out = flibs.regrid_sigma(sig, temp_old, temp_new, Nw_new, w_scale)
    with FortranFile(out_path or path, "w") as f:
        f.write_record(mu)
        f.write_record(mu_old)
        f.write_record(np.ascontiguousarray(out).ravel())
        f.write_record(np.array([temp_new, float(Nw_new), float(Norb), float(Nk)]))
    return Nk, Nw_new
