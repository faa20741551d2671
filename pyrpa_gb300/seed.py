"""Self-energy seeds on a new Matsubara mesh (plibs.regrid_sigma_bin).

``regrid_sigma_bin`` keeps the signature, defaults, return value and error
cases of plibs.regrid_sigma_bin (libs/plibs/_calc.py:52-182), which a pyrpa
script calls between two ``mkself`` runs at different temperatures.  All of
the work happens in libfmod.so (``pyrpa_gb_regrid_sigma_file``): it parses the
gfortran sequential records that io_sigma writes (mu, mu_OLD, Sigma in
Fortran order, and the optional (temp, Nw, Norb, Nk) record), checks the
arguments against that record, regrids on the GPU and writes the new file
with the record of the new mesh.  Problems the caller has to fix arrive here
as ValueError, as in the reference.
"""
from __future__ import annotations

from . import flibs


def regrid_sigma_bin(temp_old: float | None = None, temp_new: float | None = None, Norb: int | None = None,
                     Nw_old: int | None = None, Nw_new: int | None = None, w_scale: float | None = None,
                     path: str = "sigma.bin", out_path: str | None = None):
    """Regrid the sigma.bin at ``path`` onto Nw_new frequencies at temp_new
    and write it to ``out_path`` (default: in place).  Arguments left None
    are read from the file; returns (Nk, Nw_new)."""
    if temp_new is None:
        raise ValueError("regrid_sigma_bin needs the target temperature temp_new")
    return flibs.regrid_sigma_file(path, out_path or path, temp_old, temp_new, Norb, Nw_old, Nw_new,
                                   1.0 if w_scale is None else w_scale)
