"""CPU tests of the sigma.bin checks of pyrpa_gb300.seed.regrid_sigma_bin.

The library parses the io_sigma records (fself.f90:742-780) and checks the
arguments against the file before it touches the GPU, so every case where
plibs.regrid_sigma_bin (libs/plibs/_calc.py:105-150) raises ValueError is
exercised here without a device: a missing target temperature, a file
without the (temp, Nw, Norb, Nk) record and arguments missing, arguments
that contradict that record, a Sigma record whose size is not a multiple of
Nw_old*Norb^2, and an Nk that disagrees with the record.  A damaged last
record reads as an absent one.  A well-formed file reaches the GPU regrid,
which fails loudly without a device, never silently on the CPU (with a
device it simply runs).
"""
import struct

import numpy as np
import pytest


def _record(payload: bytes) -> bytes:
    n = struct.pack("<i", len(payload))
    return n + payload + n


def _regrid_or_no_device(seed, **kw):
    try:
        return seed.regrid_sigma_bin(**kw)
    except RuntimeError as e:
        assert "CUDA device" in str(e)
        return None


def _write(path, nk=3, nw=8, norb=2, footer=(0.05, 8.0, 2.0, 3.0), extra=0, damage_footer=False):
    sig = (np.arange(nk * nw * norb * norb + extra) * (1 + 0.5j)).astype(np.complex128)
    blob = _record(np.array([0.1]).tobytes()) + _record(np.array([0.2]).tobytes()) + _record(sig.tobytes())
    if footer is not None:
        rec = _record(np.array(footer, dtype=np.float64).tobytes())
        blob += rec[:-2] if damage_footer else rec
    path.write_bytes(blob)
    return str(path)


@pytest.fixture(scope="module")
def seed():
    from pyrpa_gb300 import build, flibs, seed as S
    flibs.load_library(build.LIB if build.LIB.exists() else build.build())
    return S


def test_target_temperature_required(seed, tmp_path):
    with pytest.raises(ValueError, match="temp_new"):
        seed.regrid_sigma_bin(path=_write(tmp_path / "s.bin"))


def test_missing_file(seed, tmp_path):
    with pytest.raises(ValueError, match="cannot open"):
        seed.regrid_sigma_bin(temp_new=0.04, path=str(tmp_path / "absent.bin"))


def test_no_footer_needs_the_mesh_arguments(seed, tmp_path):
    p = _write(tmp_path / "s.bin", footer=None)
    for kw in ({}, {"temp_old": 0.05}, {"temp_old": 0.05, "Norb": 2}, {"Norb": 2, "Nw_old": 8}):
        with pytest.raises(ValueError, match="temp_old, Norb and Nw_old"):
            seed.regrid_sigma_bin(temp_new=0.04, path=p, **kw)


@pytest.mark.parametrize("kw", [{"temp_old": 0.06}, {"Nw_old": 16}, {"Norb": 1}])
def test_arguments_contradicting_the_footer(seed, tmp_path, kw):
    with pytest.raises(ValueError, match="disagrees"):
        seed.regrid_sigma_bin(temp_new=0.04, path=_write(tmp_path / "s.bin"), **kw)


def test_footer_agreement_is_relative(seed, tmp_path):
    """A temp_old within 1e-8 relative of the stored one is accepted (the
    reference's np.isclose(rtol=1e-8, atol=0)): the call gets past the
    checks."""
    p = _write(tmp_path / "s.bin")
    out = _regrid_or_no_device(seed, temp_old=0.05 * (1 + 5e-9), temp_new=0.04, path=p)
    assert out in (None, (3, 8))


def test_size_not_a_multiple_of_the_mesh(seed, tmp_path):
    p = _write(tmp_path / "s.bin", footer=None, extra=3)
    with pytest.raises(ValueError, match="not a multiple"):
        seed.regrid_sigma_bin(temp_old=0.05, temp_new=0.04, Norb=2, Nw_old=8, path=p)


def test_nk_contradicting_the_footer(seed, tmp_path):
    p = _write(tmp_path / "s.bin", footer=(0.05, 8.0, 2.0, 4.0))
    with pytest.raises(ValueError, match="Nk = 3"):
        seed.regrid_sigma_bin(temp_new=0.04, path=p)


def test_damaged_footer_reads_as_absent(seed, tmp_path):
    p = _write(tmp_path / "s.bin", damage_footer=True)
    with pytest.raises(ValueError, match="temp_old, Norb and Nw_old"):
        seed.regrid_sigma_bin(temp_new=0.04, path=p)


def test_truncated_sigma_record(seed, tmp_path):
    p = tmp_path / "s.bin"
    _write(p)
    p.write_bytes(p.read_bytes()[:40])
    with pytest.raises(ValueError, match="mu, mu_OLD and Sigma"):
        seed.regrid_sigma_bin(temp_new=0.04, path=str(p))


def test_well_formed_file_reaches_the_gpu(seed, tmp_path):
    out = _regrid_or_no_device(seed, temp_new=0.04, Nw_new=12, path=_write(tmp_path / "s.bin"),
                               out_path=str(tmp_path / "o.bin"))
    assert out in (None, (3, 12))
