"""Builds ``pyrpa_gb300/libfmod.so`` for sm_103a with nvcc, in tree.

Each translation unit of ``csrc/`` compiles in parallel into ``_build/``; the
shared object is linked next to this file, where ``pyrpa_gb300.flibs`` loads
it and where a pyrpa checkout can take it as its ``libs/libfmod.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libfmod.so"
SOURCES = ["fft.cu", "flex.cu", "drivers.cu", "lws.cu", "abi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is needed to build libfmod.so")


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.cuh"))
    return any(d.stat().st_mtime > obj.stat().st_mtime for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    jobs = []
    for s in SOURCES:
        src, obj = CSRC / s, BUILD / (Path(s).stem + ".o")
        if force or _stale(obj, src):
            jobs.append([nvcc, *ARCH, *FLAGS, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if res.returncode != 0:
                raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
            if verbose:
                print(" ".join(cmd[-3:]), flush=True)
    objs = [str(BUILD / (Path(s).stem + ".o")) for s in SOURCES]
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        res = subprocess.run([nvcc, *ARCH, "-shared", "-o", str(tmp), *objs], capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n" + res.stdout + res.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
