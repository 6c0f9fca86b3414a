"""Builds libqgybj.so in-tree (qgybj/libqgybj.so) with nvcc for sm_103a.

Translation units are compiled in parallel; a unit is rebuilt when any
source or header under csrc/ or include/ is newer than its object.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
OUTDIR = HERE / "qgybj"
BUILD = HERE / "_build"
LIB = OUTDIR / "libqgybj.so"

UNITS = ["capi", "engine_fp32", "engine_fp64", "noalloc"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no floating-point contraction, so the host-built tables (DGTSV
# factors, integrating factors) round identically on x86-64 and aarch64
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", str(INCLUDE)]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or Path(c).exists()):
            return c
    return "nvcc"


def _newest_dep() -> float:
    files = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return max(f.stat().st_mtime for f in files)


def _compile(unit: str, extra: list[str]) -> tuple[str, int, str]:
    obj = BUILD / f"{unit}.o"
    cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(CSRC / f"{unit}.cu"), "-o", str(obj)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    return unit, p.returncode, p.stdout + p.stderr


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    newest = _newest_dep()
    stale = [u for u in UNITS
             if force or not (BUILD / f"{u}.o").exists() or (BUILD / f"{u}.o").stat().st_mtime < newest]
    extra = list(extra_flags or [])
    if stale:
        with ThreadPoolExecutor(max_workers=len(stale)) as ex:
            results = list(ex.map(lambda u: _compile(u, extra), stale))
        for unit, rc, out in results:
            if verbose or rc:
                sys.stderr.write(f"[nvcc {unit}] rc={rc}\n{out}")
            if rc:
                raise RuntimeError(f"nvcc failed for {unit}")
    if stale or not LIB.exists() or LIB.stat().st_mtime < newest:
        objs = [str(BUILD / f"{u}.o") for u in UNITS]
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [_nvcc(), *ARCH, "-shared", *objs, "-o", str(tmp), "-lcudart"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode:
            raise RuntimeError(f"link failed: {p.stdout}{p.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
