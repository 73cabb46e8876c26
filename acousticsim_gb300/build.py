"""Builds the native parts in-tree.

    python -m acousticsim_gb300.build          # library + oracle

Products:
  acousticsim_gb300/libcloth_gb300.so   CUDA kernels (sm_103a) + C ABI + C++ host
  oracle/libcloth_oracle.so             CPU restatement used by the tests as checker

Translation units compile in parallel; nothing is rebuilt when the outputs
are newer than every source.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libcloth_gb300.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "libcloth_oracle.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no implicit multiply-add contraction in device code, so a
# result does not depend on how the compiler shaped a kernel variant (fused
# multiply-adds are written out as fmaf where they are wanted)
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "--fmad=false", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: Path, srcs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(s.stat().st_mtime > t for s in srcs)


def _lib_sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp")) + \
        sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def build_library(force: bool = False) -> Path:
    srcs = _lib_sources()
    if not force and not _stale(LIB, srcs + [Path(__file__)]):
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for cu in sorted(CSRC.glob("*.cu")):
        o = BUILD / (cu.stem + ".o")
        objs.append(o)
        jobs.append([nvcc, *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(cu), "-o", str(o)])
    for cpp in sorted(CSRC.glob("*.cpp")):
        o = BUILD / (cpp.stem + ".o")
        objs.append(o)
        jobs.append(["g++", *CXX_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(cpp), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        list(ex.map(_run, jobs))
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


def build_oracle(force: bool = False) -> Path:
    srcs = [ORACLE_DIR / "cloth_oracle.c", ORACLE_DIR / "cloth_oracle.h"]
    if not force and not _stale(ORACLE_LIB, srcs + [Path(__file__)]):
        return ORACLE_LIB
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    _run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
          "-o", str(tmp), str(ORACLE_DIR / "cloth_oracle.c"), "-lm"])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_library, force)
        b = ex.submit(build_oracle, force)
        a.result()
        b.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)
    print(ORACLE_LIB)
