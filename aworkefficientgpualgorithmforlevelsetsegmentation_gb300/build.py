"""Build recipe of liblss.so (the C-ABI library of include/lss.h).

nvcc compiles every translation unit for sm_103a in parallel, then links one
shared library with the CUDA runtime linked statically, so the library loads
on machines without a GPU driver (nothing in it touches the GPU until an
engine is created).  Output: <package>/_build/liblss.so (git-ignored).

The synthetic-volume generators of include/lss_phantom.h are also built on
their own, host code only, into _build/libphantom.so: a process that only
needs the workloads' inputs (the CPU baseline) loads that one and not the
solver library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "liblss.so")
PHANTOM_LIB = os.path.join(BUILD, "libphantom.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
               "-ffp-contract=off", "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]

# (source, extra flags).  The REF translation unit disables FMA contraction so
# that every float operation is one IEEE-754 operation in the reference's order.
UNITS = [
    ("ref_engine.cu", ["-fmad=false"]),
    ("ns_engine.cu", []),
    ("engine_host.cu", []),
    ("lss_api.cpp", ["-x", "cu"]),
    ("compact_api.cu", []),
    ("ns_adjoint.cu", []),
    ("phantom.cpp", []),
]

HEADERS = ["common.cuh", "engine.hpp", "ns_core.hpp", "ns_kernels.cuh", "tma.cuh"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, extra: list[str]) -> str:
    out = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(INCLUDE, "lss.h"), os.path.join(INCLUDE, "lss_phantom.h"), __file__]
    if _newer(out, deps):
        cmd = [nvcc(), *ARCH, *NVCC_COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", out + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        os.replace(out + ".tmp", out)
    return out


def build_phantom() -> str:
    """libphantom.so: the generators of include/lss_phantom.h alone, built by
    the host compiler with the same IEEE settings as liblss.so (identical
    bits; tests/test_abi.py compares the two)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(CSRC, "phantom.cpp")
    deps = [src, os.path.join(INCLUDE, "lss.h"), os.path.join(INCLUDE, "lss_phantom.h"), __file__]
    if _newer(PHANTOM_LIB, deps):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
               "-I", INCLUDE, src, "-o", PHANTOM_LIB + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"phantom library build failed:\n{r.stderr}")
        os.replace(PHANTOM_LIB + ".tmp", PHANTOM_LIB)
    return PHANTOM_LIB


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    build_phantom()
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(*u), UNITS))
    if _newer(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", LIB + ".tmp", *objs,
               "-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print(LIB)
    return LIB


def ptxas_report(src: str = "ns_engine.cu") -> str:
    """Registers / spills / shared memory per kernel (nvcc -Xptxas -v)."""
    cmd = [nvcc(), *ARCH, *NVCC_COMMON, "-Xptxas", "-v", "-c", os.path.join(CSRC, src), "-o", os.devnull]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.stderr


if __name__ == "__main__":
    if "--ptxas" in sys.argv:
        print(ptxas_report(sys.argv[-1] if sys.argv[-1].endswith(".cu") else "ns_engine.cu"))
    else:
        build(force="--force" in sys.argv, verbose=True)
