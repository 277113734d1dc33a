"""ORACLE — test infrastructure only.

Build recipe of the CPU oracle: compiles oracle/lss_oracle.cpp into
oracle/_build/liboracle.so with g++ (-ffp-contract=off, so every float
operation is one IEEE-754 operation on x86-64 and aarch64 alike).

When the reference sources are present (this happens only where they are
mounted, never on the machines that run the GPU tests), build_reference()
also compiles the reference's own kernel sources for the CPU; see
oracle/ref_shim/build_ref.py.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

CXXFLAGS = ["-O2", "-std=c++20", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
            "-fno-fast-math", "-Wall", "-Wno-unused-function"]


def _stale(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("lss_oracle.cpp", "ref_model.hpp", "ns_model.hpp", "ns_adjoint.hpp")]
    if force or _stale(LIB, srcs):
        cmd = ["g++", *CXXFLAGS, "-I", HERE, srcs[0], "-o", LIB + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def build_reference() -> str | None:
    """Compiles the reference's kernels for the CPU into oracle/_ref/ when the
    reference sources exist here; returns the library path or None."""
    sys.path.insert(0, os.path.join(HERE, "ref_shim"))
    try:
        import build_ref  # type: ignore
    finally:
        sys.path.pop(0)
    return build_ref.build()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    if "--reference" in sys.argv:
        print(build_reference())
