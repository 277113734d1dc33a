"""ORACLE — test infrastructure only.

Recipe that compiles the reference's own kernel sources for the CPU, for
pinning the restated oracle (oracle/ref_model.hpp) against them.  It reads the
sources where they lie under the reference checkout (read-only), rewrites only the
CUDA launch syntax `K<<<grid, block>>>(args)` into a call of the serial
launcher of shim_cuda.h, and writes the rewritten translation units and the
library into oracle/_ref/ (git-ignored, never committed).  Nothing else of the
reference is built: CUDPP (absent from the reference) is replaced by the
restated stable compaction and the driver is the restated Segmenter sequence
of ref_model.hpp, so this pins the kernels, not the driver.

Returns None when the reference sources are not mounted (the GPU machines).
"""
from __future__ import annotations

import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REPO = os.path.dirname(ORACLE)
OUT = os.path.join(ORACLE, "_ref")
GEN = os.path.join(OUT, "gen")
LIB = os.path.join(OUT, "libref_oracle.so")

# The kernel files on the solver path, in the order of the reference's unity
# file code/gpuseg/code/src/cuda/CudaKernels.cu (ExportLevelSetVolume.cu, which
# has no caller and uses shared memory, is left out).
FILES = ["Textures.cu", "Coordinates.cu", "Math.cu", "UpdateActiveElements.cu", "MemSetFloat.cu",
         "InitializeCoordinateVolume.cu", "InitializeActiveElementsVolume.cu",
         "InitializeLevelSetVolume.cu", "UpdateLevelSetVolume.cu",
         "UpdateActiveElementsVolume.cu", "FilterDuplicates.cu",
         "ExportActiveElementsVolume.cu"]

_LAUNCH = re.compile(r"([A-Za-z_]\w*(?:\s*<\s*[\w ]+\s*>)?)\s*<<<\s*([^<>]+?)\s*>>>\s*\(")


def rewrite(text: str) -> str:
    return _LAUNCH.sub(lambda m: f"::lss_shim::launcher({m.group(2)}, &{m.group(1)})(", text)


def reference_root() -> str | None:
    """The reference checkout: $LSS_REFERENCE_ROOT, else a directory named
    `reference` beside the repository; None when neither exists."""
    root = os.environ.get("LSS_REFERENCE_ROOT") or os.path.join(os.path.dirname(REPO), "reference")
    return root if os.path.isdir(root) else None


def code_root() -> str | None:
    """code/gpuseg/code of the reference checkout, or None."""
    root = reference_root()
    return os.path.join(root, "code", "gpuseg", "code") if root else None


def build() -> str | None:
    ref = code_root()
    if ref is None:
        return None
    src_dir = os.path.join(ref, "src", "cuda")
    if not os.path.isdir(src_dir):
        return None
    os.makedirs(GEN, exist_ok=True)
    for f in FILES:
        with open(os.path.join(src_dir, f)) as fh:
            text = fh.read()
        with open(os.path.join(GEN, f + ".cpp"), "w") as fh:
            fh.write(rewrite(text))
    cmd = ["g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-w", "-DLSS_ORACLE_REFERENCE_KERNELS", "-DCUDA_ARCH_SM_13",
           "-I", ORACLE, "-I", HERE, "-I", OUT, "-I", ref,
           os.path.join(ORACLE, "lss_oracle.cpp"), "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build())
