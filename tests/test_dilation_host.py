"""Host build and run of tests/dilation_check.cu: the bit-parallel brick
dilation of the NS kernels against brute force (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_bit_parallel_dilation_matches_brute_force(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "dilation_check")
    csrc = os.path.join(ROOT, "aworkefficientgpualgorithmforlevelsetsegmentation_gb300", "csrc")
    subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-O1", "-I", os.path.join(ROOT, "include"),
                    "-I", csrc, "-gencode", "arch=compute_103a,code=sm_103a",
                    os.path.join(HERE, "dilation_check.cu"), "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr
