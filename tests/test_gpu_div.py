"""The sweeps' division with a precomputed reciprocal pair (csrc/rc_div.cuh,
Markstein's method) against CUDA's IEEE FP64 division, and the exact 0.5 * x
and 0.0 + x on the integer pipe against the FP64 multiply and add, bit for
bit (needs a GB300 and nvcc)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "rocketcombustor_gb300", "csrc")


def test_div_rn_equals_ieee_division(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "div_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    f"-I{CSRC}", "-o", exe, os.path.join(HERE, "cuda", "div_check.cu")], check=True)
    r = subprocess.run([exe, str(1 << 28)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout


def test_half_and_plus_zero_equal_the_fp64_operations(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "exact_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    f"-I{CSRC}", "-o", exe, os.path.join(HERE, "cuda", "exact_check.cu")], check=True)
    r = subprocess.run([exe, str(1 << 28)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
