"""The portable exp/log/pow of include/rc_math.h give the same bits on the GPU
as on the host CPU (needs a GB300 and nvcc): the FP64 kernels and the oracle
rely on it for their bit-identical results."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
INCLUDE = os.path.join(os.path.dirname(HERE), "include")


def test_exp_log_pow_identical_on_gpu_and_host(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "math_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    "-Xcompiler", "-ffp-contract=off", f"-I{INCLUDE}", "-o", exe,
                    os.path.join(HERE, "cuda", "math_check.cu")], check=True)
    r = subprocess.run([exe, str(1 << 22)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches exp 0 log 0 pow 0" in r.stdout
