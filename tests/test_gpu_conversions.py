"""The integer-arithmetic FP32<->FP64 conversions used on the solve path
(ugcore_gb300/csrc/common.cuh) agree bit for bit with the hardware
conversions: a small CUDA program (tests/cuda/conv_check.cu) checks 2^25
random and edge-case values on the GPU."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_conversions_match_hardware(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "conv_check")
    src = os.path.join(ROOT, "tests", "cuda", "conv_check.cu")
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                        "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include"), "-o", exe, src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("mismatches 0 ")
