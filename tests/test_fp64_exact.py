"""The FP64 helpers that replace an FP64 operation by integer work or skip it (qdiv, scale2, neg1, times_sign, the
bit-pattern comparisons, minmod_x, unit_weight_exact, div3) give the same double as the operation itself, on the
GPU, for zeros, subnormals, the ends of the normal range, infinities, NaN, every power of two and random values
(tests/cuda/fp64_exact_check.cu, built here with nvcc -fmad=false like the FP64 kernels)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "fp64_exact_check")
    subprocess.run([nvcc, "-gencode=arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-fmad=false",
                    "-I", os.path.join(ROOT, "casl_p4est_gb300", "csrc"), os.path.join(ROOT, "tests", "cuda", "fp64_exact_check.cu"),
                    "-o", exe], check=True)
    return exe


@pytest.mark.gpu
def test_fp64_helpers_equal_the_operations_they_replace(tmp_path):
    out = subprocess.run([_build(tmp_path)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "fp64 helpers ok" in out.stdout
