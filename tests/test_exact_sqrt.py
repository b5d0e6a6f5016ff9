"""The integer-pipe double square root used by the BETA rule's sampled mean
distance equals the correctly rounded sqrt: on the host on 45 million inputs
(random bit patterns over the whole positive range, subnormals included; sums
of two squared floats, the estimator's own terms; perfect squares and their
neighbours), and on the GPU, built by nvcc, on 1.3 billion more."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_exact_sqrt_matches_libm(tmp_path):
    exe = tmp_path / "exact_sqrt_check"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                           "-I", os.path.join(ROOT, "hybrid_k_nearest_neighbor_self_join_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "exact_sqrt_check.cpp"), "-o", str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout
    assert "bad=0" in out.stdout


@pytest.mark.gpu
def test_exact_sqrt_matches_gpu_sqrt(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "exact_sqrt_gpu_check"
    subprocess.check_call([nvcc, "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                           "-I", os.path.join(ROOT, "hybrid_k_nearest_neighbor_self_join_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "exact_sqrt_gpu_check.cu"), "-o", str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout
    assert "bad=0" in out.stdout
