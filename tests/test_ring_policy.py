"""The retry loop's grid-rebuild policy (csrc/ring_policy.h, shared by the host
loop and the CUDA graph's step kernel): the regrid limit is exactly the
largest radius whose ring fits the row budget, and every radius the search
is asked to take has a ring of at most 2^20 rows (a wider one forces a
rebuild sized for it).  Checked on the host over random widths and radii."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_ring_policy(tmp_path):
    exe = tmp_path / "ring_policy_check"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                           "-I", os.path.join(ROOT, "hybrid_k_nearest_neighbor_self_join_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "ring_policy_check.cpp"), "-o", str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout
    assert "bad=0" in out.stdout
