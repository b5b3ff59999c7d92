"""The fused kernels' run schedule (lb_fused.cuh: plan_runs, sched_units,
sched_run), checked on the host: every plane of every tile in a plane range
is covered by exactly one run, runs are at most run_len long and the long
runs come first (tests/sched_check.cu, compiled with nvcc as host code)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_run_schedule_covers_every_plane_once(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "sched_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", "--expt-relaxed-constexpr", os.path.join(HERE, "sched_check.cu"),
                    "-o", exe], check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
