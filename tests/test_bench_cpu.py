"""bench.py on the CPU: the reference arm's JSON line (the oracle on the host
cores, here on a small lattice) and the roofline arithmetic of the native
arm."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _run(args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, env=e,
                       capture_output=True, text=True, timeout=600)
    return r


def test_reference_arm_prints_one_contract_line():
    r = _run(["--impl", "reference", "--lattice", "24,16,16", "--steps", "2", "--warmup", "1"])
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "MLUPS" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["config"]["lattice"] == [24, 16, 16] and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the rate is the lattice's sites over the timed steps
    assert abs(d["value"] - 24 * 16 * 16 * 2 / (d["ms_per_step"] * 2e-3) / 1e6) <= 0.01 * d["value"] + 1e-3


def test_reference_arm_other_ranks_print_nothing():
    r = _run(["--impl", "reference", "--lattice", "8,8,8", "--steps", "1"], env={"RANK": "1"})
    assert r.returncode == 0 and r.stdout.strip() == ""


@pytest.mark.parametrize("prec,walls,q,want", [(0, True, 19, 609), (1, True, 19, 305), (2, True, 19, 153),
                                               (3, False, 19, 152), (1, False, 9, 144), (2, False, 9, 72)])
def test_algorithmic_bytes_per_site(prec, walls, q, want):
    assert bench.bytes_per_site(prec, walls, q) == want


def test_roofline_fraction_is_algorithmic_bytes_over_time_and_peak():
    sites = 4_194_304
    r = bench.roofline(1, sites, 0.5, 6650.0, "measured", None, walls=True)
    alg = 305 * sites
    assert r["algorithmic_bytes"] == alg
    assert abs(r["achieved"] - alg / 0.5e-3 / 1e9) < 0.1
    assert abs(r["frac"] - r["achieved"] / 6650.0) < 1e-4
    assert r["traffic"] is None and r["bound"] == "hbm" and r["unit"] == "GB/s"


def test_recorded_traffic_covers_the_bandwidth_forms():
    """Every bandwidth form the bench reports has a recorded DRAM traffic
    figure with its capture's command and commit."""
    for key in ["channel256x128x128/" + f for f in ("fp64", "fp32", "fp16", "i16")] + \
               ["spinodal512/" + f for f in ("fp32", "fp16", "i16")] + ["d2q9_4096/fp32", "d2q9_4096/fp16"]:
        t = bench.read_traffic(key)
        assert t is not None and t["bytes"] > 0 and "commit" in t["source"], key


def test_kernel_labels_follow_the_dispatch():
    from dlbc_gb300 import lbgpu

    assert bench.step_kernel(lbgpu.FP64, True) == "k_collide"
    assert bench.step_kernel(lbgpu.FP16, True) == "k_pairs"  # planar z-walls of the channel
    assert bench.step_kernel(lbgpu.FP16, True, planar_walls=False) == "k_fused"
    assert bench.step_kernel(lbgpu.FP32, True) == "k_fused" and bench.step_kernel(lbgpu.I16, True) == "k_fused"
    assert bench.step_kernel(lbgpu.FP16, True, unit_tau=False) == "k_fused"
    assert bench.step_kernel(lbgpu.FP32, False) == "k_pairs" and bench.step_kernel(lbgpu.I16, False, False) == "k_pairs"
    assert bench.step_kernel(lbgpu.FP16, False, q=9) == "k_pairs2d"
    assert bench.step_kernel(lbgpu.FP32, False, q=9) == "k_fused2d"


def test_traffic_of_another_kernel_is_not_reported():
    t = {"bytes": 123, "source": "capture", "kernel": "k_fused"}
    r = bench.roofline(2, 1000, 0.01, 6650.0, "measured", t, walls=True)
    assert r["kernel"] == "k_pairs" and r["traffic"] is None and r["traffic_source"] is None
    r = bench.roofline(1, 1000, 0.01, 6650.0, "measured", t, walls=True)
    assert r["kernel"] == "k_fused" and r["traffic"] == 123
