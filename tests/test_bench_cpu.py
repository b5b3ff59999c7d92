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
