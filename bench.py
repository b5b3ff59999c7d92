#!/usr/bin/env python3
"""Benchmark of the lattice-Boltzmann timestep on GB300.

Workload (one "step" = one D3Q19 two-component Shan-Chen timestep over the
whole lattice): the droplet-in-channel configuration, 256x128x128 sites,
bounce-back walls on the z = 0 and z = 127 planes, periodic in x and y, a red
sphere of radius 24 (rho_red 1.0 / rho_blue 0.05) in a blue bath (0.05 / 1.0),
body force 1e-6 along x, tau = 1, g = 3.6, psi = 1 - exp(-rho), BDist2
equilibrium.  The headline form is FP64 (the reference's arithmetic); beside
it in the same JSON line:

* ``forms``: the FP32, FP16-offset and I16-offset forms of the same
  workload, each with its roofline and end-to-end figure;
* ``general_tau``: FP32 and FP16 on the same channel with tau = 0.9 (the
  general collision);
* ``d2q9``: the 4096^2 D2Q9 periodic spinodal in FP64, FP32 and FP16;
* ``spinodal512``: the 512^3 periodic spinodal in every form;
* ``batched`` and ``served``: 256 lattices in one batch, and Poisson request
  streams through the serving loop;
* ``e2e``, ``cpu_baseline``, ``clocks``, ``gpu_launches`` and ``roofline``
  of the headline form.

Prints one JSON line (rank 0).  ``--impl reference`` times the reference's
algorithm on the host cores instead (the CPU oracle, all threads).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MLUPS (D3Q19 2-comp Shan-Chen timestep)"
UNIT = "MLUPS"
WORKLOAD = "droplet-channel 256x128x128 D3Q19 two-component Shan-Chen, walls z=0/127, body force 1e-6"
LATTICE = (256, 128, 128)


def workload_params(n=None, eq="BDist2", tau=1.0):
    from dlbc_gb300 import params
    n = LATTICE if n is None else n
    lines = [
        "[lattice]", f"gn = [{n[0]}, {n[1]}, {n[2]}]",
        "[lb]", "components = 2", 'fieldNames = ["red", "blue"]', f"tau = [{tau!r}, {tau!r}]",
        f"eqdist.eqDistForm = {eq}",
        "force.enableShanChen = true", "force.gcc = [[0.0, 3.6], [3.6, 0.0]]",
        "force.psiForm = Exponential", "force.globalAcc = [1e-6, 0.0, 0.0]",
        "init.fluidInit = [EqDistSphere, EqDistSphere]",
        "init.fluidDensities = [[1.0, 0.05], [0.05, 1.0]]",
        "init.initRadius = 24.0", "init.interfaceThickness = 0.0",
        "mask.maskInit = Walls",
        "mask.dimensionHasWall = [[false, false], [false, false], [true, true]]",
        "mask.wallThickness = 1",
    ]
    return params.LBParams.from_dict(params.parse_lines(lines), "d3q19")


def bytes_per_site(precision: int, walls: bool = True, q: int = 19) -> int:
    """Algorithmic bytes per site-update: every population read once and
    written once (2 components x q), plus the 1-byte mask when walls exist."""
    s = {0: 8, 1: 4, 2: 2, 3: 2}[precision]
    return 2 * 2 * q * s + (1 if walls else 0)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def time_form(p, fluids, mask, precision, steps, warmup, device, torch):
    """Device-timed steps of one form: (ms/step, collide-kernel ms/launch,
    density/psi-kernel ms/launch, kernel launches in the timed region)."""
    from dlbc_gb300 import lbgpu
    g = lbgpu.GPULattice(p, precision=precision, device=device)
    g.upload(fluids, mask)
    stream = torch.cuda.Stream(device=device)
    g.set_stream(stream.cuda_stream)
    g.step(warmup)
    g.synchronize()
    g.profile(True)
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    n0 = g.launch_count
    start.record(stream)
    g.step(steps)
    stop.record(stream)
    stop.synchronize()
    torch.cuda.synchronize(device)
    ms = start.elapsed_time(stop)
    launches = g.launch_count - n0
    k1_ms, k1_n = g.kernel_time(0)
    k2_ms, k2_n = g.kernel_time(1)
    g.profile(False)
    g.close()
    return ms / steps, k2_ms / max(k2_n, 1), k1_ms / max(k1_n, 1), launches


def time_form_device(p, precision, steps, warmup, device, torch, seed=11):
    """time_form for a lattice initialised on the device (lbgpu_init_fields):
    no host copy of the fields, for lattices too large to build on the host."""
    from dlbc_gb300 import lbgpu
    g = lbgpu.GPULattice(p, precision=precision, device=device)
    g.init_device(seed)
    stream = torch.cuda.Stream(device=device)
    g.set_stream(stream.cuda_stream)
    g.step(warmup)
    g.synchronize()
    g.profile(True)
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    n0 = g.launch_count
    start.record(stream)
    g.step(steps)
    stop.record(stream)
    stop.synchronize()
    torch.cuda.synchronize(device)
    ms = start.elapsed_time(stop)
    launches = g.launch_count - n0
    k1_ms, k1_n = g.kernel_time(0)
    k2_ms, k2_n = g.kernel_time(1)
    g.profile(False)
    g.close()
    return ms / steps, k2_ms / max(k2_n, 1), k1_ms / max(k1_n, 1), launches


def storage_scale(fluids, precision, q=19):
    """The FP16 / I16 offsets' rest density and scale that an upload of
    these fields derives (the rules of lbgpu_upload), to pin them."""
    import numpy as np
    from dlbc_gb300 import lbgpu
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    rho0, scale = [], []
    for f in fluids:
        a = f[2:-2, 2:-2, 2:-2]
        r = float(a.sum(axis=-1).mean())
        dev = float(np.abs(a / w - r).max())
        rho0.append(r)
        scale.append(max(abs(r), 4 * dev) / 1024 if precision == lbgpu.FP16 else 3 * max(abs(r), dev) / 32767)
    return rho0, scale


def e2e_form(p, fluids, hb, hm, precision, n_e2e, device, world, sites, barrier, dist):
    """End to end through the C ABI: per step, one lbgpu_step_host call on
    pinned host AoS arrays (inputs in, the same arrays out), and beside it
    lbgpu_upload + lbgpu_step(1) + lbgpu_download one after another.  FP16
    and I16 pin their storage scale first (the wavefront needs it)."""
    from dlbc_gb300 import lbgpu, replicas
    g = lbgpu.GPULattice(p, precision=precision, device=device)
    if precision in (lbgpu.FP16, lbgpu.I16):
        g.set_storage_scale(*storage_scale(fluids, precision))
    g.upload(hb, hm)

    def timed(one_step):
        for _ in range(3):
            one_step()
        barrier()
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            one_step()
        barrier()
        dt = replicas.max_over_ranks(time.perf_counter() - t0, dist, device=f"cuda:{device}")
        return world * sites * n_e2e / dt / 1e6

    def three_calls():
        g.upload(hb, hm)
        g.step(1)
        g.download(hb)

    # fresh inputs each time: the arrays hold the fields of the last step
    e2e_value = timed(lambda: g.step_host(hb, hm, hb))
    e2e_seq = timed(three_calls)
    g.close()
    for h, f in zip(hb, fluids):
        h.copy_(__import__("torch").from_numpy(f))
    return {"value": round(e2e_value, 2), "unit": UNIT,
            "h2d_bytes_per_step": sum(int(x.numel()) * 8 for x in hb) + int(hm.numel()) * 4,
            "d2h_bytes_per_step": sum(int(x.numel()) * 8 for x in hb), "steps": n_e2e,
            "call": "lbgpu_step_host(pinned AoS haloed fluids + mask in, the same arrays out): input copies, "
                    "kernels and output copies overlap by chunks of 8 x-planes",
            "three_calls_value": round(e2e_seq, 2),
            "three_calls": "lbgpu_upload -> lbgpu_step(1) -> lbgpu_download, one after another"}


GENERAL_TAU = 0.9
D2Q9_N = 4096
SPINODAL_N = 512
SPINODAL_WORKLOAD = (f"periodic spinodal {SPINODAL_N}^3 D3Q19 two-component Shan-Chen, rho 0.7 +- 0.02, "
                     f"tau 1, g 3.6, BDist2")


def run_spinodal(device, torch, peak, peak_kind, fp64_peak, dist=None, n=SPINODAL_N, forms=None):
    """The precision-study lattice (512^3 periodic spinodal decomposition,
    134 M sites) in every form, initialised on the device: MLUPS, ms/step and
    the dominant kernel's HBM roofline per form."""
    from dlbc_gb300 import lbgpu, precision_study, replicas
    p = precision_study.spinodal_params(n, 0.02)
    sites = n ** 3
    world = dist.get_world_size() if dist is not None else 1
    out = {"workload": SPINODAL_WORKLOAD.replace(str(SPINODAL_N), str(n)), "lattice": [n, n, n],
           "init": "device (lbgpu_init_fields, counter-based noise)",
           "l2": "inputs larger than L2 (FP16 populations alone 10.2 GB)", "forms": {}}
    for name, prec, steps in (("fp64", lbgpu.FP64, 10), ("fp32", lbgpu.FP32, 40), ("fp16", lbgpu.FP16, 40),
                              ("i16", lbgpu.I16, 40)):
        if forms and name not in forms:
            continue
        ms, k2, k1, launches = time_form_device(p, prec, steps, 3, device, torch)
        ms = replicas.max_over_ranks(ms, dist, device=f"cuda:{device}")
        out["forms"][name] = {
            "value": round(world * sites / (ms * 1e-3) / 1e6, 1), "unit": UNIT, "ms_per_step": round(ms, 4),
            "steps": steps, "warmup": 3, "gpu_launches": launches,
            "roofline": roofline(prec, sites, k2, peak, peak_kind, read_traffic(f"spinodal{n}/{name}"),
                                 fp64_peak, walls=False),
            "step_roofline_frac": round(bytes_per_site(prec, False) * sites / (ms * 1e-3) / 1e9 / peak, 4)}
    return out


def run_d2q9(device, torch, peak, peak_kind, dist=None, n=D2Q9_N, forms=None):
    """The D2Q9 spinodal (n^2 periodic sites, the D3Q19 spinodal's physics:
    rho 0.7 +- 0.02, tau = 1, g = 3.6, BDist2), initialised on the device, in
    the FP64 two-kernel form and the fused FP32 / FP16 forms (k_fused2d)."""
    from dlbc_gb300 import lbgpu, precision_study, replicas
    p = precision_study.spinodal_params(n, 0.02, d=2)
    sites = n * n
    world = dist.get_world_size() if dist is not None else 1
    out = {"workload": f"periodic spinodal {n}^2 D2Q9 two-component Shan-Chen, rho 0.7 +- 0.02, tau 1, g 3.6, "
                       f"BDist2", "lattice": [n, n], "init": "device (lbgpu_init_fields, counter-based noise)",
           "l2": f"inputs larger than L2 (FP16 populations, both buffers: {2 * 2 * 9 * 2 * sites / 1e9:.2f} GB)",
           "forms": {}}
    for name, prec, steps in (("fp64", lbgpu.FP64, 10), ("fp32", lbgpu.FP32, 40), ("fp16", lbgpu.FP16, 40)):
        if forms and name not in forms:
            continue
        ms, k2, k1, launches = time_form_device(p, prec, steps, 3, device, torch)
        ms = replicas.max_over_ranks(ms, dist, device=f"cuda:{device}")
        out["forms"][name] = {
            "value": round(world * sites / (ms * 1e-3) / 1e6, 1), "unit": UNIT, "ms_per_step": round(ms, 4),
            "steps": steps, "warmup": 3, "gpu_launches": launches,
            "roofline": roofline(prec, sites, k2, peak, peak_kind, read_traffic(f"d2q9_{n}/{name}"), None,
                                 walls=False, q=9),
            "step_roofline_frac": round(bytes_per_site(prec, False, 9) * sites / (ms * 1e-3) / 1e9 / peak, 4)}
    return out


# FP64 operations per site of k_collide (D3Q19, two components, BDist2,
# tau = 1, z walls): ncu counted 4.0 M DMUL + 3.9 M DADD warp instructions
# (no DFMA: the reference's arithmetic without contraction) for the 524,288
# sites of the 128x64x64 case of this workload, i.e. 7.9 M x 32 / 524,288.
K_COLLIDE_FP64_OPS_PER_SITE = 482


def fp64_rate(device):
    """Measured FP64 instruction rate of this GPU (DADD, DMUL and DFMA
    dependency chains over every SM, timed with CUDA events; the
    microbenchmark in dlbc_gb300/csrc/peak_fp64.cu), in G thread operations
    per second; None if it cannot run."""
    import ctypes
    from dlbc_gb300 import build
    try:
        L = ctypes.CDLL(build.PEAK_LIB)
        L.peak_fp64_rates.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        rates = (ctypes.c_double * 3)()
        if L.peak_fp64_rates(device, 16384, rates) != 0:
            return None
        return {"dadd": rates[0] / 1e9, "dmul": rates[1] / 1e9, "dfma": rates[2] / 1e9}
    except OSError:
        return None


def step_kernel(precision, walls, unit_tau=True, nz_even=True, q=19, planar_walls=True):
    """The kernel that runs the BDist2 step (the library's dispatch rules,
    lbk::pairs_eligible and lbk::pairs2d_eligible): k_collide for FP64; for
    D2Q9 k_pairs2d for FP16 with every tau = 1, no solid site and an even ny
    (nz_even stands for it), k_fused2d otherwise; for D3Q19 k_pairs without
    solid sites and with an even nz for I16 and for FP32/FP16 with every
    tau = 1, and for FP16 with every tau = 1 also with planar z-walls (the
    channel's: solid exactly at z = 0 and nz - 1, nz a multiple of 64, no
    wall force; planar_walls); k_fused otherwise."""
    from dlbc_gb300 import lbgpu
    if precision == lbgpu.FP64:
        return "k_collide"
    if q == 9:
        return "k_pairs2d" if precision == lbgpu.FP16 and unit_tau and not walls and nz_even else "k_fused2d"
    if not walls and nz_even and (precision == lbgpu.I16 or unit_tau):
        return "k_pairs"
    if walls and planar_walls and nz_even and precision == lbgpu.FP16 and unit_tau:
        return "k_pairs"
    return "k_fused"


def roofline(precision, sites, kernel_ms, peak, peak_kind, traffic=None, fp64_peak=None, walls=True,
             kernel=None, q=19):
    """HBM roofline of the dominant kernel: k_collide (FP64 two-kernel step),
    k_fused or k_pairs (the single-pass step).  k_collide is limited by the
    FP64 pipe, not by HBM: its FP64 instruction rate against the FP64 rate
    measured on this GPU goes beside the HBM figures."""
    alg = bytes_per_site(precision, walls, q) * sites
    achieved = alg / (kernel_ms * 1e-3) / 1e9
    from dlbc_gb300 import lbgpu
    if kernel is None:
        kernel = step_kernel(precision, walls, q=q)
    if traffic and traffic.get("kernel") not in (None, kernel):
        traffic = None  # the recorded capture is of another kernel
    out = {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 1), "peak": peak,
           "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
           "traffic": traffic["bytes"] if traffic else None,
           "traffic_source": traffic["source"] if traffic else None, "algorithmic_bytes": alg,
           "kernel_ms": round(kernel_ms, 5)}
    if precision == lbgpu.FP64 and q == 19:
        g = K_COLLIDE_FP64_OPS_PER_SITE * sites / (kernel_ms * 1e-3) / 1e9
        lim = {"pipe": "fp64", "ops_per_site": K_COLLIDE_FP64_OPS_PER_SITE, "achieved": round(g, 1),
               "unit": "G FP64 thread instructions/s"}
        if fp64_peak:
            # k_collide issues DADD and DMUL only (no contraction)
            pk = 0.5 * (fp64_peak["dadd"] + fp64_peak["dmul"])
            lim.update({"peak": round(pk, 1), "peak_kind": "measured (DADD/DMUL chains, peak_fp64.cu)",
                        "frac": round(g / pk, 4), "measured_rates": {k: round(v, 1) for k, v in fp64_peak.items()}})
        out["limiter"] = lim
    return out


def read_traffic(key):
    """DRAM bytes (read + write) per launch of the dominant kernel for a
    workload and form, from the one-pass ncu capture recorded in
    profiles/traffic.json (with the commit the capture ran at), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        e = d["captures"][key]
        src = f"ncu one-pass capture of {e['kernel']} at commit {e['commit']} ({e['command']})"
        if e.get("scaled"):
            src += "; " + e["scaled"]
        return {"bytes": e["bytes"], "source": src, "kernel": e["kernel"].split("<")[0]}
    except Exception:
        return None


def cpu_baseline(p, budget_s=12.0, threads=None):
    """The CPU oracle on the host cores, on a bounded number of steps of
    the same lattice."""
    from oracle import oracle as orc
    threads = threads or os.cpu_count() or 1
    o = orc.Oracle(p, exp_mode=1, threads=threads)
    t0 = time.perf_counter()
    o.run(1)
    t1 = time.perf_counter() - t0
    steps = max(1, min(50, int(budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    sites = p.gn[0] * p.gn[1] * p.gn[2]
    return {"value": round(sites * steps / dt / 1e6, 3), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} timesteps of the full {p.gn[0]}x{p.gn[1]}x{p.gn[2]} lattice after 1 untimed "
                      f"step (FP64 oracle, OpenMP over x-slabs)"}


def batched_params(n_sims=256, seed=3):
    """The batched workload: cubic periodic lattices, L in {32, 48, 64, 80, 96}, two red
    spheres of radius L/6 with a 2-site gap along x in a blue bath, tau ~
    U[0.8, 1.2] (both components), g ~ U[3.2, 4.0]."""
    import numpy as np
    from dlbc_gb300 import params
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_sims):
        L = int(rng.choice([32, 48, 64, 80, 96]))
        tau = float(rng.uniform(0.8, 1.2))
        g = float(rng.uniform(3.2, 4.0))
        r = L / 6.0
        lines = [
            "[lattice]", f"gn = [{L}, {L}, {L}]",
            "[lb]", "components = 2", 'fieldNames = ["red", "blue"]', f"tau = [{tau!r}, {tau!r}]",
            "eqdist.eqDistForm = BDist2", "force.enableShanChen = true",
            f"force.gcc = [[0.0, {g!r}], [{g!r}, 0.0]]", "force.psiForm = Exponential",
            "force.globalAcc = [0.0, 0.0, 0.0]",
            "init.fluidInit = [EqDistTwoSpheres, EqDistTwoSpheres]",
            "init.fluidDensities = [[1.0, 0.05], [0.05, 1.0]]",
            f"init.initRadius = {r!r}", f"init.initSeparation = [{2 * r + 2!r}, 0.0, 0.0]",
            "init.interfaceThickness = 0.0",
        ]
        out.append(params.LBParams.from_dict(params.parse_lines(lines), "d3q19"))
    return out


def run_batched(device, torch, n_sims=256, steps=2000, baseline_steps=20, dist=None):
    """The batched workload in one batch (FP16 offset storage, FP32 arithmetic), timed with
    CUDA events on the batch's stream; the sequential baseline runs each size
    class alone in the plain FP64 form for a few steps and extrapolates.  With
    several ranks the lattices are split over them by size (no exchange) and
    the time is the slowest rank's."""
    from dlbc_gb300 import lbgpu, replicas
    all_ps = batched_params(n_sims)
    world = dist.get_world_size() if dist is not None else 1
    rank = dist.get_rank() if dist is not None else 0
    mine = replicas.shard([q.gn[0] * q.gn[1] * q.gn[2] for q in all_ps], world)[rank]
    ps = [all_ps[i] for i in mine]
    b = lbgpu.Batch(precision=lbgpu.FP16, device=device)
    for p in ps:
        b.add_device(p)
    stream = torch.cuda.Stream(device=device)
    b.set_stream(stream.cuda_stream)
    b.step(12)  # autotune (8 steps) + graph capture, untimed
    b.synchronize()
    shape = b.launch_shape()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    n0 = b.launch_count
    start.record(stream)
    b.step(steps)
    stop.record(stream)
    stop.synchronize()
    ms = replicas.max_over_ranks(start.elapsed_time(stop), dist, device=f"cuda:{device}")
    launches = b.launch_count - n0
    sites = sum(p.gn[0] * p.gn[1] * p.gn[2] for p in all_ps)
    dev_bytes = b.device_bytes
    b.close()
    ps = all_ps
    # sequential baselines per size class: the plain FP64 form, and the
    # same FP16 form one lattice at a time (what batching itself gains)
    def sequential(prec, nsteps):
        per_step = {}
        for L in sorted({p.gn[0] for p in ps}):
            p = next(q for q in ps if q.gn[0] == L)
            g = lbgpu.GPULattice(p, precision=prec, device=device)
            g.init_device()
            g.step(3)
            g.synchronize()
            t0 = time.perf_counter()
            g.step(nsteps)
            g.synchronize()
            per_step[L] = (time.perf_counter() - t0) / nsteps
            g.close()
        return sum(per_step[p.gn[0]] * steps for p in ps)

    seq_s = sequential(lbgpu.FP64, baseline_steps)
    seq16_s = sequential(lbgpu.FP16, 10 * baseline_steps)
    return {
        "workload": f"{n_sims} periodic D3Q19 two-sphere lattices, L in {{32,48,64,80,96}}, {steps} steps, "
                    f"tau~U[0.8,1.2], g~U[3.2,4.0]",
        "form": "fp16 offset storage, fp32 arithmetic", "sims": n_sims, "steps": steps,
        "ranks": world, "sharding": "whole lattices, balanced by sites (largest first), no exchange",
        "total_sites": int(sites), "time_s": round(ms / 1e3, 3), "sims_per_s": round(n_sims / (ms / 1e3), 3),
        "aggregate_mlups": round(sites * steps / (ms / 1e3) / 1e6, 1), "launch_shape": list(shape),
        "kernel_launches": launches, "device_bytes": int(dev_bytes),
        "sequential_fp64_baseline": {"sims_per_s": round(n_sims / seq_s, 4), "time_s": round(seq_s, 1),
                                     "how": f"each size class alone, plain FP64 form, {baseline_steps} timed "
                                            f"steps, extrapolated to {steps} steps x {n_sims} sims"},
        "speedup_vs_sequential_fp64": round(seq_s / (ms / 1e3), 1),
        "sequential_fp16_baseline": {"sims_per_s": round(n_sims / seq16_s, 4), "time_s": round(seq16_s, 1),
                                     "how": f"each size class alone, the same FP16 form, {10 * baseline_steps} "
                                            f"timed steps (host-timed, one launch per step), extrapolated"},
        "speedup_vs_sequential_fp16": round(seq16_s / (ms / 1e3), 2),
    }


def _serve_stream(device, n_requests, rate, step_scale, budget_gb, dist, seed):
    import numpy as np
    from dlbc_gb300 import lbgpu, replicas, serve
    reqs = serve.request_stream(n_requests, rate=rate, seed=seed, step_scale=step_scale)
    world = dist.get_world_size() if dist is not None else 1
    rank = dist.get_rank() if dist is not None else 0
    srv = serve.Server(precision=lbgpu.FP16, budget_bytes=budget_gb * 1e9, device=device)
    out = srv.run([r for r in reqs if r.rid % world == rank])
    srv.batch.close()
    parts = replicas.gather_to_root(out, dist)
    if rank != 0:
        return None, reqs
    if world > 1:
        results = [r for part in parts for r in part["results"]]
        lat = np.array([r["latency"] for r in results])
        wall = max(part["makespan_s"] for part in parts)
        work = sum(r["sites"] * r["steps"] for r in results)
        out = {"requests": len(results), "p50_latency_s": float(np.percentile(lat, 50)),
               "p99_latency_s": float(np.percentile(lat, 99)), "makespan_s": wall,
               "aggregate_mlups": work / wall / 1e6, "site_steps": sum(p["site_steps"] for p in parts),
               "peak_members": max(p["peak_members"] for p in parts),
               "peak_device_bytes": max(p["peak_device_bytes"] for p in parts), "results": results}
    results = out.pop("results")
    out["mean_queue_s"] = float(np.mean([r["queue"] for r in results]))
    out["ranks"] = world
    out["workload"] = (f"{n_requests} droplet-channel requests, Poisson {rate:.3g}/s, x~U[48,256], y=z~U[32,128], "
                       f"radius~U[6,y/4], steps~U[2000,20000] x {step_scale}, acc~U[0,1e-5], "
                       f"budget {budget_gb} GB, fp16 storage")
    for k in ("p50_latency_s", "p99_latency_s", "makespan_s", "aggregate_mlups", "mean_queue_s"):
        out[k] = round(out[k], 3)
    return out, reqs


def run_served(device, n_requests=200, n_sustained=100, step_scale=1.0, rate=50.0, budget_gb=120.0, dist=None):
    """The served workload with full-length requests: a Poisson stream at
    `rate` (50/s, far beyond what one GPU sustains: latency is queueing),
    then a second stream at 0.9 x the sustainable rate measured on the
    first (requests/s the aggregate MLUPS can serve).  Poisson arrivals,
    admission by an HBM budget, continuous batching.  With several ranks,
    request i goes to rank i mod N (each GPU serves its own stream, no
    exchange); latencies are gathered on rank 0."""
    import numpy as np
    over, reqs = _serve_stream(device, n_requests, rate, step_scale, budget_gb, dist, seed=2024)
    sustainable = None
    if over is not None:
        mean_work = float(np.mean([r.sites * r.steps for r in reqs]))
        sustainable = over["aggregate_mlups"] * 1e6 / mean_work
        over["sustainable_rate_per_s"] = round(sustainable, 3)
    if dist is not None:
        import torch
        t = torch.tensor([sustainable or 0.0], device=f"cuda:{device}")
        dist.broadcast(t, 0)
        sustainable = float(t.item())
    steady = None
    if n_sustained > 0 and sustainable and sustainable > 0:
        steady, _ = _serve_stream(device, n_sustained, 0.9 * sustainable, step_scale, budget_gb, dist, seed=2025)
    if over is None:
        return None
    return {"oversubscribed": over, "sustained": steady, "step_scale": step_scale}


def run_reference(args):
    """--impl reference: the reference's CPU algorithm (the oracle) on all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import oracle as orc
    p = workload_params()
    threads = os.cpu_count() or 1
    o = orc.Oracle(p, exp_mode=1, threads=threads)
    o.run(max(0, min(args.warmup, 3)))
    steps = max(1, min(args.steps, 20))
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    sites = LATTICE[0] * LATTICE[1] * LATTICE[2]
    v = sites * steps / dt / 1e6
    line = {
        "metric": METRIC, "value": round(v, 3), "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
        "warmup": min(args.warmup, 3), "ms_per_step": round(dt / steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "lattice": list(LATTICE), "form": "fp64", "eq_form": "BDist2"},
        "impl": "reference",
        "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{steps} timesteps of the full lattice (the reference's D/MPI build cannot "
                                   f"be compiled: no D toolchain and an empty 'unstandard' submodule)"},
        "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--served-requests", type=int, default=200,
                    help="requests of the oversubscribed served stream (0.3 x as many at the sustainable rate)")
    ap.add_argument("--no-spinodal", action="store_true", help="skip the 512^3 spinodal block")
    ap.add_argument("--no-general-tau", action="store_true", help="skip the tau != 1 block")
    ap.add_argument("--no-d2q9", action="store_true", help="skip the D2Q9 block")
    ap.add_argument("--d2q9-n", type=int, default=D2Q9_N, help="edge of the D2Q9 lattice")
    ap.add_argument("--d2q9-forms", default=None, help="comma-separated forms of the D2Q9 block (default all)")
    ap.add_argument("--spinodal-n", type=int, default=SPINODAL_N, help="edge of the spinodal lattice")
    ap.add_argument("--spinodal-forms", default=None, help="comma-separated forms of the spinodal block (default all)")
    ap.add_argument("--form", default="fp64", choices=["fp64", "fp32", "fp16", "i16"],
                    help="headline form (the others are reported under 'forms')")
    ap.add_argument("--lattice", default=None,
                    help="override the lattice as X,Y,Z (small cases for profiling; the default is the workload)")
    args = ap.parse_args()
    if args.lattice:
        global LATTICE
        LATTICE = tuple(int(v) for v in args.lattice.split(","))
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    device = local

    from dlbc_gb300 import build, init, lbgpu, replicas
    build.build()
    p = workload_params(LATTICE)
    fluids, mask = init.init_fields(p)
    sites = LATTICE[0] * LATTICE[1] * LATTICE[2]
    peak, peak_kind = measured_peaks()
    fp64_peak = fp64_rate(device)
    forms_all = {"fp64": lbgpu.FP64, "fp32": lbgpu.FP32, "fp16": lbgpu.FP16, "i16": lbgpu.I16}
    head = forms_all[args.form]
    dtype = {"fp64": "f64", "fp32": "f32", "fp16": "f16-storage/f32", "i16": "i16-storage/f32"}[args.form]

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(device)

    # ---- headline form, inputs resident in HBM
    barrier()
    with ClockSampler(device) as clk:
        ms_step, k2_ms, k1_ms, launches = time_form(p, fluids, mask, head, args.steps, args.warmup, device, torch)
    barrier()
    ms_max = replicas.max_over_ranks(ms_step, dist, device=f"cuda:{device}")
    value = world * sites / (ms_max * 1e-3) / 1e6

    # ---- end to end through the C ABI with pinned host buffers:
    # per step, upload the state (populations + mask), one timestep, download
    e2e = None
    hb = hm = None
    if args.e2e_steps > 0:
        hb = [torch.from_numpy(f).pin_memory() for f in fluids]
        hm = torch.from_numpy(mask).pin_memory()
        e2e = e2e_form(p, fluids, hb, hm, head, args.e2e_steps, device, world, sites, barrier, dist)

    # ---- the other forms of the same workload
    forms = {}
    if not args.no_forms:
        for name, prec in forms_all.items():
            if name == args.form:
                continue
            f_ms, f_k2, f_k1, _ = time_form(p, fluids, mask, prec, args.steps, args.warmup, device, torch)
            forms[name] = {"value": round(world * sites / (f_ms * 1e-3) / 1e6, 1),
                           "ms_per_step": round(f_ms, 4),
                           "k_density_psi_ms": round(f_k1, 4), "k_collide_ms": round(f_k2, 4),
                           "roofline": roofline(prec, sites, f_k2, peak, peak_kind,
                                                read_traffic(f"channel{'x'.join(map(str, LATTICE))}/{name}"),
                                                fp64_peak),
                           "step_roofline_frac": round(bytes_per_site(prec) * sites / (f_ms * 1e-3) / 1e9 / peak,
                                                       4)}
            if hb is not None:
                forms[name]["e2e"] = e2e_form(p, fluids, hb, hm, prec, args.e2e_steps, device, world, sites,
                                              barrier, dist)

    # ---- the general collision (tau != 1) of the bandwidth forms, beside
    # the tau = 1 figures above
    general_tau = None
    if not args.no_general_tau:
        p9 = workload_params(LATTICE, tau=GENERAL_TAU)
        f9, m9 = init.init_fields(p9)
        general_tau = {"workload": f"the same channel with tau = {GENERAL_TAU} for both components", "forms": {}}
        for name in ("fp32", "fp16"):
            prec = forms_all[name]
            g_ms, g_k2, _, _ = time_form(p9, f9, m9, prec, args.steps, args.warmup, device, torch)
            g_ms = replicas.max_over_ranks(g_ms, dist, device=f"cuda:{device}")
            v = world * sites / (g_ms * 1e-3) / 1e6
            e = {"value": round(v, 1), "ms_per_step": round(g_ms, 4),
                 "roofline": roofline(prec, sites, g_k2, peak, peak_kind, None, None, kernel="k_fused")}
            unit = forms.get(name, {}).get("value") if name != args.form else value
            if unit:
                e["vs_tau_1"] = round(v / unit, 4)
            general_tau["forms"][name] = e

    d2q9 = None if args.no_d2q9 else run_d2q9(device, torch, peak, peak_kind, dist=dist, n=args.d2q9_n,
                                              forms=args.d2q9_forms.split(",") if args.d2q9_forms else None)
    spinodal = None if args.no_spinodal else run_spinodal(device, torch, peak, peak_kind, fp64_peak, dist=dist,
                                                            n=args.spinodal_n,
                                                            forms=args.spinodal_forms.split(",") if args.spinodal_forms
                                                            else None)
    del hb, hm
    batched = None if args.no_batched else run_batched(device, torch, dist=dist)
    served = None if args.no_served else run_served(device, n_requests=args.served_requests,
                                                    n_sustained=max(10, (3 * args.served_requests) // 10), dist=dist)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(p)

    if rank == 0:
        pop_gb = 2 * 2 * 19 * {0: 8, 1: 4, 2: 2, 3: 2}[head] * sites / 1e9
        l2_note = ("inputs larger than L2" if pop_gb > 0.129 else "inputs smaller than L2 (129 MB)") + \
            f" (populations, both buffers: {pop_gb:.2f} GB), no flush between steps"
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_max, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": {"workload": WORKLOAD if LATTICE == (256, 128, 128) else f"droplet-channel {LATTICE}",
                       "lattice": list(LATTICE), "form": args.form, "eq_form": "BDist2",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": l2_note},
            "roofline": roofline(head, sites, k2_ms, peak, peak_kind,
                                 read_traffic(f"channel{'x'.join(map(str, LATTICE))}/{args.form}"), fp64_peak),
            "kernels_ms": {"k_density_psi": round(k1_ms, 4), "k_collide": round(k2_ms, 4)},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "forms": forms,
            "general_tau": general_tau,
            "d2q9": d2q9,
            "spinodal512": spinodal,
            "batched": batched,
            "served": served,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
