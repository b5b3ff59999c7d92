"""Serving loop: continuous batching of lattice-Boltzmann requests on one GPU.

Requests (droplet-in-channel simulations of random size and length) arrive
as a Poisson stream and wait until the batch can admit them within the
device-memory budget (lbgpu_batch_add_init: the initial fields are computed
on the device, so nothing but the parameters crosses the bus).  Admission
is fit-first with aging: waiting requests are scanned in arrival order and
every one that fits is admitted, so a large request at the head does not
hold back smaller ones behind it, until the head has waited longer than
`age_limit_s`; from then on nothing overtakes it.  Admitted requests step
together in one persistent launch per timestep (lbgpu_batch_step), in
chunks of steps that end when the first member finishes and, while the
budget has room, near the next arrival (estimated from the measured step
rate), so that a new request joins within a fraction of a chunk; a request
leaves the batch the moment it has done its steps, which frees its memory
for the next waiting request.  The clock is real: arrivals are replayed at
their times, and a request's latency is its completion time minus its
arrival time (queueing included).

Every member computes exactly what it would compute alone (the batch kernel's
per-site arithmetic does not depend on the other members), so a request's
result is the same in the mix and alone; tests/test_gpu_serve.py checks it.
"""
from __future__ import annotations

import argparse
import collections
import dataclasses
import json
import time
from typing import Dict, List, Optional

import numpy as np

from . import lbgpu, params


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the stream
    gn: tuple
    radius: float
    steps: int
    acc: float
    p: Optional[params.LBParams] = None

    @property
    def sites(self) -> int:
        return int(self.gn[0] * self.gn[1] * self.gn[2])


def droplet_channel_params(gn, radius, acc, tau=1.0, g=3.6) -> params.LBParams:
    """A red sphere (1.0 / 0.05) in a blue bath (0.05 / 1.0) between walls on
    the z = 0 and z = nz-1 planes, body force `acc` along x."""
    lines = [
        "[lattice]", f"gn = [{gn[0]}, {gn[1]}, {gn[2]}]",
        "[lb]", "components = 2", 'fieldNames = ["red", "blue"]', f"tau = [{tau}, {tau}]",
        "eqdist.eqDistForm = BDist2", "force.enableShanChen = true",
        f"force.gcc = [[0.0, {g}], [{g}, 0.0]]", "force.psiForm = Exponential",
        f"force.globalAcc = [{acc!r}, 0.0, 0.0]",
        "init.fluidInit = [EqDistSphere, EqDistSphere]",
        "init.fluidDensities = [[1.0, 0.05], [0.05, 1.0]]",
        f"init.initRadius = {radius!r}", "init.interfaceThickness = 0.0",
        "mask.maskInit = Walls",
        "mask.dimensionHasWall = [[false, false], [false, false], [true, true]]",
        "mask.wallThickness = 1",
    ]
    return params.LBParams.from_dict(params.parse_lines(lines), "d3q19")


def request_stream(n: int, rate: float = 50.0, seed: int = 2024, step_scale: float = 1.0) -> List[Request]:
    """Poisson arrivals at `rate`/s; x ~ U[48, 256], y = z ~ U[32, 128],
    sphere radius ~ U[6, y/4], steps ~ U[2000, 20000] (times step_scale),
    body force ~ U[0, 1e-5]."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    for i in range(n):
        t += float(rng.exponential(1.0 / rate))
        x = int(rng.integers(48, 257))
        y = int(rng.integers(32, 129))
        radius = float(rng.uniform(6.0, y / 4.0))
        steps = max(1, int(round(int(rng.integers(2000, 20001)) * step_scale)))
        acc = float(rng.uniform(0.0, 1e-5))
        r = Request(i, t, (x, y, y), radius, steps, acc)
        r.p = droplet_channel_params(r.gn, radius, acc)
        out.append(r)
    return out


class Server:
    """Continuous-batching loop over one lbgpu batch."""

    def __init__(self, precision: int = lbgpu.FP16, budget_bytes: float = 120e9, device: int = 0,
                 max_chunk: int = 500, min_chunk: int = 25, age_limit_s: float = 5.0, keep_state: bool = False):
        self.batch = lbgpu.Batch(precision=precision, device=device, hbm_budget_bytes=int(budget_bytes))
        # memberships change constantly: one fixed launch shape, graph replay
        self.batch.set_tuning(autotune=False, tile_height=8, ctas_per_sm=0, use_graph=True)
        self.max_chunk = max_chunk
        self.min_chunk = min_chunk
        self.age_limit_s = age_limit_s
        self.keep_state = keep_state

    def run(self, requests: List[Request], realtime: bool = True) -> Dict:
        b = self.batch
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting: collections.deque = collections.deque()
        active: Dict[int, list] = {}
        results = []
        peak_members = 0
        peak_bytes = 0
        t0 = time.perf_counter()
        site_steps = 0
        step_rate = 0.0  # steps per second of the last chunk
        while pending or waiting or active:
            now = time.perf_counter() - t0
            if not realtime:
                while pending:
                    waiting.append(pending.popleft())
            while pending and pending[0].arrival <= now:
                waiting.append(pending.popleft())
            # fit-first admission with aging
            kept: collections.deque = collections.deque()
            blocked = False
            while waiting:
                r = waiting.popleft()
                if blocked:
                    kept.append(r)
                    continue
                try:
                    sid = b.add_device(r.p)
                except lbgpu.BudgetExceeded:
                    if not active:
                        raise
                    kept.append(r)
                    # the oldest waiting request has aged: nothing overtakes it
                    if len(kept) == 1 and now - r.arrival > self.age_limit_s:
                        blocked = True
                    continue
                active[sid] = [r, r.steps, time.perf_counter() - t0]
            waiting = kept
            peak_members = max(peak_members, len(active))
            peak_bytes = max(peak_bytes, b.device_bytes)
            if not active:
                if pending:
                    time.sleep(max(0.0, pending[0].arrival - (time.perf_counter() - t0)))
                continue
            k = min(self.max_chunk, min(v[1] for v in active.values()))
            # while nothing waits (the budget had room for every request so
            # far), end the chunk near the next arrival so that it joins soon;
            # while requests wait for room, chunks end when a member finishes
            if pending and not waiting and step_rate > 0.0:
                until = pending[0].arrival - (time.perf_counter() - t0)
                k = max(min(k, self.min_chunk), min(k, int(until * step_rate)))
            t_launch = time.perf_counter()
            b.step(k)
            b.synchronize()
            dt = time.perf_counter() - t_launch
            if dt > 0.0:
                step_rate = k / dt
            site_steps += k * sum(v[0].sites for v in active.values())
            done_t = time.perf_counter() - t0
            for sid in [s for s, v in active.items() if v[1] - k == 0]:
                r, _, admit = active.pop(sid)
                m = b.member(sid)
                mass, mom = m.reduce()
                rec = {"rid": r.rid, "arrival": r.arrival, "admitted": admit, "completed": done_t,
                       "latency": done_t - r.arrival, "queue": admit - r.arrival, "steps": r.steps,
                       "sites": r.sites, "mass": mass.tolist(), "momentum": mom.tolist()}
                if self.keep_state:
                    rec["population"] = m.population()
                results.append(rec)
                b.remove(sid)
            for v in active.values():
                v[1] -= k
        wall = time.perf_counter() - t0
        lat = np.array([r["latency"] for r in results])
        work = sum(r["sites"] * r["steps"] for r in results)
        return {
            "requests": len(results),
            "p50_latency_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "makespan_s": wall,
            "aggregate_mlups": work / wall / 1e6,
            "site_steps": int(site_steps),
            "peak_members": peak_members,
            "peak_device_bytes": int(peak_bytes),
            "results": sorted(results, key=lambda r: r["rid"]),
        }


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--requests", type=int, default=32)
    ap.add_argument("--rate", type=float, default=50.0)
    ap.add_argument("--step-scale", type=float, default=1.0)
    ap.add_argument("--budget-gb", type=float, default=120.0)
    ap.add_argument("--precision", default="fp16", choices=["fp32", "fp16", "i16"])
    ap.add_argument("--seed", type=int, default=2024)
    args = ap.parse_args()
    reqs = request_stream(args.requests, args.rate, args.seed, args.step_scale)
    srv = Server(lbgpu.PRECISIONS[args.precision], args.budget_gb * 1e9)
    out = srv.run(reqs)
    mean_work = np.mean([r.sites * r.steps for r in reqs])
    out["sustainable_rate_per_s"] = out["aggregate_mlups"] * 1e6 / mean_work
    out.pop("results")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
