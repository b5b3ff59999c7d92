"""Precision study: FP32, FP16-offset and 16-bit fixed-point (I16) storage
against FP64 on a large spinodal decomposition, or on the droplet channel.

Spinodal: two-component D3Q19 Shan-Chen, periodic, rho = 0.7 +- `perturb`
per site and component (device-side counter-based noise, the same initial
state for every form up to the storage rounding), tau = 1, g = 3.6,
psi = 1 - exp(-rho), BDist2.  Channel (--workload channel): the benchmark's
256x128x128 droplet channel, a flow that stays near its initial densities.
Every form runs the same number of steps from the same initial fields; the
FP64 form is the reference for the errors (it is bit-identical to the CPU
restatement of the reference, checked at small sizes by the tests).

Reported per form: time and MLUPS, relative L2 error of each component's
density and velocity against FP64 at checkpoints, the fraction of sites
whose phase (sign of rho_red - rho_blue) differs from FP64's (the interface
position error), and the relative change of each component's total mass.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import lbgpu, params


def spinodal_params(n: int, perturb: float, d: int = 3) -> params.LBParams:
    """The spinodal lattice: n^3 D3Q19, or n^2 D2Q9 with d = 2."""
    lines = [
        "[lattice]", f"gn = [{', '.join([str(n)] * d)}]",
        "[lb]", "components = 2", 'fieldNames = ["red", "blue"]', "tau = [1.0, 1.0]",
        "eqdist.eqDistForm = BDist2", "force.enableShanChen = true",
        "force.gcc = [[0.0, 3.6], [3.6, 0.0]]", "force.psiForm = Exponential",
        f"force.globalAcc = [{', '.join(['0.0'] * d)}]",
        "init.fluidInit = [EqDistPerturb, EqDistPerturb]", "init.fluidDensities = [[0.7], [0.7]]",
        f"init.fluidPerturb = [{perturb}, {perturb}]",
    ]
    return params.LBParams.from_dict(params.parse_lines(lines), "d3q19" if d == 3 else "d2q9")


def channel_params(n=(256, 128, 128)) -> params.LBParams:
    """The droplet channel: a red sphere of radius 24 (1.0 / 0.05) in a blue
    bath (0.05 / 1.0), bounce-back walls on z = 0 and z = nz - 1, body force
    1e-6 along x, tau = 1, g = 3.6, BDist2: a flow that stays near its
    initial densities, unlike the spinodal."""
    lines = [
        "[lattice]", f"gn = [{n[0]}, {n[1]}, {n[2]}]",
        "[lb]", "components = 2", 'fieldNames = ["red", "blue"]', "tau = [1.0, 1.0]",
        "eqdist.eqDistForm = BDist2", "force.enableShanChen = true",
        "force.gcc = [[0.0, 3.6], [3.6, 0.0]]", "force.psiForm = Exponential",
        "force.globalAcc = [1e-6, 0.0, 0.0]",
        "init.fluidInit = [EqDistSphere, EqDistSphere]",
        "init.fluidDensities = [[1.0, 0.05], [0.05, 1.0]]",
        "init.initRadius = 24.0", "init.interfaceThickness = 0.0",
        "mask.maskInit = Walls",
        "mask.dimensionHasWall = [[false, false], [false, false], [true, true]]",
        "mask.wallThickness = 1",
    ]
    return params.LBParams.from_dict(params.parse_lines(lines), "d3q19")


def run_form(p, precision, steps, checkpoints, seed, device=0, rho0=(0.0, 0.0)):
    g = lbgpu.GPULattice(p, precision=precision, device=device, rho0=rho0)
    g.init_device(seed)
    mass0, _ = g.reduce()
    out = {}
    done = 0
    t_total = 0.0
    for cp in checkpoints:
        g.synchronize()
        t0 = time.perf_counter()
        g.step(cp - done)
        g.synchronize()
        t_total += time.perf_counter() - t0
        done = cp
        dens = g.density()
        vel = g.velocity()
        mass, _ = g.reduce()
        drift = [float((mass[c] - mass0[c]) / mass0[c]) for c in range(len(mass))]
        out[cp] = ([d.astype(np.float64) for d in dens], [v.astype(np.float64) for v in vel], drift)
    g.close()
    return out, t_total


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--workload", choices=["spinodal", "channel"], default="spinodal",
                    help="the n^3 spinodal, or the 256x128x128 droplet channel (--n ignored)")
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--perturb", type=float, default=0.02)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--checkpoints", default="500,1000,2000,5000")
    ap.add_argument("--forms", default="fp32,fp16,i16",
                    help="comma-separated forms compared with FP64 (which always runs)")
    ap.add_argument("--fp16-origin", type=float, action="append", default=[],
                    help="also run the FP16 form with offsets from this density instead of the mean "
                         "(a tiny value such as 1e-12 stores plain scaled f_q / w_q)")
    args = ap.parse_args()
    cps = sorted({int(c) for c in args.checkpoints.split(",") if int(c) <= args.steps} | {args.steps})
    if args.workload == "channel":
        p = channel_params()
        sites = 256 * 128 * 128
        what = (f"256x128x128 droplet channel (walls z = 0 / 127, body force 1e-6, radius 24), "
                f"{args.steps} steps, BDist2, g 3.6")
    else:
        p = spinodal_params(args.n, args.perturb)
        sites = args.n ** 3
        what = f"{args.n}^3 periodic spinodal decomposition, rho 0.7 +- {args.perturb}, {args.steps} steps, BDist2, g 3.6"
    ref, t64 = run_form(p, lbgpu.FP64, args.steps, cps, args.seed)
    report = {"workload": what,
              "fp64": {"time_s": round(t64, 2), "mlups": round(sites * args.steps / t64 / 1e6, 1),
                       "mass_drift": {cp: ref[cp][2] for cp in cps}}}
    wanted = set(args.forms.split(","))
    forms = [(n, prec, (0.0, 0.0)) for n, prec in (("fp32", lbgpu.FP32), ("fp16", lbgpu.FP16), ("i16", lbgpu.I16))
             if n in wanted]
    forms += [(f"fp16 origin {v:g}", lbgpu.FP16, (v, v)) for v in args.fp16_origin]
    for name, prec, rho0 in forms:
        res, t = run_form(p, prec, args.steps, cps, args.seed, rho0=rho0)
        errs = {}
        for cp in cps:
            (d, v, drift), (d64, v64, _) = res[cp], ref[cp]
            phase = np.mean(np.sign(d[0] - d[1]) != np.sign(d64[0] - d64[1]))
            errs[cp] = {"rho_l2": [rel_l2(d[c], d64[c]) for c in range(2)],
                        "u_l2": [rel_l2(v[c], v64[c]) for c in range(2)],
                        "phase_mismatch_fraction": float(phase),
                        "mass_drift": drift}
        report[name] = {"time_s": round(t, 2), "mlups": round(sites * args.steps / t / 1e6, 1), "errors": errs}
        del res
    print(json.dumps(report))


if __name__ == "__main__":
    main()
