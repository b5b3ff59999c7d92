#!/usr/bin/env python3
"""Turn the reference's HDF5 golden files into small committed fixtures.

Run from the repository root with the path of a reference checkout:

    python tests/golden/make_fixtures.py <reference checkout> [case ...]

For every case it stores, in ``tests/golden/<case>.npz``:

* the parameter file text and the connectivity (so tests need no reference
  checkout at run time);
* per golden file: the SHA-256 of the whole ``/OutArray`` (bitwise checks of
  exact goldens), its shape, min/max/sum, and either the full array (2D
  cases) or two x-planes of it (3D cases, to keep the fixtures small).
"""
import glob
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from dlbc_gb300 import h5  # noqa: E402

# (case name, test dir, input file, connectivity, golden glob, timesteps, tolerance per t)
CASES = [
    ("merging-droplets-3d", "lb/merging-droplets-3d", "merging-droplets-3d.in", "d3q19",
     "reference-data/*-t%08d.h5", {0: 0.0, 10: 1e-15, 1000: 1e-14}),
    ("bdist2-sc-3d", "lb/bdist2-sc-3d", "bdist2-sc-3d.in", "d3q19",
     "reference-data/*-t%08d.h5", {0: 0.0, 10: 1e-15, 100: 1e-15}),
    ("laplace-droplet-3d", "lb/laplace-droplet-3d", "laplace-droplet-3d.in", "d3q19",
     "reference-data/*-t%08d.h5", {0: 0.0, 10: 1e-15, 100: 1e-15}),
    ("merging-droplets-2d", "lb/merging-droplets-2d", "merging-droplets-2d.in", "d2q9",
     "reference-data/*-t%08d.h5", {0: 0.0, 100: 1e-15, 1000: 1e-14}),
    ("bdist2-sc-2d", "lb/bdist2-sc-2d", "bdist2-sc-2d.in", "d2q9",
     "reference-data/*-t%08d.h5", {0: 0.0, 10: 1e-15, 100: 1e-14}),
    ("poiseuille-2d", "lb/poiseuille-2d", "poiseuille-2d.in", "d2q9",
     "reference-data/*-t%08d.h5", {0: 0.0, 1000: 0.0}),
    ("laplace-quasi-1d-d2q9", "lb/laplace-quasi-1d", "laplace-quasi-1d-d2q9.in", "d2q9",
     "reference-data/d2q9/*-t%08d.h5", {0: 0.0, 1000: 1e-15}),
    ("laplace-quasi-1d-d1q3", "lb/laplace-quasi-1d", "laplace-quasi-1d-d1q3.in", "d1q3",
     "reference-data/d1q3/*-t%08d.h5", {0: 0.0, 1000: 1e-15}),
    # restored from the t = 0 checkpoint, 5 steps; the test compares without a tolerance
    ("checkpoint-3d", "technical/checkpoint-3d", "checkpoint-3d.in.source", "d3q19",
     "reference-data/*-t%08d.h5", {0: 0.0, 5: 0.0}),
]

# checkpoint files stored whole (case, directory, file stem, checkpoint name)
CHECKPOINTS = [
    ("checkpoint-3d", "technical/checkpoint-3d/reference-data/cp", ["cp-fluids0", "cp-fluids1", "cp-mask"],
     "checkpoint-3d-t00000000"),
]

# init-2d: every initialiser and mask at t = 0 (exact goldens)
INIT_2D = [
    "fluid-init-const-2d", "fluid-init-constrandom-2d", "fluid-init-eqdist-2d",
    "fluid-init-eqdistcylinder-x-2d", "fluid-init-eqdistcylinder-y-2d",
    "fluid-init-eqdistcylinder-z-2d", "fluid-init-eqdistcylinderfrac-x-2d",
    "fluid-init-eqdistcylinderfrac-y-2d", "fluid-init-eqdistcylinderfrac-z-2d",
    "fluid-init-eqdistlamellae-x-2d", "fluid-init-eqdistlamellae-y-2d",
    "fluid-init-eqdistlamellaefrac-x-2d", "fluid-init-eqdistlamellaefrac-y-2d",
    "fluid-init-eqdistperturb-2d", "fluid-init-eqdistperturbfrac-2d",
    "fluid-init-eqdistrandom-2d", "fluid-init-eqdistsphere-2d",
    "fluid-init-eqdistspherefrac-2d", "fluid-init-eqdistspherefrac-boundary-2d",
    "fluid-init-eqdisttwospheres-2d", "fluid-init-eqdisttwospheresfrac-2d",
    "mask-init-box-2d", "mask-init-none-2d", "mask-init-plates-x-2d", "mask-init-plates-y-2d",
    "mask-init-tube-x-2d", "mask-init-tube-y-2d", "mask-init-tube-z-2d", "mask-init-walls-2d",
]


def sha(a: np.ndarray) -> str:
    """SHA-256 of the array bytes, with every NaN in one canonical encoding
    (never-initialised populations are NaN in the reference)."""
    a = np.array(a, copy=True)
    if a.dtype.kind == "f":
        a[np.isnan(a)] = np.nan
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def golden_kind(base: str) -> str:
    for k in ("population", "density", "colour", "velocity", "force", "mask"):
        if base.startswith(k + "-"):
            return k
    return ""


def store(out: dict, key: str, a: np.ndarray, full: bool):
    out[key + "/sha256"] = np.array(sha(a))
    out[key + "/dtype"] = np.array(str(a.dtype))
    out[key + "/shape"] = np.array(a.shape)
    out[key + "/stats"] = np.array([a.min(), a.max(), a.astype(np.float64).sum()], np.float64)
    if full:
        out[key + "/data"] = a
    else:
        nx = a.shape[0]
        out[key + "/planes"] = np.array([nx // 4, nx // 2])
        out[key + "/data"] = a[[nx // 4, nx // 2]]


def main(ref: str, only=()):
    tests = os.path.join(ref, "tests", "runnable", "tests")
    for name, tdir, inp, dq, pattern, tsteps in CASES:
        if only and name not in only:
            continue
        root = os.path.join(tests, tdir)
        out = {"input": np.array(open(os.path.join(root, inp)).read()), "dq": np.array(dq)}
        keys = []
        for t, tol in sorted(tsteps.items()):
            for f in sorted(glob.glob(os.path.join(root, pattern % t))):
                base = os.path.basename(f)
                kind = golden_kind(base)
                if not kind:
                    continue
                field = base.split("-")[1] if kind not in ("colour", "mask") else ""
                a = h5.read_field(f)
                key = f"t{t}/{kind}" + (f"-{field}" if field else "")
                store(out, key, a, full=(dq != "d3q19"))
                out[key + "/tol"] = np.array(tol)
                keys.append(key)
        out["keys"] = np.array(keys)
        for cname, cdir, stems, cpname in CHECKPOINTS:
            if cname != name:
                continue
            out["checkpoint/name"] = np.array(cpname)
            for stem in stems:
                f = os.path.join(tests, cdir, f"{stem}-{cpname}.h5")
                out[f"checkpoint/{stem}"] = h5.read_field(f)
                out[f"checkpoint/{stem}/timestep"] = np.array(
                    h5.read_attrs(f, "globals")["dlbc.lb.lb.timestep"]).ravel()
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {len(keys)} arrays, {os.path.getsize(path)} bytes")

    if only and "init-2d" not in only:
        return
    root = os.path.join(tests, "lb", "init-2d")
    out = {}
    names = []
    for case in INIT_2D:
        out[case + "/input"] = np.array(open(os.path.join(root, case + ".in")).read())
        for f in sorted(glob.glob(os.path.join(root, "reference-data", f"*-{case}-t00000000.h5"))):
            base = os.path.basename(f)
            kind = golden_kind(base)
            if not kind:
                continue
            field = base.split("-")[1] if kind not in ("colour", "mask") else ""
            a = h5.read_field(f)
            key = f"{case}/{kind}" + (f"-{field}" if field else "")
            out[key + "/sha256"] = np.array(sha(a))
            out[key + "/shape"] = np.array(a.shape)
            names.append(key)
    out["keys"] = np.array(names)
    out["cases"] = np.array(INIT_2D)
    # maskInit = File: the case's input text, its mask file and the hashes of
    # its t = 0 dumps (the fluid File case reads 0.6 MB population files and
    # is covered with synthetic files instead)
    case = "mask-init-file-2d"
    out["file/" + case + "/input"] = np.array(open(os.path.join(root, case + ".in")).read())
    out["file/" + case + "/mask"] = h5.read_field(os.path.join(root, "reference-data", f"mask-{case}-t00000000.h5"))
    for f in sorted(glob.glob(os.path.join(root, "reference-data", f"*-{case}-t00000000.h5"))):
        base = os.path.basename(f)
        kind = golden_kind(base)
        field = base.split("-")[1] if kind not in ("colour", "mask") else ""
        key = f"file/{case}/{kind}" + (f"-{field}" if field else "")
        out[key + "/sha256"] = np.array(sha(h5.read_field(f)))
    path = os.path.join(HERE, "init-2d.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {len(names)} hashes, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_fixtures.py <reference checkout> [case ...]")
    # optional further arguments: only these cases (the rest are left as they are)
    main(sys.argv[1], tuple(sys.argv[2:]))
