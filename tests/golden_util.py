"""Helpers to load the committed golden fixtures (tests/golden/*.npz)."""
import hashlib
import os

import numpy as np

from dlbc_gb300 import params

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_case(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    text = str(z["input"])
    dq = str(z["dq"])
    p = params.LBParams.from_dict(params.parse_lines(text.splitlines()), dq)
    return z, p


def sha(a):
    """SHA-256 as tests/golden/make_fixtures.py computes it (NaNs canonical)."""
    a = np.array(a, copy=True)
    if a.dtype.kind == "f":
        a[np.isnan(a)] = np.nan
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def times(z):
    return sorted({int(k.split("/")[0][1:]) for k in z["keys"]})


def golden_arrays(z, t):
    for k in z["keys"]:
        k = str(k)
        if k.startswith(f"t{t}/"):
            yield k, k.split("/")[1]


def compare(z, key, a, tol):
    """Compare an oracle/kernel output with a golden entry.

    tol == 0: bitwise (SHA-256 of the whole array); otherwise the stored
    data (full array or planes) within |a - b| <= tol, and stats close."""
    shape = tuple(z[key + "/shape"])
    assert a.shape == shape, (key, a.shape, shape)
    if tol == 0.0:
        return sha(a.astype(np.dtype(str(z[key + "/dtype"])))) == str(z[key + "/sha256"])
    data = z[key + "/data"]
    if (key + "/planes") in z.files:
        a = a[list(z[key + "/planes"])]
    return bool(np.all(np.abs(a - data) <= tol))


def oracle_output(o, p, kind):
    """Output named like the reference's dump files."""
    if kind == "colour":
        return o.colour(0, 1)
    if kind == "mask":
        return o.mask()
    what, name = kind.split("-", 1)
    c = p.field_names.index(name)
    return {"population": o.population, "density": o.density,
            "velocity": o.velocity, "force": o.force}[what](c)
