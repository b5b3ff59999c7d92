"""Host-side initialisers (dlbc_gb300.init) against the oracle's restatement
and the reference's init goldens."""
import os

import numpy as np
import pytest

from dlbc_gb300 import init, params
from golden_util import GOLDEN, load_case, sha
from oracle import oracle as orc

CASES = ["merging-droplets-3d", "bdist2-sc-3d", "laplace-droplet-3d", "merging-droplets-2d",
         "bdist2-sc-2d", "poiseuille-2d", "laplace-quasi-1d-d2q9"]


@pytest.mark.parametrize("name", CASES)
def test_host_init_equals_oracle_init(name):
    z, p = load_case(name)
    fl, m = init.init_fields(p)
    o = orc.Oracle(p)
    for c in range(p.components):
        assert sha(fl[c]) == sha(o.fluid_haloed(c))
    assert np.array_equal(m, o.mask_haloed())


def test_host_init_matches_init_goldens():
    z = np.load(os.path.join(GOLDEN, "init-2d.npz"))
    keys = [str(k) for k in z["keys"]]
    for case in z["cases"]:
        case = str(case)
        p = params.LBParams.from_dict(params.parse_lines(str(z[case + "/input"]).splitlines()), "d2q9")
        fl, m = init.init_fields(p)
        phys = (slice(2, -2), slice(2, -2))
        for key in keys:
            if not key.startswith(case + "/"):
                continue
            kind = key.split("/")[1]
            if kind.startswith("population-"):
                c = p.field_names.index(kind.split("-", 1)[1])
                assert sha(fl[c][phys]) == str(z[key + "/sha256"]), key
            elif kind == "mask":
                assert sha(m[phys]) == str(z[key + "/sha256"]), key


def test_periodic_halo_fill():
    a = np.arange(6 * 5 * 4, dtype=np.float64).reshape(6, 5, 4, 1)
    h = init.periodic_fill(np.pad(a, [(2, 2), (2, 2), (2, 2), (0, 0)]), 3)
    assert h.shape == (10, 9, 8, 1)
    assert h[0, 2, 2, 0] == a[4, 0, 0, 0] and h[9, 8, 7, 0] == a[1, 1, 1, 0]
