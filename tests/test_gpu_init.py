"""Device-side initial fields (lbgpu_init_fields) against the host
restatement of the reference's initialisers (bitwise for the deterministic
ones, statistically for the counter-based random ones)."""
import os

import numpy as np
import pytest

from dlbc_gb300 import init, lbgpu, params
from golden_util import GOLDEN, load_case
from lbcases import droplet_channel, spinodal

pytestmark = pytest.mark.gpu

RANDOM = {"EqDistPerturb", "EqDistPerturbFrac", "EqDistRandom", "ConstRandom"}


def device_fields(p, seed=0):
    # the init-only inputs (timesteps = 0) leave tau unset; the fields do not depend on it
    p.tau = [t if t > 0 else 1.0 for t in (p.tau or [1.0] * p.components)]
    g = lbgpu.GPULattice(p, precision=lbgpu.FP64)
    g.init_device(seed)
    return g.download(), g


def deterministic_cases():
    out = []
    for name in ["merging-droplets-3d", "bdist2-sc-3d", "laplace-droplet-3d", "merging-droplets-2d",
                 "bdist2-sc-2d", "poiseuille-2d", "laplace-quasi-1d-d2q9"]:
        out.append((name, load_case(name)[1]))
    z = np.load(os.path.join(GOLDEN, "init-2d.npz"))
    for case in z["cases"]:
        case = str(case)
        p = params.LBParams.from_dict(params.parse_lines(str(z[case + "/input"]).splitlines()), "d2q9")
        if any(params.FLUID_INITS[fi] in RANDOM | {"File"} for fi in p.fluid_init):
            continue
        p.nc = [1, 1]
        out.append((case, p))
    out.append(("droplet-channel", droplet_channel((24, 16, 20), radius=5.5)))
    return out


@pytest.mark.parametrize("name,p", deterministic_cases(), ids=lambda v: v if isinstance(v, str) else "")
def test_device_init_equals_host_init(name, p):
    fl, m = init.init_fields(p)
    got, g = device_fields(p)
    for c in range(p.components):
        assert np.array_equal(got[c], fl[c], equal_nan=True), (name, c)


def test_random_initialisers_statistics():
    p = spinodal((32, 32, 32), perturb=0.02)
    got, g = device_fields(p, seed=5)
    w = init.weights(19)
    for c in range(2):
        rho = got[c][2:-2, 2:-2, 2:-2].sum(axis=-1)
        assert abs(rho.mean() - 0.7) < 1e-3
        assert rho.min() >= 0.68 - 1e-12 and rho.max() < 0.72 + 1e-12
        # populations are rho * w_q
        assert np.allclose(got[c][2:-2, 2:-2, 2:-2] / w, rho[..., None], rtol=1e-14)
    assert not np.array_equal(got[0], got[1])  # components draw independent numbers
    again, _ = device_fields(p, seed=5)
    assert np.array_equal(again[0], got[0])  # deterministic in the seed


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16])
def test_device_init_batch_member_steps_like_lone_lattice(precision):
    p = droplet_channel((40, 24, 36), radius=6.0, acc=1e-4)
    b = lbgpu.Batch(precision=precision)
    sid = b.add_device(p)
    b.step(17)
    got = b.member(sid).population()
    g = lbgpu.GPULattice(p, precision=precision)
    g.init_device()
    g.step(17)
    ref = g.population()
    for c in range(2):
        assert np.array_equal(got[c], ref[c])
