"""Device-side initial fields (lbgpu_init_fields) against the host
restatement of the reference's initialisers: bitwise for the deterministic
ones and for the random ones drawing the reference's Mt19937 sequences
(rng = 1), statistically for the counter-based draws."""
import os

import numpy as np
import pytest

from dlbc_gb300 import init, lbgpu, params
from golden_util import GOLDEN, load_case, sha
from lbcases import droplet_channel, spinodal

pytestmark = pytest.mark.gpu

RANDOM = {"EqDistPerturb", "EqDistPerturbFrac", "EqDistRandom", "ConstRandom"}


def device_fields(p, seed=0, reference_rng=False):
    # the init-only inputs (timesteps = 0) leave tau unset; the fields do not depend on it
    p.tau = [t if t > 0 else 1.0 for t in (p.tau or [1.0] * p.components)]
    g = lbgpu.GPULattice(p, precision=lbgpu.FP64)
    g.init_device(seed, reference_rng=reference_rng)
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


def random_cases():
    """The reference's random-initialiser goldens (four ranks, reseeded
    components), a 3D spinodal on one rank and on a 2 x 1 x 2 grid, and a
    ConstRandom / EqDistRandom mix without reseeding."""
    out = []
    z = np.load(os.path.join(GOLDEN, "init-2d.npz"))
    for case in z["cases"]:
        case = str(case)
        p = params.LBParams.from_dict(params.parse_lines(str(z[case + "/input"]).splitlines()), "d2q9")
        if any(params.FLUID_INITS[fi] in RANDOM for fi in p.fluid_init):
            out.append((case, p))
    p = spinodal((24, 20, 16), perturb=0.02, seed=11)
    out.append(("spinodal-1-rank", p))
    p = spinodal((24, 20, 16), perturb=0.02, seed=-3)
    p.nc = [2, 1, 2]
    out.append(("spinodal-4-ranks", p))
    p = spinodal((12, 10, 8), seed=5)
    p.fluid_init = [params.FLUID_INITS.index("ConstRandom"), params.FLUID_INITS.index("EqDistRandom")]
    p.shift_seed_by_rank = False
    p.nc = [2, 1, 1]
    out.append(("constrandom-eqdistrandom", p))
    return out


@pytest.mark.parametrize("name,p", random_cases(), ids=lambda v: v if isinstance(v, str) else "")
def test_device_init_reference_rng_equals_host_init(name, p):
    fl, m = init.init_fields(p)
    got, g = device_fields(p, reference_rng=True)
    for c in range(p.components):
        assert np.array_equal(got[c], fl[c], equal_nan=True), (name, c)


def test_device_init_reference_rng_matches_goldens():
    """rng = 1 against the reference's own output: the populations of every
    random initialiser of init-2d (EqDistPerturb, EqDistPerturbFrac,
    EqDistRandom, ConstRandom; four ranks, reseeded components), by hash."""
    z = np.load(os.path.join(GOLDEN, "init-2d.npz"))
    keys = [str(k) for k in z["keys"]]
    checked = 0
    for case in z["cases"]:
        case = str(case)
        p = params.LBParams.from_dict(params.parse_lines(str(z[case + "/input"]).splitlines()), "d2q9")
        if not any(params.FLUID_INITS[fi] in RANDOM for fi in p.fluid_init):
            continue
        got, g = device_fields(p, reference_rng=True)
        for key in keys:
            kind = key.split("/")[1] if key.startswith(case + "/") else ""
            if kind.startswith("population-"):
                c = p.field_names.index(kind.split("-", 1)[1])
                assert sha(got[c][2:-2, 2:-2]) == str(z[key + "/sha256"]), key
                checked += 1
    assert checked == 8
