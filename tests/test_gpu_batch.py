"""Batches (lbgpu_batch_*): many independent lattices in one persistent
launch per step.  Each member must step exactly like the same lattice run
alone, whatever the launch shape, graph replay or the other members."""
import numpy as np
import pytest

from dlbc_gb300 import init, lbgpu
from lbcases import droplet_channel, spinodal

pytestmark = pytest.mark.gpu


def two_spheres(L, tau=1.0, g=3.6, radius=None):
    from dlbc_gb300 import params
    r = L / 6.0 if radius is None else radius
    lines = [
        "[lattice]", f"gn = [{L}, {L}, {L}]",
        "[lb]", "components = 2", 'fieldNames = ["red", "blue"]', f"tau = [{tau}, {tau}]",
        "eqdist.eqDistForm = BDist2", "force.enableShanChen = true",
        f"force.gcc = [[0.0, {g}], [{g}, 0.0]]", "force.psiForm = Exponential",
        "force.globalAcc = [0.0, 0.0, 0.0]",
        "init.fluidInit = [EqDistTwoSpheres, EqDistTwoSpheres]",
        "init.fluidDensities = [[1.0, 0.05], [0.05, 1.0]]",
        f"init.initRadius = {r}", f"init.initSeparation = [{2 * r + 2}, 0.0, 0.0]",
        "init.interfaceThickness = 0.0",
    ]
    return params.LBParams.from_dict(params.parse_lines(lines), "d3q19")


def members():
    # even z extents run the pair kernel, the odd one (21) the one-site-per-
    # thread fused kernel: one batch step launches both
    return [two_spheres(32, tau=0.9, g=3.5), spinodal((24, 20, 40)), two_spheres(48, tau=1.1, g=3.9),
            droplet_channel((20, 18, 36), radius=5.0, acc=1e-3, gwc=(0.2, -0.1)),
            droplet_channel((14, 12, 21), radius=3.0, acc=1e-3, tau=(0.9, 0.9))]


def alone(p, precision, steps):
    fl, m = init.init_fields(p)
    g = lbgpu.GPULattice(p, precision=precision)
    g.upload(fl, m)
    g.step(steps)
    return g.population()


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16, lbgpu.I16])
@pytest.mark.parametrize("shape", ["autotune", (8, 2), (4, 4), "nograph"])
def test_batch_members_step_like_lone_lattices(precision, shape):
    ps = members()
    if precision == lbgpu.I16:  # the I16 form needs an even z extent
        ps = [p for p in ps if p.gn[2] % 2 == 0]
    steps = 23
    b = lbgpu.Batch(precision=precision)
    if shape == "nograph":
        b.set_tuning(autotune=False, tile_height=8, ctas_per_sm=0, use_graph=False)
    elif shape != "autotune":
        b.set_tuning(autotune=False, tile_height=shape[0], ctas_per_sm=shape[1], use_graph=True)
    ids = []
    for p in ps:
        fl, m = init.init_fields(p)
        ids.append(b.add(p, fl, m))
    b.step(steps)
    for sid, p in zip(ids, ps):
        got = b.member(sid).population()
        ref = alone(p, precision, steps)
        for c in range(2):
            assert np.array_equal(got[c], ref[c]), (sid, c, np.abs(got[c] - ref[c]).max())


def test_batch_join_leave_mid_run():
    """Members that join and leave between steps do not disturb the others."""
    ps = members()
    b = lbgpu.Batch(precision=lbgpu.FP32)
    fl0, m0 = init.init_fields(ps[0])
    s0 = b.add(ps[0], fl0, m0)
    b.step(5)
    fl1, m1 = init.init_fields(ps[1])
    s1 = b.add(ps[1], fl1, m1)
    fl2, m2 = init.init_fields(ps[3])
    s2 = b.add(ps[3], fl2, m2)
    b.step(7)
    b.remove(s1)
    b.step(4)
    assert np.array_equal(b.member(s0).population()[0], alone(ps[0], lbgpu.FP32, 16)[0])
    assert np.array_equal(b.member(s2).population()[1], alone(ps[3], lbgpu.FP32, 11)[1])


def test_batch_budget_admission():
    p = two_spheres(32)
    fl, m = init.init_fields(p)
    per = 2 * 2 * 19 * 32 ** 3 * 2 + 32 ** 3  # FP16 member bytes (two buffers + mask)
    b = lbgpu.Batch(precision=lbgpu.FP16, hbm_budget_bytes=int(per * 2.5))
    a = b.add(p, fl, m)
    b.add(p, fl, m)
    with pytest.raises(lbgpu.BudgetExceeded):
        b.add(p, fl, m)
    b.remove(a)
    b.add(p, fl, m)
    assert b.device_bytes <= per * 2.5
