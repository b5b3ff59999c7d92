"""The reference's unit-test known answers through the C ABI (FP64 form):
density.d:50-61 (densities 0.1 and 0.5), velocity.d:59-74 / 122-160 (raw
velocities (1, 1, 0) and (-0.2, -0.2, 0.2), NaN where the density is 0,
0 on solid sites) and momentum.d:91-119 (momentum (-0.1, -0.1, 0.1), none
on solid sites), on a 4^3 lattice holding the test populations."""
import numpy as np
import pytest

from dlbc_gb300 import lbgpu
from lbcases import spinodal

pytestmark = pytest.mark.gpu

POP_A = [0.0] * 7 + [0.1] + [0.0] * 11
POP_B = [0.1, 0.0, 0.1, 0.0, 0.0, 0.0, 0.0, 0.1, 0.0, 0.0, 0.1, 0.0, 0.0, 0.0, 0.1, 0.0, 0.0, 0.0, 0.0]


def kat_lattice(sites, solid=()):
    p = spinodal((4, 4, 4))
    nH = (8, 8, 8)
    fluids = []
    for _ in range(p.components):
        a = np.zeros(nH + (19,))
        for (x, y, z), pop in sites.items():
            a[x + 2, y + 2, z + 2] = pop
        fluids.append(a)
    mask = np.zeros(nH, np.int32)
    for (x, y, z) in solid:
        mask[x + 2, y + 2, z + 2] = 1
    g = lbgpu.GPULattice(p, precision=lbgpu.FP64)
    g.upload(fluids, mask)
    return g


def test_density_and_velocity_known_answers():
    g = kat_lattice({(0, 0, 0): POP_A, (1, 2, 3): POP_B})
    dens, vel = g.density(), g.velocity()
    for c in range(2):
        assert dens[c][0, 0, 0] == 0.1 and dens[c][1, 2, 3] == 0.5 and dens[c][3, 3, 3] == 0.0
        assert vel[c][0, 0, 0].tolist() == [1.0, 1.0, 0.0]
        assert vel[c][1, 2, 3].tolist() == [-0.2, -0.2, 0.2]
        assert np.all(np.isnan(vel[c][0, 1, 3]))


def test_momentum_known_answer():
    g = kat_lattice({(1, 2, 3): POP_B})
    mass, mom = g.reduce()
    for c in range(2):
        assert mass[c] == 0.5
        assert mom[c].tolist() == [-0.1, -0.1, 0.1]


def test_solid_sites_carry_no_velocity_or_momentum():
    g = kat_lattice({(1, 2, 3): POP_B}, solid=[(1, 2, 3), (0, 1, 3)])
    vel = g.velocity()
    mass, mom = g.reduce()
    for c in range(2):
        assert vel[c][1, 2, 3].tolist() == [0.0, 0.0, 0.0] and vel[c][0, 1, 3].tolist() == [0.0, 0.0, 0.0]
        assert mass[c] == 0.0 and mom[c].tolist() == [0.0, 0.0, 0.0]
    assert g.colour()[1, 2, 3] == 0.0
