"""The reference's unit tests (known answers and properties) on the CPU
oracle and on the kernels' connectivity tables.

Each test names the reference unittest it restates:
density.d:50-61, velocity.d:59-74 / 122-160, momentum.d:91-119,
force.d:370-384 (psi), eqdist.d:317-360 (conservation of every equilibrium)
and connectivity.d:433-480 (bounce-back, weights, speed of sound).  The
oracle runs them through its lattice entry points (a 4^3 lattice holding
the test populations), the way the kernels compute them.
"""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from lbcases import spinodal
from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))

# the populations of the reference's tests (D3Q19)
POP_A = [0.0] * 7 + [0.1] + [0.0] * 11
POP_B = [0.1, 0.0, 0.1, 0.0, 0.0, 0.0, 0.0, 0.1, 0.0, 0.0, 0.1, 0.0, 0.0, 0.0, 0.1, 0.0, 0.0, 0.0, 0.0]

# D3Q19 velocities in the reference's order (connectivity.d:401-418)
D3Q19 = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
         (1, 1, 0), (-1, 1, 0), (0, 1, 1), (0, -1, 1), (1, 0, 1), (1, 0, -1), (1, -1, 0),
         (-1, -1, 0), (0, 1, -1), (0, -1, -1), (-1, 0, 1), (-1, 0, -1)]
# D2Q9 (connectivity.d:372-381)
D2Q9 = [(0, 0), (1, 0), (-1, 0), (0, 1), (0, -1), (1, 1), (1, -1), (-1, 1), (-1, -1)]


def kat_lattice(sites, solid=()):
    """A 4^3 D3Q19 oracle lattice, all populations zero but the given sites
    (physical coordinates -> population), `solid` sites masked."""
    p = spinodal((4, 4, 4))
    o = orc.Oracle(p, init=False)
    h = o.halo
    for c in range(p.components):
        a = np.zeros(o.nH + (19,))
        for (x, y, z), pop in sites.items():
            a[x + h, y + h, z + h] = pop
        o.set_fluid_haloed(c, a)
    m = np.zeros(o.nH, np.int32)
    for (x, y, z) in solid:
        m[x + h, y + h, z + h] = 1
    o.set_mask_haloed(m)
    return o


def test_density_known_answers():
    """density.d:50-61: 0.1 and 0.5, exactly."""
    o = kat_lattice({(0, 0, 0): POP_A, (1, 2, 3): POP_B})
    for c in range(2):
        d = o.density(c)
        assert d[0, 0, 0] == 0.1 and d[1, 2, 3] == 0.5
        assert d[3, 3, 3] == 0.0


def test_raw_velocity_known_answers():
    """velocity.d:59-74 and 122-160: raw velocity (1, 1, 0) and (-0.2, -0.2,
    0.2) exactly; NaN where the density is 0; 0 on solid sites."""
    o = kat_lattice({(0, 0, 0): POP_A, (1, 2, 3): POP_B})
    for c in range(2):
        v = o.velocity(c)
        assert v[0, 0, 0].tolist() == [1.0, 1.0, 0.0]
        assert v[1, 2, 3].tolist() == [-0.2, -0.2, 0.2]
        assert np.all(np.isnan(v[0, 1, 3]))
    o = kat_lattice({(1, 2, 3): POP_B}, solid=[(1, 2, 3), (0, 1, 3)])
    for c in range(2):
        v = o.velocity(c)
        assert v[1, 2, 3].tolist() == [0.0, 0.0, 0.0] and v[0, 1, 3].tolist() == [0.0, 0.0, 0.0]


def test_momentum_known_answer():
    """momentum.d:91-119: the momentum of POP_B is (-0.1, -0.1, 0.1), the
    density times the raw velocity, exactly."""
    o = kat_lattice({(1, 2, 3): POP_B})
    for c in range(2):
        m = o.density(c)[1, 2, 3] * o.velocity(c)[1, 2, 3]
        assert m.tolist() == [-0.1, -0.1, 0.1]


@pytest.mark.parametrize("mode", [0, 1])
def test_psi_known_answers(mode):
    """force.d:370-384: psi = 1 - exp(-rho) at 0, 0.7, 1, 2 to the digits
    the reference gives (1e-11), with both of the oracle's exp, and within
    an ulp of the host's exp."""
    want = {0.0: 0.0, 0.7: 0.5034146962, 1.0: 0.63212055882, 2.0: 0.86466471676}
    x = np.array([-r for r in want], np.float64)
    got = 1.0 - orc.exp(x, mode)
    for g, (rho, w) in zip(got, want.items()):
        assert abs(g - w) < 1e-11, (rho, g, w)
        assert g == 1.0 - math.exp(-rho) or abs(g - (1.0 - math.exp(-rho))) <= 2.3e-16


@pytest.mark.parametrize("eq", ["SecondOrder", "ThirdOrder", "BDist2"])
@pytest.mark.parametrize("d", [3, 2])
def test_equilibria_conserve_mass_and_momentum(eq, d):
    """eqdist.d:317-360: every equilibrium conserves the mass of the
    populations it is computed from, and all but BDist2 their momentum
    (shifted by dv = 0 without forces).  One oracle step of a random
    one-component lattice without Shan-Chen forces, tau = 1: each site's
    new populations are the equilibrium of the populations streamed into
    it."""
    p = spinodal((6, 5, 4) if d == 3 else (6, 5), eq=eq, d=d)
    p.components = 1
    p.tau = [1.0]
    p.shan_chen = False
    o = orc.Oracle(p, init=False)
    q = p.q
    rng = np.random.default_rng(3)
    a = rng.uniform(0.0, 1.0, o.nH + (q,))
    o.set_fluid_haloed(0, a)
    o.exchange_halo()
    pop = o.population(0)
    if d == 3:
        cvec = np.array(D3Q19)
    else:
        cvec = np.array(D2Q9)
    streamed = np.empty_like(pop)
    for k in range(q):
        streamed[..., k] = np.roll(pop[..., k], shift=tuple(cvec[k]), axis=tuple(range(d)))
    o.run(1)
    rho0 = streamed.sum(axis=-1)
    rho1 = o.density(0)
    assert np.allclose(rho1, rho0, rtol=1e-13, atol=0)
    if eq != "BDist2":
        j0 = np.einsum("...q,qd->...d", streamed, cvec)
        j1 = rho1[..., None] * o.velocity(0)
        assert np.allclose(j1, j0, rtol=1e-12, atol=1e-14)


@pytest.fixture(scope="module")
def conn_tables(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("conn") / "conn_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", os.path.join(HERE, "conn_check.cu"), "-o", exe], check=True,
                   capture_output=True, text=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=60).stdout
    tables = {}
    for line in out.split("\n"):
        if line.strip():
            Q, qq, cx, cy, cz, b, w, css = line.split()
            tables.setdefault(int(Q), []).append(((int(cx), int(cy), int(cz)), int(b), float(w), float(css)))
    return tables


def test_kernels_velocity_order(conn_tables):
    """The kernels' D3Q19 and D2Q9 velocities in the reference's order."""
    assert [c for c, _, _, _ in conn_tables[19]] == D3Q19
    assert [c for c, _, _, _ in conn_tables[9]] == [v + (0,) for v in D2Q9]


@pytest.mark.parametrize("Q", [19, 9, 5, 3])
def test_connectivity_properties(conn_tables, Q):
    """connectivity.d:433-480: bounce-back reverses every velocity, the
    weights sum to 1 and the speed of sound sum_q w_q c_qx^2 is 1/3 (1 for
    D1Q5)."""
    t = conn_tables[Q]
    for c, b, w, css in t:
        assert t[b][0] == tuple(-v for v in c)
    assert abs(sum(w for _, _, w, _ in t) - 1.0) <= 1e-15
    cs2 = sum(w * c[0] * c[0] for c, _, w, _ in t)
    want = 1.0 if Q == 5 else 1.0 / 3.0
    assert abs(cs2 - want) <= 1e-15 and t[0][3] == want
