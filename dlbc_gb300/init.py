"""Initial fields in the reference's layout (host side, numpy).

Restates ``initMask`` (src/dlbc/lb/mask.d:134-172) and ``initFluids``
(src/dlbc/lb/init.d:77-134) with the field initialisers of
src/dlbc/fields/init.d, producing what ``L.fluids[i].arr`` and ``L.mask.arr``
hold before the first timestep: haloed arrays (halo 2, row-major [x][y][z],
the Q populations of a site contiguous), with the halo filled by periodic
images as ``exchangeHalo`` leaves it (src/main.d:142).

Random numbers follow the reference exactly: Mt19937 seeded with
``seed (+ rank)`` (src/dlbc/random.d:43-53), one ``uniform(a, b)`` draw per
haloed site of each process's local block in row-major order, fluid 0 before
fluid 1 unless ``randomReseed`` (src/dlbc/lb/init.d:109-122).  The process
grid ``parallel.nc`` is honoured so that a lattice initialised on N MPI
ranks is reproduced bit for bit.
"""
from __future__ import annotations

from typing import List, Tuple

import numpy as np

from .params import FLUID_INITS, LBParams

HALO = 2
_FI = {name: i for i, name in enumerate(FLUID_INITS)}


def weights(q: int) -> np.ndarray:
    """generateWeights (src/dlbc/lb/connectivity.d:250-295)."""
    if q == 19:
        return np.array([1.0 / 3.0] + [1.0 / 18.0] * 6 + [1.0 / 36.0] * 12)
    if q == 9:
        return np.array([4.0 / 9.0] + [1.0 / 9.0] * 4 + [1.0 / 36.0] * 4)
    if q == 3:
        return np.array([4.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0])
    if q == 5:
        return np.array([6.0 / 12.0, 2.0 / 12.0, 2.0 / 12.0, 1.0 / 12.0, 1.0 / 12.0])
    raise ValueError(q)


def eq_dist_unity(q: int, eq_form: int) -> np.ndarray:
    """eqDistUnity (src/dlbc/lb/eqdist.d:310-315): the equilibrium of unit
    density at rest.  It equals the lattice weights except for BDist2 on
    D2Q9, whose constants (eqdist.d:186-230) give 1/2, 1/12 and 1/24, and
    BDist2 on D1Q3/D1Q5, which returns the population itself
    (eqdist.d:268-272): (1, 0, ..., 0)."""
    if eq_form == 2 and q in (3, 5):
        return np.array([1.0] + [0.0] * (q - 1))
    if eq_form == 2 and q == 9:
        aN1 = 1.0 / 24.0
        return np.array([0.5] + [2.0 * aN1] * 4 + [aN1] * 4)
    return weights(q)


class _Rng:
    """Mt19937 with Phobos' uniform(a, b) for doubles."""

    def __init__(self, seed: int):
        self.rs = np.random.RandomState(seed & 0xFFFFFFFF)

    def uniform(self, a: float, b: float, n: int) -> np.ndarray:
        u = self.rs.randint(0, 2 ** 32, size=n, dtype=np.uint32).astype(np.float64)
        bb = np.nextafter(b, -np.inf)
        return a + (bb - a) * u / 4294967295.0


def _slt(pos, width, negval, posval):
    """symmetricLinearTransition (src/dlbc/fields/init.d:346-366), elementwise."""
    pos = np.asarray(pos, np.float64)
    if width == 0.0:
        return np.where(pos < 0, negval, posval).astype(np.float64)
    with np.errstate(all="ignore"):
        mid = negval * (0.5 - pos / width) + posval * (0.5 + pos / width)
    return np.where(pos < -0.5 * width, negval, np.where(pos > 0.5 * width, posval, mid)).astype(np.float64)


def _dot(offs: List[np.ndarray]) -> np.ndarray:
    s = np.zeros_like(offs[0])
    for o in offs:
        s = s + o * o
    return s


def _local_mask(p: LBParams, nl, nc, cc, nlH) -> np.ndarray:
    d = p.d
    grids = np.meshgrid(*[np.arange(nlH[i]) for i in range(d)], indexing="ij")
    g = [grids[i] + cc[i] * nl[i] - HALO for i in range(d)]
    m = np.zeros(nlH, np.int32)
    mi = p.mask_init
    if mi == 0:
        return m
    if mi == 2:  # Plates
        ax = p.mask_axis
        N = nl[ax] * nc[ax]
        m[(g[ax] == p.wall_offset) | (g[ax] == N - 1 - p.wall_offset)] = 1
    elif mi in (3, 4):  # Tube / Box
        for vd in range(d):
            if mi == 3 and vd == p.mask_axis:
                continue
            m[(g[vd] == 0) | (g[vd] == nl[vd] * nc[vd] - 1)] = 1
    elif mi == 5:  # Walls
        for vd in range(d):
            if p.dimension_has_wall[vd][0]:
                m[g[vd] < p.wall_thickness] = 1
            if p.dimension_has_wall[vd][1]:
                m[g[vd] >= nl[vd] * nc[vd] - p.wall_thickness] = 1
    elif mi == 1:  # File (mask.d:153-155): the global mask, this process's block
        gm = _read_global(p.mask_file, tuple(int(x) for x in p.gn[:d]), "mask.maskFile")
        block = tuple(slice(cc[i] * nl[i], (cc[i] + 1) * nl[i]) for i in range(d))
        m[tuple(slice(HALO, HALO + nl[i]) for i in range(d))] = gm[block]
    else:
        raise ValueError(f"unsupported maskInit {mi}")
    return m


def _read_global(path: str, shape, what: str) -> np.ndarray:
    """A field file as readField reads it (src/dlbc/io/hdf5.d:309): the
    /OutArray of the global lattice, checked against the lattice size."""
    from . import h5
    if not path:
        raise ValueError(f"{what} is not set")
    a = h5.read_field(path)
    if tuple(a.shape[: len(shape)]) != tuple(shape):
        raise ValueError(f"{what} {path}: shape {a.shape} does not match the lattice {shape}")
    return a


def _local_fluid(p: LBParams, f: int, rng: _Rng, nl, nc, cc, nlH) -> np.ndarray:
    d, q = p.d, p.q
    eqpop = eq_dist_unity(q, p.eq_form)
    size = int(np.prod(nlH))
    fi = p.fluid_init[f]
    dens = p.fluid_densities[f]
    gsz = [int(x) for x in p.gn[:d]]
    grids = np.meshgrid(*[np.arange(nlH[i], dtype=np.float64) for i in range(d)], indexing="ij")

    def gcoord(i):
        return (grids[i] + float(cc[i] * nl[i])) - float(HALO)

    out = np.full(tuple(nlH) + (q,), np.nan)
    if fi == _FI["None"]:
        return out
    if fi == _FI["File"]:  # init.d:272-275: this process's block of the file
        ga = _read_global(p.fluid_files[f] if f < len(p.fluid_files) else "", tuple(gsz), "init.fluidFiles")
        if ga.shape != tuple(gsz) + (q,):
            raise ValueError(f"init.fluidFiles {p.fluid_files[f]}: shape {ga.shape}, expected {tuple(gsz) + (q,)}")
        block = tuple(slice(cc[i] * nl[i], (cc[i] + 1) * nl[i]) for i in range(d))
        out[tuple(slice(HALO, HALO + nl[i]) for i in range(d))] = ga[block]
        return out
    if fi == _FI["Const"]:
        out[...] = dens[0]
        return out
    if fi == _FI["ConstRandom"]:
        out[...] = (dens[0] * rng.uniform(0.0, 2.0, size * q)).reshape(out.shape)
        return out
    if fi == _FI["EqDist"]:
        out[...] = dens[0] * eqpop
        return out
    if fi == _FI["EqDistRandom"]:
        val = dens[0] * rng.uniform(0.0, 2.0, size)
    elif fi == _FI["EqDistPerturb"]:
        val = dens[0] + rng.uniform(-p.fluid_perturb[f], p.fluid_perturb[f], size)
    elif fi == _FI["EqDistPerturbFrac"]:
        val = dens[0] * (1.0 + rng.uniform(-p.fluid_perturb[f], p.fluid_perturb[f], size))
    elif fi in (_FI["EqDistSphere"], _FI["EqDistSphereFrac"], _FI["EqDistTwoSpheres"],
                _FI["EqDistTwoSpheresFrac"], _FI["EqDistCylinder"], _FI["EqDistCylinderFrac"]):
        R = p.init_radius
        off = list(p.init_offset)
        sep = list(p.init_separation)
        if fi in (_FI["EqDistSphereFrac"], _FI["EqDistTwoSpheresFrac"]):
            small = min(gsz)
            R = p.init_radius * small
            off = [p.init_offset[i] * gsz[i] for i in range(d)]
            sep = [p.init_separation[i] * gsz[i] for i in range(d)]
        if fi == _FI["EqDistCylinderFrac"]:
            small = 0
            for vd in range(d):
                if vd != p.init_axis and (gsz[vd] < small or small == 0):
                    small = gsz[vd]
            R = p.init_radius * small
            off = [p.init_offset[i] * gsz[i] for i in range(d)]
        centre = [float(nc[i] * nl[i]) * 0.5 for i in range(d)]
        if fi in (_FI["EqDistTwoSpheres"], _FI["EqDistTwoSpheresFrac"]):
            o1 = [gcoord(i) - (centre[i] + off[i] - 0.5 * sep[i]) + 0.5 for i in range(d)]
            o2 = [gcoord(i) - (centre[i] + off[i] + 0.5 * sep[i]) + 0.5 for i in range(d)]
            relpos = np.minimum(np.sqrt(_dot(o1)) - R, np.sqrt(_dot(o2)) - R)
        elif fi in (_FI["EqDistCylinder"], _FI["EqDistCylinderFrac"]):
            o = [np.zeros_like(grids[0]) if i == p.init_axis else gcoord(i) - (centre[i] + off[i]) + 0.5
                 for i in range(d)]
            relpos = np.sqrt(_dot(o)) - R
        else:
            o = [gcoord(i) - (centre[i] + off[i]) + 0.5 for i in range(d)]
            relpos = np.sqrt(_dot(o)) - R
        val = _slt(relpos, p.interface_thickness, dens[0], dens[1])
    elif fi in (_FI["EqDistLamellae"], _FI["EqDistLamellaeFrac"]):
        ax = p.init_axis
        widths = list(p.lamellae_widths)
        if fi == _FI["EqDistLamellaeFrac"]:
            widths = [w * gsz[ax] for w in widths]
        interfaces = [0.0] + widths
        for i in range(1, len(interfaces)):
            interfaces[i] += interfaces[i - 1]
        interfaces = [v - 0.5 for v in interfaces]
        gp = gcoord(ax)
        diffs = np.stack([np.abs(iv - gp) for iv in interfaces])
        ci = np.argmin(diffs, axis=0)  # first minimum, as findClosestInterface
        mind = gp - np.asarray(interfaces)[ci]
        nv = len(dens)
        val = np.empty_like(gp)
        for k in range(len(interfaces)):
            sel = ci == k
            if k == 0:
                neg, pos = dens[nv - 1], dens[0]
            elif k == nv:
                neg, pos = dens[k - 1], dens[0]
            else:
                neg, pos = dens[k - 1], dens[k]
            val[sel] = _slt(mind[sel], p.interface_thickness, neg, pos)
    else:
        raise ValueError(f"unsupported fluidInit {fi}")
    val = np.asarray(val, np.float64).reshape(nlH)
    out[...] = val[..., None] * eqpop
    return out


def periodic_fill(a: np.ndarray, d: int) -> np.ndarray:
    """exchangeHalo on one process: halo sites become periodic images."""
    sl = tuple(slice(HALO, -HALO) for _ in range(d))
    phys = a[sl]
    pad = [(HALO, HALO)] * d + [(0, 0)] * (a.ndim - d)
    return np.pad(phys, pad, mode="wrap")


def init_fields(p: LBParams) -> Tuple[List[np.ndarray], np.ndarray]:
    """(fluids, mask): haloed arrays as the reference holds them after
    initMask + initFluids + exchangeHalo."""
    d, q = p.d, p.q
    n = [int(x) for x in p.gn[:d]]
    nc = [max(1, int(p.nc[i])) if i < len(p.nc) else 1 for i in range(d)]
    nl = []
    for i in range(d):
        if n[i] % nc[i]:
            raise ValueError(f"Cannot divide lattice {n} evenly over a {nc} grid of processes.")
        nl.append(n[i] // nc[i])
    nlH = [x + 2 * HALO for x in nl]
    nH = [x + 2 * HALO for x in n]
    fluids = [np.zeros(tuple(nH) + (q,), np.float64) for _ in range(p.components)]
    mask = np.zeros(tuple(nH), np.int32)
    nranks = int(np.prod(nc))
    for rank in range(nranks):
        cc = []
        r = rank
        for i in reversed(range(d)):  # last dimension fastest
            cc.insert(0, r % nc[i])
            r //= nc[i]
        lm = _local_mask(p, nl, nc, cc, nlH)
        grng = _Rng(p.seed + (rank if p.shift_seed_by_rank else 0))
        phys_l = tuple(slice(HALO, HALO + nl[i]) for i in range(d))
        phys_g = tuple(slice(HALO + cc[i] * nl[i], HALO + (cc[i] + 1) * nl[i]) for i in range(d))
        mask[phys_g] = lm[phys_l]
        for f in range(p.components):
            rng = grng
            if p.random_reseed[f]:
                rng = _Rng(p.random_seed[f] + (rank if p.shift_seed_by_rank else 0))
            lf = _local_fluid(p, f, rng, nl, nc, cc, nlH)
            # initEqDistWall (src/dlbc/fields/init.d:469-477)
            solid = lm == 1
            lf[solid] = 0.0
            lf[solid, 0] = 1.0
            fluids[f][phys_g] = lf[phys_l]
    fluids = [np.ascontiguousarray(periodic_fill(a, d)) for a in fluids]
    mask = np.ascontiguousarray(periodic_fill(mask, d))
    return fluids, mask
