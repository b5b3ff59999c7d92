"""The pair kernel (two z-adjacent sites per thread, lb_pairs.cuh): the
fused single-pass step of lattices without solid sites, with an even z
extent and the BDist2 equilibrium, in the I16 form and, with every tau = 1,
the FP32 and FP16 forms; in FP16 also lattices whose solid sites are
exactly the planes z = 0 and z = nz - 1 (planar walls, nz a multiple of 64,
no wall force).  Elsewhere the one-site-per-thread kernel (lb_fused.cuh)
runs, which the same tests cover (the other walled cases).

* Against the two-kernel float step (LBGPU_TWO_KERNEL=1, a different
  kernel with the reference's per-site operation order): populations within
  the tolerances of the fused-versus-two-kernel test (2e-6 of the largest
  population in FP32, 2e-3 in FP16), forces within 3e-7 / 3e-4, over tile
  edges in y and z, partial tiles, tiny extents, walls with the wall force,
  tau != 1 and one component.  I16 (both kernels, tau != 1 included)
  against FP32 within the FP16 tolerances.
* Translation invariance, bit for bit (every form, walls included): a
  lattice shifted periodically by
  (3, 5, 2), by 66 sites along z or by (1, 8, 64) steps to the shifted
  result.  The shifted sites move to other lanes, warps, tiles and ring
  gathers, so this checks that a site's arithmetic does not depend on where
  it is computed.
* Mass conservation and no spurious momentum over a phase separation.
"""
import os

import numpy as np
import pytest

from dlbc_gb300 import init, lbgpu
from lbcases import droplet_channel, spinodal

pytestmark = pytest.mark.gpu


def _with_env(env, fn):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        return fn()
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


def _run(p, steps, precision, fields=None, two_kernel=False, record_force=True, rho0=(0.0, 0.0)):
    def go():
        fl, m = fields if fields is not None else init.init_fields(p)
        g = lbgpu.GPULattice(p, precision=precision, rho0=rho0)
        g.upload(fl, m)
        return g
    g = _with_env({"LBGPU_TWO_KERNEL": "1" if two_kernel else "0"}, go)
    if record_force:
        g.set_record_force(True)
    g.step(steps)
    pops = g.population()
    fo = g.force() if record_force else None
    g.close()
    return pops, fo


def _one_component(p):
    p.components = 1
    p.field_names = p.field_names[:1]
    p.tau = p.tau[:1]
    p.gcc = [[0.0]]
    p.gwc = p.gwc[:1]
    p.fluid_init = p.fluid_init[:1]
    p.fluid_densities = p.fluid_densities[:1]
    p.fluid_perturb = p.fluid_perturb[:1]
    p.random_reseed = p.random_reseed[:1]
    p.random_seed = p.random_seed[:1]
    return p


CASES = {
    "two-z-tiles": lambda: spinodal((12, 16, 128), perturb=0.03),
    "partial-tiles": lambda: spinodal((10, 13, 70), perturb=0.03),
    "nz2": lambda: spinodal((6, 9, 2), perturb=0.03),
    "nz4-ny2": lambda: spinodal((5, 2, 4), perturb=0.03),
    "walls": lambda: droplet_channel((14, 18, 36), radius=5.0, acc=1e-3),
    "wall-force": lambda: droplet_channel((12, 10, 66), radius=4.0, acc=1e-3, gwc=(0.25, -0.15)),
    "tau": lambda: droplet_channel((12, 11, 40), radius=4.0, acc=1e-3, gwc=(0.1, 0.0), tau=(0.8, 1.3)),
    "one-component": lambda: _one_component(spinodal((10, 12, 64), perturb=0.03)),
    # planar z-walls (the FP16 pair kernel's walled case): one z-tile holding
    # both wall lanes, and two z-tiles with one each, partial y tiles
    "planar-walls": lambda: droplet_channel((14, 18, 64), radius=5.0, acc=1e-3),
    "planar-walls-2tiles": lambda: droplet_channel((10, 9, 128), radius=4.0, acc=1e-3),
}


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16])
@pytest.mark.parametrize("case", list(CASES))
def test_pairs_match_two_kernel_step(case, precision):
    p = CASES[case]()
    a, fa = _run(p, 20, precision)
    b, fb = _run(p, 20, precision, two_kernel=True)
    tol = 2e-6 if precision == lbgpu.FP32 else 2e-3
    ftol = 3e-7 if precision == lbgpu.FP32 else 3e-4
    for c in range(p.components):
        scale = np.abs(b[c]).max()
        assert np.all(np.isfinite(a[c]))
        assert np.abs(a[c] - b[c]).max() <= tol * scale, (c, np.abs(a[c] - b[c]).max() / scale)
        assert np.nanmax(np.abs(fa[c] - fb[c])) <= ftol, (c, np.nanmax(np.abs(fa[c] - fb[c])))


@pytest.mark.parametrize("case", ["two-z-tiles", "partial-tiles", "nz2", "walls", "wall-force", "tau",
                                  "one-component", "planar-walls", "planar-walls-2tiles"])
def test_i16_close_to_fp32(case):
    """The 16-bit fixed-point form (I16): populations after 20 steps within
    2e-3 of the largest population of the FP32 form's, forces within 3e-4
    (the FP16 form's tolerances against float arithmetic)."""
    p = CASES[case]()
    a, fa = _run(p, 20, lbgpu.I16)
    b, fb = _run(p, 20, lbgpu.FP32)
    for c in range(p.components):
        scale = np.abs(b[c]).max()
        assert np.all(np.isfinite(a[c]))
        assert np.abs(a[c] - b[c]).max() <= 2e-3 * scale, (c, np.abs(a[c] - b[c]).max() / scale)
        assert np.nanmax(np.abs(fa[c] - fb[c])) <= 3e-4, (c, np.nanmax(np.abs(fa[c] - fb[c])))


def _shifted(fields, mask, shift):
    d = len(shift)
    sl = (slice(2, -2),) * d
    axes = tuple(range(d))
    fl = [np.roll(f[sl], shift, axis=axes) for f in fields]
    m = np.roll(mask[sl], shift, axis=axes)
    pad = lambda a: np.pad(a, [(2, 2)] * d + [(0, 0)] * (a.ndim - d), mode="wrap")  # noqa: E731
    return [pad(f) for f in fl], pad(m)


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16, lbgpu.I16])
@pytest.mark.parametrize("shift", [(3, 5, 2), (0, 0, 66), (1, 8, 64)])
def test_pairs_translation_invariant_bitwise(precision, shift):
    p = spinodal((12, 20, 132), perturb=0.05)
    fl, m = init.init_fields(p)
    # a fixed reference density for the offset forms: the mean at upload
    # could round differently for the permuted lattice
    a, fa = _run(p, 15, precision, fields=(fl, m), rho0=(0.7, 0.7))
    fs, ms = _shifted(fl, m, shift)
    b, fb = _run(p, 15, precision, fields=(fs, ms), rho0=(0.7, 0.7))
    for c in range(2):
        assert np.array_equal(np.roll(a[c], shift, axis=(0, 1, 2)), b[c]), c
        assert np.array_equal(np.roll(fa[c], shift, axis=(0, 1, 2)), fb[c], equal_nan=True), c


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16, lbgpu.I16])
@pytest.mark.parametrize("shift", [(3, 5, 0), (1, 8, 0)])
def test_pairs_walled_channel_translation_invariant_bitwise(precision, shift):
    """The same with z walls (shifted along x and y only; the one-site
    kernel, whose tiles next to a wall run the wall code): bounce-back, the
    wall force reading the solid sites' densities, and still every site
    computes the same bits wherever it sits."""
    p = droplet_channel((12, 20, 70), radius=4.0, acc=1e-3, gwc=(0.2, -0.1))
    fl, m = init.init_fields(p)
    a, fa = _run(p, 15, precision, fields=(fl, m), rho0=(0.5, 0.5))
    fs, ms = _shifted(fl, m, shift)
    b, fb = _run(p, 15, precision, fields=(fs, ms), rho0=(0.5, 0.5))
    for c in range(2):
        assert np.array_equal(np.roll(a[c], shift, axis=(0, 1, 2)), b[c]), c
        assert np.array_equal(np.roll(fa[c], shift, axis=(0, 1, 2)), fb[c], equal_nan=True), c


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16, lbgpu.I16])
@pytest.mark.parametrize("shift", [(3, 5, 0), (1, 8, 0)])
def test_pairs_planar_walls_translation_invariant_bitwise(precision, shift):
    """Planar z-walls (walls exactly at z = 0 and z = nz - 1, no wall force,
    tau = 1: FP16 on the pair kernel's wall lanes, FP32 and I16 on the
    one-site kernel), shifted along x and y: the wall lanes' bounce-back,
    psi and stores give every site the same bits wherever it sits."""
    p = droplet_channel((12, 20, 128), radius=4.0, acc=1e-3)
    fl, m = init.init_fields(p)
    a, fa = _run(p, 15, precision, fields=(fl, m), rho0=(0.5, 0.5))
    fs, ms = _shifted(fl, m, shift)
    b, fb = _run(p, 15, precision, fields=(fs, ms), rho0=(0.5, 0.5))
    for c in range(2):
        assert np.array_equal(np.roll(a[c], shift, axis=(0, 1, 2)), b[c]), c
        assert np.array_equal(np.roll(fa[c], shift, axis=(0, 1, 2)), fb[c], equal_nan=True), c


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16, lbgpu.I16])
def test_pairs_conserve_mass_over_phase_separation(precision):
    """A spinodal decomposition through phase separation: the total mass of
    each component drifts by rounding only (I16: its collision conserves
    every site's integer mass exactly, except where the rest population
    saturates at +-32767, which the violent separation of this lattice
    reaches at a few sites: 3e-8), the total momentum stays at its (zero)
    initial value to rounding."""
    p = spinodal((32, 32, 64), perturb=0.05)
    fl, m = init.init_fields(p)
    g = lbgpu.GPULattice(p, precision=precision)
    g.upload(fl, m)
    mass0, _ = g.reduce()
    g.step(600)
    mass1, mom1 = g.reduce()
    d = g.density()
    assert all(np.all(np.isfinite(x)) for x in d)
    assert d[0].max() - d[0].min() > 0.3  # separated
    drift = {lbgpu.FP32: 1e-4, lbgpu.FP16: 2e-2, lbgpu.I16: 2e-7}[precision]
    assert np.all(np.abs(mass1 - mass0) <= drift * np.abs(mass0)), (mass0, mass1)
    total = np.asarray(mom1, dtype=np.float64).reshape(p.components, 3).sum(axis=0)
    assert np.abs(total).max() <= 1e-3 * float(np.sum(mass1)), mom1


@pytest.mark.parametrize("tau", [(1.0, 1.0), (0.95, 1.05)])
def test_i16_conserves_mass_exactly_with_walls(tau):
    """The I16 form on the one-site kernel (walls, the wall force, tau = 1
    and tau != 1) conserves each component's total mass exactly: 2000 steps
    of a droplet in a channel, where a uniform bath rounds the same way at
    every site and every step (the FP16 form drifts there)."""
    p = droplet_channel((24, 20, 36), radius=5.0, acc=1e-5, gwc=(0.1, -0.05), tau=tau)
    fl, m = init.init_fields(p)
    g = lbgpu.GPULattice(p, precision=lbgpu.I16)
    g.upload(fl, m)
    mass0, _ = g.reduce()
    g.step(2000)
    mass1, _ = g.reduce()
    assert np.all(np.isfinite(mass1))
    assert np.all(np.abs(mass1 - mass0) <= 1e-12 * np.abs(mass0)), (mass0, mass1)


# The D2Q9 pair kernel (lb_pairs2d.cuh, the FP16 form; FP32 runs the
# one-site D2Q9 kernel on the same lattices): every tau = 1, BDist2, an even
# ny, no solid site; tiles of 256 y, the second partial, and tiny extents.
CASES_2D = {
    "d2q9-two-tiles": lambda: spinodal((12, 300), perturb=0.03, d=2),
    "d2q9-ny2": lambda: spinodal((6, 2), perturb=0.03, d=2),
    "d2q9-ny258": lambda: spinodal((5, 258), perturb=0.03, d=2),
}


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16])
@pytest.mark.parametrize("case", list(CASES_2D))
def test_pairs2d_match_two_kernel_step(case, precision):
    p = CASES_2D[case]()
    a, fa = _run(p, 20, precision)
    b, fb = _run(p, 20, precision, two_kernel=True)
    tol = 2e-6 if precision == lbgpu.FP32 else 2e-3
    ftol = 3e-7 if precision == lbgpu.FP32 else 3e-4
    for c in range(p.components):
        scale = np.abs(b[c]).max()
        assert np.all(np.isfinite(a[c]))
        assert np.abs(a[c] - b[c]).max() <= tol * scale, (c, np.abs(a[c] - b[c]).max() / scale)
        assert np.nanmax(np.abs(fa[c] - fb[c])) <= ftol, (c, np.nanmax(np.abs(fa[c] - fb[c])))


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16])
@pytest.mark.parametrize("shift", [(3, 5), (0, 66), (1, 256)])
def test_pairs2d_translation_invariant_bitwise(precision, shift):
    """Shifted sites move to other lanes, warps (the shuffles' edge loads),
    tiles and ring gathers, and still compute the same bits."""
    p = spinodal((12, 300), perturb=0.05, d=2)
    fl, m = init.init_fields(p)
    a, fa = _run(p, 15, precision, fields=(fl, m), rho0=(0.7, 0.7))
    fs, ms = _shifted(fl, m, shift)
    b, fb = _run(p, 15, precision, fields=(fs, ms), rho0=(0.7, 0.7))
    for c in range(2):
        assert np.array_equal(np.roll(a[c], shift, axis=(0, 1)), b[c]), c
        assert np.array_equal(np.roll(fa[c], shift, axis=(0, 1)), fb[c], equal_nan=True), c
