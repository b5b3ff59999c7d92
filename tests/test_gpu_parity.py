"""CUDA path (through the C ABI) against the CPU oracle on the same inputs.

The FP64 form must be bit-identical to the oracle run with the kernels' exp
(exp_mode=1): both evaluate the reference's operations in the same order in
IEEE double without contraction.  Reduced-precision forms are checked
against the FP64 oracle within stated error bounds.
"""
import numpy as np
import pytest

from dlbc_gb300 import init, lbgpu
from golden_util import compare, golden_arrays, load_case, times
from lbcases import droplet_channel, spinodal
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def run_both(p, steps, precision=lbgpu.FP64, record_force=False):
    fl, m = init.init_fields(p)
    o = orc.Oracle(p, exp_mode=1, threads=8)
    g = lbgpu.GPULattice(p, precision=precision)
    g.upload(fl, m)
    if record_force:
        g.set_record_force(True)
    o.run(steps)
    g.step(steps)
    g.synchronize()
    return o, g


def assert_bitwise(o, g, p, check_force=False):
    pops = g.population()
    for c in range(p.components):
        a, b = pops[c], o.population(c)
        assert np.array_equal(a, b), f"component {c}: max |diff| {np.nanmax(np.abs(a - b)):.3e}"
    dens = g.density()
    vel = g.velocity()
    for c in range(p.components):
        assert np.array_equal(dens[c], o.density(c))
        assert np.array_equal(vel[c], o.velocity(c))
    if p.components == 2:
        assert np.array_equal(g.colour(), o.colour(0, 1))
    if check_force:
        fo = g.force()
        for c in range(p.components):
            assert np.array_equal(fo[c], o.force(c))


@pytest.mark.parametrize("eq", ["BDist2", "SecondOrder", "ThirdOrder"])
def test_fp64_spinodal_bitwise(eq):
    p = spinodal((24, 20, 16), eq=eq)
    o, g = run_both(p, 50, record_force=True)
    assert_bitwise(o, g, p, check_force=True)


def test_fp64_spinodal_long_run_bitwise():
    """Config-0 physics at 32^3 for 300 steps: chaotic enough that any
    last-bit difference would have grown visibly."""
    p = spinodal((32, 32, 32), eq="BDist2")
    o, g = run_both(p, 300)
    assert_bitwise(o, g, p)


@pytest.mark.parametrize("gwc", [(0.0, 0.0), (0.3, -0.2)])
def test_fp64_droplet_channel_walls_bitwise(gwc):
    """Config-1 physics (walls, body force, sphere) incl. the wall force."""
    p = droplet_channel((24, 12, 14), radius=4.0, acc=1e-3, gwc=gwc)
    o, g = run_both(p, 40, record_force=True)
    assert_bitwise(o, g, p, check_force=True)


def test_fp64_odd_and_minimal_sizes():
    for n in [(5, 7, 3), (2, 2, 2), (3, 2, 9)]:
        p = spinodal(n, eq="BDist2")
        o, g = run_both(p, 7)
        assert_bitwise(o, g, p)


def test_fp64_unequal_tau_and_single_component():
    p = droplet_channel((16, 10, 12), radius=3.0, acc=2e-4, tau=(0.8, 1.3), eq="SecondOrder")
    o, g = run_both(p, 20)
    assert_bitwise(o, g, p)
    p1 = spinodal((12, 10, 8))
    p1.components = 1
    p1.field_names = ["red"]
    p1.tau = [0.9]
    p1.gcc = [[-4.0]]
    p1.gwc = [0.0]
    p1.fluid_init = p1.fluid_init[:1]
    p1.fluid_densities = p1.fluid_densities[:1]
    p1.fluid_perturb = p1.fluid_perturb[:1]
    p1.random_reseed = p1.random_reseed[:1]
    p1.random_seed = p1.random_seed[:1]
    o, g = run_both(p1, 15)
    assert_bitwise(o, g, p1)


@pytest.mark.parametrize("name", ["merging-droplets-3d", "bdist2-sc-3d", "laplace-droplet-3d",
                                  "merging-droplets-2d", "bdist2-sc-2d", "poiseuille-2d",
                                  "laplace-quasi-1d-d2q9", "laplace-quasi-1d-d1q3", "checkpoint-3d"])
def test_fp64_reference_cases_bitwise_and_goldens(name):
    """The reference's own test inputs: bitwise vs the oracle, and within the
    reference's accuracies of its golden files at the first dump times
    (bit for bit for the D3Q19 BDist2 Shan-Chen cases)."""
    exact = name in ("bdist2-sc-3d", "checkpoint-3d")
    z, p = load_case(name)
    fl, m = init.init_fields(p)
    g = lbgpu.GPULattice(p)
    g.upload(fl, m)
    o = orc.Oracle(p, exp_mode=1, threads=8)
    t_now = 0
    small = int(np.prod(p.gn[: p.d])) <= 4096
    for t in times(z):
        if t > 100 and not (small and t <= 1000):
            break
        g.step(t - t_now)
        o.run(t - t_now)
        t_now = t
        assert_bitwise(o, g, p)
        for key, kind in golden_arrays(z, t):
            if kind.startswith("force") or kind == "mask":
                continue
            tol = 0.0 if exact else max(float(z[key + "/tol"]), 2.5e-15 if t > 0 else 0.0)
            if kind == "colour":
                a = g.colour()
            else:
                what, nm = kind.split("-", 1)
                c = p.field_names.index(nm)
                a = {"density": g.density, "velocity": g.velocity, "population": g.population}[what]()[c]
            assert compare(z, key, a, tol), key


def _lattice_1d(dq, eq, walls=False, tau=(1.0, 1.0), n=48, gwc=(0.0, 0.0)):
    from dlbc_gb300 import params
    lines = ["[lattice]", f"gn = [{n}]", "[lb]", "components = 2", 'fieldNames = ["red", "blue"]',
             f"tau = [{tau[0]}, {tau[1]}]", f"eqdist.eqDistForm = {eq}", "force.enableShanChen = true",
             "force.gcc = [[0.0, 3.6], [3.6, 0.0]]", "force.psiForm = Exponential",
             f"force.gwc = [{gwc[0]}, {gwc[1]}]", "force.globalAcc = [2e-5]",
             "init.fluidInit = [EqDistSphereFrac, EqDistSphereFrac]",
             "init.fluidDensities = [[0.7, 0.5], [0.5, 0.7]]", "init.initRadius = 0.25",
             "init.interfaceThickness = 5.0", "[random]", "seed = 4"]
    if walls:
        lines += ["[lb]", "mask.maskInit = Walls", "mask.dimensionHasWall = [[true, true]]"]
    return params.LBParams.from_dict(params.parse_lines(lines), dq)


@pytest.mark.parametrize("dq", ["d1q3", "d1q5"])
@pytest.mark.parametrize("eq", ["SecondOrder", "ThirdOrder", "BDist2"])
def test_fp64_one_dimensional_bitwise(dq, eq):
    """D1Q3 and D1Q5 (including D1Q5's |c| = 2 velocities in streaming, the
    Shan-Chen sum and the moments, its c_s^2 = 1, and BDist2's 1D no-op)
    bit for bit against the oracle, periodic and between walls."""
    for walls, tau, gwc in ((False, (1.0, 1.0), (0.0, 0.0)), (True, (0.8, 1.3), (0.2, -0.1))):
        p = _lattice_1d(dq, eq, walls=walls, tau=tau, gwc=gwc)
        o, g = run_both(p, 60, record_force=True)
        assert_bitwise(o, g, p, check_force=True)
        mass, mom = g.reduce()
        for c in range(2):
            assert abs(mass[c] - o.total_mass(c)) <= 1e-14 * abs(o.total_mass(c))


@pytest.mark.parametrize("dq", ["d1q3", "d1q5"])
@pytest.mark.parametrize("precision,tol", [(lbgpu.FP32, 1e-5), (lbgpu.FP16, 2e-3)])
def test_reduced_precision_one_dimensional(dq, precision, tol):
    p = _lattice_1d(dq, "ThirdOrder", walls=True)
    o, g = run_both(p, 200, precision=precision)
    d = g.density()
    for c in range(2):
        ref = o.density(c)
        assert np.linalg.norm(d[c] - ref) / np.linalg.norm(ref) < tol


@pytest.mark.parametrize("precision", [lbgpu.FP64, lbgpu.FP32, lbgpu.FP16])
def test_roundtrip_through_many_staging_chunks(precision):
    """Upload and download of a lattice whose haloed x-planes (14 MB each)
    need several chunks of each half of the staging buffer per component:
    the copies on the copy stream and the transposes on the step stream
    alternate between the halves without overwriting a chunk in use.  FP64
    and FP32 round-trip exactly (FP32: the stored floats, and a second
    round trip is the identity); FP16 stores offsets with a scale taken from
    the data, so its round trip is checked within half's resolution."""
    p = spinodal((40, 300, 300), perturb=0.05)
    fl, m = init.init_fields(p)
    rng = np.random.default_rng(3)
    for a in fl:
        a += rng.uniform(-1e-3, 1e-3, a.shape)  # distinct values everywhere
        a[...] = init.periodic_fill(a, 3)
    g = lbgpu.GPULattice(p, precision=precision)
    g.upload(fl, m)
    back = g.download()
    for c in range(2):
        if precision == lbgpu.FP64:
            assert np.array_equal(back[c], fl[c])
        elif precision == lbgpu.FP32:
            assert np.array_equal(back[c], fl[c].astype(np.float32).astype(np.float64))
        else:
            assert np.abs(back[c] - fl[c]).max() < 2e-3
    if precision != lbgpu.FP16:
        g2 = lbgpu.GPULattice(p, precision=precision)
        g2.upload(back, m)
        again = g2.download()
        for c in range(2):
            assert np.array_equal(again[c], back[c])


def test_download_roundtrip_and_halo():
    p = droplet_channel((10, 8, 6), radius=2.0)
    fl, m = init.init_fields(p)
    g = lbgpu.GPULattice(p)
    g.upload(fl, m)
    back = g.download()
    for c in range(2):
        assert np.array_equal(back[c], fl[c])


@pytest.mark.parametrize("precision", [lbgpu.FP64, lbgpu.FP32, lbgpu.FP16])
def test_pinned_host_arrays(precision):
    """Page-locked host arrays (pinned torch tensors, as the end-to-end
    benchmark passes) give the same results as pageable numpy arrays, halo
    images included."""
    import torch
    p = droplet_channel((12, 10, 16), radius=3.0, acc=1e-4)
    fl, m = init.init_fields(p)
    a = lbgpu.GPULattice(p, precision=precision)
    a.upload(fl, m)
    a.step(3)
    ra = a.download()
    b = lbgpu.GPULattice(p, precision=precision)
    pf = [torch.from_numpy(x.copy()).pin_memory() for x in fl]
    pm = torch.from_numpy(m.copy()).pin_memory()
    b.upload(pf, pm)
    b.step(3)
    out = [torch.empty(x.shape, dtype=torch.float64).pin_memory() for x in fl]
    b.download(out)
    for c in range(2):
        assert np.array_equal(out[c].numpy(), ra[c], equal_nan=True)


def test_mass_conservation_and_reduction():
    p = spinodal((32, 24, 16))
    o, g = run_both(p, 100)
    mass, mom = g.reduce()
    for c in range(2):
        ref = o.total_mass(c)
        assert abs(mass[c] - ref) <= 1e-13 * abs(ref)
    fl, _ = init.init_fields(p)
    m0 = [fl[c][2:-2, 2:-2, 2:-2].sum() for c in range(2)]
    for c in range(2):
        assert abs(mass[c] - m0[c]) <= 1e-12 * m0[c]


@pytest.mark.parametrize("precision,tol", [(lbgpu.FP32, 2e-5), (lbgpu.FP16, 2e-3)])
def test_reduced_precision_error_vs_fp64(precision, tol):
    """Relative L2 density error of the FP32 / FP16-storage forms against the
    FP64 oracle after 100 steps of spinodal decomposition."""
    p = spinodal((32, 32, 32), perturb=0.02)
    o, g = run_both(p, 100, precision=precision)
    dens = g.density()
    for c in range(2):
        ref = o.density(c)
        err = np.linalg.norm(dens[c] - ref) / np.linalg.norm(ref)
        assert err < tol, (c, err)


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16])
def test_reduced_precision_through_phase_separation(precision):
    """Spinodal decomposition run until the components have separated
    (densities far outside their initial +-0.05 spread): the FP32 and
    FP16-offset forms stay finite, conserve mass, and separate like FP64."""
    p = spinodal((32, 32, 32), perturb=0.05)
    fl, m = init.init_fields(p)
    ref = lbgpu.GPULattice(p)
    ref.upload(fl, None)
    g = lbgpu.GPULattice(p, precision=precision)
    g.upload(fl, None)
    mass0, _ = g.reduce()
    ref.step(1500)
    g.step(1500)
    d64 = ref.density()
    d = g.density()
    for c in range(2):
        assert np.all(np.isfinite(d[c]))
        assert d64[c].max() - d64[c].min() > 0.5  # separated
        assert np.abs(d[c].max() - d64[c].max()) < 0.05 * d64[c].max()
    mass1, _ = g.reduce()
    # FP32 conserves mass to float rounding; half offsets keep 11 significant
    # bits, and the rounding of separated bulk phases (all 19 offsets of a
    # site nearly equal, so their rounding errors add up) lets the total mass
    # drift by a few 1e-3 over this run
    drift = 1e-4 if precision == lbgpu.FP32 else 1e-2
    assert np.all(np.abs(mass1 - mass0) <= drift * np.abs(mass0)), (mass0, mass1)
    phase = np.mean(np.sign(d[0] - d[1]) != np.sign(d64[0] - d64[1]))
    assert phase < 0.05, phase


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16])
@pytest.mark.parametrize("d", [3, 2])
def test_fused_step_leaves_solid_sites_unchanged(precision, d):
    """The fused step writes fluid sites only; both population buffers hold
    the solid sites' populations, so they read back bit for bit as uploaded
    after any number of steps (odd and even)."""
    n = (12, 10, 16) if d == 3 else (12, 20)
    p = droplet_channel(n, radius=3.0, acc=1e-4, gwc=(0.2, -0.1), d=d)
    fl, m = init.init_fields(p)
    g = lbgpu.GPULattice(p, precision=precision)
    g.upload(fl, m)
    d0 = g.population()
    solid = m[(slice(2, -2),) * d] != 0
    assert solid.any()
    for n in (1, 2, 5):
        g.step(n)
        d = g.population()
        for c in range(2):
            assert np.array_equal(d[c][solid], d0[c][solid])
            assert not np.array_equal(d[c][~solid], d0[c][~solid])


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16])
def test_reupload_with_new_mask_matches_fresh_lattice(precision):
    """A state uploaded over a running lattice, at odd parity and with a
    different mask (an obstacle added), steps exactly like the same state
    uploaded into a new handle: the solid sites of the other buffer are
    refreshed before the next fused step."""
    p = droplet_channel((14, 16, 32), radius=4.0, acc=1e-4, gwc=(0.2, -0.1))
    fl, m = init.init_fields(p)
    g = lbgpu.GPULattice(p, precision=precision)
    g.upload(fl, m)
    g.step(3)
    m2 = m.copy()
    m2[6:10, 6:9, 12:15] = 1  # an obstacle (haloed indices)
    fl2 = [f.copy() for f in fl]
    g.upload(fl2, m2)
    g.step(4)
    a = g.population()
    h = lbgpu.GPULattice(p, precision=precision)
    h.upload(fl2, m2)
    h.step(4)
    b = h.population()
    for c in range(2):
        assert np.array_equal(a[c], b[c])


def test_launch_count_and_errors():
    p = spinodal((8, 8, 8))
    fl, m = init.init_fields(p)
    g = lbgpu.GPULattice(p)
    with pytest.raises(lbgpu.LbgpuError):
        g.step(1)  # before upload
    g.upload(fl, m)
    n0 = g.launch_count
    g.step(5)
    assert g.launch_count - n0 == 10
    with pytest.raises(lbgpu.LbgpuError):
        g.force()  # force not recorded


def _run_form(p, steps, precision, two_kernel, record_force=False):
    import os
    old = os.environ.get("LBGPU_TWO_KERNEL")
    os.environ["LBGPU_TWO_KERNEL"] = "1" if two_kernel else "0"
    try:
        fl, m = init.init_fields(p)
        g = lbgpu.GPULattice(p, precision=precision)
    finally:
        if old is None:
            del os.environ["LBGPU_TWO_KERNEL"]
        else:
            os.environ["LBGPU_TWO_KERNEL"] = old
    g.upload(fl, m)
    if record_force:
        g.set_record_force(True)
    g.step(steps)
    out = g.population()
    f = g.force() if record_force else None
    return out, f


FUSED_CASES = {
    "spinodal": lambda: spinodal((24, 20, 40), eq="BDist2"),
    "walls": lambda: droplet_channel((20, 18, 36), radius=5.0, acc=1e-3, gwc=(0.25, -0.15)),
    "partial_tiles": lambda: spinodal((7, 13, 37), eq="SecondOrder"),
    # D2Q9 (lb_fused2d.cuh): two 256-site tiles, the second partial
    "d2q9-spinodal": lambda: spinodal((40, 300), d=2),
    "d2q9-walls": lambda: droplet_channel((36, 70), radius=8.0, acc=1e-3, gwc=(0.25, -0.15), d=2),
    # (tau = 0.8 / 1.3 is unstable for this 2D case in the reference's
    # arithmetic too: the CPU oracle overflows within 30 steps)
    "d2q9-unequal-tau": lambda: droplet_channel((30, 40), radius=6.0, acc=1e-3, tau=(0.9, 1.1), d=2),
    "d2q9-third-order": lambda: spinodal((7, 37), eq="ThirdOrder", d=2),
}


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16])
@pytest.mark.parametrize("case", list(FUSED_CASES))
def test_fused_step_matches_two_kernel_step(precision, case):
    """The fused single-pass kernel computes the same per-site arithmetic as
    the two-kernel step; only FMA contraction may differ (float)."""
    p = FUSED_CASES[case]()
    a, fa = _run_form(p, 30, precision, two_kernel=False, record_force=True)
    b, fb = _run_form(p, 30, precision, two_kernel=True, record_force=True)
    tol = 2e-6 if precision == lbgpu.FP32 else 2e-3
    # the force is a cancelling sum of terms w_q*psi*psi*g ~ 0.03: compare it
    # on that scale (the fused kernel sums the stencil in another order)
    ftol = 3e-7 if precision == lbgpu.FP32 else 3e-4
    for c in range(2):
        scale = np.abs(b[c]).max()
        assert np.abs(a[c] - b[c]).max() <= tol * scale, (c, np.abs(a[c] - b[c]).max())
        assert np.abs(fa[c] - fb[c]).max() <= ftol, (c, np.abs(fa[c] - fb[c]).max())
