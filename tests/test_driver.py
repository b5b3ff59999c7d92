"""The reference-style driver: file names, parameter input, HDF5 dumps,
checkpoint write/rotate/restore and hooks.

CPU tests run the driver over a stand-in lattice backed by the oracle (test
infrastructure only: the driver's own default is the CUDA lattice) to check
its file handling; the GPU tests run the same paths on the CUDA lattice.
The checkpoint-3d case is the reference's own restore test
(tests/runnable/tests/technical/checkpoint-3d): restore from its t = 0
checkpoint files, run 5 steps, compare the dumps with its goldens exactly.
"""
import os
import re

import numpy as np
import pytest

from dlbc_gb300 import driver, h5, init, lbgpu
from golden_util import compare, golden_arrays, load_case, sha
from lbcases import D3Q19_VELOCITIES, spinodal
from oracle import oracle as orc


class OracleLattice:
    """The CPU oracle behind GPULattice's interface (test stand-in)."""

    def __init__(self, p, precision=0, device=0):
        self.p = p
        self.o = orc.Oracle(p, exp_mode=1, threads=4, init=False)
        self.n = tuple(p.gn[: p.d])
        self.record = False

    def upload(self, fluids, mask=None):
        for c, a in enumerate(fluids):
            self.o.set_fluid_haloed(c, a)
        m = mask if mask is not None else np.zeros(self.o.nH, np.int32)
        self.o.set_mask_haloed(m)

    def download(self, out=None):
        out = out or [np.empty(self.o.nH + (self.p.q,)) for _ in range(self.p.components)]
        self.o.exchange_halo()
        for c in range(self.p.components):
            out[c][...] = self.o.fluid_haloed(c)
        return out

    def step(self, n=1):
        self.o.run(n)

    def step_host(self, fluids, mask=None, out=None):
        self.upload(fluids, mask)
        self.step(1)
        return self.download(out)

    def advect(self):
        pass

    def collide(self):
        self.o.run(1)

    def set_record_force(self, on=True):
        self.record = on

    def density(self):
        return [self.o.density(c) for c in range(self.p.components)]

    def velocity(self):
        return [self.o.velocity(c) for c in range(self.p.components)]

    def colour(self):
        return self.o.colour(0, 1)

    def force(self):
        return [self.o.force(c) for c in range(self.p.components)]

    def synchronize(self):
        pass

    def close(self):
        pass


# ---------------------------------------------------------------------------
# names, tokens, cadence, input
# ---------------------------------------------------------------------------

def test_file_names_follow_the_reference():
    # the example of the reference's usage text (src/dlbc/getopt.d:44-48)
    assert driver.filename_cp_output("out", "cp", "cp-red", "foobar", "20140527T135106", 60) == \
        "out/cp/cp-red-foobar-20140527T135106-t00000060.h5"
    assert driver.filename_cp_restore("out", "cp", "cp-red", "foobar-20140527T135106-t00000060") == \
        "out/cp/cp-red-foobar-20140527T135106-t00000060.h5"
    assert driver.filename_output(".", "density-red", "sim", "20140527T135106", 7) == \
        "./density-red-sim-20140527T135106-t00000007.h5"
    assert re.fullmatch(r"\d{8}T\d{6}", driver.simulation_id())


def test_dump_cadence_and_tokens():
    assert driver.dump_now(5, 10) and not driver.dump_now(5, 11) and not driver.dump_now(0, 0)
    raw = {"lb.force.gcc": [[0.0, 3.6], [3.6, 0.0]], "lb.tau": [1.0, 0.8], "lattice.gn": [16, 8, 4],
           "lb.force.enableShanChen": True}
    s = driver.replace_fname_tokens("sc-%lb.force.gcc[0][1]%-%lb.tau[1]%-%lattice.gn[0]%-%lb.force.enableShanChen%"
                                    "-%unset.key%", raw)
    assert s == "sc-3.6-0.8-16-true-%unset.key%"


def test_parameters_from_h5_input_and_command_line(tmp_path):
    f = str(tmp_path / "prev.h5")
    h5.write_field(f, np.zeros((2, 2, 2)), input_lines=["[lb]", "timesteps = 3", "tau = [1.0]"])
    d, lines = driver.read_input([f], ["lb.timesteps=7"])
    assert d["lb.timesteps"] == 7 and d["lb.tau"] == [1.0]
    assert lines == ["[lb]", "timesteps = 3", "tau = [1.0]", "[]", "lb.timesteps=7"]
    with pytest.raises(Exception):
        driver.read_input([])


def test_h5_writer_roundtrip(tmp_path):
    f = str(tmp_path / "a.h5")
    a = np.random.default_rng(0).random((3, 4, 5, 19))
    h5.write_field(f, a, input_lines=["x = 1"], metadata={"revisionHash": "abc"},
                   globals_={"dlbc.lb.lb.timestep": 42})
    assert np.array_equal(h5.read_field(f), a)
    assert h5.list_links(f) == ["OutArray", "globals", "metadata"]
    assert h5.read_attrs(f)["input"] == ["x = 1"]
    assert h5.read_attrs(f, "metadata")["revisionHash"] == ["abc"]
    assert int(h5.read_attrs(f, "globals")["dlbc.lb.lb.timestep"][0]) == 42
    m = np.zeros((4, 3), np.int32)
    m[1, 2] = 1
    h5.write_field(f, m)
    got = h5.read_field(f)
    assert got.dtype == np.int32 and np.array_equal(got, m)


def test_hook_list():
    calls = []
    hl = driver.HookList("postAdvectionHooks")
    hl.registerFunction(lambda s: calls.append(("a", s)), "a")
    hl.registerFunction(lambda s: calls.append(("b", s)), "b")
    hl.execute(7)
    assert calls == [("a", 7), ("b", 7)] and hl.showAllRegisteredFunctions() == ["a", "b"]


# ---------------------------------------------------------------------------
# the checkpoint-3d case through the driver
# ---------------------------------------------------------------------------

def _stage_checkpoint_case(tmp_path):
    """Lay out the reference test directory: the parameter file, the
    restore files under reference-data/cp, output/ for the run."""
    z, p = load_case("checkpoint-3d")
    cpdir = tmp_path / "reference-data" / "cp"
    cpdir.mkdir(parents=True)
    name = str(z["checkpoint/name"])
    for stem in ("cp-fluids0", "cp-fluids1", "cp-mask"):
        t = int(z[f"checkpoint/{stem}/timestep"][0])
        h5.write_field(str(cpdir / f"{stem}-{name}.h5"), z[f"checkpoint/{stem}"],
                       input_lines=str(z["input"]).splitlines(), globals_={"dlbc.lb.lb.timestep": t})
    inp = tmp_path / "checkpoint-3d.in"
    inp.write_text(str(z["input"]))
    return z, p, str(inp), name


def _check_outputs(z, outdir, sim_id):
    checked = 0
    for t in (0, 5):
        for key, kind in golden_arrays(z, t):
            stem = "colour-red-blue" if kind == "colour" else kind
            f = os.path.join(outdir, f"{stem}-checkpoint-3d-{sim_id}-t{t:08d}.h5")
            assert compare(z, key, h5.read_field(f), 0.0), key
            checked += 1
    assert checked == 10


def _run_checkpoint_case(tmp_path, monkeypatch, lattice_cls):
    z, p, inp, name = _stage_checkpoint_case(tmp_path)
    monkeypatch.chdir(tmp_path)
    sim = driver.Simulation([inp], restore=name, sim_id="20261204T000000", lattice_cls=lattice_cls)
    sim.setup()
    assert sim.timestep == 0
    sim.run()
    sim.close()
    _check_outputs(z, str(tmp_path / "output"), "20261204T000000")
    # checkpoints: t = 5 written, t = 0 rotated out (cpKeep = 1), timestep in /globals
    cp5 = tmp_path / "output" / "cp" / "cp-fluids0-checkpoint-3d-20261204T000000-t00000005.h5"
    cp0 = tmp_path / "output" / "cp" / "cp-fluids0-checkpoint-3d-20261204T000000-t00000000.h5"
    assert cp5.exists() and not cp0.exists()
    assert int(h5.read_attrs(str(cp5), "globals")["dlbc.lb.lb.timestep"][0]) == 5
    assert sha(h5.read_field(str(cp5))) == str(z["t5/population-red/sha256"])
    assert h5.read_attrs(str(cp5))["input"] == str(z["input"]).splitlines()


def test_checkpoint_3d_restore_case_cpu(tmp_path, monkeypatch):
    _run_checkpoint_case(tmp_path, monkeypatch, OracleLattice)


def _restart_case(tmp_path, monkeypatch, lattice_cls, hooks=False):
    """6 steps in one go against 3 + restore + 3: bitwise equal dumps."""
    monkeypatch.chdir(tmp_path)
    inp = tmp_path / "sd.in"
    inp.write_text("\n".join([
        "[lattice]", "gn = [12, 10, 8]",
        "[lb]", "timesteps = 6", "components = 2", 'fieldNames = ["red", "blue"]', "tau = [1.0, 0.9]",
        "eqdist.eqDistForm = BDist2", "force.enableShanChen = true", "force.gcc = [[0.0, 3.6], [3.6, 0.0]]",
        "force.psiForm = Exponential", "force.globalAcc = [1e-5, 0.0, 0.0]",
        "init.fluidInit = [EqDistPerturb, EqDistPerturb]", "init.fluidDensities = [[0.7], [0.7]]",
        "init.fluidPerturb = [0.02, 0.02]", "io.populationFreq = 6", "io.densityFreq = 3",
        "mask.maskInit = Walls", "mask.dimensionHasWall = [[false, false], [false, false], [true, true]]",
        "[io]", "simulationName = sd", "outputPath = out", "checkpoint.cpFreq = 3", "checkpoint.cpPath = cp",
        "checkpoint.cpRestorePath = cp", "checkpoint.cpKeep = 2",
        "[random]", "seed = 3"]))
    a = driver.Simulation([str(inp)], sim_id="A", lattice_cls=lattice_cls)
    if hooks:
        a.postCollisionHooks.registerFunction(lambda s: None, "noop")
    a.setup()
    a.run()
    a.close()
    b = driver.Simulation([str(inp)], cli=["lb.timesteps=3"], sim_id="B", lattice_cls=lattice_cls)
    b.setup()
    b.run()
    b.close()
    c = driver.Simulation([str(inp)], restore="sd-B-t00000003", sim_id="C", lattice_cls=lattice_cls)
    c.setup()
    assert c.timestep == 3
    c.run()
    c.close()
    for comp in ("red", "blue"):
        fa = h5.read_field(f"out/population-{comp}-sd-A-t00000006.h5")
        fc = h5.read_field(f"out/population-{comp}-sd-C-t00000006.h5")
        assert np.array_equal(fa, fc)
        assert np.array_equal(h5.read_field(f"out/density-{comp}-sd-A-t00000003.h5"),
                              h5.read_field(f"out/density-{comp}-sd-B-t00000003.h5"))
    # cpKeep = 2: both checkpoints of run A are kept
    assert os.path.exists("out/cp/cp-mask-sd-A-t00000003.h5") and os.path.exists("out/cp/cp-mask-sd-A-t00000006.h5")
    assert np.array_equal(h5.read_field("out/cp/cp-mask-sd-A-t00000003.h5")[:, :, 0], np.ones((12, 10), np.int32))


def test_restore_continues_exactly_cpu(tmp_path, monkeypatch):
    _restart_case(tmp_path, monkeypatch, OracleLattice)


def hook_paths_case(tmp_path, monkeypatch, lattice_cls):
    """Hooks that change the host fields before advection and after
    collision: the one-call path (lbgpu_step_host, taken when no hook sits
    between advection and collision) and the split path (forced here by a
    no-op post-advection hook) write the same populations."""
    monkeypatch.chdir(tmp_path)
    inp = tmp_path / "hp.in"
    inp.write_text("\n".join([
        "[lattice]", "gn = [24, 10, 8]",
        "[lb]", "timesteps = 4", "components = 2", 'fieldNames = ["red", "blue"]', "tau = [1.0, 0.9]",
        "eqdist.eqDistForm = BDist2", "force.enableShanChen = true", "force.gcc = [[0.0, 3.6], [3.6, 0.0]]",
        "force.psiForm = Exponential", "force.globalAcc = [1e-5, 0.0, 0.0]",
        "init.fluidInit = [EqDistPerturb, EqDistPerturb]", "init.fluidDensities = [[0.7], [0.7]]",
        "init.fluidPerturb = [0.02, 0.02]", "io.populationFreq = 4",
        "mask.maskInit = Walls", "mask.dimensionHasWall = [[false, false], [false, false], [true, true]]",
        "[io]", "simulationName = hp", "outputPath = out",
        "[random]", "seed = 5"]))

    def pre(sim):
        sim.fluids[0][..., 0] *= 1.001

    def post(sim):
        sim.fluids[1][..., 1] *= 0.999

    runs = {}
    for name, split in (("one", False), ("split", True)):
        sim = driver.Simulation([str(inp)], sim_id=name, lattice_cls=lattice_cls)
        sim.preAdvectionHooks.registerFunction(pre, "pre")
        sim.postCollisionHooks.registerFunction(post, "post")
        if split:
            sim.postAdvectionHooks.registerFunction(lambda s: None, "noop")
        sim.setup()
        sim.run()
        sim.close()
        runs[name] = [h5.read_field(f"out/population-{c}-hp-{name}-t00000004.h5") for c in ("red", "blue")]
    for a, b in zip(runs["one"], runs["split"]):
        assert np.array_equal(a, b)


def test_hook_paths_agree_cpu(tmp_path, monkeypatch):
    calls = []

    class Counting(OracleLattice):
        def step_host(self, fluids, mask=None, out=None):
            calls.append(1)
            return super().step_host(fluids, mask, out)

    hook_paths_case(tmp_path, monkeypatch, Counting)
    assert len(calls) == 4  # the one-call run used it every step, the split run never


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

@pytest.mark.gpu
def test_checkpoint_3d_restore_case_gpu(tmp_path, monkeypatch):
    """The reference's restore test on the CUDA lattice (FP64): every dump
    at t = 0 and t = 5 equals the reference's golden files exactly."""
    _run_checkpoint_case(tmp_path, monkeypatch, lbgpu.GPULattice)


@pytest.mark.gpu
@pytest.mark.parametrize("hooks", [False, True])
def test_restore_continues_exactly_gpu(tmp_path, monkeypatch, hooks):
    _restart_case(tmp_path, monkeypatch, lbgpu.GPULattice, hooks=hooks)


@pytest.mark.gpu
@pytest.mark.parametrize("walls", [False, True])
def test_split_phases_equal_full_step(walls):
    """lbgpu_advect + lbgpu_collide == lbgpu_step(1), bit for bit (FP64)."""
    from lbcases import droplet_channel
    p = droplet_channel((14, 10, 12), radius=3.0, acc=1e-4) if walls else spinodal((12, 10, 8), perturb=0.02)
    fl, m = init.init_fields(p)
    a = lbgpu.GPULattice(p)
    b = lbgpu.GPULattice(p)
    a.upload(fl, m if walls else None)
    b.upload(fl, m if walls else None)
    for _ in range(4):
        a.step(1)
        b.advect()
        b.collide()
    ra, rb = a.download(), b.download()
    for c in range(2):
        assert np.array_equal(ra[c], rb[c], equal_nan=True)
    with pytest.raises(lbgpu.LbgpuError):
        b.collide()  # collide without advect
    b.advect()
    with pytest.raises(lbgpu.LbgpuError):
        b.step(1)  # a full step between the phases


@pytest.mark.gpu
def test_post_advection_hook_sees_streamed_populations(tmp_path, monkeypatch):
    """A post-advection hook gets f_q(x - c_q) (periodic), and what it
    changes is what collides."""
    monkeypatch.chdir(tmp_path)
    inp = tmp_path / "h.in"
    inp.write_text("\n".join([
        "[lattice]", "gn = [8, 6, 4]",
        "[lb]", "timesteps = 2", "components = 2", 'fieldNames = ["red", "blue"]', "tau = [1.0, 1.0]",
        "eqdist.eqDistForm = BDist2", "force.enableShanChen = true", "force.gcc = [[0.0, 3.6], [3.6, 0.0]]",
        "force.psiForm = Exponential", "init.fluidInit = [EqDistPerturb, EqDistPerturb]",
        "init.fluidDensities = [[0.7], [0.7]]", "init.fluidPerturb = [0.02, 0.02]",
        "[io]", "enableIO = false"]))
    sim = driver.Simulation([str(inp)], lattice_cls=lbgpu.GPULattice)
    seen = {}

    def pre(s):
        seen["pre"] = [a.copy() for a in s.fluids]

    def post(s):
        seen["post"] = [a.copy() for a in s.fluids]

    sim.preAdvectionHooks.registerFunction(pre, "pre")
    sim.postAdvectionHooks.registerFunction(post, "post")
    sim.setup()
    sim.run()
    sim.close()
    cv = D3Q19_VELOCITIES
    for c in range(2):
        before, after = seen["pre"][c][2:-2, 2:-2, 2:-2], seen["post"][c][2:-2, 2:-2, 2:-2]
        for q in range(19):
            want = np.roll(before[..., q], shift=tuple(cv[q]), axis=(0, 1, 2))
            assert np.array_equal(after[..., q], want), (c, q)


# ---------------------------------------------------------------------------
# a one-dimensional reference input through the driver
# ---------------------------------------------------------------------------

def _run_quasi_1d(tmp_path, monkeypatch, lattice_cls):
    """The reference's laplace-quasi-1d D1Q3 input run by the driver for its
    1000 steps: the density and colour dumps at t = 0 and t = 1000 under the
    reference's names, within the reference's accuracy of its goldens (the
    t = 1000 allowance as in the oracle's golden tests)."""
    z, p = load_case("laplace-quasi-1d-d1q3")
    inp = tmp_path / "laplace-quasi-1d-d1q3.in"
    inp.write_text(str(z["input"]))
    monkeypatch.chdir(tmp_path)
    sim = driver.Simulation([str(inp)], sim_id="20261204T000000", lattice_cls=lattice_cls)
    sim.setup()
    sim.run()
    sim.close()
    checked = 0
    for t in (0, 1000):
        for key, kind in golden_arrays(z, t):
            stem = "colour-red-blue" if kind == "colour" else kind
            f = tmp_path / "output" / "d1q3" / f"{stem}-laplace-d1q3-gcc3.6-20261204T000000-t{t:08d}.h5"
            tol = 0.0 if t == 0 else 2.5e-15
            assert compare(z, key, h5.read_field(str(f)), tol), key
            checked += 1
    assert checked == 6


def test_quasi_1d_d1q3_case_cpu(tmp_path, monkeypatch):
    _run_quasi_1d(tmp_path, monkeypatch, OracleLattice)


@pytest.mark.gpu
def test_quasi_1d_d1q3_case_gpu(tmp_path, monkeypatch):
    _run_quasi_1d(tmp_path, monkeypatch, lbgpu.GPULattice)
