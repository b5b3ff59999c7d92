"""Run driver in the reference's shape: command line, parameter files, the
time loop with its hook points, data dumps and checkpoints, on the GPU
lattice of :mod:`dlbc_gb300.lbgpu`.

It mirrors, one for one:

* ``processCLI`` (src/dlbc/getopt.d:67-124): ``-p``/``--parameterfile``
  (repeatable; a ``.h5`` file contributes its ``input`` attribute, as
  ``readParameterSetFromHdf5File`` does, src/dlbc/parameters.d:339-350),
  ``--parameter "key=value"`` (repeatable, fully qualified), ``-r``/
  ``--restore <name>``, ``--show-input``;
* ``main`` (src/main.d:91-163): initial fields (or a restored checkpoint),
  the first dump at the start timestep, then ``runTimeloop``
  (src/main.d:174-200);
* the hook lists of src/dlbc/hooks.d:57-118 (pre/post advection, pre/post
  collision, pre/post LB init) and the plugin register (hooks.d:21-45);
* ``dumpData`` (src/dlbc/io/io.d:198-213) and ``dumpLBData``
  (src/dlbc/lb/io.d:56-101) with the reference's file names
  (``makeFilenameOutput`` io.d:160-172, ``makeFilenameCpOutput`` /
  ``makeFilenameCpRestore`` src/dlbc/io/checkpoint.d:183-240) and HDF5
  layout (src/dlbc/io/hdf5.d:125-299, through :mod:`dlbc_gb300.h5`);
* checkpoints (checkpoint.d:80-160, 248-313): ``cp-fluids<i>`` and
  ``cp-mask`` files with the ``globals`` group holding
  ``dlbc.lb.lb.timestep``, rotation by ``cpFreq``/``cpKeep``.

The lattice lives on the GPU.  With no hook registered, the driver steps
``lbgpu_step(k)`` between dump times; the host mirror (``fluids``, ``mask``:
haloed arrays in the reference's layout) is refreshed only at dumps and
checkpoints.  A registered hook sees the host mirror, synchronised before it
runs and uploaded after it (the hook may change it); hooks between advection
and collision run between ``lbgpu_advect`` and ``lbgpu_collide``.  The
reference's own stale-marking hooks (``markDensitiesAsStale``,
src/dlbc/lb/density.d:338; ``markPsiAsStale``, src/dlbc/lb/force.d:131)
have nothing to mark here and are not registered.

Plugins are Python callables registered with :data:`pluginRegister`; each is
called with the :class:`Simulation` after the parameters are read and
registers its hooks on it (the reference's plugin init functions take no
argument and register into module-level hook lists).
"""
from __future__ import annotations

import argparse
import datetime
import os
import re
import sys
from typing import Any, Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import h5, init, lbgpu, params

HookFn = Callable[["Simulation"], None]


class HookList:
    """``TVoidHooks`` (src/dlbc/hooks.d:57-118): named functions run in
    registration order."""

    def __init__(self, name: str):
        self.name = name
        self.functions: List[Tuple[HookFn, str]] = []

    def registerFunction(self, fn: HookFn, fname: str) -> None:  # noqa: N802 (reference name)
        self.functions.append((fn, fname))

    def execute(self, sim: "Simulation") -> None:
        for fn, _ in self.functions:
            fn(sim)

    def showAllRegisteredFunctions(self) -> List[str]:  # noqa: N802
        return [n for _, n in self.functions]

    def __len__(self) -> int:
        return len(self.functions)


class PluginRegister:
    """``pluginRegister`` (src/dlbc/hooks.d:21-45)."""

    def __init__(self):
        self.plugins: List[Callable[["Simulation"], None]] = []

    def registerPlugin(self, fn: Callable[["Simulation"], None]) -> None:  # noqa: N802
        self.plugins.append(fn)

    def execute(self, sim: "Simulation") -> None:
        for fn in self.plugins:
            fn(sim)


pluginRegister = PluginRegister()


# ---------------------------------------------------------------------------
# names and cadence
# ---------------------------------------------------------------------------

def dump_now(freq: int, t: int) -> bool:
    """``dumpNow`` (src/dlbc/io/io.d:224-226)."""
    return freq > 0 and t % freq == 0


def simulation_id(now: Optional[datetime.datetime] = None) -> str:
    """``initSimulationId`` (src/dlbc/io/io.d:86-92): the first 15 characters
    of the ISO basic timestamp, ``YYYYMMDDTHHMMSS``."""
    now = now or datetime.datetime.now()
    return now.strftime("%Y%m%dT%H%M%S")


def _d_to_string(v: Any) -> str:
    """``std.conv.to!string`` of a parameter value, as used for file name
    tokens: bools lower case, floats with six significant digits."""
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, float):
        return f"{v:g}"
    if isinstance(v, list):
        return "[" + ", ".join(_d_to_string(x) for x in v) + "]"
    return str(v)


def replace_fname_tokens(name: str, raw: Dict[str, Any]) -> str:
    """``replaceFnameTokens`` (src/dlbc/parameters.d:507-527): ``%key%``,
    ``%key[i]%`` and ``%key[i][j]%`` become the parameter's value.  Tokens
    naming a parameter that was not set are left as they are."""

    def sub(m: "re.Match[str]") -> str:
        key, idx = m.group(1), m.group(2)
        if key not in raw:
            return m.group(0)
        v = raw[key]
        for i in re.findall(r"\[([0-9]+)\]", idx or ""):
            v = v[int(i)]
        return _d_to_string(v)

    return re.sub(r"%([A-Za-z0-9_.]+)((?:\[[0-9]+\]){0,2})%", sub, name)


def filename_output(output_path: str, name: str, sim_name: str, sim_id: str, t: int) -> str:
    """``makeFilenameOutput`` (src/dlbc/io/io.d:160-172)."""
    return f"{output_path}/{name}-{sim_name}-{sim_id}-t{t:08d}.h5"


def filename_cp_output(output_path: str, cp_path: str, name: str, sim_name: str, sim_id: str, t: int) -> str:
    """``makeFilenameCpOutput`` (src/dlbc/io/checkpoint.d:183-201)."""
    return f"{output_path}/{cp_path}/{name}-{sim_name}-{sim_id}-t{t:08d}.h5"


def filename_cp_restore(output_path: str, cp_restore_path: str, name: str, restore: str) -> str:
    """``makeFilenameCpRestore`` (src/dlbc/io/checkpoint.d:212-240).  Like the
    reference, the file is looked up under ``cpRestorePath`` even when that
    is empty (the reference computes a fallback to ``cpPath`` but does not
    use it)."""
    return f"{output_path}/{cp_restore_path}/{name}-{restore}.h5"


# ---------------------------------------------------------------------------
# parameters
# ---------------------------------------------------------------------------

def read_input(files: Sequence[str], cli: Sequence[str] = ()) -> Tuple[Dict[str, Any], List[str]]:
    """Parameter files in order (text, or ``.h5`` with an ``input``
    attribute), then the command-line overrides after a ``[]`` line
    (src/dlbc/parameters.d:166-196).  Returns the parsed values and the
    input lines the reference stores in every output file's ``input``
    attribute."""
    if not files:
        raise params.ParameterError("Parameter filename not set, please specify using the -p <filename> option.")
    d: Dict[str, Any] = {}
    lines_all: List[str] = []
    for f in files:
        if f.endswith(".h5"):
            lines = list(h5.read_attrs(f)["input"])
        else:
            with open(f) as fh:
                lines = fh.read().splitlines()
        lines_all += lines
        params.parse_lines(lines, d)
    if cli:
        lines_all.append("[]")
        lines_all += list(cli)
        params.parse_lines(list(cli), d, section="")
    return d, lines_all


def _connectivity(d: Dict[str, Any], dq: Optional[str]) -> str:
    if dq:
        return dq
    # one extent: D1Q3, the reference's tested 1D build (D1Q5 on request)
    return {1: "d1q3", 2: "d2q9"}.get(len(d.get("lattice.gn", [])), "d3q19")


# ---------------------------------------------------------------------------
# the simulation
# ---------------------------------------------------------------------------

class Simulation:
    """One run: parameters, GPU lattice, host mirror, hooks, output."""

    def __init__(self, files: Sequence[str], cli: Sequence[str] = (), restore: str = "",
                 precision: int = lbgpu.FP64, device: int = 0, dq: Optional[str] = None,
                 device_init: bool = False, sim_id: Optional[str] = None, log: Callable[[str], None] = None,
                 lattice_cls: Callable = lbgpu.GPULattice):
        self.raw, self.input_lines = read_input(files, cli)
        self.dq = _connectivity(self.raw, dq)
        self.p = params.LBParams.from_dict(self.raw, self.dq)
        self.log = log or (lambda msg: None)
        if bool(self.raw.get("elec.enableElec", False)):
            raise params.ParameterError("elec.enableElec: the electrokinetic solver is not part of the GPU path")
        if int(self.raw.get("lb.laplaceFreq", 0)) > 0:
            self.log("lb.laplaceFreq is set: Laplace analysis output is not written")
        p = self.p
        self.restore = restore
        self.precision = precision
        self.device_init = device_init
        self.sim_name = replace_fname_tokens(p.simulation_name, self.raw)
        self.output_path = replace_fname_tokens(p.output_path, self.raw)
        self.sim_id = sim_id if sim_id is not None else simulation_id()
        self.cp_path = p.cp_path
        self.cp_restore_path = str(self.raw.get("io.checkpoint.cpRestorePath", ""))
        self.create_path = bool(self.raw.get("io.createPath", True))
        self.timestep = 0
        self.preAdvectionHooks = HookList("preAdvectionHooks")
        self.postAdvectionHooks = HookList("postAdvectionHooks")
        self.preCollisionHooks = HookList("preCollisionHooks")
        self.postCollisionHooks = HookList("postCollisionHooks")
        self.preLbInitHooks = HookList("preLbInitHooks")
        self.postLbInitHooks = HookList("postLbInitHooks")
        self.fluids: List[np.ndarray] = []
        self.mask: Optional[np.ndarray] = None
        # lattice_cls(p, precision=, device=) holds the fields; the default
        # is the CUDA lattice (the tests substitute a CPU stand-in only to
        # check this module's file handling without a GPU)
        self.lattice = lattice_cls(p, precision=precision, device=device)
        self.written: List[str] = []
        self._host_valid = False
        pluginRegister.execute(self)

    # -- host mirror -------------------------------------------------------------
    def _walls(self) -> bool:
        return self.mask is not None and bool(np.any(self.mask))

    def sync_to_host(self) -> None:
        """Refresh ``fluids`` (halo included, periodic images) from the device."""
        if not self._host_valid:
            self.lattice.download(self.fluids)
            self._host_valid = True

    def sync_to_device(self) -> None:
        self.lattice.upload(self.fluids, self.mask if self._walls() else None)

    def _run_hooks(self, hooks: Sequence[HookList]) -> None:
        if not any(len(h) for h in hooks):
            return
        self.sync_to_host()
        for h in hooks:
            h.execute(self)
        self.sync_to_device()

    # -- setup -------------------------------------------------------------------
    def setup(self) -> None:
        """``main`` up to the first dump (src/main.d:131-148)."""
        p = self.p
        if self.enable_io() and self.create_path:
            for path in (self.output_path, f"{self.output_path}/{self.cp_path}"):
                os.makedirs(path, exist_ok=True)
        shape = tuple(n + 4 for n in p.gn[: p.d])
        self.fluids = [np.empty(shape + (p.q,), np.float64) for _ in range(p.components)]
        if self.restore:
            self.read_checkpoint()
            self.sync_to_device()
            self._host_valid = True
        else:
            self.preLbInitHooks.execute(self)
            if self.device_init:
                self.lattice.init_device()
                self.mask = None
                self._host_valid = False
                self.sync_to_host()
                self.mask = self._device_mask(shape)
            else:
                self.fluids, self.mask = init.init_fields(p)
                self.sync_to_device()
                self._host_valid = True
            if len(self.postLbInitHooks):
                self.sync_to_host()
                self.postLbInitHooks.execute(self)
                self.sync_to_device()
        if int(p.freqs.get("force", 0)) > 0:
            self.lattice.set_record_force(True)
        self.dump_data(self.timestep)

    def _device_mask(self, shape) -> np.ndarray:
        # the mask initialisers are deterministic: the host restatement gives
        # the same mask the device computed
        _, m = init.init_fields(self._mask_only_params())
        assert m.shape == shape
        return m

    def _mask_only_params(self) -> params.LBParams:
        import copy
        q = copy.deepcopy(self.p)
        q.fluid_init = [0] * q.components
        return q

    # -- the time loop -------------------------------------------------------------
    def _hooked(self) -> bool:
        return any(len(h) for h in (self.preAdvectionHooks, self.postAdvectionHooks,
                                    self.preCollisionHooks, self.postCollisionHooks))

    def _next_stop(self) -> int:
        """The next timestep after which something is written."""
        p = self.p
        t_end = p.timesteps
        stop = t_end
        if self.enable_io():
            for f in list(p.freqs.values()) + [p.cp_freq]:
                if f > 0:
                    stop = min(stop, (self.timestep // f + 1) * f)
        return max(stop, self.timestep + 1)

    def step_once(self) -> None:
        """One iteration of ``runTimeloop``'s body (src/main.d:175-199) with
        the hook points of advectFields / collideFields."""
        mid = len(self.postAdvectionHooks) or len(self.preCollisionHooks)
        if not mid and len(self.postCollisionHooks):
            # the host fields go through the timestep in one call
            # (lbgpu_step_host: upload, step and download overlapped) and
            # come back for the post-collision hooks
            self.sync_to_host()
            self.preAdvectionHooks.execute(self)
            self.lattice.step_host(self.fluids, self.mask if self._walls() else None, self.fluids)
            self.postCollisionHooks.execute(self)
            self.sync_to_device()
            self._host_valid = True  # the device holds what the hooks left
            return
        self._host_valid = False
        self._run_hooks([self.preAdvectionHooks])
        if len(self.postAdvectionHooks) or len(self.preCollisionHooks):
            self.lattice.advect()
            self._host_valid = False
            self._run_hooks([self.postAdvectionHooks, self.preCollisionHooks])
            self.lattice.collide()
        else:
            self.lattice.step(1)
        self._host_valid = False
        self._run_hooks([self.postCollisionHooks])
        self._host_valid = False

    def run(self) -> None:
        """``runTimeloop`` (src/main.d:174-200)."""
        p = self.p
        while self.timestep < p.timesteps:
            if self._hooked():
                self.timestep += 1
                self.step_once()
            else:
                k = min(self._next_stop(), p.timesteps) - self.timestep
                self.lattice.step(k)
                self._host_valid = False
                self.timestep += k
            self.dump_data(self.timestep)
        self.lattice.synchronize()

    # -- output ------------------------------------------------------------------
    def enable_io(self) -> bool:
        return bool(self.p.enable_io)

    def _write(self, path: str, arr: np.ndarray, checkpoint_t: Optional[int] = None) -> None:
        meta = {"revisionHash": "dlbc_gb300", "revisionDesc": "dlbc_gb300", "revisionBranch": "",
                "revisionChanged": 0, "revisionChanges": ""}
        glob = {"dlbc.lb.lb.timestep": int(checkpoint_t)} if checkpoint_t is not None else None
        h5.write_field(path, arr, input_lines=self.input_lines, metadata=meta, globals_=glob)
        self.written.append(path)
        self.log(f"  HDF writing to file '{path}'.")

    def _physical(self, a: np.ndarray) -> np.ndarray:
        sl = tuple(slice(2, 2 + n) for n in self.p.gn[: self.p.d])
        return np.ascontiguousarray(a[sl])

    def dump_data(self, t: int) -> None:
        """``dumpData`` (src/dlbc/io/io.d:198-213)."""
        p = self.p
        if not self.enable_io() or t < p.start_output:
            return
        if dump_now(p.cp_freq, t):
            self.dump_checkpoint(t)
            self.remove_checkpoint(t - p.cp_freq * p.cp_keep)
        self.dump_lb_data(t)

    def dump_lb_data(self, t: int) -> None:
        """``dumpLBData`` (src/dlbc/lb/io.d:56-101)."""
        p, L = self.p, self.lattice
        out = self.output_path
        names = p.field_names
        fr = p.freqs
        if dump_now(fr.get("population", 0), t):
            self.sync_to_host()
            for i, a in enumerate(self.fluids):
                self._write(filename_output(out, "population-" + names[i], self.sim_name, self.sim_id, t),
                            self._physical(a))
        if dump_now(fr.get("density", 0), t):
            for i, a in enumerate(L.density()):
                self._write(filename_output(out, "density-" + names[i], self.sim_name, self.sim_id, t), a)
        if dump_now(fr.get("colour", 0), t) and p.components == 2:
            self._write(filename_output(out, f"colour-{names[0]}-{names[1]}", self.sim_name, self.sim_id, t),
                        L.colour())
        if dump_now(fr.get("velocity", 0), t):
            for i, a in enumerate(L.velocity()):
                self._write(filename_output(out, "velocity-" + names[i], self.sim_name, self.sim_id, t), a)
        if dump_now(fr.get("force", 0), t) and t > 0:
            for i, a in enumerate(L.force()):
                self._write(filename_output(out, "force-" + names[i], self.sim_name, self.sim_id, t), a)
        if dump_now(fr.get("mask", 0), t):
            m = self.mask if self.mask is not None else np.zeros(tuple(n + 4 for n in p.gn[: p.d]), np.int32)
            self._write(filename_output(out, "mask", self.sim_name, self.sim_id, t), self._physical(m))

    # -- checkpoints ---------------------------------------------------------------
    def _cp_names(self) -> List[str]:
        return [f"cp-fluids{i}" for i in range(self.p.components)] + ["cp-mask"]

    def dump_checkpoint(self, t: int) -> None:
        """``dumpCheckpoint`` (src/dlbc/io/checkpoint.d:116-121)."""
        self.sync_to_host()
        p = self.p
        m = self.mask if self.mask is not None else np.zeros(tuple(n + 4 for n in p.gn[: p.d]), np.int32)
        arrays = [self._physical(a) for a in self.fluids] + [self._physical(m)]
        for name, a in zip(self._cp_names(), arrays):
            self._write(filename_cp_output(self.output_path, self.cp_path, name, self.sim_name, self.sim_id, t),
                        a, checkpoint_t=t)

    def remove_checkpoint(self, t: int) -> None:
        """``removeCheckpoint`` (src/dlbc/io/checkpoint.d:150-157)."""
        if t < 0:
            return
        for name in self._cp_names():
            f = filename_cp_output(self.output_path, self.cp_path, name, self.sim_name, self.sim_id, t)
            if os.path.exists(f):
                os.remove(f)

    def read_checkpoint(self) -> None:
        """``readCheckpoint`` (src/dlbc/io/checkpoint.d:132-141): populations
        and mask from ``cp-*-<restore>.h5``, the timestep from the files'
        ``globals`` group; halos are periodic images (``exchangeHalo``)."""
        p = self.p
        gn = tuple(p.gn[: p.d])
        for i in range(p.components):
            f = filename_cp_restore(self.output_path, self.cp_restore_path, f"cp-fluids{i}", self.restore)
            a = h5.read_field(f)
            if a.shape != gn + (p.q,):
                raise params.ParameterError(f"{f}: shape {a.shape}, expected {gn + (p.q,)}")
            self.fluids[i] = init.periodic_fill(_haloed(a, p.d), p.d)
            self.timestep = int(np.asarray(h5.read_attrs(f, "globals")["dlbc.lb.lb.timestep"]).ravel()[0])
        f = filename_cp_restore(self.output_path, self.cp_restore_path, "cp-mask", self.restore)
        m = h5.read_field(f).astype(np.int32)
        if m.shape != gn:
            raise params.ParameterError(f"{f}: shape {m.shape}, expected {gn}")
        self.mask = init.periodic_fill(_haloed(m, p.d), p.d)

    def close(self) -> None:
        self.lattice.close()


def _haloed(a: np.ndarray, d: int) -> np.ndarray:
    pad = [(2, 2)] * d + [(0, 0)] * (a.ndim - d)
    return np.ascontiguousarray(np.pad(a, pad))


# ---------------------------------------------------------------------------
# command line
# ---------------------------------------------------------------------------

def main(argv: Optional[Sequence[str]] = None) -> int:
    ap = argparse.ArgumentParser(prog="dlbc_gb300.driver",
                                 description="Lattice-Boltzmann run on the GPU with the reference's "
                                             "parameter files, dumps and checkpoints.")
    ap.add_argument("-p", "--parameterfile", action="append", default=[], help="parameter file (repeatable)")
    ap.add_argument("--parameter", action="append", default=[], help='override "key=value" (repeatable)')
    ap.add_argument("-r", "--restore", default="", help="restore from checkpoint <name>-<id>-t<time>")
    ap.add_argument("--show-input", action="store_true", help="print the parameter input and exit")
    ap.add_argument("--precision", choices=sorted(lbgpu.PRECISIONS), default="fp64")
    ap.add_argument("--connectivity", choices=["d3q19", "d2q9", "d1q3", "d1q5"], default=None)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--device-init", action="store_true",
                    help="compute initial fields on the device (random initialisers then use a "
                         "counter-based generator instead of the reference's Mt19937 stream)")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    if a.show_input:
        _, lines = read_input(a.parameterfile, a.parameter)
        print("\n".join(lines))
        return 0
    log = (lambda m: print(m, file=sys.stderr)) if a.verbose else None
    sim = Simulation(a.parameterfile, a.parameter, restore=a.restore, precision=lbgpu.PRECISIONS[a.precision],
                     device=a.device, dq=a.connectivity, device_init=a.device_init, log=log)
    try:
        sim.setup()
        sim.run()
    finally:
        sim.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
