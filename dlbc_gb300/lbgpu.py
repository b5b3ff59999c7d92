"""ctypes binding of the C ABI in include/lbgpu.h (``liblbgpu.so``).

This is how the Python host side (tests, bench, the reference-style driver
in :mod:`dlbc_gb300.driver`) reaches the CUDA kernels: exactly the calls a
D program would make through ``extern(C)``.  The library is loaded from the
package's ``_build`` directory; if it is missing the import fails loudly
(there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblbgpu.so")

FP64, FP32, FP16, I16 = 0, 1, 2, 3
PRECISIONS = {"fp64": FP64, "fp32": FP32, "fp16": FP16, "i16": I16}
MAXC = 2

ERRORS = {0: "OK", -1: "LBGPU_E_INVALID", -2: "LBGPU_E_NOMEM", -3: "LBGPU_E_CUDA", -4: "LBGPU_E_BUDGET",
          -5: "LBGPU_E_NOTREADY", -6: "LBGPU_E_NONFINITE"}

EXPORTED = ["lbgpu_abi_version", "lbgpu_create", "lbgpu_destroy", "lbgpu_upload", "lbgpu_step",
            "lbgpu_advect", "lbgpu_collide",
            "lbgpu_download", "lbgpu_step_host", "lbgpu_moments", "lbgpu_set_record_force", "lbgpu_force", "lbgpu_reduce",
            "lbgpu_synchronize", "lbgpu_set_stream", "lbgpu_profile", "lbgpu_kernel_time",
            "lbgpu_launch_count", "lbgpu_device_bytes", "lbgpu_last_error", "lbgpu_set_storage_scale"]


class LbgpuConfig(C.Structure):
    _fields_ = [
        ("d", C.c_int32), ("q", C.c_int32), ("gn", C.c_int32 * 3), ("components", C.c_int32),
        ("shan_chen", C.c_int32), ("psi_form", C.c_int32), ("eq_form", C.c_int32),
        ("precision", C.c_int32), ("device", C.c_int32),
        ("tau", C.c_double * MAXC), ("gcc", (C.c_double * MAXC) * MAXC), ("gwc", C.c_double * MAXC),
        ("global_acc", C.c_double * 3), ("rho0", C.c_double * MAXC),
    ]


class LbgpuError(RuntimeError):
    pass


_lib: Optional[C.CDLL] = None


def lib() -> C.CDLL:
    """Load liblbgpu.so (built by dlbc_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise LbgpuError(f"{LIB_PATH} is missing: run `python -m dlbc_gb300.build` (needs nvcc)")
        L = C.CDLL(LIB_PATH)
        H = C.c_void_p
        PP = C.POINTER(C.c_void_p)
        L.lbgpu_abi_version.restype = C.c_int32
        L.lbgpu_create.argtypes = [C.POINTER(LbgpuConfig), C.POINTER(H)]
        L.lbgpu_destroy.argtypes = [H]
        L.lbgpu_destroy.restype = None
        L.lbgpu_upload.argtypes = [H, PP, C.c_void_p]
        L.lbgpu_step.argtypes = [H, C.c_int32]
        L.lbgpu_advect.argtypes = [H]
        L.lbgpu_collide.argtypes = [H]
        L.lbgpu_download.argtypes = [H, PP]
        L.lbgpu_step_host.argtypes = [H, PP, C.c_void_p, PP]
        L.lbgpu_moments.argtypes = [H, PP, PP, C.c_void_p]
        L.lbgpu_set_record_force.argtypes = [H, C.c_int32]
        L.lbgpu_force.argtypes = [H, PP]
        L.lbgpu_reduce.argtypes = [H, C.c_void_p, C.c_void_p]
        L.lbgpu_synchronize.argtypes = [H]
        L.lbgpu_set_stream.argtypes = [H, C.c_void_p]
        L.lbgpu_profile.argtypes = [H, C.c_int32]
        L.lbgpu_kernel_time.argtypes = [H, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
        L.lbgpu_set_storage_scale.argtypes = [H, C.c_void_p, C.c_void_p]
        L.lbgpu_launch_count.argtypes = [H]
        L.lbgpu_launch_count.restype = C.c_int64
        L.lbgpu_device_bytes.argtypes = [H]
        L.lbgpu_device_bytes.restype = C.c_int64
        L.lbgpu_last_error.argtypes = [H]
        L.lbgpu_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def make_config(p, precision: int = FP64, device: int = 0, rho0: Sequence[float] = (0.0, 0.0)) -> LbgpuConfig:
    """C config from :class:`dlbc_gb300.params.LBParams`."""
    c = LbgpuConfig()
    c.d, c.q = p.d, p.q
    for i in range(p.d):
        c.gn[i] = int(p.gn[i])
    c.components = p.components
    c.shan_chen = int(p.shan_chen)
    c.psi_form = int(p.psi_form)
    c.eq_form = int(p.eq_form)
    c.precision = int(precision)
    c.device = int(device)
    for f in range(p.components):
        c.tau[f] = p.tau[f] if p.tau else 1.0
        c.gwc[f] = p.gwc[f]
        c.rho0[f] = rho0[f] if f < len(rho0) else 0.0
        for g in range(p.components):
            c.gcc[f][g] = p.gcc[f][g]
    for i in range(p.d):
        c.global_acc[i] = p.global_acc[i]
    return c


def _ptrs(arrays: Sequence[Optional[np.ndarray]], n: int):
    arr = (C.c_void_p * n)()
    for i in range(n):
        a = arrays[i] if i < len(arrays) else None
        arr[i] = None if a is None else a.ctypes.data
    return arr


def _ptr_of(a) -> int:
    """Address of a numpy array or a (host) torch tensor."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


class GPULattice:
    """One device-resident lattice behind the C ABI."""

    def __init__(self, p, precision: int = FP64, device: int = 0, rho0: Sequence[float] = (0.0, 0.0)):
        self.p = p
        self.precision = precision
        self.cfg = make_config(p, precision, device, rho0)
        self.h = C.c_void_p()
        rc = lib().lbgpu_create(C.byref(self.cfg), C.byref(self.h))
        if rc != 0:
            raise LbgpuError(f"lbgpu_create: {ERRORS.get(rc, rc)}: {lib().lbgpu_last_error(None).decode()}")
        self.n = tuple(int(x) for x in p.gn[: p.d])
        self.nH = tuple(x + 4 for x in self.n)

    def _check(self, rc: int, what: str):
        if rc != 0:
            raise LbgpuError(f"{what}: {ERRORS.get(rc, rc)}: {lib().lbgpu_last_error(self.h).decode()}")

    def close(self):
        if self.h:
            lib().lbgpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- reference-layout transfers -----------------------------------------
    def upload(self, fluids: List, mask=None) -> None:
        """fluids[c]: haloed AoS float64 arrays (nH..., q); mask: haloed int32 or None.
        Accepts numpy arrays or pinned host torch tensors."""
        ptrs = (C.c_void_p * MAXC)()
        for i, a in enumerate(fluids):
            if isinstance(a, np.ndarray):
                assert a.dtype == np.float64 and a.flags.c_contiguous and a.shape == self.nH + (self.p.q,)
            ptrs[i] = _ptr_of(a)
        m = None
        if mask is not None:
            if isinstance(mask, np.ndarray):
                assert mask.dtype == np.int32 and mask.flags.c_contiguous and mask.shape == self.nH
            m = _ptr_of(mask)
        self._check(lib().lbgpu_upload(self.h, ptrs, m), "lbgpu_upload")

    def download(self, out: Optional[List] = None) -> List:
        if out is None:
            out = [np.empty(self.nH + (self.p.q,), np.float64) for _ in range(self.p.components)]
        ptrs = (C.c_void_p * MAXC)()
        for i, a in enumerate(out):
            ptrs[i] = _ptr_of(a)
        self._check(lib().lbgpu_download(self.h, ptrs), "lbgpu_download")
        return out

    def set_storage_scale(self, rho0: Optional[Sequence[float]], scale: Optional[Sequence[float]]) -> None:
        """FP16 / I16: pin the stored offsets' rest density and scale (None
        unpins); before the first upload."""
        if rho0 is None or scale is None:
            self._check(lib().lbgpu_set_storage_scale(self.h, None, None), "lbgpu_set_storage_scale")
            return
        r = np.ascontiguousarray(rho0, dtype=np.float64)
        s = np.ascontiguousarray(scale, dtype=np.float64)
        self._check(lib().lbgpu_set_storage_scale(self.h, r.ctypes.data, s.ctypes.data), "lbgpu_set_storage_scale")

    def step(self, n: int = 1) -> None:
        self._check(lib().lbgpu_step(self.h, int(n)), "lbgpu_step")

    def step_host(self, fluids: List, mask=None, out: Optional[List] = None) -> List:
        """One timestep from host fields to host fields (``lbgpu_step_host``):
        the same as upload(fluids, mask), step(1), download(out).  ``out``
        may be ``fluids`` itself."""
        if out is None:
            out = [np.empty(self.nH + (self.p.q,), np.float64) for _ in range(self.p.components)]
        pin = (C.c_void_p * MAXC)()
        for i, a in enumerate(fluids):
            if isinstance(a, np.ndarray):
                assert a.dtype == np.float64 and a.flags.c_contiguous and a.shape == self.nH + (self.p.q,)
            pin[i] = _ptr_of(a)
        pout = (C.c_void_p * MAXC)()
        for i, a in enumerate(out):
            if isinstance(a, np.ndarray):
                assert a.dtype == np.float64 and a.flags.c_contiguous and a.shape == self.nH + (self.p.q,)
            pout[i] = _ptr_of(a)
        m = None
        if mask is not None:
            if isinstance(mask, np.ndarray):
                assert mask.dtype == np.int32 and mask.flags.c_contiguous and mask.shape == self.nH
            m = _ptr_of(mask)
        self._check(lib().lbgpu_step_host(self.h, pin, m, pout), "lbgpu_step_host")
        return out

    def advect(self) -> None:
        """First phase of a timestep (streaming); :meth:`collide` completes it."""
        self._check(lib().lbgpu_advect(self.h), "lbgpu_advect")

    def collide(self) -> None:
        """Second phase: densities, psi, forces and collision of the advected state."""
        self._check(lib().lbgpu_collide(self.h), "lbgpu_collide")

    def synchronize(self) -> None:
        self._check(lib().lbgpu_synchronize(self.h), "lbgpu_synchronize")

    def set_stream(self, stream_handle: Optional[int]) -> None:
        """Queue work on a caller-owned cudaStream_t (an integer handle, e.g.
        ``torch.cuda.Stream().cuda_stream``); None restores the own stream."""
        self._check(lib().lbgpu_set_stream(self.h, stream_handle), "lbgpu_set_stream")

    def profile(self, on: bool = True) -> None:
        self._check(lib().lbgpu_profile(self.h, int(on)), "lbgpu_profile")

    def kernel_time(self, which: int):
        """(total ms, launches) of kernel 0 (density/psi) or 1 (collide)."""
        ms = C.c_double()
        n = C.c_int64()
        self._check(lib().lbgpu_kernel_time(self.h, which, C.byref(ms), C.byref(n)), "lbgpu_kernel_time")
        return ms.value, n.value

    def set_record_force(self, on: bool = True) -> None:
        self._check(lib().lbgpu_set_record_force(self.h, int(on)), "lbgpu_set_record_force")

    # -- outputs -----------------------------------------------------------------
    def density(self) -> List[np.ndarray]:
        out = [np.empty(self.n, np.float64) for _ in range(self.p.components)]
        self._check(lib().lbgpu_moments(self.h, _ptrs(out, MAXC), None, None), "lbgpu_moments")
        return out

    def velocity(self) -> List[np.ndarray]:
        out = [np.empty(self.n + (self.p.d,), np.float64) for _ in range(self.p.components)]
        self._check(lib().lbgpu_moments(self.h, None, _ptrs(out, MAXC), None), "lbgpu_moments")
        return out

    def colour(self) -> np.ndarray:
        out = np.empty(self.n, np.float64)
        self._check(lib().lbgpu_moments(self.h, None, None, out.ctypes.data), "lbgpu_moments")
        return out

    def force(self) -> List[np.ndarray]:
        out = [np.empty(self.n + (self.p.d,), np.float64) for _ in range(self.p.components)]
        self._check(lib().lbgpu_force(self.h, _ptrs(out, MAXC)), "lbgpu_force")
        return out

    def population(self) -> List[np.ndarray]:
        """Physical-site populations [x][y][z][q] (like the population dumps)."""
        full = self.download()
        sl = tuple(slice(2, 2 + n) for n in self.n)
        return [np.ascontiguousarray(a[sl]) for a in full]

    def reduce(self):
        C_ = self.p.components
        mass = np.zeros(C_, np.float64)
        mom = np.zeros(C_ * self.p.d, np.float64)
        self._check(lib().lbgpu_reduce(self.h, mass.ctypes.data, mom.ctypes.data), "lbgpu_reduce")
        return mass, mom.reshape(C_, self.p.d)

    @property
    def launch_count(self) -> int:
        return int(lib().lbgpu_launch_count(self.h))

    @property
    def device_bytes(self) -> int:
        return int(lib().lbgpu_device_bytes(self.h))


# ---------------------------------------------------------------------------
# batches (lbgpu_batch_* in include/lbgpu.h)
# ---------------------------------------------------------------------------
EXPORTED += ["lbgpu_batch_create", "lbgpu_batch_destroy", "lbgpu_batch_add", "lbgpu_batch_remove",
             "lbgpu_batch_step", "lbgpu_batch_member", "lbgpu_batch_set_stream", "lbgpu_batch_synchronize",
             "lbgpu_batch_device_bytes", "lbgpu_batch_launch_count", "lbgpu_batch_set_tuning",
             "lbgpu_batch_launch_shape", "lbgpu_batch_last_error", "lbgpu_step_noalloc"]

_batch_ready = False


def _batch_lib() -> C.CDLL:
    global _batch_ready
    L = lib()
    if not _batch_ready:
        H = C.c_void_p
        L.lbgpu_batch_create.argtypes = [C.c_int32, C.c_int32, C.c_int64, C.POINTER(H)]
        L.lbgpu_batch_destroy.argtypes = [H]
        L.lbgpu_batch_destroy.restype = None
        L.lbgpu_batch_add.argtypes = [H, C.POINTER(LbgpuConfig), C.POINTER(C.c_void_p), C.c_void_p,
                                      C.POINTER(C.c_int32)]
        L.lbgpu_batch_remove.argtypes = [H, C.c_int32]
        L.lbgpu_batch_step.argtypes = [H, C.c_int32]
        L.lbgpu_batch_member.argtypes = [H, C.c_int32]
        L.lbgpu_batch_member.restype = H
        L.lbgpu_batch_set_stream.argtypes = [H, C.c_void_p]
        L.lbgpu_batch_synchronize.argtypes = [H]
        L.lbgpu_batch_device_bytes.argtypes = [H]
        L.lbgpu_batch_device_bytes.restype = C.c_int64
        L.lbgpu_batch_launch_count.argtypes = [H]
        L.lbgpu_batch_launch_count.restype = C.c_int64
        L.lbgpu_batch_set_tuning.argtypes = [H, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
        L.lbgpu_batch_launch_shape.argtypes = [H, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.lbgpu_batch_last_error.argtypes = [H]
        L.lbgpu_batch_last_error.restype = C.c_char_p
        _batch_ready = True
    return L


class BudgetExceeded(LbgpuError):
    """lbgpu_batch_add refused a lattice that does not fit the HBM budget."""


class _MemberView(GPULattice):
    """A batch member's handle (owned by the batch)."""

    def __init__(self, p, precision, h):
        self.p = p
        self.precision = precision
        self.h = C.c_void_p(h)
        self.n = tuple(int(x) for x in p.gn[: p.d])
        self.nH = tuple(x + 4 for x in self.n)

    def close(self):
        self.h = C.c_void_p()

    def step(self, n: int = 1) -> None:
        raise LbgpuError("batch members advance with Batch.step")


class Batch:
    """Independent lattices advanced together (lbgpu_batch_*)."""

    def __init__(self, precision: int = FP16, device: int = 0, hbm_budget_bytes: int = 0):
        self.L = _batch_lib()
        self.precision = precision
        self.device = device
        self.h = C.c_void_p()
        rc = self.L.lbgpu_batch_create(device, precision, int(hbm_budget_bytes), C.byref(self.h))
        if rc != 0:
            raise LbgpuError(f"lbgpu_batch_create: {ERRORS.get(rc, rc)}: "
                             f"{self.L.lbgpu_batch_last_error(None).decode()}")
        self.params = {}

    def _check(self, rc, what):
        if rc == -4:
            raise BudgetExceeded(f"{what}: {self.L.lbgpu_batch_last_error(self.h).decode()}")
        if rc != 0:
            raise LbgpuError(f"{what}: {ERRORS.get(rc, rc)}: {self.L.lbgpu_batch_last_error(self.h).decode()}")

    def add(self, p, fluids, mask=None, rho0=(0.0, 0.0)) -> int:
        cfg = make_config(p, self.precision, self.device, rho0)
        ptrs = (C.c_void_p * MAXC)()
        for i, a in enumerate(fluids):
            ptrs[i] = _ptr_of(a)
        sid = C.c_int32()
        self._check(self.L.lbgpu_batch_add(self.h, C.byref(cfg), ptrs, _ptr_of(mask), C.byref(sid)),
                    "lbgpu_batch_add")
        self.params[sid.value] = p
        return sid.value

    def remove(self, sid: int) -> None:
        self._check(self.L.lbgpu_batch_remove(self.h, sid), "lbgpu_batch_remove")
        self.params.pop(sid, None)

    def step(self, n: int = 1) -> None:
        self._check(self.L.lbgpu_batch_step(self.h, int(n)), "lbgpu_batch_step")

    def member(self, sid: int) -> GPULattice:
        h = self.L.lbgpu_batch_member(self.h, sid)
        if not h:
            raise LbgpuError(f"no batch member {sid}")
        return _MemberView(self.params[sid], self.precision, h)

    def set_stream(self, stream_handle) -> None:
        self._check(self.L.lbgpu_batch_set_stream(self.h, stream_handle), "lbgpu_batch_set_stream")

    def synchronize(self) -> None:
        self._check(self.L.lbgpu_batch_synchronize(self.h), "lbgpu_batch_synchronize")

    def set_tuning(self, autotune=True, tile_height=0, ctas_per_sm=0, use_graph=True) -> None:
        self._check(self.L.lbgpu_batch_set_tuning(self.h, int(autotune), int(tile_height), int(ctas_per_sm),
                                                  int(use_graph)), "lbgpu_batch_set_tuning")

    def launch_shape(self):
        ty = C.c_int32()
        cps = C.c_int32()
        self._check(self.L.lbgpu_batch_launch_shape(self.h, C.byref(ty), C.byref(cps)), "lbgpu_batch_launch_shape")
        return ty.value, cps.value

    @property
    def device_bytes(self) -> int:
        return int(self.L.lbgpu_batch_device_bytes(self.h))

    @property
    def launch_count(self) -> int:
        return int(self.L.lbgpu_batch_launch_count(self.h))

    def close(self):
        if self.h:
            self.L.lbgpu_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# device-side initial fields (lbgpu_init_fields / lbgpu_batch_add_init)
# ---------------------------------------------------------------------------
EXPORTED += ["lbgpu_init_fields", "lbgpu_batch_add_init"]


class LbgpuInit(C.Structure):
    _fields_ = [
        ("fluid_init", C.c_int32 * MAXC), ("n_densities", C.c_int32 * MAXC),
        ("densities", (C.c_double * 8) * MAXC), ("perturb", C.c_double * MAXC), ("seed", C.c_uint64),
        ("init_radius", C.c_double), ("init_offset", C.c_double * 3), ("init_separation", C.c_double * 3),
        ("init_axis", C.c_int32), ("interface_thickness", C.c_double), ("n_lamellae", C.c_int32),
        ("lamellae_widths", C.c_double * 8), ("mask_init", C.c_int32), ("mask_axis", C.c_int32),
        ("wall_offset", C.c_int32), ("wall_thickness", C.c_int32), ("dimension_has_wall", (C.c_int32 * 2) * 3),
        ("rng", C.c_int32), ("random_reseed", C.c_int32 * MAXC), ("nc", C.c_int32 * 3),
        ("shift_seed_by_rank", C.c_int32), ("random_seed", C.c_uint64 * MAXC),
    ]


def make_init(p, seed: int = 0, reference_rng: bool = False) -> LbgpuInit:
    """Device initialiser description from :class:`dlbc_gb300.params.LBParams`.

    ``reference_rng``: the random initialisers draw the reference's Mt19937
    sequences on the process grid ``p.nc``, seeded with ``p.seed`` (``seed``
    is then unused) and ``p.random_seed`` where ``p.random_reseed``, plus the
    rank where ``p.shift_seed_by_rank``; otherwise counter-based draws keyed
    by ``seed``."""
    ini = LbgpuInit()
    for f in range(p.components):
        ini.fluid_init[f] = p.fluid_init[f]
        dens = p.fluid_densities[f]
        ini.n_densities[f] = len(dens)
        for j, v in enumerate(dens[:8]):
            ini.densities[f][j] = v
        ini.perturb[f] = p.fluid_perturb[f]
    ini.seed = seed & 0xFFFFFFFFFFFFFFFF
    if reference_rng:
        ini.rng = 1
        ini.seed = int(p.seed) & 0xFFFFFFFFFFFFFFFF
        ini.shift_seed_by_rank = int(bool(p.shift_seed_by_rank))
        for i in range(min(p.d, 3, len(p.nc))):
            ini.nc[i] = max(1, int(p.nc[i]))
        for f in range(p.components):
            if f < len(p.random_reseed) and p.random_reseed[f]:
                ini.random_reseed[f] = 1
                ini.random_seed[f] = int(p.random_seed[f]) & 0xFFFFFFFFFFFFFFFF
    ini.init_radius = p.init_radius
    for i in range(p.d):
        ini.init_offset[i] = p.init_offset[i]
        ini.init_separation[i] = p.init_separation[i]
        ini.dimension_has_wall[i][0] = int(p.dimension_has_wall[i][0])
        ini.dimension_has_wall[i][1] = int(p.dimension_has_wall[i][1])
    ini.init_axis = p.init_axis
    ini.interface_thickness = p.interface_thickness
    ini.n_lamellae = len(p.lamellae_widths)
    for j, w in enumerate(p.lamellae_widths[:8]):
        ini.lamellae_widths[j] = w
    ini.mask_init = p.mask_init
    ini.mask_axis = p.mask_axis
    ini.wall_offset = p.wall_offset
    ini.wall_thickness = p.wall_thickness
    return ini


def _init_lib():
    L = _batch_lib()
    if not getattr(L, "_init_ready", False):
        L.lbgpu_init_fields.argtypes = [C.c_void_p, C.POINTER(LbgpuInit)]
        L.lbgpu_batch_add_init.argtypes = [C.c_void_p, C.POINTER(LbgpuConfig), C.POINTER(LbgpuInit),
                                           C.POINTER(C.c_int32)]
        L._init_ready = True
    return L


def _gpulattice_init_device(self, seed: int = 0, reference_rng: bool = False) -> None:
    """Fill the lattice on the device from its parameters (lbgpu_init_fields);
    ``reference_rng`` as :func:`make_init`."""
    ini = make_init(self.p, seed, reference_rng)
    self._check(_init_lib().lbgpu_init_fields(self.h, C.byref(ini)), "lbgpu_init_fields")


GPULattice.init_device = _gpulattice_init_device


def _batch_add_device(self, p, seed: int = 0, rho0=(0.0, 0.0), reference_rng: bool = False) -> int:
    """Admit a lattice whose initial fields are computed on the device
    (``reference_rng`` as :func:`make_init`)."""
    cfg = make_config(p, self.precision, self.device, rho0)
    ini = make_init(p, seed, reference_rng)
    sid = C.c_int32()
    self._check(_init_lib().lbgpu_batch_add_init(self.h, C.byref(cfg), C.byref(ini), C.byref(sid)),
                "lbgpu_batch_add_init")
    self.params[sid.value] = p
    return sid.value


Batch.add_device = _batch_add_device
