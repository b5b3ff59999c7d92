"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module: it is the checker for the CUDA path, never part of it.  The
library is built from ``oracle/lb_oracle.cpp`` by ``oracle/Makefile``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblb_oracle.so")
MAXC = 4


class OrConfig(C.Structure):
    _fields_ = [
        ("d", C.c_int32), ("q", C.c_int32), ("gn", C.c_int32 * 3), ("components", C.c_int32),
        ("shan_chen", C.c_int32), ("psi_form", C.c_int32), ("eq_form", C.c_int32),
        ("exp_mode", C.c_int32), ("sum_mode", C.c_int32), ("threads", C.c_int32),
        ("tau", C.c_double * MAXC), ("gcc", (C.c_double * MAXC) * MAXC), ("gwc", C.c_double * MAXC),
        ("global_acc", C.c_double * 3),
    ]


class OrInit(C.Structure):
    _fields_ = [
        ("fluid_init", C.c_int32 * MAXC), ("n_dens", C.c_int32 * MAXC),
        ("densities", (C.c_double * 8) * MAXC), ("perturb", C.c_double * MAXC),
        ("random_reseed", C.c_int32 * MAXC), ("random_seed", C.c_int32 * MAXC),
        ("seed", C.c_int32), ("shift_seed_by_rank", C.c_int32), ("init_radius", C.c_double),
        ("init_offset", C.c_double * 3), ("init_separation", C.c_double * 3),
        ("init_axis", C.c_int32), ("interface_thickness", C.c_double), ("n_lamellae", C.c_int32),
        ("lamellae_widths", C.c_double * 8), ("mask_init", C.c_int32), ("mask_axis", C.c_int32),
        ("wall_offset", C.c_int32), ("wall_thickness", C.c_int32),
        ("dimension_has_wall", (C.c_int32 * 2) * 3), ("nc", C.c_int32 * 3),
    ]


_lib: Optional[C.CDLL] = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        L.or_create.restype = P
        L.or_create.argtypes = [C.POINTER(OrConfig)]
        L.or_destroy.argtypes = [P]
        L.or_lengths_h.argtypes = [P, C.c_int32 * 3, C.POINTER(C.c_int32)]
        L.or_init_lattice.argtypes = [P, C.POINTER(OrInit)]
        L.or_init_lattice.restype = C.c_int
        for fn in ("or_get_fluid", "or_set_fluid", "or_population", "or_density", "or_velocity", "or_force"):
            getattr(L, fn).argtypes = [P, C.c_int, dp]
        L.or_colour.argtypes = [P, C.c_int, C.c_int, dp]
        L.or_get_mask.argtypes = [P, ip]
        L.or_set_mask.argtypes = [P, ip]
        L.or_mask_phys.argtypes = [P, ip]
        L.or_exchange_halo.argtypes = [P]
        L.or_run.argtypes = [P, C.c_int]
        L.or_total_mass.argtypes = [P, C.c_int]
        L.or_total_mass.restype = C.c_double
        L.or_uniform_sequence.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_int, dp]
        L.or_uniform_sequence.restype = C.c_double
        L.or_exp.argtypes = [C.c_int, C.c_int, dp, dp]
        L.or_exp.restype = None
        L.or_div.argtypes = [C.c_int, dp, dp, dp]
        L.or_div.restype = None
        _lib = L
    return _lib


def exp(x, mode: int = 1):
    """exp of a float64 array: mode 1 the kernels' lbmath::lb_exp, mode 2
    its FP64 routine for arguments outside the integer range
    (lbmath::lb_exp_fp64), mode 0 long double expl rounded to double."""
    x = np.ascontiguousarray(x, np.float64)
    out = np.empty_like(x)
    lib().or_exp(mode, x.size, x, out)
    return out


def div(a, b):
    """a / b elementwise by the kernels' integer IEEE division."""
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    out = np.empty_like(a)
    lib().or_div(a.size, a, b, out)
    return out


def make_config(p, exp_mode: int = 0, sum_mode: int = 0, threads: int = 1) -> OrConfig:
    """Oracle configuration from a :class:`dlbc_gb300.params.LBParams`."""
    c = OrConfig()
    c.d, c.q = p.d, p.q
    for i in range(p.d):
        c.gn[i] = p.gn[i]
    c.components = p.components
    c.shan_chen = int(p.shan_chen)
    c.psi_form = p.psi_form
    c.eq_form = p.eq_form
    c.exp_mode = exp_mode
    c.sum_mode = sum_mode
    c.threads = threads
    for f in range(p.components):
        c.tau[f] = p.tau[f] if p.tau else 1.0
        c.gwc[f] = p.gwc[f]
        for g in range(p.components):
            c.gcc[f][g] = p.gcc[f][g]
    for i in range(p.d):
        c.global_acc[i] = p.global_acc[i]
    return c


def make_init(p) -> OrInit:
    ini = OrInit()
    for f in range(p.components):
        ini.fluid_init[f] = p.fluid_init[f]
        dens = p.fluid_densities[f]
        ini.n_dens[f] = len(dens)
        for j, v in enumerate(dens[:8]):
            ini.densities[f][j] = v
        ini.perturb[f] = p.fluid_perturb[f]
        ini.random_reseed[f] = int(p.random_reseed[f])
        ini.random_seed[f] = p.random_seed[f]
    ini.seed = p.seed
    ini.shift_seed_by_rank = int(p.shift_seed_by_rank)
    ini.init_radius = p.init_radius
    for i in range(p.d):
        ini.init_offset[i] = p.init_offset[i]
        ini.init_separation[i] = p.init_separation[i]
        ini.dimension_has_wall[i][0] = int(p.dimension_has_wall[i][0])
        ini.dimension_has_wall[i][1] = int(p.dimension_has_wall[i][1])
        ini.nc[i] = p.nc[i] if i < len(p.nc) else 0
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


class Oracle:
    """One lattice held by the CPU oracle."""

    def __init__(self, p, exp_mode: int = 0, sum_mode: int = 0, threads: int = 1, init: bool = True):
        self.p = p
        self.cfg = make_config(p, exp_mode, sum_mode, threads)
        self.h = lib().or_create(C.byref(self.cfg))
        if not self.h:
            raise ValueError("oracle rejected the configuration")
        nh = (C.c_int32 * 3)()
        halo = C.c_int32()
        lib().or_lengths_h(self.h, nh, C.byref(halo))
        self.nH = tuple(nh[i] for i in range(p.d))
        self.halo = halo.value
        self.n = tuple(p.gn[: p.d])
        if init:
            rc = lib().or_init_lattice(self.h, C.byref(make_init(p)))
            if rc != 0:
                raise ValueError(f"oracle init failed ({rc})")

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_destroy(self.h)
            self.h = None

    def run(self, n: int) -> None:
        lib().or_run(self.h, n)

    def exchange_halo(self) -> None:
        lib().or_exchange_halo(self.h)

    def fluid_haloed(self, c: int) -> np.ndarray:
        a = np.empty(self.nH + (self.p.q,), np.float64)
        lib().or_get_fluid(self.h, c, a)
        return a

    def set_fluid_haloed(self, c: int, a: np.ndarray) -> None:
        lib().or_set_fluid(self.h, c, np.ascontiguousarray(a, np.float64))

    def mask_haloed(self) -> np.ndarray:
        a = np.empty(self.nH, np.int32)
        lib().or_get_mask(self.h, a)
        return a

    def set_mask_haloed(self, m: np.ndarray) -> None:
        lib().or_set_mask(self.h, np.ascontiguousarray(m, np.int32))

    def population(self, c: int) -> np.ndarray:
        a = np.empty(self.n + (self.p.q,), np.float64)
        lib().or_population(self.h, c, a)
        return a

    def density(self, c: int) -> np.ndarray:
        a = np.empty(self.n, np.float64)
        lib().or_density(self.h, c, a)
        return a

    def colour(self, c1: int = 0, c2: int = 1) -> np.ndarray:
        a = np.empty(self.n, np.float64)
        lib().or_colour(self.h, c1, c2, a)
        return a

    def velocity(self, c: int) -> np.ndarray:
        a = np.empty(self.n + (self.p.d,), np.float64)
        lib().or_velocity(self.h, c, a)
        return a

    def force(self, c: int) -> np.ndarray:
        a = np.empty(self.n + (self.p.d,), np.float64)
        lib().or_force(self.h, c, a)
        return a

    def mask(self) -> np.ndarray:
        a = np.empty(self.n, np.int32)
        lib().or_mask_phys(self.h, a)
        return a

    def total_mass(self, c: int) -> float:
        return lib().or_total_mass(self.h, c)


def uniform_sequence(seed: int, a: float, b: float, n: int) -> np.ndarray:
    out = np.empty(n, np.float64)
    lib().or_uniform_sequence(seed & 0xFFFFFFFF, a, b, n, out)
    return out
