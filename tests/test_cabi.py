"""The C-ABI library: builds, loads and exports every entry point that
include/lbgpu.h declares.  No compute calls (no GPU here)."""
import ctypes
import os
import re

import pytest

from dlbc_gb300 import build, lbgpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "lbgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lbgpu_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def libpath():
    return build.build()


def test_library_exports_all_declared_symbols(libpath):
    names = declared_functions()
    assert len(names) >= 14
    lib = ctypes.CDLL(libpath)
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(lbgpu.EXPORTED) | (set(names) - set(lbgpu.EXPORTED))


def test_abi_version_without_gpu(libpath):
    lib = ctypes.CDLL(libpath)
    assert lib.lbgpu_abi_version() == 1


def test_create_rejects_bad_configs_without_touching_the_gpu(libpath):
    from dlbc_gb300 import params
    L = lbgpu.lib()
    base = params.LBParams(d=3, q=19, gn=[8, 8, 8], components=2, tau=[1.0, 1.0], gcc=[[0, 0], [0, 0]],
                           gwc=[0, 0], global_acc=[0, 0, 0])
    for mutate in (lambda c: setattr(c, "q", 27), lambda c: setattr(c, "components", 3),
                   lambda c: c.gn.__setitem__(0, 1), lambda c: setattr(c, "precision", 9),
                   lambda c: c.tau.__setitem__(0, 0.0)):
        cfg = lbgpu.make_config(base)
        mutate(cfg)
        h = ctypes.c_void_p()
        rc = L.lbgpu_create(ctypes.byref(cfg), ctypes.byref(h))
        assert rc == -1 and not h.value
        assert L.lbgpu_last_error(None)
