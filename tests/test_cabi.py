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
    assert lib.lbgpu_abi_version() == 2


def test_create_rejects_bad_configs_without_touching_the_gpu(libpath):
    from dlbc_gb300 import params
    L = lbgpu.lib()
    base = params.LBParams(d=3, q=19, gn=[8, 8, 8], components=2, tau=[1.0, 1.0], gcc=[[0, 0], [0, 0]],
                           gwc=[0, 0], global_acc=[0, 0, 0])
    for mutate in (lambda c: setattr(c, "q", 27), lambda c: setattr(c, "components", 3),
                   lambda c: c.gn.__setitem__(0, 1), lambda c: setattr(c, "precision", 9),
                   lambda c: c.tau.__setitem__(0, 0.0),
                   # 4096 x 4096 x 256 = 2^32 sites: above the 2^31-site limit
                   lambda c: [c.gn.__setitem__(i, v) for i, v in enumerate((4096, 4096, 256))]):
        cfg = lbgpu.make_config(base)
        mutate(cfg)
        h = ctypes.c_void_p()
        rc = L.lbgpu_create(ctypes.byref(cfg), ctypes.byref(h))
        assert rc == -1 and not h.value
        assert L.lbgpu_last_error(None)


C_CONSUMER = r"""
#include <stdio.h>
#include <string.h>
#include "lbgpu.h"

int main(void) {
  lbgpu_config cfg;
  lbgpu_handle* h = NULL;
  memset(&cfg, 0, sizeof cfg);
  cfg.d = 3;
  cfg.q = 27; /* no such connectivity: refused before any device work */
  cfg.gn[0] = cfg.gn[1] = cfg.gn[2] = 8;
  cfg.components = 2;
  cfg.tau[0] = cfg.tau[1] = 1.0;
  int rc = lbgpu_create(&cfg, &h);
  const char* msg = lbgpu_last_error(NULL);
  printf("%d %d %d %s\n", lbgpu_abi_version(), rc, h == NULL, msg ? "msg" : "none");
  return 0;
}
"""


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_header_compiles_links_and_runs_from_c_and_cpp(libpath, tmp_path, lang):
    """A C99 and a C++17 host include include/lbgpu.h, link liblbgpu.so and
    call it: the ABI version and a configuration refused without a GPU."""
    import shutil
    import subprocess
    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip(f"no {lang} compiler")
    src = tmp_path / ("consumer.c" if lang == "c" else "consumer.cpp")
    src.write_text(C_CONSUMER)
    exe = tmp_path / "consumer"
    libdir = os.path.dirname(libpath)
    std = "-std=c99" if lang == "c" else "-std=c++17"
    subprocess.run([cc, std, "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-llbgpu", f"-Wl,-rpath,{libdir}"], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert out == ["2", "-1", "1", "msg"], out


def test_noalloc_rejects_lattices_beyond_the_scratch(libpath):
    """lbgpu_step_noalloc refuses a lattice whose scratch does not fit its
    static 64 MiB array before any device work (so it runs without a GPU)."""
    from lbcases import spinodal
    fn = lbgpu.lib().lbgpu_step_noalloc
    fn.argtypes = [ctypes.POINTER(lbgpu.LbgpuConfig), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
    fn.restype = ctypes.c_int
    err = ctypes.create_string_buffer(512)
    # 256 x 128 x 128 two-component FP64 needs 128 MiB of scratch; 256 x 256 x 128 FP32 the same
    cfg = lbgpu.make_config(spinodal((256, 128, 128)), precision=lbgpu.FP64, device=0)
    rc = fn(ctypes.byref(cfg), ctypes.c_void_p(16), ctypes.c_void_p(32), None, None, err, len(err))
    assert rc == -1
    assert b"scratch" in err.value
    cfg = lbgpu.make_config(spinodal((256, 256, 128)), precision=lbgpu.FP32, device=0)
    rc = fn(ctypes.byref(cfg), ctypes.c_void_p(16), ctypes.c_void_p(32), None, None, err, len(err))
    assert rc == -1
    assert b"scratch" in err.value
    # a configuration the entry point does not support is refused the same way
    cfg = lbgpu.make_config(spinodal((8, 8, 8)), precision=lbgpu.FP16, device=0)
    rc = fn(ctypes.byref(cfg), ctypes.c_void_p(16), ctypes.c_void_p(32), None, None, err, len(err))
    assert rc == -1


def test_i16_rejects_lattices_off_the_pair_kernel(libpath):
    """The 16-bit fixed-point form (LBGPU_I16) runs only on the pair kernel:
    D3Q19, an even z extent and BDist2.  Other lattices are refused at
    creation, before any device work."""
    from lbcases import spinodal
    L = lbgpu.lib()
    for p in (spinodal((8, 8, 9)), spinodal((8, 8, 8), eq="SecondOrder"), spinodal((8, 8), d=2)):
        cfg = lbgpu.make_config(p, precision=lbgpu.I16)
        h = ctypes.c_void_p()
        assert L.lbgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == -1 and not h.value
        assert b"I16" in L.lbgpu_last_error(None)
