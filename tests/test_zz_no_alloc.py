"""lbgpu_step_noalloc: the allocation-free timestep for callers that cannot
let the library allocate device memory (their framework's pool owns the GPU,
or they cannot accept cudaMalloc's implicit synchronisation mid-run).

It must give the same populations as the regular entry points
(lbgpu_create/lbgpu_upload/lbgpu_step) on two calls in a row: bit for bit
in FP64, the tolerance every FP64 parity test here uses.  The caller owns the
population buffers (torch CUDA tensors here); the scratch is the library's
static device array, shared by all calls.
"""
import ctypes

import numpy as np
import pytest

from dlbc_gb300 import init, lbgpu
from lbcases import droplet_channel, spinodal

pytestmark = pytest.mark.gpu


def _noalloc():
    L = lbgpu.lib()
    fn = L.lbgpu_step_noalloc
    fn.argtypes = [ctypes.POINTER(lbgpu.LbgpuConfig), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
    fn.restype = ctypes.c_int
    return fn


def _to_soa(fluids, p):
    """Haloed AoS host arrays -> [c][q][x][y][z] physical SoA."""
    sl = tuple(slice(2, -2) for _ in range(p.d))
    return np.ascontiguousarray(np.stack([np.moveaxis(f[sl], -1, 0) for f in fluids]))


def _from_soa(a):
    return [np.ascontiguousarray(np.moveaxis(a[c], 0, -1)) for c in range(a.shape[0])]


@pytest.mark.parametrize("case", ["spinodal", "walls"])
def test_noalloc_matches_regular_step_twice(case):
    import torch
    p = spinodal((24, 20, 16)) if case == "spinodal" else droplet_channel((20, 12, 14), radius=4.0, acc=1e-3,
                                                                          gwc=(0.2, -0.1))
    fl, m = init.init_fields(p)

    # the regular, allocating entry points
    g = lbgpu.GPULattice(p, precision=lbgpu.FP64)
    g.upload(fl, m)
    g.step(1)
    ref1 = g.population()
    g.step(1)
    ref2 = g.population()
    g.close()

    # the allocation-free entry point on caller-owned device buffers
    dev = torch.device("cuda", 0)
    a = torch.from_numpy(_to_soa(fl, p)).to(dev)
    b = torch.empty_like(a)
    mask = None
    if case == "walls":
        mask = torch.from_numpy(np.ascontiguousarray(m[2:-2, 2:-2, 2:-2].astype(np.uint8))).to(dev)
    cfg = lbgpu.make_config(p, precision=lbgpu.FP64, device=0)
    err = ctypes.create_string_buffer(512)
    fn = _noalloc()
    stream = torch.cuda.current_stream(dev).cuda_stream

    rc = fn(ctypes.byref(cfg), a.data_ptr(), b.data_ptr(), None if mask is None else mask.data_ptr(), stream,
            err, len(err))
    assert rc == 0, err.value.decode()
    torch.cuda.synchronize(dev)
    out1 = _from_soa(b.cpu().numpy())

    rc = fn(ctypes.byref(cfg), b.data_ptr(), a.data_ptr(), None if mask is None else mask.data_ptr(), stream,
            err, len(err))
    assert rc == 0, err.value.decode()
    torch.cuda.synchronize(dev)
    out2 = _from_soa(a.cpu().numpy())

    for c in range(p.components):
        assert np.array_equal(out1[c], ref1[c]), f"first call, component {c}"
        assert np.array_equal(out2[c], ref2[c]), f"second call, component {c}"


def test_noalloc_rejects_lattices_beyond_the_scratch():
    p = spinodal((256, 128, 128))
    cfg = lbgpu.make_config(p, precision=lbgpu.FP64, device=0)
    err = ctypes.create_string_buffer(512)
    dummy = ctypes.c_void_p(16)
    rc = _noalloc()(ctypes.byref(cfg), dummy, ctypes.c_void_p(32), None, None, err, len(err))
    assert rc == -1
    assert b"scratch" in err.value
