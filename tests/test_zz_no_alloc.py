"""lbgpu_step_noalloc: the allocation-free timestep for callers that cannot
let the library allocate device memory (their framework's pool owns the GPU,
or they cannot accept cudaMalloc's implicit synchronisation mid-run).

It must give the same populations as the regular entry points
(lbgpu_create/lbgpu_upload/lbgpu_step) on two calls in a row: bit for bit
in FP64, the tolerance every FP64 parity test here uses; in FP32 within the
tolerance the fused-versus-two-kernel FP32 test uses (2e-6 of the largest
population), because lbgpu_step runs the fused single-pass kernel for FP32
D3Q19 and D2Q9 and this entry point the two-kernel float step.  The caller owns the
population buffers (torch CUDA tensors here); the scratch is the library's
static device array, shared by all calls.  (Its size check, which needs no
GPU, is in test_cabi.py.)
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


def _to_soa(fluids, p, dtype):
    """Haloed AoS host arrays -> [c][q][x][y](z) physical SoA."""
    sl = tuple(slice(2, -2) for _ in range(p.d))
    return np.ascontiguousarray(np.stack([np.moveaxis(f[sl], -1, 0) for f in fluids]).astype(dtype))


def _from_soa(a):
    return [np.ascontiguousarray(np.moveaxis(a[c], 0, -1)).astype(np.float64) for c in range(a.shape[0])]


CASES = {
    "spinodal": lambda: spinodal((24, 20, 16)),
    "walls": lambda: droplet_channel((20, 12, 14), radius=4.0, acc=1e-3, gwc=(0.2, -0.1)),
    "unequal-tau": lambda: droplet_channel((16, 10, 12), radius=3.0, acc=1e-3, tau=(0.8, 1.3)),
    "d2q9": lambda: spinodal((40, 36), d=2),
}


@pytest.mark.parametrize("precision", [lbgpu.FP64, lbgpu.FP32])
@pytest.mark.parametrize("case", list(CASES))
def test_noalloc_matches_regular_step_twice(case, precision):
    import torch
    p = CASES[case]()
    fl, m = init.init_fields(p)

    # the regular, allocating entry points
    g = lbgpu.GPULattice(p, precision=precision)
    g.upload(fl, m)
    g.step(1)
    ref1 = g.population()
    g.step(1)
    ref2 = g.population()
    g.close()

    # the allocation-free entry point on caller-owned device buffers
    dev = torch.device("cuda", 0)
    dtype = np.float64 if precision == lbgpu.FP64 else np.float32
    a = torch.from_numpy(_to_soa(fl, p, dtype)).to(dev)
    b = torch.empty_like(a)
    mask = None
    if m is not None and np.any(m):
        sl = tuple(slice(2, -2) for _ in range(p.d))
        mask = torch.from_numpy(np.ascontiguousarray(m[sl].astype(np.uint8))).to(dev)
    cfg = lbgpu.make_config(p, precision=precision, device=0)
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
        if precision == lbgpu.FP64:
            assert np.array_equal(out1[c], ref1[c]), f"first call, component {c}"
            assert np.array_equal(out2[c], ref2[c]), f"second call, component {c}"
        else:
            for k, (o, r) in enumerate(((out1[c], ref1[c]), (out2[c], ref2[c]))):
                err_max = float(np.abs(o - r).max())
                assert err_max <= 2e-6 * float(np.abs(r).max()), (f"call {k + 1}, component {c}", err_max)
