"""lbgpu_step_host (one timestep from host fields to host fields) against the
sequence it stands for, lbgpu_upload + lbgpu_step(1) + lbgpu_download: the
same bits, step after step, with the output array used as the next input.

The FP64 form, the FP32 form and (with their storage scale pinned) the
FP16 and I16 forms run as a wavefront over chunks of x-planes (copies in,
kernels, copies out overlapping; the reduced forms' fused kernel over plane
ranges); lattices too small for it, profiled handles and unpinned FP16/I16
run the three calls in turn.  The launch counts tell the two apart: the
wavefront launches the step kernels once per chunk, the fallback exactly as
the sequence does.
"""
import numpy as np
import pytest

from dlbc_gb300 import init, lbgpu
from lbcases import droplet_channel, spinodal
from test_driver import hook_paths_case
from test_gpu_parity import _lattice_1d

pytestmark = pytest.mark.gpu


def _cases():
    return {
        "channel-walls-force": (droplet_channel((40, 12, 14), radius=4.0, acc=1e-3, gwc=(0.3, -0.2)), True),
        "spinodal-odd-sizes": (spinodal((37, 10, 9)), True),
        "d2q9": (spinodal((64, 40), d=2), True),
        "d1q5-walls": (_lattice_1d("d1q5", "ThirdOrder", walls=True, n=48), True),
        "d1q3": (_lattice_1d("d1q3", "SecondOrder", n=200), True),
        "too-small": (spinodal((5, 7, 3)), False),
    }


def _compare(p, precision, steps, wave, pinned=False, record_force=False, scale=None):
    fl, m = init.init_fields(p)
    seq = lbgpu.GPULattice(p, precision=precision)
    one = lbgpu.GPULattice(p, precision=precision)
    if scale is not None:
        seq.set_storage_scale(*scale)
        one.set_storage_scale(*scale)
    if record_force:
        seq.set_record_force(True)
        one.set_record_force(True)
    state_seq = [a.copy() for a in fl]
    if pinned:
        import torch
        state = [torch.from_numpy(a.copy()).pin_memory() for a in fl]
        mask = None if m is None else torch.from_numpy(m.copy()).pin_memory()
        view = [t.numpy() for t in state]
    else:
        state = [a.copy() for a in fl]
        mask = m
        view = state
    for t in range(steps):
        n0 = seq.launch_count
        seq.upload(state_seq, m)
        seq.step(1)
        seq.download(state_seq)
        n_seq = seq.launch_count - n0
        n0 = one.launch_count
        one.step_host(state, mask, state)  # output into the input arrays
        n_one = one.launch_count - n0
        for c in range(p.components):
            assert np.array_equal(view[c], state_seq[c], equal_nan=True), (t, c)
        if wave:
            assert n_one > n_seq, (n_one, n_seq)
        else:
            assert n_one == n_seq, (n_one, n_seq)
    if record_force:
        fa, fb = seq.force(), one.force()
        for c in range(p.components):
            assert np.array_equal(fa[c], fb[c])
    # the device state after the call is the sequence's: stepping on agrees
    seq.step(3)
    one.step(3)
    pa, pb = seq.population(), one.population()
    for c in range(p.components):
        assert np.array_equal(pa[c], pb[c], equal_nan=True)


@pytest.mark.parametrize("name", list(_cases()))
def test_step_host_fp64_equals_upload_step_download(name):
    p, wave = _cases()[name]
    _compare(p, lbgpu.FP64, 4, wave, record_force=name.startswith("channel"))


def test_step_host_pinned_host_arrays():
    p = droplet_channel((40, 12, 14), radius=4.0, acc=1e-3)
    _compare(p, lbgpu.FP64, 3, True, pinned=True)


# pinned offsets: rest density and scale per component
SCALES = {lbgpu.FP16: ((0.5, 0.5), (1.0 / 1024, 1.0 / 1024)), lbgpu.I16: ((0.5, 0.5), (3.0 / 32767, 3.0 / 32767))}


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16, lbgpu.I16])
@pytest.mark.parametrize("pin", [False, True])
def test_step_host_reduced_forms(precision, pin):
    """FP32 runs the wavefront; FP16 and I16 run it once their scale is
    pinned, the three calls otherwise (the upload derives the scale from the
    whole input).  Walls with the wall force: the wavefront's upload writes
    the solid sites into both population buffers."""
    if precision == lbgpu.FP32 and pin:
        pytest.skip("FP32 has no storage scale")
    p = droplet_channel((40, 12, 14), radius=4.0, acc=1e-3, gwc=(0.3, -0.2))
    _compare(p, precision, 3, precision == lbgpu.FP32 or pin, record_force=True,
             scale=SCALES[precision] if pin else None)


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16])
@pytest.mark.parametrize("case", ["walls", "periodic"])
def test_step_host_d2q9_fused_wavefront(precision, case):
    """The D2Q9 fused kernels over row ranges (the wavefront) compute the
    bits of their whole-lattice launch: the one-site kernel with walls, the
    wall force and a partial tile; the pair kernel on a periodic lattice."""
    if case == "walls":
        p = droplet_channel((48, 300), radius=8.0, acc=1e-3, gwc=(0.3, -0.2), d=2)
    else:
        p = spinodal((48, 300), perturb=0.03, d=2)
    _compare(p, precision, 3, True, record_force=True, scale=SCALES.get(precision))


def test_step_host_fp32_one_site_kernel_wavefront():
    """An odd z extent runs the one-site-per-thread fused kernel: its plane
    ranges make the same wavefront."""
    p = spinodal((37, 10, 9))
    _compare(p, lbgpu.FP32, 3, True)


@pytest.mark.parametrize("precision", [lbgpu.FP32, lbgpu.FP16])
def test_step_host_full_size_channel_reduced(precision):
    p = droplet_channel((256, 128, 128), radius=24.0, acc=1e-6)
    _compare(p, precision, 2, True, pinned=True, scale=SCALES.get(precision))


def test_step_host_full_size_channel():
    """The 256x128x128 droplet channel of the end-to-end measurement (32
    chunks of 8 planes through the 256 MiB staging buffer), pinned arrays."""
    p = droplet_channel((256, 128, 128), radius=24.0, acc=1e-6)
    _compare(p, lbgpu.FP64, 2, True, pinned=True)


def test_step_host_rejects_bad_calls():
    p = spinodal((16, 8, 8))
    fl, m = init.init_fields(p)
    g = lbgpu.GPULattice(p)
    g.upload(fl, m)
    g.advect()
    with pytest.raises(lbgpu.LbgpuError, match="NOTREADY"):
        g.step_host(fl, m, [a.copy() for a in fl])
    g.collide()
    out = g.step_host(fl, m)
    seq = lbgpu.GPULattice(p)
    seq.upload(fl, m)
    seq.step(1)
    ref = seq.download()
    for c in range(2):
        assert np.array_equal(out[c], ref[c])


def test_driver_hook_paths_agree_gpu(tmp_path, monkeypatch):
    """The driver's one-call path (host hooks before advection and after
    collision) and its split path write the same populations on the GPU."""
    hook_paths_case(tmp_path, monkeypatch, lbgpu.GPULattice)
