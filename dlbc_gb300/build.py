"""Build the CUDA library ``dlbc_gb300/_build/liblbgpu.so`` for sm_103a.

Translation units compiled in parallel with one ``-gencode``:

* ``lb_step_f64.cu``, ``lb_api.cu`` and ``lb_init.cu`` with ``-fmad=false``
  (the FP64 form and the double-precision moments must round every product
  and sum as the reference does);
* the fused FP32 / FP16 / I16-storage steps (``lb_fused*.cu``, split by
  storage type, connectivity and batching) also with ``-fmad=false``: their
  fused multiply-adds are explicit, so all variants of a kernel give the
  same bits;
* the two-kernel FP32 / FP16 step and the rest (``lb_step_lp.cu``,
  ``lb_batch.cu``, ``lb_noalloc.cu``) with contraction allowed.

Beside it, ``_build/libpeak_fp64.so`` (``peak_fp64.cu``): the FP64
instruction-rate microbenchmark the benchmark reports the FP64 form against.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liblbgpu.so")
PEAK_LIB = os.path.join(OUT, "libpeak_fp64.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr"]
UNITS = {
    "lb_step_f64.cu": ["-fmad=false"],
    "lb_api.cu": ["-fmad=false"],
    "lb_init.cu": ["-fmad=false"],
    "lb_step_lp.cu": [],
    # the fused kernels: explicit fmaf only, so that every variant of the
    # step computes the same bits
    "lb_fused.cu": ["-fmad=false"],
    "lb_fused_f32.cu": ["-fmad=false"],
    "lb_fused_f16.cu": ["-fmad=false"],
    "lb_fused_batch.cu": ["-fmad=false"],
    "lb_fused2d.cu": ["-fmad=false"],
    "lb_batch.cu": [],
    "lb_noalloc.cu": [],
}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _sources_mtime() -> float:
    m = 0.0
    for root in (CSRC, os.path.join(os.path.dirname(HERE), "include")):
        for f in os.listdir(root):
            m = max(m, os.path.getmtime(os.path.join(root, f)))
    return max(m, os.path.getmtime(__file__))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if stale) and return the library path."""
    if (not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime()
            and os.path.exists(PEAK_LIB) and os.path.getmtime(PEAK_LIB) >= _sources_mtime()):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    peak = subprocess.Popen([nv, *ARCH, *COMMON, "-shared", os.path.join(CSRC, "peak_fp64.cu"), "-o",
                             PEAK_LIB + ".tmp", "-lcudart"], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                            text=True)

    def compile_unit(item):
        src, extra = item
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [nv, *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    _, perr = peak.communicate()
    if peak.returncode != 0:
        raise RuntimeError(f"nvcc failed for peak_fp64.cu:\n{perr}")
    os.replace(PEAK_LIB + ".tmp", PEAK_LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
