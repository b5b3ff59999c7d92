// lbgpu_step_noalloc: one timestep on caller-owned device buffers, without
// allocating any device memory.
//
// lbgpu_create/lbgpu_step keep their populations and their psi/rho scratch
// in memory the library allocates with cudaMalloc.  Some callers cannot let
// a library allocate: a host framework whose pool already owns the GPU's
// memory (every byte is handed out by that pool, so a stray cudaMalloc may
// fail or break its accounting), or a caller that cannot accept the
// device-wide synchronisation cudaMalloc/cudaFree may imply while its other
// streams are running.  This entry point serves them: the caller passes the
// populations (in and out) as device pointers it owns, and the timestep's
// scratch (the densities and psi values the Shan-Chen stencil reads) lives in
// the file-scope array below.
//
// FP32 runs the two-kernel float step (the step lbgpu_create selects with
// LBGPU_TWO_KERNEL=1), not the fused single-pass kernel lbgpu_step runs for
// FP32 D3Q19 by default, so its FP32 populations agree with lbgpu_step's
// within the FP32 form's rounding, not bit for bit; FP64 agrees bit for bit.
//
// Scratch: kNoallocScratchBytes (64 MiB) of static device memory.  Every GPU
// that loads this library holds that array until the process exits.  The
// timestep needs components * 2 values per site of the arithmetic type
// (double for LBGPU_FP64, float for LBGPU_FP32), so the largest lattice is
// 64 MiB / (components * 2 * 8) sites in FP64 (2,097,152 = 128^3 sites for
// two components) and twice that in FP32; larger lattices are rejected.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress (with that device current) and caches it; make
// that first call before any stream capture.  The scratch holds the last
// call's densities and psi values; the timestep overwrites all of them before
// reading any, so nothing needs clearing.  All calls share the one array:
// calls whose kernels overlap on the GPU (different streams, or host threads,
// without ordering between them) race on it and must be serialised by the
// caller.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "../../include/lbgpu.h"
#include "lb_launch.h"

namespace {

constexpr size_t kNoallocScratchBytes = size_t(64) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

int noalloc_fail(int code, char* errbuf, size_t errlen, const char* fmt, long long a = 0, long long b = 0,
                 long long c = 0) {
  if (errbuf && errlen) snprintf(errbuf, errlen, fmt, a, b, c);
  return code;
}

}  // namespace

extern "C" int lbgpu_step_noalloc(const lbgpu_config* cfg, const void* f_in, void* f_out, const uint8_t* mask,
                                  void* stream, char* errbuf, size_t errbuf_len) {
  if (errbuf && errbuf_len) errbuf[0] = '\0';
  if (!cfg || !f_in || !f_out)
    return noalloc_fail(LBGPU_E_INVALID, errbuf, errbuf_len, "null config or population pointer");
  if (f_in == f_out)
    return noalloc_fail(LBGPU_E_INVALID, errbuf, errbuf_len, "f_in and f_out must be different buffers");
  if (!((cfg->d == 3 && cfg->q == 19) || (cfg->d == 2 && cfg->q == 9)))
    return noalloc_fail(LBGPU_E_INVALID, errbuf, errbuf_len, "only D3Q19 and D2Q9 are supported");
  if (cfg->components < 1 || cfg->components > LBGPU_MAX_COMPONENTS)
    return noalloc_fail(LBGPU_E_INVALID, errbuf, errbuf_len, "components must be 1 or 2");
  if (cfg->precision != LBGPU_FP64 && cfg->precision != LBGPU_FP32)
    return noalloc_fail(LBGPU_E_INVALID, errbuf, errbuf_len,
                        "the allocation-free step supports LBGPU_FP64 and LBGPU_FP32 only");
  if (cfg->eq_form < 0 || cfg->eq_form > 2 || cfg->psi_form < 0 || cfg->psi_form > 1)
    return noalloc_fail(LBGPU_E_INVALID, errbuf, errbuf_len, "unknown eqDistForm or psiForm");
  if (cfg->device < 0 || cfg->device >= kMaxDevices)
    return noalloc_fail(LBGPU_E_INVALID, errbuf, errbuf_len, "device ordinal out of range");
  const int C = cfg->components;
  const int nx = cfg->gn[0], ny = cfg->gn[1], nz = cfg->d == 3 ? cfg->gn[2] : 1;
  if (nx < 2 || ny < 2 || (cfg->d == 3 && nz < 2))
    return noalloc_fail(LBGPU_E_INVALID, errbuf, errbuf_len, "every lattice extent must be >= 2");
  for (int c = 0; c < C; ++c)
    if (!(cfg->tau[c] > 0.0)) return noalloc_fail(LBGPU_E_INVALID, errbuf, errbuf_len, "tau must be positive");
  const long long n = (long long)nx * ny * nz;
  const size_t arith = cfg->precision == LBGPU_FP64 ? sizeof(double) : sizeof(float);
  const size_t need = size_t(n) * C * 2 * arith;
  if (need > kNoallocScratchBytes)
    return noalloc_fail(LBGPU_E_INVALID, errbuf, errbuf_len,
                        "lattice of %lld sites needs %lld bytes of scratch; the allocation-free step has %lld "
                        "(use lbgpu_create/lbgpu_step for larger lattices)",
                        n, (long long)need, (long long)kNoallocScratchBytes);

  int prev = -1;
  cudaError_t e = cudaGetDevice(&prev);
  if (e != cudaSuccess) return noalloc_fail(LBGPU_E_CUDA, errbuf, errbuf_len, "cudaGetDevice failed");
  if (prev != cfg->device) {
    e = cudaSetDevice(cfg->device);
    if (e != cudaSuccess) return noalloc_fail(LBGPU_E_CUDA, errbuf, errbuf_len, "cudaSetDevice failed");
  }

  // once per device, with that device current: the scratch array's address
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[cfg->device]) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        if (prev != cfg->device) cudaSetDevice(prev);
        return noalloc_fail(LBGPU_E_CUDA, errbuf, errbuf_len, "cudaGetSymbolAddress of the scratch array failed");
      }
      g_scratch_addr[cfg->device] = ptr;
    }
    scratch = g_scratch_addr[cfg->device];
  }

  lbk::StepParams P{};
  P.nx = nx;
  P.ny = ny;
  P.nz = nz;
  P.n = n;
  P.shan_chen = cfg->shan_chen;
  P.psi_form = cfg->psi_form;
  P.eq_form = cfg->eq_form;
  P.record_force = 0;
  // every tau == 1: the relaxation is the equilibrium itself (the exact
  // shortcut lbgpu_create enables for the same configuration)
  P.unit_tau = 1;
  for (int c = 0; c < C; ++c)
    if (cfg->tau[c] != 1.0) P.unit_tau = 0;
  for (int c = 0; c < 2; ++c) {
    const double tau = c < C ? cfg->tau[c] : 1.0;
    P.tau[c] = tau;
    P.omega[c] = 1.0 / tau;
    P.one_minus_omega[c] = 1.0 - P.omega[c];
    P.gwc[c] = c < C ? cfg->gwc[c] : 0.0;
    for (int c2 = 0; c2 < 2; ++c2) P.gcc[c][c2] = (c < C && c2 < C) ? cfg->gcc[c][c2] : 0.0;
    P.rho0[c] = 0.f;
    P.scale[c] = 1.f;
    P.inv_scale[c] = 1.f;
  }
  for (int i = 0; i < 3; ++i) P.acc[i] = i < cfg->d ? cfg->global_acc[i] : 0.0;

  lbk::StepBuffers b;
  b.f = f_in;
  b.fout = f_out;
  b.mask = mask;
  b.rho = scratch;
  b.psi = static_cast<unsigned char*>(scratch) + size_t(n) * C * arith;
  b.force = nullptr;
  int64_t launches = 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  e = cfg->precision == LBGPU_FP64 ? lbk::launch_step_f64(cfg->q, C, b, P, st, &launches, nullptr)
                                   : lbk::launch_step_f32(cfg->q, C, b, P, st, &launches, nullptr);
  if (prev != cfg->device) cudaSetDevice(prev);
  if (e != cudaSuccess) return noalloc_fail(LBGPU_E_CUDA, errbuf, errbuf_len, "timestep launch failed");
  return LBGPU_OK;
}
