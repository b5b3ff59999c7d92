// C-ABI of the GB300 lattice-Boltzmann timestep (declared in include/lbgpu.h).
//
// Device layout (SoA, physical sites only, no halo):
//   populations  f[buf][c][q][site], two buffers (streaming is pull: read one,
//                write the other, swap), site = (x*ny + y)*nz + z;
//   mask         uint8 [site], only when the lattice has a solid site;
//   rho, psi     [c][site] scratch for the timestep's psi stencil;
//   force        [c][site][d] doubles, only while force recording is on.
// Host transfers go through a bounded device staging buffer holding whole
// haloed x-planes of the reference's AoS layout.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/lbgpu.h"
#include "lb_launch.h"

namespace {

constexpr size_t kStagingBytes = size_t(256) << 20;

thread_local std::string g_create_error;

size_t storage_size(int precision) { return precision == LBGPU_FP64 ? 8 : precision == LBGPU_FP32 ? 4 : 2; }

int storage_kind(int precision) {
  return precision == LBGPU_FP16 ? lbk::kStoreF16 : precision == LBGPU_I16 ? lbk::kStoreI16 : lbk::kStoreF32;
}

}  // namespace

// I16: 16-bit fixed point over offsets up to 3 max(rho0, initial spread)
// from rho0, i.e. f/w from -2 rho0 to 4 rho0 for a lattice that starts near
// rho0: phase separation (a Shan-Chen component's dense phase about twice
// its mean density) and the force-shifted equilibrium's velocity terms stay
// inside; values beyond saturate
double i16_scale(double rho0, double maxdev) {
  const double range = 3.0 * std::max(fabs(rho0), maxdev);
  return range > 0.0 ? range / 32767.0 : 1.0 / 32767.0;
}

namespace {
size_t arith_size(int precision) { return precision == LBGPU_FP64 ? 8 : 4; }

}  // namespace

#include "lb_handle.h"

namespace {

// --------------------------------------------------------------------------
// transfer kernels
// --------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T to_storage(double v, int q, int c, const StepParams& P, int Q);

template <>
__device__ __forceinline__ double to_storage<double>(double v, int, int, const StepParams&, int) {
  return v;
}
template <>
__device__ __forceinline__ float to_storage<float>(double v, int, int, const StepParams&, int) {
  return float(v);
}
__device__ __forceinline__ float wq(int Q, int q) { return float(lbk::weight_of(Q, q)); }
template <>
__device__ __forceinline__ __half to_storage<__half>(double v, int q, int c, const StepParams& P, int Q) {
  return __float2half_rn((float(v) * (1.0f / wq(Q, q)) - P.rho0[c]) * P.inv_scale[c]);
}

// I16: round((f/w - rho0) / scale), saturated to +-32767
template <>
__device__ __forceinline__ int16_t to_storage<int16_t>(double v, int q, int c, const StepParams& P, int Q) {
  const int h = __float2int_rn((float(v) * (1.0f / wq(Q, q)) - P.rho0[c]) * P.inv_scale[c]);
  return int16_t(h < -32767 ? -32767 : (h > 32767 ? 32767 : h));
}

template <typename T>
__device__ __forceinline__ double from_storage(T v, int q, int c, const StepParams& P, int Q);
template <>
__device__ __forceinline__ double from_storage<double>(double v, int, int, const StepParams&, int) {
  return v;
}
template <>
__device__ __forceinline__ double from_storage<float>(float v, int, int, const StepParams&, int) {
  return double(v);
}
template <>
__device__ __forceinline__ double from_storage<__half>(__half v, int q, int c, const StepParams& P, int Q) {
  return double(wq(Q, q) * fmaf(P.scale[c], __half2float(v), P.rho0[c]));
}
// I16 in double: the sums of a lattice whose integer offsets are conserved
// (the I16 collision conserves every site's mass exactly) then are too, to
// double rounding
template <>
__device__ __forceinline__ double from_storage<int16_t>(int16_t v, int q, int c, const StepParams& P, int Q) {
  return lbk::weight_of(Q, q) * (double(P.rho0[c]) + double(P.scale[c]) * double(v));
}

struct Geo {
  int nx, ny, nz, nxh, nyh, nzh, hy, hz, Q;  // hy, hz: halo in y, z (0 where the lattice has no such axis)
  int64_t n;
};

// AoS haloed staging (haloed x-planes [xh0, xh0 + nplanes)) -> SoA physical
// AoS haloed staging -> SoA physical; with f_solid (and mask), solid sites are
// written into f_solid as well (the fused steps do not write solid sites, so
// both population buffers must hold them)
template <typename T>
__global__ void k_upload(const double* __restrict__ stage, T* __restrict__ f, int c, int xh0, int nplanes, Geo g,
                         StepParams P, T* __restrict__ f_solid = nullptr, const uint8_t* __restrict__ mask = nullptr) {
  const int64_t per_plane = int64_t(g.ny) * g.nz;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= per_plane * nplanes) return;
  const int pl = int(i / per_plane);
  const int64_t r = i - int64_t(pl) * per_plane;
  const int y = int(r / g.nz), z = int(r - int64_t(y) * g.nz);
  const int xh = xh0 + pl;
  const int x = xh - kHalo;
  if (x < 0 || x >= g.nx) return;
  const double* src = stage + ((int64_t(pl) * g.nyh + (y + g.hy)) * g.nzh + (z + g.hz)) * g.Q;
  const int64_t site = (int64_t(x) * g.ny + y) * g.nz + z;
  T* fc = f + int64_t(c) * g.Q * g.n;
  T* fs = (f_solid && mask && mask[site]) ? f_solid + int64_t(c) * g.Q * g.n : nullptr;
  for (int q = 0; q < g.Q; ++q) {
    const T v = to_storage<T>(src[q], q, c, P, g.Q);
    fc[int64_t(q) * g.n + site] = v;
    if (fs) fs[int64_t(q) * g.n + site] = v;
  }
}

// SoA physical -> AoS haloed staging (halo sites get periodic images)
template <typename T>
__global__ void k_download(double* __restrict__ stage, const T* __restrict__ f, int c, int xh0, int nplanes, Geo g,
                           StepParams P) {
  const int64_t per_plane = int64_t(g.nyh) * g.nzh;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= per_plane * nplanes) return;
  const int pl = int(i / per_plane);
  const int64_t r = i - int64_t(pl) * per_plane;
  const int yh = int(r / g.nzh), zh = int(r - int64_t(yh) * g.nzh);
  const int x = ((xh0 + pl - kHalo) % g.nx + g.nx) % g.nx;
  const int y = ((yh - g.hy) % g.ny + g.ny) % g.ny;
  const int z = ((zh - g.hz) % g.nz + g.nz) % g.nz;
  const int64_t site = (int64_t(x) * g.ny + y) * g.nz + z;
  double* dst = stage + i * g.Q;
  const T* fc = f + int64_t(c) * g.Q * g.n;
  for (int q = 0; q < g.Q; ++q) dst[q] = from_storage<T>(fc[int64_t(q) * g.n + site], q, c, P, g.Q);
}

__global__ void k_upload_mask(const int32_t* __restrict__ stage_mask, uint8_t* __restrict__ mask, int xh0,
                              int nplanes, Geo g, int* __restrict__ nsolid) {
  const int64_t per_plane = int64_t(g.ny) * g.nz;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= per_plane * nplanes) return;
  const int pl = int(i / per_plane);
  const int64_t r = i - int64_t(pl) * per_plane;
  const int y = int(r / g.nz), z = int(r - int64_t(y) * g.nz);
  const int x = xh0 + pl - kHalo;
  if (x < 0 || x >= g.nx) return;
  const int v = stage_mask[(int64_t(pl) * g.nyh + (y + g.hy)) * g.nzh + (z + g.hz)];
  mask[(int64_t(x) * g.ny + y) * g.nz + z] = v != 0;
  if (v != 0) atomicAdd(nsolid, 1);
}

// moments in double: density (pairwise sum), raw velocity, colour
template <typename T, int Q>
__global__ void k_moments(const T* __restrict__ f, const uint8_t* __restrict__ mask, int C, Geo g, StepParams P,
                          double* __restrict__ den_out, double* __restrict__ vel_out, double* __restrict__ col_out) {
  constexpr int D = lbk::Conn<Q>::D;
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= g.n) return;
  const bool solid = mask && mask[s];
  double den[2] = {0.0, 0.0};
  for (int c = 0; c < C; ++c) {
    double pop[Q];
    const T* fc = f + int64_t(c) * Q * g.n;
#pragma unroll
    for (int q = 0; q < Q; ++q) pop[q] = from_storage<T>(fc[int64_t(q) * g.n + s], q, c, P, Q);
    den[c] = lbk::density<Q, double>(pop);
    if (den_out) den_out[int64_t(c) * g.n + s] = den[c];
    if (vel_out) {
      const double recip = 1.0 / den[c];
#pragma unroll
      for (int vd = 0; vd < D; ++vd)
        vel_out[(int64_t(c) * g.n + s) * D + vd] = solid ? 0.0 : lbk::moment<Q, double>(pop, vd) * recip;
    }
  }
  if (col_out && C > 1) col_out[s] = solid ? 0.0 : den[0] - den[1];
}

// deterministic reduction: per-block sums in a fixed tree order, then one
// block sums the partials in block order
constexpr int kRedThreads = 256;

template <typename T, int Q>
__global__ void k_reduce_partial(const T* __restrict__ f, const uint8_t* __restrict__ mask, int C, Geo g,
                                 StepParams P, int64_t per_block, double* __restrict__ partial) {
  constexpr int D = lbk::Conn<Q>::D;
  constexpr int NV = 2 * (1 + 3);
  __shared__ double sh[kRedThreads][NV];
  double acc[NV];
  for (int k = 0; k < NV; ++k) acc[k] = 0.0;
  const int64_t s0 = int64_t(blockIdx.x) * per_block;
  const int64_t s1 = min(g.n, s0 + per_block);
  for (int64_t s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
    if (mask && mask[s]) continue;
    for (int c = 0; c < C; ++c) {
      double pop[Q];
      const T* fc = f + int64_t(c) * Q * g.n;
#pragma unroll
      for (int q = 0; q < Q; ++q) pop[q] = from_storage<T>(fc[int64_t(q) * g.n + s], q, c, P, Q);
      acc[c * 4] += lbk::density<Q, double>(pop);
#pragma unroll
      for (int vd = 0; vd < D; ++vd) acc[c * 4 + 1 + vd] += lbk::moment<Q, double>(pop, vd);
    }
  }
  for (int k = 0; k < NV; ++k) sh[threadIdx.x][k] = acc[k];
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < NV; ++k) sh[threadIdx.x][k] += sh[threadIdx.x + w][k];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < NV; ++k) partial[int64_t(blockIdx.x) * NV + k] = sh[0][k];
}

__global__ void k_reduce_final(const double* __restrict__ partial, int nblocks, double* __restrict__ out) {
  constexpr int NV = 8;
  if (threadIdx.x < NV) {
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += partial[int64_t(b) * NV + threadIdx.x];
    out[threadIdx.x] = s;
  }
}

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

Geo geo_of(const lbgpu_handle* h) {
  Geo g;
  g.nx = h->nx;
  g.ny = h->ny;
  g.nz = h->nz;
  g.nxh = h->nxh;
  g.nyh = h->nyh;
  g.nzh = h->nzh;
  g.hy = h->hy;
  g.hz = h->hz;
  g.Q = h->Q;
  g.n = h->n;
  return g;
}

template <typename T>
cudaError_t launch_upload(lbgpu_handle* h, const double* stage, int c, int xh0, int np) {
  const Geo g = geo_of(h);
  const int64_t work = int64_t(g.ny) * g.nz * np;
  k_upload<T><<<unsigned(ceil_div(work, 256)), 256, 0, h->stream>>>(stage, static_cast<T*>(h->f[h->cur]), c, xh0,
                                                                     np, g, h->P);
  h->launches++;
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_download(lbgpu_handle* h, double* stage, int c, int xh0, int np) {
  const Geo g = geo_of(h);
  const int64_t work = int64_t(g.nyh) * g.nzh * np;
  k_download<T><<<unsigned(ceil_div(work, 256)), 256, 0, h->stream>>>(
      stage, static_cast<const T*>(h->f[h->cur]), c, xh0, np, g, h->P);
  h->launches++;
  return cudaGetLastError();
}

// the copy stream and its events (created on first use)
cudaError_t xfer_setup(lbgpu_handle* h) {
  if (h->copy_stream) return cudaSuccess;
  cudaError_t e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking);
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&h->xfer_ev[i], cudaEventDisableTiming);
  return e;
}

// half `buf` of the staging buffer (256-byte aligned halves)
double* stage_half(const lbgpu_handle* h, int buf) {
  const size_t half = (h->staging_bytes / 2) & ~size_t(255);
  return reinterpret_cast<double*>(reinterpret_cast<char*>(h->staging) + size_t(buf) * half);
}

template <typename T>
cudaError_t launch_moments(lbgpu_handle* h, double* den, double* vel, double* col) {
  const Geo g = geo_of(h);
  const unsigned blocks = unsigned(ceil_div(g.n, 128));
  const T* f = static_cast<const T*>(h->f[h->cur]);
  if (h->Q == 19)
    k_moments<T, 19><<<blocks, 128, 0, h->stream>>>(f, h->mask, h->C, g, h->P, den, vel, col);
  else if (h->Q == 9)
    k_moments<T, 9><<<blocks, 128, 0, h->stream>>>(f, h->mask, h->C, g, h->P, den, vel, col);
  else if (h->Q == 5)
    k_moments<T, 5><<<blocks, 128, 0, h->stream>>>(f, h->mask, h->C, g, h->P, den, vel, col);
  else
    k_moments<T, 3><<<blocks, 128, 0, h->stream>>>(f, h->mask, h->C, g, h->P, den, vel, col);
  h->launches++;
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_reduce(lbgpu_handle* h, double* partial, int nblocks, int64_t per_block, double* out) {
  const Geo g = geo_of(h);
  const T* f = static_cast<const T*>(h->f[h->cur]);
  if (h->Q == 19)
    k_reduce_partial<T, 19><<<nblocks, kRedThreads, 0, h->stream>>>(f, h->mask, h->C, g, h->P, per_block, partial);
  else if (h->Q == 9)
    k_reduce_partial<T, 9><<<nblocks, kRedThreads, 0, h->stream>>>(f, h->mask, h->C, g, h->P, per_block, partial);
  else if (h->Q == 5)
    k_reduce_partial<T, 5><<<nblocks, kRedThreads, 0, h->stream>>>(f, h->mask, h->C, g, h->P, per_block, partial);
  else
    k_reduce_partial<T, 3><<<nblocks, kRedThreads, 0, h->stream>>>(f, h->mask, h->C, g, h->P, per_block, partial);
  k_reduce_final<<<1, 32, 0, h->stream>>>(partial, nblocks, out);
  h->launches += 2;
  return cudaGetLastError();
}

int validate(const lbgpu_config* c, std::string* why) {
  if (!c) {
    *why = "null config";
    return LBGPU_E_INVALID;
  }
  if (!((c->d == 3 && c->q == 19) || (c->d == 2 && c->q == 9) || (c->d == 1 && (c->q == 3 || c->q == 5)))) {
    *why = "only D3Q19, D2Q9, D1Q3 and D1Q5 are supported";
    return LBGPU_E_INVALID;
  }
  if (c->components < 1 || c->components > LBGPU_MAX_COMPONENTS) {
    *why = "components must be 1 or 2";
    return LBGPU_E_INVALID;
  }
  for (int i = 0; i < c->d; ++i)
    if (c->gn[i] < 2) {
      *why = "every lattice extent must be >= 2 (the halo of 2 holds periodic images)";
      return LBGPU_E_INVALID;
    }
  int64_t n = 1;
  for (int i = 0; i < c->d; ++i) n *= c->gn[i];
  if (n > (int64_t(1) << 31)) {
    *why = "lattice larger than 2^31 sites";
    return LBGPU_E_INVALID;
  }
  if (c->precision < LBGPU_FP64 || c->precision > LBGPU_I16) {
    *why = "unknown precision";
    return LBGPU_E_INVALID;
  }
  if (c->precision == LBGPU_I16 && !(c->d == 3 && c->q == 19 && c->gn[2] % 2 == 0 && c->eq_form == LBGPU_EQ_BDIST2)) {
    *why = "the I16 form runs D3Q19 lattices with an even z extent and the BDist2 equilibrium";
    return LBGPU_E_INVALID;
  }
  if (c->eq_form < 0 || c->eq_form > 2 || c->psi_form < 0 || c->psi_form > 1) {
    *why = "unknown eqDistForm or psiForm";
    return LBGPU_E_INVALID;
  }
  for (int i = 0; i < c->components; ++i)
    if (!(c->tau[i] > 0.0)) {
      *why = "tau must be positive";
      return LBGPU_E_INVALID;
    }
  return LBGPU_OK;
}

// accumulate the elapsed times of all recorded steps (synchronizes)
cudaError_t fold_kernel_times(lbgpu_handle* h) {
  if (h->ev_pending.empty()) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return e;
  for (auto& se : h->ev_pending) {
    float a = 0.f, b = 0.f;
    cudaEventElapsedTime(&a, se.ev[0], se.ev[1]);
    cudaEventElapsedTime(&b, se.ev[1], se.ev[2]);
    h->kernel_ms[0] += a;
    h->kernel_ms[1] += b;
    h->kernel_n[0]++;
    h->kernel_n[1]++;
    h->ev_pool.push_back(se);
  }
  h->ev_pending.clear();
  return cudaSuccess;
}

}  // namespace

int lb_handle_create(const lbgpu_config* cfg, bool lite, double* staging, size_t staging_bytes,
                     cudaStream_t stream, lbgpu_handle** out, std::string* err) {
  if (!out) return LBGPU_E_INVALID;
  *out = nullptr;
  int rc = validate(cfg, err);
  if (rc) return rc;
  cudaError_t e = cudaSetDevice(cfg->device);
  if (e != cudaSuccess) {
    *err = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
    return LBGPU_E_CUDA;
  }
  lbgpu_handle* h = new lbgpu_handle;
  h->cfg = *cfg;
  h->d = cfg->d;
  h->Q = cfg->q;
  h->C = cfg->components;
  h->nx = cfg->gn[0];
  h->ny = cfg->d >= 2 ? cfg->gn[1] : 1;
  h->nz = cfg->d == 3 ? cfg->gn[2] : 1;
  h->hy = cfg->d >= 2 ? kHalo : 0;
  h->hz = cfg->d == 3 ? kHalo : 0;
  h->nxh = h->nx + 2 * kHalo;
  h->nyh = h->ny + 2 * h->hy;
  h->nzh = h->nz + 2 * h->hz;
  h->n = int64_t(h->nx) * h->ny * h->nz;
  h->lite = lite;
  {
    const char* tk = getenv("LBGPU_TWO_KERNEL");
    // the fused kernel indexes a component's populations with 32-bit offsets
    h->fused = cfg->precision != LBGPU_FP64 && (cfg->q == 19 || (cfg->q == 9 && cfg->precision != LBGPU_I16)) &&
               (cfg->precision == LBGPU_I16 || !(tk && tk[0] == '1' && !lite)) && 19 * h->n < (int64_t(1) << 32);
  }
  if (cfg->precision == LBGPU_I16 && !h->fused) {
    *err = "the I16 form needs fewer than 2^32/19 sites";
    delete h;
    return LBGPU_E_INVALID;
  }
  if (lite && (!h->fused || cfg->q != 19)) {
    *err = "batch members must be FP32/FP16 D3Q19 lattices below 2^32/19 sites";
    delete h;
    return LBGPU_E_INVALID;
  }

  StepParams& P = h->P;
  P.nx = h->nx;
  P.ny = h->ny;
  P.nz = h->nz;
  P.n = h->n;
  P.shan_chen = cfg->shan_chen;
  P.psi_form = cfg->psi_form;
  P.eq_form = cfg->eq_form;
  P.record_force = 0;
  for (int c = 0; c < 2; ++c) {
    const double tau = c < h->C ? cfg->tau[c] : 1.0;
    P.tau[c] = tau;
    P.omega[c] = 1.0 / tau;               // collision.d:99
    P.one_minus_omega[c] = 1.0 - P.omega[c];
    P.gwc[c] = c < h->C ? cfg->gwc[c] : 0.0;
    for (int c2 = 0; c2 < 2; ++c2) P.gcc[c][c2] = (c < h->C && c2 < h->C) ? cfg->gcc[c][c2] : 0.0;
    P.rho0[c] = 0.f;
    P.scale[c] = 1.f;
    P.inv_scale[c] = 1.f;
  }
  for (int i = 0; i < 3; ++i) P.acc[i] = i < cfg->d ? cfg->global_acc[i] : 0.0;
  P.unit_tau = 1;
  for (int c = 0; c < h->C; ++c)
    if (cfg->tau[c] != 1.0) P.unit_tau = 0;

  if (lite) {
    h->stream = stream;
    h->staging = staging;
    h->staging_bytes = staging_bytes;
    h->owns_staging = false;
  } else {
    e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    h->stream = h->own_stream;
    if (e != cudaSuccess) {
      *err = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
      delete h;
      return LBGPU_E_CUDA;
    }
  }
  const size_t fbytes = size_t(h->C) * h->Q * h->n * storage_size(cfg->precision);
  const size_t sbytes = lite ? 0 : size_t(h->C) * h->n * arith_size(cfg->precision);
  const size_t plane_bytes = size_t(h->nyh) * h->nzh * h->Q * sizeof(double);
  if (!lite) h->staging_bytes = std::max(plane_bytes, std::min(kStagingBytes, plane_bytes * h->nxh));
  h->moments_bytes = size_t(h->C) * h->n * sizeof(double);
  void* ptrs[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  const size_t sizes[5] = {fbytes, fbytes, sbytes, sbytes, lite ? 0 : h->staging_bytes};
  for (int i = 0; i < 5; ++i) {
    if (sizes[i] == 0) continue;
    e = cudaMalloc(&ptrs[i], sizes[i]);
    if (e != cudaSuccess) {
      for (int j = 0; j < i; ++j)
        if (ptrs[j]) cudaFree(ptrs[j]);
      if (h->own_stream) cudaStreamDestroy(h->own_stream);
      *err = std::string("device allocation of ") + std::to_string(sizes[i]) + " bytes failed: " +
             cudaGetErrorString(e);
      cudaGetLastError();
      delete h;
      return LBGPU_E_NOMEM;
    }
    h->device_bytes += int64_t(sizes[i]);
  }
  h->f[0] = ptrs[0];
  h->f[1] = ptrs[1];
  h->fbytes = fbytes;
  h->rho = ptrs[2];
  h->psi = ptrs[3];
  if (h->fused && !lite) {
    e = cudaMalloc(&h->work_counter, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(h->work_counter, 0, sizeof(int));
    if (e != cudaSuccess) {
      cudaGetLastError();
      if (h->work_counter) cudaFree(h->work_counter);
      h->work_counter = nullptr;  // static scheduling
    } else {
      h->device_bytes += sizeof(int);
    }
  }
  if (!lite) h->staging = static_cast<double*>(ptrs[4]);
  *out = h;
  return LBGPU_OK;
}

int64_t lb_member_bytes(const lbgpu_config* cfg) {
  int64_t n = 1;
  for (int i = 0; i < cfg->d; ++i) n *= cfg->gn[i];
  // populations (two buffers), mask byte and 32-bit neighbour mask
  return 2 * int64_t(cfg->components) * cfg->q * n * int64_t(storage_size(cfg->precision)) + 5 * n + 1;
}

// Neighbour mask of every site: bit 0 the site's own solid flag, bit q the
// solid flag of x + c_q (periodic), for the fused step's bounce-back, stencil
// and wall-force tests (any connectivity; nz = 1 in 2D, ny = nz = 1 in 1D).
template <int Q>
__global__ void k_nbmask(const uint8_t* __restrict__ mask, uint32_t* __restrict__ nbm, Geo g) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= g.n) return;
  const int64_t yz = int64_t(g.ny) * g.nz;
  const int x = int(s / yz);
  const int64_t r = s - int64_t(x) * yz;
  const int y = int(r / g.nz), z = int(r - int64_t(y) * g.nz);
  uint32_t bits = mask[s] ? 1u : 0u;
#pragma unroll
  for (int q = 1; q < Q; ++q) {
    const int xn = (x + lbk::Conn<Q>::cx(q) + g.nx) % g.nx;
    const int yn = (y + lbk::Conn<Q>::cy(q) + g.ny) % g.ny;
    const int zn = (z + lbk::Conn<Q>::cz(q) + g.nz) % g.nz;
    if (mask[(int64_t(xn) * g.ny + yn) * g.nz + zn]) bits |= 1u << q;
  }
  nbm[s] = bits;
}

// Wall flag of every (x, tile) for the fused step's 8 x 32 tiles: 1 if a
// site of the tile or of its one-site ring in plane x has a nonzero
// neighbour mask.
__global__ void k_tile_walls(const uint32_t* __restrict__ nbm, uint8_t* __restrict__ out, Geo g, int tiles_y,
                             int tiles_z) {
  const int tiles = tiles_y * tiles_z;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= int64_t(g.nx) * tiles) return;
  const int x = int(i / tiles);
  const int tile = int(i - int64_t(x) * tiles);
  const int y0 = (tile / tiles_z) * 8, z0 = (tile % tiles_z) * 32;
  const int tyv = min(8, g.ny - y0), tzv = min(32, g.nz - z0);
  uint32_t any = 0;
  for (int yy = -1; yy <= tyv; ++yy) {
    const int y = (y0 + yy + g.ny) % g.ny;
    for (int zz = -1; zz <= tzv; ++zz) {
      const int z = (z0 + zz + g.nz) % g.nz;
      any |= nbm[(int64_t(x) * g.ny + y) * g.nz + z];
    }
  }
  out[i] = any != 0;
}

// Sets *bad if a site's solid flag differs from "z = 0 or z = nz - 1" (the
// channel's planar walls, which the pair kernel handles on its edge lanes).
__global__ void k_zwall_check(const uint8_t* __restrict__ mask, Geo g, int* __restrict__ bad) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= g.n) return;
  const int z = int(s % g.nz);
  const bool wall = z == 0 || z == g.nz - 1;
  if ((mask[s] != 0) != wall) *bad = 1;
}

int lb_sync_solids(lbgpu_handle* h, int cur, cudaStream_t st) {
  if (!h->mask || !h->fused || h->solids_synced) return LBGPU_OK;
  cudaError_t e = cudaMemcpyAsync(h->f[1 - cur], h->f[cur], h->fbytes, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return h->cuda_fail(e, "solid-site copy");
  h->solids_synced = true;
  return LBGPU_OK;
}

int lb_update_nbmask(lbgpu_handle* h) {
  h->solids_synced = false;  // new populations or a new mask
  // every walled lattice: the two-kernel step reads them too (one 32-bit
  // load per site instead of one mask byte per neighbour)
  const bool want = h->mask != nullptr;
  const int tiles_y = (h->ny + 7) / 8, tiles_z = (h->nz + 31) / 32;
  const int64_t nflags = int64_t(h->nx) * tiles_y * tiles_z;
  // the flags, then (4-byte aligned) the planar-wall check's result
  const int64_t flag_off = (nflags + 3) / 4 * 4, tw_bytes = flag_off + 4;
  h->zwall = false;
  if (!want) {
    if (h->nbmask) {
      cudaFree(h->nbmask);
      h->device_bytes -= 4 * h->n;
      h->nbmask = nullptr;
    }
    if (h->tile_walls) {
      cudaFree(h->tile_walls);
      h->device_bytes -= tw_bytes;
      h->tile_walls = nullptr;
    }
    return LBGPU_OK;
  }
  if (!h->nbmask) {
    cudaError_t e = cudaMalloc(&h->nbmask, size_t(h->n) * sizeof(uint32_t));
    if (e != cudaSuccess) {
      cudaGetLastError();
      h->nbmask = nullptr;
      return h->fail(LBGPU_E_NOMEM, "neighbour mask allocation failed");
    }
    h->device_bytes += 4 * h->n;
  }
  const unsigned nb_blocks = unsigned(ceil_div(h->n, 256));
  if (h->Q == 19)
    k_nbmask<19><<<nb_blocks, 256, 0, h->stream>>>(h->mask, h->nbmask, geo_of(h));
  else if (h->Q == 9)
    k_nbmask<9><<<nb_blocks, 256, 0, h->stream>>>(h->mask, h->nbmask, geo_of(h));
  else if (h->Q == 5)
    k_nbmask<5><<<nb_blocks, 256, 0, h->stream>>>(h->mask, h->nbmask, geo_of(h));
  else
    k_nbmask<3><<<nb_blocks, 256, 0, h->stream>>>(h->mask, h->nbmask, geo_of(h));
  h->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return h->cuda_fail(e, "neighbour mask kernel");
  // the tile wall flags: the D3Q19 one-site fused kernel of a lone lattice
  // (batch members use other tile shapes)
  if (h->Q != 19 || !h->fused || h->lite) return LBGPU_OK;
  if (!h->tile_walls) {
    e = cudaMalloc(&h->tile_walls, size_t(tw_bytes));
    if (e != cudaSuccess) {
      cudaGetLastError();
      h->tile_walls = nullptr;
      return h->fail(LBGPU_E_NOMEM, "tile wall flags allocation failed");
    }
    h->device_bytes += tw_bytes;
  }
  k_tile_walls<<<unsigned(ceil_div(nflags, 128)), 128, 0, h->stream>>>(h->nbmask, h->tile_walls, geo_of(h), tiles_y,
                                                                    tiles_z);
  h->launches++;
  e = cudaGetLastError();
  if (e != cudaSuccess) return h->cuda_fail(e, "tile wall flags kernel");
  // planar z-walls (the pair kernel's walled case)
  {
    int* d_bad = reinterpret_cast<int*>(h->tile_walls + flag_off);
    int bad = 1;
    e = cudaMemsetAsync(d_bad, 0, sizeof(int), h->stream);
    if (e == cudaSuccess) {
      k_zwall_check<<<nb_blocks, 256, 0, h->stream>>>(h->mask, geo_of(h), d_bad);
      h->launches++;
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "planar wall check");
    h->zwall = bad == 0 && h->d == 3 && h->nz >= 4;
  }
  return LBGPU_OK;
}

int lb_ensure_moments(lbgpu_handle* h) {
  if (h->moments) return LBGPU_OK;
  cudaError_t e = cudaMalloc(&h->moments, h->moments_bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    h->moments = nullptr;
    return h->fail(LBGPU_E_NOMEM, "moments scratch allocation failed");
  }
  h->device_bytes += int64_t(h->moments_bytes);
  return LBGPU_OK;
}

extern "C" {

int32_t lbgpu_abi_version(void) { return LBGPU_ABI_VERSION; }

const char* lbgpu_last_error(const lbgpu_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int lbgpu_create(const lbgpu_config* cfg, lbgpu_handle** out) {
  std::string why;
  const int rc = lb_handle_create(cfg, false, nullptr, 0, nullptr, out, &why);
  if (rc) g_create_error = why;
  return rc;
}

void lbgpu_destroy(lbgpu_handle* h) {
  if (!h) return;
  cudaSetDevice(h->cfg.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaFree(h->f[0]);
  cudaFree(h->f[1]);
  if (h->rho) cudaFree(h->rho);
  if (h->psi) cudaFree(h->psi);
  if (h->owns_staging && h->staging) cudaFree(h->staging);
  if (h->moments) cudaFree(h->moments);
  if (h->mask) cudaFree(h->mask);
  if (h->nbmask) cudaFree(h->nbmask);
  if (h->tile_walls) cudaFree(h->tile_walls);
  if (h->work_counter) cudaFree(h->work_counter);
  if (h->force) cudaFree(h->force);
  for (auto& e : h->ev_pending)
    for (auto ev : e.ev) cudaEventDestroy(ev);
  for (auto& e : h->ev_pool)
    for (auto ev : e.ev) cudaEventDestroy(ev);
  if (h->copy_stream) {
    cudaStreamSynchronize(h->copy_stream);
    for (auto ev : h->xfer_ev)
      if (ev) cudaEventDestroy(ev);
    cudaStreamDestroy(h->copy_stream);
  }
  if (h->copy_stream2) {
    cudaStreamSynchronize(h->copy_stream2);
    cudaStreamDestroy(h->copy_stream2);
  }
  for (auto ev : h->pipe_ev)
    if (ev) cudaEventDestroy(ev);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
}

// mask: int32 haloed -> uint8 physical (through the staging buffer, on
// h->stream); dropped when nothing is solid
static int upload_mask(lbgpu_handle* h, const int32_t* mask) {
  cudaError_t e;
  if (mask) {
    if (!h->mask) {
      e = cudaMalloc(&h->mask, size_t(h->n));
      if (e != cudaSuccess) return h->cuda_fail(e, "mask allocation");
      h->device_bytes += h->n;
    }
    // the solid-site counter lives in the last 256 bytes of the staging buffer
    const size_t usable = h->staging_bytes - 256;
    int* d_count = reinterpret_cast<int*>(reinterpret_cast<char*>(h->staging) + usable);
    cudaMemsetAsync(d_count, 0, sizeof(int), h->stream);
    const size_t plane_m = size_t(h->nyh) * h->nzh;
    const int ppc = int(std::max<size_t>(1, usable / (plane_m * sizeof(int32_t))));
    for (int xh0 = 0; xh0 < h->nxh; xh0 += ppc) {
      const int np = std::min(ppc, h->nxh - xh0);
      if (xh0 + np <= kHalo || xh0 >= h->nx + kHalo) continue;
      e = cudaMemcpyAsync(h->staging, mask + size_t(xh0) * plane_m, size_t(np) * plane_m * sizeof(int32_t),
                          cudaMemcpyHostToDevice, h->stream);
      if (e != cudaSuccess) return h->cuda_fail(e, "mask copy");
      const Geo g = geo_of(h);
      const int64_t work = int64_t(g.ny) * g.nz * np;
      k_upload_mask<<<unsigned(ceil_div(work, 256)), 256, 0, h->stream>>>(
          reinterpret_cast<const int32_t*>(h->staging), h->mask, xh0, np, g, d_count);
      h->launches++;
    }
    int nsolid = 0;
    e = cudaMemcpyAsync(&nsolid, d_count, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "mask upload");
    if (nsolid == 0) {
      cudaFree(h->mask);
      h->device_bytes -= h->n;
      h->mask = nullptr;
    }
  } else if (h->mask) {
    cudaFree(h->mask);
    h->device_bytes -= h->n;
    h->mask = nullptr;
  }
  return LBGPU_OK;
}

int lbgpu_upload(lbgpu_handle* h, const double* const* fluids, const int32_t* mask) {
  if (!h || !fluids) return LBGPU_E_INVALID;
  for (int c = 0; c < h->C; ++c)
    if (!fluids[c]) return h->fail(LBGPU_E_INVALID, "null fluid array");
  cudaSetDevice(h->cfg.device);
  cudaError_t e;
  const size_t plane_vals = size_t(h->nyh) * h->nzh * h->Q;

  // FP16 / I16 offset storage: rest density and scale per component (unless
  // the caller pinned them, lbgpu_set_storage_scale)
  if ((h->cfg.precision == LBGPU_FP16 || h->cfg.precision == LBGPU_I16) && !h->scale_pinned) {
    for (int c = 0; c < h->C; ++c) {
      double rho0 = h->cfg.rho0[c];
      double maxdev = 0.0;
      const double* a = fluids[c];
      // mean density and the largest |f_q / w_q - rho0| over physical sites
      double sum = 0.0;
      int64_t cnt = 0;
      for (int x = kHalo; x < h->nx + kHalo; ++x)
        for (int y = h->hy; y < h->ny + h->hy; ++y)
          for (int z = h->hz; z < h->nz + h->hz; ++z) {
            const double* p = a + ((int64_t(x) * h->nyh + y) * h->nzh + z) * h->Q;
            double s = 0.0;
            for (int q = 0; q < h->Q; ++q) s += p[q];
            sum += s;
            ++cnt;
          }
      if (rho0 <= 0.0) rho0 = sum / double(cnt);
      for (int x = kHalo; x < h->nx + kHalo; ++x)
        for (int y = h->hy; y < h->ny + h->hy; ++y)
          for (int z = h->hz; z < h->nz + h->hz; ++z) {
            const double* p = a + ((int64_t(x) * h->nyh + y) * h->nzh + z) * h->Q;
            for (int q = 0; q < h->Q; ++q) {
              const double w = lbk::weight_of(h->Q, q);
              maxdev = std::max(maxdev, fabs(p[q] / w - rho0));
            }
          }
      // half is a floating-point format: every stored offset keeps 11
      // significant bits whatever the scale, which therefore only sets the
      // range.  Offsets up to 64 * max(rho0, 4 * initial spread) stay finite,
      // so phase separation, which moves densities far beyond their initial
      // spread, cannot overflow; offsets below 6e-8 of that lose precision.
      double scale;
      if (h->cfg.precision == LBGPU_FP16) {
        const double span = std::max(fabs(rho0), 4.0 * maxdev);
        scale = span > 0.0 ? span / 1024.0 : 1.0 / 4096.0;
      } else {
        scale = i16_scale(rho0, maxdev);
      }
      h->P.rho0[c] = float(rho0);
      h->P.scale[c] = float(scale);
      h->P.inv_scale[c] = float(1.0 / scale);
    }
  }

  // chunks of whole haloed x-planes through alternating staging halves: the
  // copy of one chunk (copy stream) overlaps the transpose of the previous
  // one (h->stream)
  e = xfer_setup(h);
  if (e != cudaSuccess) return h->cuda_fail(e, "transfer stream");
  const int ppc = int(std::max<size_t>(1, ((h->staging_bytes / 2) & ~size_t(255)) / (plane_vals * sizeof(double))));
  cudaEventRecord(h->xfer_ev[2], h->stream);  // earlier work on the staging buffer
  cudaEventRecord(h->xfer_ev[3], h->stream);
  int k = 0;
  for (int c = 0; c < h->C; ++c) {
    for (int xh0 = 0; xh0 < h->nxh; xh0 += ppc) {
      const int np = std::min(ppc, h->nxh - xh0);
      // only planes that hold physical sites matter
      if (xh0 + np <= kHalo || xh0 >= h->nx + kHalo) continue;
      const int buf = k & 1;
      double* stage = stage_half(h, buf);
      cudaStreamWaitEvent(h->copy_stream, h->xfer_ev[2 + buf], 0);  // the half's previous transpose is done
      e = cudaMemcpyAsync(stage, fluids[c] + size_t(xh0) * plane_vals, size_t(np) * plane_vals * sizeof(double),
                          cudaMemcpyHostToDevice, h->copy_stream);
      if (e != cudaSuccess) return h->cuda_fail(e, "upload copy");
      cudaEventRecord(h->xfer_ev[buf], h->copy_stream);
      cudaStreamWaitEvent(h->stream, h->xfer_ev[buf], 0);
      if (h->cfg.precision == LBGPU_FP64)
        e = launch_upload<double>(h, stage, c, xh0, np);
      else if (h->cfg.precision == LBGPU_FP32)
        e = launch_upload<float>(h, stage, c, xh0, np);
      else if (h->cfg.precision == LBGPU_I16)
        e = launch_upload<int16_t>(h, stage, c, xh0, np);
      else
        e = launch_upload<__half>(h, stage, c, xh0, np);
      if (e != cudaSuccess) return h->cuda_fail(e, "upload kernel");
      cudaEventRecord(h->xfer_ev[2 + buf], h->stream);
      ++k;
    }
  }

  if (int rc = upload_mask(h, mask)) return rc;
  if (int rc = lb_update_nbmask(h)) return rc;
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "upload");
  h->uploaded = true;
  h->force_valid = 0;
  return LBGPU_OK;
}

int lbgpu_set_record_force(lbgpu_handle* h, int32_t enable) {
  if (!h) return LBGPU_E_INVALID;
  cudaSetDevice(h->cfg.device);
  if (enable && !h->force) {
    const size_t bytes = size_t(h->C) * h->n * h->d * sizeof(double);
    cudaError_t e = cudaMalloc(&h->force, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return h->fail(LBGPU_E_NOMEM, "force buffer allocation failed");
    }
    h->device_bytes += int64_t(bytes);
  }
  h->record_force = enable ? 1 : 0;
  return LBGPU_OK;
}

static int run_phase(lbgpu_handle* h, int phase) {
  if (!h) return LBGPU_E_INVALID;
  if (!h->uploaded) return h->fail(LBGPU_E_NOTREADY, "timestep phase before lbgpu_upload");
  if (h->lite || !h->rho) return h->fail(LBGPU_E_INVALID, "batch members step with their batch");
  if (h->cfg.precision == LBGPU_I16)
    return h->fail(LBGPU_E_INVALID, "the I16 form has no split timestep (use lbgpu_step)");
  if (phase == lbk::kPhaseAdvect && h->advected)
    return h->fail(LBGPU_E_NOTREADY, "lbgpu_advect twice: lbgpu_collide completes the timestep");
  if (phase == lbk::kPhaseCollide && !h->advected)
    return h->fail(LBGPU_E_NOTREADY, "lbgpu_collide without lbgpu_advect");
  cudaSetDevice(h->cfg.device);
  lbk::StepBuffers b;
  b.f = h->f[h->cur];
  b.fout = h->f[1 - h->cur];
  b.mask = h->mask;
  b.rho = h->rho;
  b.psi = h->psi;
  b.force = h->force;
  StepParams P = h->P;
  P.record_force = (h->record_force && phase == lbk::kPhaseCollide) ? 1 : 0;
  cudaError_t e;
  if (h->cfg.precision == LBGPU_FP64)
    e = lbk::launch_phase_f64(phase, h->Q, h->C, b, P, h->stream, &h->launches);
  else if (h->cfg.precision == LBGPU_FP32)
    e = lbk::launch_phase_f32(phase, h->Q, h->C, b, P, h->stream, &h->launches);
  else
    e = lbk::launch_phase_f16(phase, h->Q, h->C, b, P, h->stream, &h->launches);
  if (e != cudaSuccess) return h->cuda_fail(e, "phase launch");
  h->cur = 1 - h->cur;
  h->advected = phase == lbk::kPhaseAdvect;
  if (P.record_force) h->force_valid = 1;
  return LBGPU_OK;
}

int lbgpu_advect(lbgpu_handle* h) { return run_phase(h, lbk::kPhaseAdvect); }

int lbgpu_collide(lbgpu_handle* h) { return run_phase(h, lbk::kPhaseCollide); }

int lbgpu_step(lbgpu_handle* h, int32_t nsteps) {
  if (!h || nsteps < 0) return LBGPU_E_INVALID;
  if (!h->uploaded) return h->fail(LBGPU_E_NOTREADY, "lbgpu_step before lbgpu_upload");
  if (h->advected) return h->fail(LBGPU_E_NOTREADY, "lbgpu_step between lbgpu_advect and lbgpu_collide");
  cudaSetDevice(h->cfg.device);
  for (int t = 0; t < nsteps; ++t) {
    lbk::StepBuffers b;
    b.f = h->f[h->cur];
    b.fout = h->f[1 - h->cur];
    b.mask = h->mask;
    b.nbmask = h->nbmask;
    b.tile_walls = h->tile_walls;
    b.zwall = h->zwall ? 1 : 0;
    b.work_counter = h->work_counter;
    b.rho = h->rho;
    b.psi = h->psi;
    b.force = h->force;
    StepParams P = h->P;
    P.record_force = (h->record_force && t == nsteps - 1) ? 1 : 0;
    const lbk::StepEvents* evp = nullptr;
    if (h->profiling) {
      if (h->ev_pending.size() >= 4096) {
        cudaError_t fe = fold_kernel_times(h);
        if (fe != cudaSuccess) return h->cuda_fail(fe, "kernel timing");
      }
      lbk::StepEvents se;
      if (!h->ev_pool.empty()) {
        se = h->ev_pool.back();
        h->ev_pool.pop_back();
      } else {
        for (auto& ev : se.ev) {
          cudaError_t ce = cudaEventCreate(&ev);
          if (ce != cudaSuccess) return h->cuda_fail(ce, "event create");
        }
      }
      h->ev_pending.push_back(se);
      evp = &h->ev_pending.back();
    }
    cudaError_t e;
    if (h->cfg.precision == LBGPU_FP64)
      e = lbk::launch_step_f64(h->Q, h->C, b, P, h->stream, &h->launches, evp);
    else if (h->fused) {
      if (int rc = lb_sync_solids(h, h->cur, h->stream)) return rc;
      e = lbk::launch_fused(storage_kind(h->cfg.precision), h->Q, h->C, b, P, h->stream, &h->launches, evp,
                            h->cfg.device);
    } else if (h->cfg.precision == LBGPU_FP32)
      e = lbk::launch_step_f32(h->Q, h->C, b, P, h->stream, &h->launches, evp);
    else
      e = lbk::launch_step_f16(h->Q, h->C, b, P, h->stream, &h->launches, evp);
    if (e != cudaSuccess) return h->cuda_fail(e, "step launch");
    h->cur = 1 - h->cur;
    if (P.record_force) h->force_valid = 1;
  }
  return LBGPU_OK;
}

int lbgpu_download(lbgpu_handle* h, double* const* fluids) {
  if (!h || !fluids) return LBGPU_E_INVALID;
  if (!h->uploaded) return h->fail(LBGPU_E_NOTREADY, "lbgpu_download before lbgpu_upload");
  cudaSetDevice(h->cfg.device);
  const size_t plane_vals = size_t(h->nyh) * h->nzh * h->Q;
  cudaError_t e = xfer_setup(h);
  if (e != cudaSuccess) return h->cuda_fail(e, "transfer stream");
  // as the upload, in the other direction: the transpose of one chunk
  // (h->stream) overlaps the copy of the previous one (copy stream)
  const int ppc = int(std::max<size_t>(1, ((h->staging_bytes / 2) & ~size_t(255)) / (plane_vals * sizeof(double))));
  int k = 0;
  for (int c = 0; c < h->C; ++c) {
    if (!fluids[c]) continue;
    for (int xh0 = 0; xh0 < h->nxh; xh0 += ppc) {
      const int np = std::min(ppc, h->nxh - xh0);
      const int buf = k & 1;
      double* stage = stage_half(h, buf);
      if (k >= 2) cudaStreamWaitEvent(h->stream, h->xfer_ev[2 + buf], 0);  // the half's previous copy is done
      if (h->cfg.precision == LBGPU_FP64)
        e = launch_download<double>(h, stage, c, xh0, np);
      else if (h->cfg.precision == LBGPU_FP32)
        e = launch_download<float>(h, stage, c, xh0, np);
      else if (h->cfg.precision == LBGPU_I16)
        e = launch_download<int16_t>(h, stage, c, xh0, np);
      else
        e = launch_download<__half>(h, stage, c, xh0, np);
      if (e != cudaSuccess) return h->cuda_fail(e, "download kernel");
      cudaEventRecord(h->xfer_ev[buf], h->stream);
      cudaStreamWaitEvent(h->copy_stream, h->xfer_ev[buf], 0);
      e = cudaMemcpyAsync(fluids[c] + size_t(xh0) * plane_vals, stage, size_t(np) * plane_vals * sizeof(double),
                          cudaMemcpyDeviceToHost, h->copy_stream);
      if (e != cudaSuccess) return h->cuda_fail(e, "download copy");
      cudaEventRecord(h->xfer_ev[2 + buf], h->copy_stream);
      ++k;
    }
  }
  e = cudaStreamSynchronize(h->copy_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "download");
  return LBGPU_OK;
}

// --------------------------------------------------------------------------
// lbgpu_step_host: upload, one timestep and download in one call
// --------------------------------------------------------------------------
namespace {

constexpr int kWavePlanes = 8;  // x-planes per chunk of the wavefront

// the largest |c_x| of the connectivity (D1Q5 reaches x +- 2)
int reach_x(int Q) { return Q == 5 ? 2 : 1; }

cudaError_t wave_setup(lbgpu_handle* h) {
  cudaError_t e = xfer_setup(h);
  if (e == cudaSuccess && !h->copy_stream2) e = cudaStreamCreateWithFlags(&h->copy_stream2, cudaStreamNonBlocking);
  for (int i = 0; i < 9 && e == cudaSuccess; ++i)
    if (!h->pipe_ev[i]) e = cudaEventCreateWithFlags(&h->pipe_ev[i], cudaEventDisableTiming);
  return e;
}

// x-planes per chunk of the wavefront, 0 when the lattice is too small or
// too wide for it (then the call runs upload, step and download in turn)
int wave_planes(const lbgpu_handle* h) {
  const size_t plane_bytes = size_t(h->nyh) * h->nzh * h->Q * sizeof(double);
  const size_t slot_bytes = (h->staging_bytes / 8) & ~size_t(255);
  const int k = int(std::min<size_t>(kWavePlanes, slot_bytes / plane_bytes));
  return (k >= 1 && h->nx >= 2 * k + 4 * reach_x(h->Q)) ? k : 0;
}

// The FP64 timestep as a wavefront over chunks of K x-planes, so that the
// input copies, the kernels and the output copies overlap.  Chunk j (physical
// planes [a, b) of every component): copy_stream copies the whole haloed
// planes into upload slot j % 2 of the staging buffer; h->stream transposes
// them into the population buffer, runs k_density_psi on the planes whose
// x +- R neighbours are now present and k_collide on the planes whose x +- R
// densities are done, and transposes the finished planes into a download
// slot; copy_stream2 copies those to the host.  Planes 0 .. 2R-1 need the
// last planes (periodic wrap) and finish after the last chunk.  The per-site
// arithmetic is lbgpu_step's, so the result is the same bits.  A plane's
// input copy completes before its output copy starts, so `out` may alias
// `in`.  Staging slots: [0, 4) upload (parity, component), [4, 8) download.
// Events: 0 start, 1-2 upload slot filled, 3-4 upload slot free, 5-6
// download slot filled, 7-8 download slot free.
extern "C++" {
template <typename T>
int step_host_wave(lbgpu_handle* h, const double* const* in, double* const* out, int K) {
  const Geo g = geo_of(h);
  const bool fp64 = h->cfg.precision == LBGPU_FP64;
  const size_t plane_vals = size_t(h->nyh) * h->nzh * h->Q;
  const size_t plane_bytes = plane_vals * sizeof(double);
  const int64_t plane_sites = int64_t(h->ny) * h->nz;
  const size_t slot_bytes = (h->staging_bytes / 8) & ~size_t(255);
  auto slot = [&](int k) {
    return reinterpret_cast<double*>(reinterpret_cast<char*>(h->staging) + size_t(k) * slot_bytes);
  };
  cudaEvent_t* ev = h->pipe_ev;
  const int R = reach_x(h->Q);
  const int nx = h->nx;
  T* fin = static_cast<T*>(h->f[h->cur]);
  T* fout = static_cast<T*>(h->f[1 - h->cur]);
  lbk::StepBuffers b;
  b.f = h->f[h->cur];
  b.fout = h->f[1 - h->cur];
  b.mask = h->mask;
  b.nbmask = h->nbmask;
  b.tile_walls = h->tile_walls;
  b.zwall = h->zwall ? 1 : 0;
  b.work_counter = h->work_counter;
  b.rho = h->rho;
  b.psi = h->psi;
  b.force = h->force;
  cudaError_t e;
  // on an error, let the copies already queued finish before returning: the
  // caller may free or reuse its host arrays once the call returns
  auto fail = [&](cudaError_t err, const char* what) {
    cudaStreamSynchronize(h->copy_stream);
    cudaStreamSynchronize(h->stream);
    cudaStreamSynchronize(h->copy_stream2);
    return h->cuda_fail(err, what);
  };

  // work queued earlier on h->stream (the mask upload, moments that use the
  // staging buffer) precedes the copies into the staging buffer
  cudaEventRecord(ev[0], h->stream);
  cudaStreamWaitEvent(h->copy_stream, ev[0], 0);
  cudaStreamWaitEvent(h->copy_stream2, ev[0], 0);

  auto part = [&](int which, int x0, int x1) -> cudaError_t {
    if (x1 <= x0) return cudaSuccess;
    StepParams P = h->P;
    P.record_force = h->record_force ? 1 : 0;
    if (!fp64) {
      // the fused forms: one pair-kernel launch per plane range (it reads
      // planes x0 - 2 .. x1 + 1, those the FP64 collide part needs)
      if (which != lbk::kPartCollide) return cudaSuccess;
      return lbk::launch_fused_range(storage_kind(h->cfg.precision), h->Q, h->C, b, P, x0, x1, h->stream, &h->launches,
                                     h->cfg.device);
    }
    P.s_begin = int64_t(x0) * plane_sites;
    P.s_end = int64_t(x1) * plane_sites;
    return lbk::launch_part_f64(which, h->Q, h->C, b, P, h->stream, &h->launches);
  };
  int nd = 0;  // download chunks queued
  // haloed planes [xh0, xh1), all of them finished
  auto download = [&](int xh0, int xh1) -> cudaError_t {
    for (int a = xh0; a < xh1; a += K) {
      const int np = std::min(K, xh1 - a);
      const int p = nd & 1;
      if (nd >= 2) cudaStreamWaitEvent(h->stream, ev[7 + p], 0);  // the slot's previous copies are done
      const int64_t work = int64_t(g.nyh) * g.nzh * np;
      for (int c = 0; c < h->C; ++c) {
        if (!out[c]) continue;
        k_download<T><<<unsigned(ceil_div(work, 256)), 256, 0, h->stream>>>(slot(4 + 2 * p + c), fout, c, a, np, g,
                                                                             h->P);
        h->launches++;
      }
      cudaError_t le = cudaGetLastError();
      if (le != cudaSuccess) return le;
      cudaEventRecord(ev[5 + p], h->stream);
      cudaStreamWaitEvent(h->copy_stream2, ev[5 + p], 0);
      for (int c = 0; c < h->C; ++c) {
        if (!out[c]) continue;
        le = cudaMemcpyAsync(out[c] + size_t(a) * plane_vals, slot(4 + 2 * p + c), size_t(np) * plane_bytes,
                             cudaMemcpyDeviceToHost, h->copy_stream2);
        if (le != cudaSuccess) return le;
      }
      cudaEventRecord(ev[7 + p], h->copy_stream2);
      ++nd;
    }
    return cudaSuccess;
  };

  int dn = R, cn = 2 * R;  // k_density_psi done on planes [R, dn), k_collide (and download) on [2R, cn)
  int j = 0;
  for (int a = 0; a < nx; a += K, ++j) {
    const int bnd = std::min(nx, a + K);
    const int p = j & 1;
    if (j >= 2) cudaStreamWaitEvent(h->copy_stream, ev[3 + p], 0);  // the slot's previous transposes are done
    for (int c = 0; c < h->C; ++c) {
      e = cudaMemcpyAsync(slot(2 * p + c), in[c] + size_t(a + kHalo) * plane_vals, size_t(bnd - a) * plane_bytes,
                          cudaMemcpyHostToDevice, h->copy_stream);
      if (e != cudaSuccess) return fail(e, "step_host input copy");
    }
    cudaEventRecord(ev[1 + p], h->copy_stream);
    cudaStreamWaitEvent(h->stream, ev[1 + p], 0);
    const int64_t work = plane_sites * (bnd - a);
    for (int c = 0; c < h->C; ++c) {
      k_upload<T><<<unsigned(ceil_div(work, 256)), 256, 0, h->stream>>>(
          slot(2 * p + c), fin, c, a + kHalo, bnd - a, g, h->P, fp64 ? nullptr : fout, fp64 ? nullptr : h->mask);
      h->launches++;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "step_host input transpose");
    cudaEventRecord(ev[3 + p], h->stream);
    const bool last = bnd == nx;
    const int dnew = last ? nx : bnd - R;
    if ((e = part(lbk::kPartDensityPsi, dn, dnew)) != cudaSuccess) return fail(e, "step_host density");
    dn = std::max(dn, dnew);
    if (last && (e = part(lbk::kPartDensityPsi, 0, R)) != cudaSuccess) return fail(e, "step_host density");
    const int cnew = last ? nx : dn - R;
    if ((e = part(lbk::kPartCollide, cn, cnew)) != cudaSuccess) return fail(e, "step_host collide");
    if (!last) {
      if (cnew > cn && (e = download(cn + kHalo, cnew + kHalo)) != cudaSuccess)
        return fail(e, "step_host output");
      cn = std::max(cn, cnew);
    } else {
      if ((e = part(lbk::kPartCollide, 0, 2 * R)) != cudaSuccess) return fail(e, "step_host collide");
      // physical planes [cn, nx) with the images of planes 0 and 1, then the
      // images of planes nx-2 and nx-1 with physical planes [0, 2R)
      if ((e = download(cn + kHalo, nx + 2 * kHalo)) != cudaSuccess) return fail(e, "step_host output");
      if ((e = download(0, 2 * R + kHalo)) != cudaSuccess) return fail(e, "step_host output");
    }
  }
  e = cudaStreamSynchronize(h->copy_stream2);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->copy_stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "step_host");
  h->cur = 1 - h->cur;
  if (h->record_force) h->force_valid = 1;
  return LBGPU_OK;
}
}  // extern "C++"

}  // namespace

int lbgpu_step_host(lbgpu_handle* h, const double* const* fluids_in, const int32_t* mask, double* const* fluids_out) {
  if (!h || !fluids_in || !fluids_out) return LBGPU_E_INVALID;
  for (int c = 0; c < h->C; ++c)
    if (!fluids_in[c]) return h->fail(LBGPU_E_INVALID, "null fluid array");
  if (h->lite || !h->rho) return h->fail(LBGPU_E_INVALID, "batch members step with their batch");
  if (h->advected) return h->fail(LBGPU_E_NOTREADY, "lbgpu_step_host between lbgpu_advect and lbgpu_collide");
  // the wavefront: FP64, and the fused forms (FP16 and I16 once their
  // offsets' scale is pinned: otherwise the upload derives it from the whole
  // input first)
  const bool fused_wave = h->fused && h->work_counter && (h->cfg.precision == LBGPU_FP32 || h->scale_pinned);
  const int K = ((h->cfg.precision == LBGPU_FP64 || fused_wave) && !h->profiling) ? wave_planes(h) : 0;
  if (K == 0) {
    // the other forms, profiled handles and lattices too small for the
    // wavefront: one after another
    if (int rc = lbgpu_upload(h, fluids_in, mask)) return rc;
    if (int rc = lbgpu_step(h, 1)) return rc;
    return lbgpu_download(h, fluids_out);
  }
  cudaSetDevice(h->cfg.device);
  cudaError_t e = wave_setup(h);
  if (e != cudaSuccess) return h->cuda_fail(e, "transfer streams");
  if (int rc = upload_mask(h, mask)) return rc;
  if (int rc = lb_update_nbmask(h)) return rc;
  h->force_valid = 0;
  int rc;
  if (h->cfg.precision == LBGPU_FP64)
    rc = step_host_wave<double>(h, fluids_in, fluids_out, K);
  else if (h->cfg.precision == LBGPU_FP32)
    rc = step_host_wave<float>(h, fluids_in, fluids_out, K);
  else if (h->cfg.precision == LBGPU_FP16)
    rc = step_host_wave<__half>(h, fluids_in, fluids_out, K);
  else
    rc = step_host_wave<int16_t>(h, fluids_in, fluids_out, K);
  if (rc) return rc;
  // the wavefront's upload wrote the solid sites into both buffers
  if (h->fused) h->solids_synced = true;
  h->uploaded = true;
  return LBGPU_OK;
}

int lbgpu_set_storage_scale(lbgpu_handle* h, const double* rho0, const double* scale) {
  if (!h) return LBGPU_E_INVALID;
  if (h->cfg.precision != LBGPU_FP16 && h->cfg.precision != LBGPU_I16)
    return h->fail(LBGPU_E_INVALID, "the storage scale belongs to the FP16 and I16 forms");
  if (!rho0 || !scale) {
    h->scale_pinned = false;
    return LBGPU_OK;
  }
  for (int c = 0; c < h->C; ++c)
    if (!(scale[c] > 0.0) || !std::isfinite(scale[c]) || !std::isfinite(rho0[c]))
      return h->fail(LBGPU_E_INVALID, "the storage scale must be positive and finite");
  if (h->uploaded)
    return h->fail(LBGPU_E_INVALID, "pin the storage scale before the first upload (the stored offsets use it)");
  for (int c = 0; c < h->C; ++c) {
    h->P.rho0[c] = float(rho0[c]);
    h->P.scale[c] = float(scale[c]);
    h->P.inv_scale[c] = float(1.0 / scale[c]);
  }
  h->scale_pinned = true;
  return LBGPU_OK;
}

int lbgpu_moments(lbgpu_handle* h, double* const* density, double* const* velocity, double* colour) {
  if (!h) return LBGPU_E_INVALID;
  if (!h->uploaded) return h->fail(LBGPU_E_NOTREADY, "lbgpu_moments before lbgpu_upload");
  cudaSetDevice(h->cfg.device);
  if (int rc = lb_ensure_moments(h)) return rc;
  // densities go through the moments buffer (C*N doubles), velocities
  // through a temporary stream-ordered device buffer (C*N*d doubles)
  cudaError_t e;
  const size_t n = size_t(h->n);
  // densities (and colour) first
  const bool want_den = density != nullptr || colour != nullptr;
  if (want_den) {
    // the colour goes through the staging buffer when N doubles fit in it,
    // else it is formed on the host from the densities
    double* col = h->staging;
    const bool col_fits = h->staging_bytes >= n * sizeof(double);
    std::vector<double> tmp;
    double* dcol = (colour && h->C > 1 && col_fits) ? col : nullptr;
    if (h->cfg.precision == LBGPU_FP64)
      e = launch_moments<double>(h, h->moments, nullptr, dcol);
    else if (h->cfg.precision == LBGPU_FP32)
      e = launch_moments<float>(h, h->moments, nullptr, dcol);
    else if (h->cfg.precision == LBGPU_I16)
      e = launch_moments<int16_t>(h, h->moments, nullptr, dcol);
    else
      e = launch_moments<__half>(h, h->moments, nullptr, dcol);
    if (e != cudaSuccess) return h->cuda_fail(e, "moments kernel");
    if (density)
      for (int c = 0; c < h->C; ++c)
        if (density[c]) {
          e = cudaMemcpyAsync(density[c], h->moments + size_t(c) * n, n * sizeof(double), cudaMemcpyDeviceToHost,
                              h->stream);
          if (e != cudaSuccess) return h->cuda_fail(e, "density copy");
        }
    if (colour && h->C > 1) {
      if (dcol) {
        e = cudaMemcpyAsync(colour, dcol, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
        if (e != cudaSuccess) return h->cuda_fail(e, "colour copy");
      } else {
        // colour = rho0 - rho1 on fluid sites from the densities
        tmp.resize(2 * n);
        e = cudaMemcpyAsync(tmp.data(), h->moments, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return h->cuda_fail(e, "colour copy");
        std::vector<uint8_t> m;
        if (h->mask) {
          m.resize(n);
          e = cudaMemcpy(m.data(), h->mask, n, cudaMemcpyDeviceToHost);
          if (e != cudaSuccess) return h->cuda_fail(e, "mask copy");
        }
        for (size_t i = 0; i < n; ++i) colour[i] = (h->mask && m[i]) ? 0.0 : tmp[i] - tmp[n + i];
      }
    }
    e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "moments");
  }
  if (velocity) {
    // d doubles per site per component do not fit the moments buffer (C*N
    // doubles): one kernel writes them into a temporary device buffer
    double* dvel = nullptr;
    const size_t vbytes = size_t(h->C) * n * h->d * sizeof(double);
    e = cudaMallocAsync(reinterpret_cast<void**>(&dvel), vbytes, h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "velocity buffer");
    if (h->cfg.precision == LBGPU_FP64)
      e = launch_moments<double>(h, nullptr, dvel, nullptr);
    else if (h->cfg.precision == LBGPU_FP32)
      e = launch_moments<float>(h, nullptr, dvel, nullptr);
    else if (h->cfg.precision == LBGPU_I16)
      e = launch_moments<int16_t>(h, nullptr, dvel, nullptr);
    else
      e = launch_moments<__half>(h, nullptr, dvel, nullptr);
    if (e != cudaSuccess) return h->cuda_fail(e, "velocity kernel");
    for (int c = 0; c < h->C; ++c)
      if (velocity[c]) {
        e = cudaMemcpyAsync(velocity[c], dvel + size_t(c) * n * h->d, n * h->d * sizeof(double),
                            cudaMemcpyDeviceToHost, h->stream);
        if (e != cudaSuccess) return h->cuda_fail(e, "velocity copy");
      }
    cudaFreeAsync(dvel, h->stream);
    e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "velocity");
  }
  return LBGPU_OK;
}

int lbgpu_force(lbgpu_handle* h, double* const* force) {
  if (!h || !force) return LBGPU_E_INVALID;
  if (!h->force || !h->force_valid)
    return h->fail(LBGPU_E_NOTREADY, "no recorded force: call lbgpu_set_record_force(h, 1) before lbgpu_step");
  cudaSetDevice(h->cfg.device);
  const size_t per = size_t(h->n) * h->d;
  for (int c = 0; c < h->C; ++c)
    if (force[c]) {
      cudaError_t e = cudaMemcpyAsync(force[c], h->force + size_t(c) * per, per * sizeof(double),
                                      cudaMemcpyDeviceToHost, h->stream);
      if (e != cudaSuccess) return h->cuda_fail(e, "force copy");
    }
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "force");
  return LBGPU_OK;
}

int lbgpu_reduce(lbgpu_handle* h, double* mass, double* momentum) {
  if (!h) return LBGPU_E_INVALID;
  if (!h->uploaded) return h->fail(LBGPU_E_NOTREADY, "lbgpu_reduce before lbgpu_upload");
  cudaSetDevice(h->cfg.device);
  if (int rc = lb_ensure_moments(h)) return rc;
  const int nblocks = int(std::min<int64_t>(1024, ceil_div(h->n, kRedThreads)));
  const int64_t per_block = ceil_div(h->n, nblocks);
  double* partial = h->moments;             // nblocks*8 doubles <= C*N doubles
  double* out = h->moments + size_t(nblocks) * 8;
  if (size_t(nblocks) * 8 + 8 > h->moments_bytes / sizeof(double))
    return h->fail(LBGPU_E_INVALID, "lattice too small for the reduction scratch");
  cudaError_t e;
  if (h->cfg.precision == LBGPU_FP64)
    e = launch_reduce<double>(h, partial, nblocks, per_block, out);
  else if (h->cfg.precision == LBGPU_FP32)
    e = launch_reduce<float>(h, partial, nblocks, per_block, out);
  else if (h->cfg.precision == LBGPU_I16)
    e = launch_reduce<int16_t>(h, partial, nblocks, per_block, out);
  else
    e = launch_reduce<__half>(h, partial, nblocks, per_block, out);
  if (e != cudaSuccess) return h->cuda_fail(e, "reduce kernel");
  double res[8];
  e = cudaMemcpyAsync(res, out, sizeof res, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "reduce");
  for (int c = 0; c < h->C && c < 2; ++c) {
    if (mass) mass[c] = res[c * 4];
    if (momentum)
      for (int vd = 0; vd < h->d && vd < 3; ++vd) momentum[c * h->d + vd] = res[c * 4 + 1 + vd];
  }
  return LBGPU_OK;
}

int lbgpu_synchronize(lbgpu_handle* h) {
  if (!h) return LBGPU_E_INVALID;
  cudaSetDevice(h->cfg.device);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "synchronize");
  return LBGPU_OK;
}

int lbgpu_set_stream(lbgpu_handle* h, void* stream) {
  if (!h) return LBGPU_E_INVALID;
  cudaSetDevice(h->cfg.device);
  cudaError_t e = fold_kernel_times(h);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "set_stream");
  h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
  return LBGPU_OK;
}

int lbgpu_profile(lbgpu_handle* h, int32_t enable) {
  if (!h) return LBGPU_E_INVALID;
  cudaSetDevice(h->cfg.device);
  cudaError_t e = fold_kernel_times(h);
  if (e != cudaSuccess) return h->cuda_fail(e, "profile");
  h->profiling = enable != 0;
  h->kernel_ms[0] = h->kernel_ms[1] = 0.0;
  h->kernel_n[0] = h->kernel_n[1] = 0;
  return LBGPU_OK;
}

int lbgpu_kernel_time(lbgpu_handle* h, int32_t which, double* total_ms, int64_t* launches) {
  if (!h || which < 0 || which > 1) return LBGPU_E_INVALID;
  cudaSetDevice(h->cfg.device);
  cudaError_t e = fold_kernel_times(h);
  if (e != cudaSuccess) return h->cuda_fail(e, "kernel_time");
  if (total_ms) *total_ms = h->kernel_ms[which];
  if (launches) *launches = h->kernel_n[which];
  return LBGPU_OK;
}

int64_t lbgpu_launch_count(const lbgpu_handle* h) { return h ? h->launches : 0; }
int64_t lbgpu_device_bytes(const lbgpu_handle* h) { return h ? h->device_bytes : 0; }

}  // extern "C"
