// Device-side initial fields (lbgpu_init_fields, lbgpu_batch_add_init).
//
// Restates, per physical site of one process, initMask (src/dlbc/lb/mask.d:134-172)
// and initFluid (src/dlbc/lb/init.d:263-339) with the field initialisers of
// src/dlbc/fields/init.d: initEqDistSphere :84-103, initEqDistSphereFrac
// :105-126, initEqDistTwoSpheres(Frac) :129-182, initEqDistCylinder(Frac)
// :184-234, initEqDistLamellae(Frac) :236-274 with symmetricLinearTransition
// :346-366, initPlates/Tube/Box/Walls :377-467 and initEqDistWall :469-477.
// Compiled with -fmad=false: the double arithmetic is the reference's, so
// the deterministic initialisers give the reference's values bit for bit.
// The random initialisers draw either the reference's sequence (Mt19937,
// generated on the host in the reference's order and copied to the device,
// lbgpu_init.rng = 1) or from a counter-based generator (splitmix64 of
// seed, component, population and site).
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/lbgpu.h"
#include "lb_core.cuh"
#include "lb_draws.h"
#include "lb_handle.h"

namespace {

struct InitDev {
  int d, Q, C;
  int nx, ny, nz;
  int fluid_init[2];
  int n_dens[2];
  double dens[2][8];
  double perturb[2];
  unsigned long long seed;
  double R[2];
  double off[2][3];
  double sep[2][3];
  int axis;
  double thick;
  int n_if[2];
  double interfaces[2][9];
  int mask_init, mask_axis, wall_offset, wall_thickness;
  int dhw[3][2];
  double eqpop[19];
  // the reference's draws of component c for the physical sites ([site]
  // or, ConstRandom, [site][q]; null: counter-based draws)
  const uint32_t* draws[2];
};

enum {
  kNone, kFile, kConst, kEqDist, kEqDistPerturb, kEqDistPerturbFrac, kConstRandom, kEqDistRandom, kEqDistSphere,
  kEqDistSphereFrac, kEqDistCylinder, kEqDistCylinderFrac, kEqDistTwoSpheres, kEqDistTwoSpheresFrac,
  kEqDistLamellae, kEqDistLamellaeFrac
};

__device__ __forceinline__ uint32_t hash_u32(unsigned long long seed, int c, int q, int64_t site) {
  // splitmix64 (Steele, Lea, Flood: "Fast splittable pseudorandom number generators", 2014)
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(site * 64 + c * 32 + q + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return uint32_t(z >> 32);
}

// draw q (0 unless ConstRandom) of component c at physical site `site`
__device__ __forceinline__ uint32_t draw_u32(const InitDev& I, int c, int q, int64_t site) {
  if (I.draws[c]) return I.draws[c][I.fluid_init[c] == kConstRandom ? site * I.Q + q : site];
  return hash_u32(I.seed, c, q, site);
}

// std.random.uniform!"[)"(a, b) with a 32-bit draw u
__device__ __forceinline__ double uniform_ab(uint32_t u, double a, double b) {
  const double bb = nextafter(b, -INFINITY);
  return a + (bb - a) * double(u) / 4294967295.0;
}

__device__ __forceinline__ double slt(double pos, double width, double negval, double posval) {
  if (width == 0.0) return pos < 0 ? negval : posval;
  if (pos < -0.5 * width) return negval;
  if (pos > 0.5 * width) return posval;
  return negval * (0.5 - pos / width) + posval * (0.5 + pos / width);
}

__device__ bool site_solid(const InitDev& I, const int g[3]) {
  const int n[3] = {I.nx, I.ny, I.nz};
  switch (I.mask_init) {
    case 2: {  // Plates
      const int a = I.mask_axis;
      return g[a] == I.wall_offset || g[a] == n[a] - 1 - I.wall_offset;
    }
    case 3:
    case 4: {  // Tube, Box
      bool s = false;
      for (int vd = 0; vd < I.d; ++vd) {
        if (I.mask_init == 3 && vd == I.mask_axis) continue;
        if (g[vd] == 0 || g[vd] == n[vd] - 1) s = true;
      }
      return s;
    }
    case 5: {  // Walls
      bool s = false;
      for (int vd = 0; vd < I.d; ++vd) {
        if (I.dhw[vd][0] && g[vd] < I.wall_thickness) s = true;
        if (I.dhw[vd][1] && g[vd] >= n[vd] - I.wall_thickness) s = true;
      }
      return s;
    }
    default:
      return false;
  }
}

// populations of component c at site g (physical coordinates)
__device__ void site_pops(const InitDev& I, int c, const int g[3], int64_t site, bool solid, double* pop) {
  const int Q = I.Q, d = I.d;
  if (solid) {
    pop[0] = 1.0;
    for (int q = 1; q < Q; ++q) pop[q] = 0.0;
    return;
  }
  const int fi = I.fluid_init[c];
  const double* dens = I.dens[c];
  const int n[3] = {I.nx, I.ny, I.nz};
  double val = 0.0;
  switch (fi) {
    case kConst:
      for (int q = 0; q < Q; ++q) pop[q] = dens[0];
      return;
    case kConstRandom:
      for (int q = 0; q < Q; ++q) pop[q] = dens[0] * uniform_ab(draw_u32(I, c, q, site), 0.0, 2.0);
      return;
    case kEqDist:
      val = dens[0];
      break;
    case kEqDistRandom:
      val = dens[0] * uniform_ab(draw_u32(I, c, 0, site), 0.0, 2.0);
      break;
    case kEqDistPerturb:
      val = dens[0] + uniform_ab(draw_u32(I, c, 0, site), -I.perturb[c], I.perturb[c]);
      break;
    case kEqDistPerturbFrac:
      val = dens[0] * (1.0 + uniform_ab(draw_u32(I, c, 0, site), -I.perturb[c], I.perturb[c]));
      break;
    case kEqDistSphere:
    case kEqDistSphereFrac:
    case kEqDistCylinder:
    case kEqDistCylinderFrac:
    case kEqDistTwoSpheres:
    case kEqDistTwoSpheresFrac: {
      const bool two = fi == kEqDistTwoSpheres || fi == kEqDistTwoSpheresFrac;
      const bool cyl = fi == kEqDistCylinder || fi == kEqDistCylinderFrac;
      double s1 = 0.0, s2 = 0.0;
      for (int i = 0; i < d; ++i) {
        const double gi = double(g[i]);
        const double centre = double(n[i]) * 0.5;
        if (two) {
          const double o1 = gi - (centre + I.off[c][i] - 0.5 * I.sep[c][i]) + 0.5;
          const double o2 = gi - (centre + I.off[c][i] + 0.5 * I.sep[c][i]) + 0.5;
          s1 = s1 + o1 * o1;
          s2 = s2 + o2 * o2;
        } else {
          const double o = (cyl && i == I.axis) ? 0.0 : gi - (centre + I.off[c][i]) + 0.5;
          s1 = s1 + o * o;
        }
      }
      double relpos = sqrt(s1) - I.R[c];
      if (two) {
        const double r2 = sqrt(s2) - I.R[c];
        relpos = r2 < relpos ? r2 : relpos;
      }
      val = slt(relpos, I.thick, dens[0], dens[1]);
      break;
    }
    case kEqDistLamellae:
    case kEqDistLamellaeFrac: {
      const double gp = double(g[I.axis]);
      const int nif = I.n_if[c];
      int ci = 0;
      double mind = fabs(I.interfaces[c][0] - gp);
      for (int i = 1; i < nif; ++i) {
        const double df = fabs(I.interfaces[c][i] - gp);
        if (df < mind) {
          mind = df;
          ci = i;
        }
      }
      const double minDiff = gp - I.interfaces[c][ci];
      const int nv = I.n_dens[c];
      if (ci == 0)
        val = slt(minDiff, I.thick, dens[nv - 1], dens[0]);
      else if (ci == nv)
        val = slt(minDiff, I.thick, dens[ci - 1], dens[0]);
      else
        val = slt(minDiff, I.thick, dens[ci - 1], dens[ci]);
      break;
    }
    default:  // None: never-initialised populations are NaN in the reference
      for (int q = 0; q < Q; ++q) pop[q] = NAN;
      return;
  }
  for (int q = 0; q < Q; ++q) pop[q] = val * I.eqpop[q];
}

__device__ __forceinline__ void site_coords(int64_t s, int ny, int nz, int g[3]) {
  const int64_t t = s / nz;
  g[2] = int(s - t * nz);
  g[0] = int(t / ny);
  g[1] = int(t - int64_t(g[0]) * ny);
}

constexpr int kInitThreads = 256;

// per-block partial sums of every component's site densities (pass 1) or
// maxima of |f_q/w_q - rho0_c| (pass 2) for the FP16 offsets
__global__ void k_init_stats(InitDev I, int64_t n, int pass, const double* __restrict__ rho0,
                             double* __restrict__ partial) {
  __shared__ double sh[kInitThreads][2];
  double acc[2] = {0.0, 0.0};
  for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < n; s += int64_t(gridDim.x) * blockDim.x) {
    int g[3];
    site_coords(s, I.ny, I.nz, g);
    const bool solid = site_solid(I, g);
    for (int c = 0; c < I.C; ++c) {
      double pop[19];
      site_pops(I, c, g, s, solid, pop);
      if (pass == 1) {
        double r = 0.0;
        for (int q = 0; q < I.Q; ++q) r += pop[q];
        acc[c] += r;
      } else {
        for (int q = 0; q < I.Q; ++q) {
          const double w = lbk::weight_of(I.Q, q);
          acc[c] = fmax(acc[c], fabs(pop[q] / w - rho0[c]));
        }
      }
    }
  }
  sh[threadIdx.x][0] = acc[0];
  sh[threadIdx.x][1] = acc[1];
  __syncthreads();
  for (int w = kInitThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int c = 0; c < 2; ++c)
        sh[threadIdx.x][c] = pass == 1 ? sh[threadIdx.x][c] + sh[threadIdx.x + w][c]
                                       : fmax(sh[threadIdx.x][c], sh[threadIdx.x + w][c]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[blockIdx.x * 2] = sh[0][0];
    partial[blockIdx.x * 2 + 1] = sh[0][1];
  }
}

template <typename T>
__device__ __forceinline__ T encode(double v, int Q, int q, int c, const StepParams& P);
template <>
__device__ __forceinline__ double encode<double>(double v, int, int, int, const StepParams&) {
  return v;
}
template <>
__device__ __forceinline__ float encode<float>(double v, int, int, int, const StepParams&) {
  return float(v);
}
template <>
__device__ __forceinline__ __half encode<__half>(double v, int Q, int q, int c, const StepParams& P) {
  const float w = float(lbk::weight_of(Q, q));
  return __float2half_rn((float(v) * (1.0f / w) - P.rho0[c]) * P.inv_scale[c]);
}

template <>
__device__ __forceinline__ int16_t encode<int16_t>(double v, int Q, int q, int c, const StepParams& P) {
  const float w = float(lbk::weight_of(Q, q));
  const int h = __float2int_rn((float(v) * (1.0f / w) - P.rho0[c]) * P.inv_scale[c]);
  return int16_t(h < -32767 ? -32767 : (h > 32767 ? 32767 : h));
}

template <typename T>
__global__ void k_init_write(InitDev I, int64_t n, StepParams P, T* __restrict__ f, uint8_t* __restrict__ mask,
                             int* __restrict__ nsolid) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int g[3];
  site_coords(s, I.ny, I.nz, g);
  const bool solid = site_solid(I, g);
  if (mask) mask[s] = solid;
  if (solid) atomicAdd(nsolid, 1);
  for (int c = 0; c < I.C; ++c) {
    double pop[19];
    site_pops(I, c, g, s, solid, pop);
    T* fc = f + int64_t(c) * I.Q * n;
    for (int q = 0; q < I.Q; ++q) fc[int64_t(q) * n + s] = encode<T>(pop[q], I.Q, q, c, P);
  }
}

// host-side resolution of the Frac forms and the lamellae interfaces
// (initEqDist*Frac, calculateInterfaces src/dlbc/fields/init.d:335-344)
int build_init(const lbgpu_handle* h, const lbgpu_init* ini, InitDev* I, std::string* err) {
  memset(I, 0, sizeof *I);
  I->d = h->d;
  I->Q = h->Q;
  I->C = h->C;
  I->nx = h->nx;
  I->ny = h->ny;
  I->nz = h->nz;
  const int gsz[3] = {h->nx, h->ny, h->nz};
  int small = gsz[0];
  for (int i = 0; i < h->d; ++i) small = std::min(small, gsz[i]);
  I->seed = ini->seed;
  I->axis = ini->init_axis;
  I->thick = ini->interface_thickness;
  I->mask_init = ini->mask_init;
  I->mask_axis = ini->mask_axis;
  I->wall_offset = ini->wall_offset;
  I->wall_thickness = ini->wall_thickness;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 2; ++j) I->dhw[i][j] = ini->dimension_has_wall[i][j];
  if (ini->mask_init == 1) {
    *err = "maskInit = File is a host-side initialiser: use lbgpu_upload";
    return LBGPU_E_INVALID;
  }
  if (ini->mask_init < 0 || ini->mask_init > 5) {
    *err = "unknown maskInit";
    return LBGPU_E_INVALID;
  }
  for (int c = 0; c < h->C; ++c) {
    const int fi = ini->fluid_init[c];
    if (fi == kFile || fi < 0 || fi > kEqDistLamellaeFrac) {
      *err = "fluidInit = File (or an unknown value) is not a device-side initialiser";
      return LBGPU_E_INVALID;
    }
    I->fluid_init[c] = fi;
    I->n_dens[c] = std::max(1, std::min(8, ini->n_densities[c]));
    for (int j = 0; j < 8; ++j) I->dens[c][j] = ini->densities[c][j];
    I->perturb[c] = ini->perturb[c];
    I->R[c] = ini->init_radius;
    for (int i = 0; i < 3; ++i) {
      I->off[c][i] = ini->init_offset[i];
      I->sep[c][i] = ini->init_separation[i];
    }
    if (fi == kEqDistSphereFrac || fi == kEqDistTwoSpheresFrac) {
      I->R[c] = ini->init_radius * double(small);
      for (int i = 0; i < h->d; ++i) {
        I->off[c][i] = ini->init_offset[i] * double(gsz[i]);
        I->sep[c][i] = ini->init_separation[i] * double(gsz[i]);
      }
    }
    if (fi == kEqDistCylinderFrac) {
      int ss = 0;
      for (int vd = 0; vd < h->d; ++vd)
        if (vd != ini->init_axis && (gsz[vd] < ss || ss == 0)) ss = gsz[vd];
      I->R[c] = ini->init_radius * double(ss);
      for (int i = 0; i < h->d; ++i) I->off[c][i] = ini->init_offset[i] * double(gsz[i]);
    }
    if (fi == kEqDistLamellae || fi == kEqDistLamellaeFrac) {
      if (ini->n_lamellae < 1 || ini->n_lamellae > 8 || ini->n_lamellae != I->n_dens[c] ||
          ini->init_axis < 0 || ini->init_axis >= h->d) {
        *err = "lamellae need 1..8 widths, one density per lamella and an axis of the lattice";
        return LBGPU_E_INVALID;
      }
      double v[9];
      v[0] = 0.0;
      for (int i = 0; i < ini->n_lamellae; ++i)
        v[i + 1] = fi == kEqDistLamellaeFrac ? ini->lamellae_widths[i] * double(gsz[ini->init_axis])
                                             : ini->lamellae_widths[i];
      for (int i = 1; i <= ini->n_lamellae; ++i) v[i] += v[i - 1];
      for (int i = 0; i <= ini->n_lamellae; ++i) I->interfaces[c][i] = v[i] - 0.5;
      I->n_if[c] = ini->n_lamellae + 1;
    }
  }
  // eqDistUnity (eqdist.d:310-315): the weights, except BDist2 on D2Q9
  for (int q = 0; q < h->Q; ++q)
    I->eqpop[q] = lbk::weight_of(h->Q, q);
  // eqDistUnity of BDist2: D1Q3/D1Q5 return the population itself (1, 0, ...)
  if ((h->Q == 3 || h->Q == 5) && h->cfg.eq_form == LBGPU_EQ_BDIST2)
    for (int q = 0; q < h->Q; ++q) I->eqpop[q] = q == 0 ? 1.0 : 0.0;
  if (h->Q == 9 && h->cfg.eq_form == LBGPU_EQ_BDIST2) {
    const double aN1 = 1.0 / 24.0;
    I->eqpop[0] = 0.5;
    for (int q = 1; q < 5; ++q) I->eqpop[q] = 2.0 * aN1;
    for (int q = 5; q < 9; ++q) I->eqpop[q] = aN1;
  }
  return LBGPU_OK;
}

bool random_init(int fi) {
  return fi == kEqDistPerturb || fi == kEqDistPerturbFrac || fi == kConstRandom || fi == kEqDistRandom;
}

// Device copies of the reference's draws, freed with the initialisation
struct ReferenceDraws {
  uint32_t* d[2] = {nullptr, nullptr};
  ~ReferenceDraws() {
    for (uint32_t* p : d)
      if (p) cudaFree(p);
  }
};

// The reference's draws of the random components (lb_draws.h), copied to
// the device
int make_reference_draws(lbgpu_handle* h, const lbgpu_init* ini, ReferenceDraws* out, InitDev* I) {
  lbk::DrawSpec S;
  S.n[0] = h->nx;
  S.n[1] = h->ny;
  S.n[2] = h->nz;
  S.halo[0] = kHalo;
  S.halo[1] = h->hy;
  S.halo[2] = h->hz;
  for (int i = 0; i < 3; ++i) S.nc[i] = (i < h->d && ini->nc[i] > 0) ? ini->nc[i] : 1;
  S.seed = uint32_t(ini->seed);
  S.shift_seed_by_rank = ini->shift_seed_by_rank != 0;
  S.components = h->C;
  bool any = false;
  for (int c = 0; c < h->C; ++c) {
    const int fi = ini->fluid_init[c];
    S.per_site[c] = !random_init(fi) ? 0 : (fi == kConstRandom ? h->Q : 1);
    S.reseed[c] = ini->random_reseed[c] != 0;
    S.random_seed[c] = uint32_t(ini->random_seed[c]);
    any = any || S.per_site[c] != 0;
  }
  if (!any) return LBGPU_OK;
  std::vector<uint32_t> host[2];
  if (!lbk::reference_draws(S, host))
    return h->fail(LBGPU_E_INVALID, "the lattice does not divide evenly over lbgpu_init.nc");
  for (int c = 0; c < h->C; ++c) {
    if (host[c].empty()) continue;
    const size_t bytes = host[c].size() * sizeof(uint32_t);
    cudaError_t e = cudaMalloc(&out->d[c], bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      out->d[c] = nullptr;
      return h->fail(LBGPU_E_NOMEM, "no device memory for the initialiser's random draws");
    }
    e = cudaMemcpyAsync(out->d[c], host[c].data(), bytes, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "initialiser draws");
    I->draws[c] = out->d[c];
  }
  return LBGPU_OK;
}

int reduce_stats(lbgpu_handle* h, const InitDev& I, int pass, const double* d_rho0, double* d_partial, int nblocks,
                 double out[2], bool is_max) {
  k_init_stats<<<nblocks, kInitThreads, 0, h->stream>>>(I, h->n, pass, d_rho0, d_partial);
  h->launches++;
  std::vector<double> part(size_t(nblocks) * 2);
  cudaError_t e = cudaMemcpyAsync(part.data(), d_partial, part.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                  h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "init statistics");
  out[0] = out[1] = 0.0;
  for (int b = 0; b < nblocks; ++b)
    for (int c = 0; c < 2; ++c)
      out[c] = is_max ? std::max(out[c], part[size_t(b) * 2 + c]) : out[c] + part[size_t(b) * 2 + c];
  return LBGPU_OK;
}

}  // namespace

extern "C" int lbgpu_init_fields(lbgpu_handle* h, const lbgpu_init* ini) {
  if (!h || !ini) return LBGPU_E_INVALID;
  cudaSetDevice(h->cfg.device);
  InitDev I;
  std::string why;
  if (int rc = build_init(h, ini, &I, &why)) return h->fail(rc, why);
  if (ini->rng != 0 && ini->rng != 1) return h->fail(LBGPU_E_INVALID, "lbgpu_init.rng must be 0 or 1");
  ReferenceDraws draws;
  if (ini->rng == 1)
    if (int rc = make_reference_draws(h, ini, &draws, &I)) return rc;
  cudaError_t e;
  // the solid-site counter and the statistics partials use the staging buffer
  const int nblocks = int(std::max<size_t>(1, std::min<size_t>(512, (h->staging_bytes / sizeof(double) - 8) / 2)));
  double* d_partial = h->staging;
  double* d_rho0 = h->staging + size_t(nblocks) * 2;
  int* d_count = reinterpret_cast<int*>(h->staging + size_t(nblocks) * 2 + 2);
  if ((h->cfg.precision == LBGPU_FP16 || h->cfg.precision == LBGPU_I16) && !h->scale_pinned) {
    double sums[2], maxdev[2];
    if (int rc = reduce_stats(h, I, 1, d_rho0, d_partial, nblocks, sums, false)) return rc;
    double rho0[2];
    for (int c = 0; c < 2; ++c) {
      rho0[c] = (c < h->C && h->cfg.rho0[c] > 0.0) ? h->cfg.rho0[c] : sums[c] / double(h->n);
      // the kernels encode with the float value of rho0
      rho0[c] = double(float(rho0[c]));
    }
    e = cudaMemcpyAsync(d_rho0, rho0, sizeof rho0, cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "init statistics");
    if (int rc = reduce_stats(h, I, 2, d_rho0, d_partial, nblocks, maxdev, true)) return rc;
    for (int c = 0; c < h->C; ++c) {
      // same rules as lbgpu_upload: FP16 offsets up to 64 * max(rho0,
      // 4 * spread); I16 fixed point over 3 max(rho0, spread)
      double scale;
      if (h->cfg.precision == LBGPU_FP16) {
        const double span = std::max(fabs(rho0[c]), 4.0 * maxdev[c]);
        scale = span > 0.0 ? span / 1024.0 : 1.0 / 4096.0;
      } else {
        scale = i16_scale(rho0[c], maxdev[c]);
      }
      h->P.rho0[c] = float(rho0[c]);
      h->P.scale[c] = float(scale);
      h->P.inv_scale[c] = float(1.0 / scale);
    }
  }
  const bool want_mask = ini->mask_init != 0;
  if (want_mask && !h->mask) {
    e = cudaMalloc(&h->mask, size_t(h->n));
    if (e != cudaSuccess) {
      cudaGetLastError();
      return h->fail(LBGPU_E_NOMEM, "mask allocation failed");
    }
    h->device_bytes += h->n;
  }
  cudaMemsetAsync(d_count, 0, sizeof(int), h->stream);
  h->cur = 0;
  const unsigned blocks = unsigned((h->n + kInitThreads - 1) / kInitThreads);
  uint8_t* m = want_mask ? h->mask : nullptr;
  if (h->cfg.precision == LBGPU_FP64)
    k_init_write<double><<<blocks, kInitThreads, 0, h->stream>>>(I, h->n, h->P, static_cast<double*>(h->f[0]), m,
                                                                  d_count);
  else if (h->cfg.precision == LBGPU_FP32)
    k_init_write<float><<<blocks, kInitThreads, 0, h->stream>>>(I, h->n, h->P, static_cast<float*>(h->f[0]), m,
                                                                 d_count);
  else if (h->cfg.precision == LBGPU_I16)
    k_init_write<int16_t><<<blocks, kInitThreads, 0, h->stream>>>(I, h->n, h->P, static_cast<int16_t*>(h->f[0]), m,
                                                                   d_count);
  else
    k_init_write<__half><<<blocks, kInitThreads, 0, h->stream>>>(I, h->n, h->P, static_cast<__half*>(h->f[0]), m,
                                                                  d_count);
  h->launches++;
  int nsolid = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&nsolid, d_count, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "init fields");
  if (h->mask && nsolid == 0) {
    cudaFree(h->mask);
    h->device_bytes -= h->n;
    h->mask = nullptr;
  }
  if (int rc = lb_update_nbmask(h)) return rc;
  h->uploaded = true;
  h->advected = false;
  h->force_valid = 0;
  return LBGPU_OK;
}
