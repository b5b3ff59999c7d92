// Fused single-pass D3Q19 timestep for the bandwidth forms (float
// arithmetic; float or half-offset storage).
//
// The two-kernel step (lb_kernels.cuh) reads every population twice: once to
// get the post-streaming densities for psi, once to collide.  This kernel
// reads them once.  A CTA owns a TY x TZ tile of the (y, z) plane and marches
// along x.  For each plane x+1 it pull-gathers the populations of the tile
// and of a one-site ring around it, computes rho and psi there and keeps them
// in a three-plane shared-memory ring; the tile's own gathered populations
// stay in shared memory until the next iteration, when plane x is collided
// with the psi stencil of planes x-1, x, x+1 and written out.  Ring sites are
// re-read by the neighbouring tile (from L2); the populations of a site are
// read from HBM once and written once.  With walls, every site carries a
// 32-bit neighbour mask (bit 0: the site is solid; bit q: the site x + c_q is
// solid, periodic images included), built once when the mask is set: the
// bounce-back choice of the gather (x - c_q = x + c_bounce(q)), the
// stencil's wall substitution and the wall force all read it, one coalesced
// 4-byte load per site instead of 37 mask lookups.
//
// Scheduling is persistent: CTAs take runs of run_len consecutive planes of
// one tile from an atomic counter (x-chunk-major, so that neighbouring tiles
// march together and share their ring sites through L2), or, without a
// counter, split the tile-major plane-tiles into equal contiguous ranges;
// every run starts with two warm-up planes.
//
// Per-site arithmetic restates the reference (addShanChenForcePsi
// force.d:238-309, distributeForce force.d:179-197,
// precalculateWeightedVelocity collision.d:156-196, collideFieldsKernel
// collision.d:90-119, eqDist eqdist.d:61-278) in float, re-associated where
// that saves work: the Shan-Chen sum of component c1 is
// -psi_c1 * sum_c2 g_c1c2 * S_c2 with S_c2 = sum_q w_q psi_c2(x + c_q) c_q
// (the same mathematical value as the reference's per-term products), and
// divisions by the density use a correctly rounded reciprocal.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include <type_traits>

#include "lb_kernels.cuh"

namespace lbk {

// Tiles are TY x 32 sites (TY = 4 or 8, a template parameter; 32 = one warp
// along the contiguous z axis), one thread per site.
constexpr int kFusedTZ = 32;
// CTAs per SM of the populations-free single-lattice kernel (28 KB of shared
// memory each): three at up to 85 registers with walls, four at 64 without
// (measured best on GB300; the wall code spills at 64)
template <bool WALLS>
constexpr int mom_ctas() { return WALLS ? 3 : 4; }
constexpr int kFusedRZ = kFusedTZ + 2;   // tile + one-site ring

// float copies of the step parameters (no double arithmetic in the kernel)
struct FusedParams {
  int32_t nx, ny, nz;
  int64_t n;
  int32_t tiles_y, tiles_z;
  int64_t work;            // tiles * nx plane-tiles
  int32_t shan_chen, psi_form, eq_form, record_force;
  int32_t unit_tau;        // every tau == 1: the relaxation is the equilibrium itself
  float tau[2], inv_tau[2], omega[2], one_minus_omega[2];
  float gcc[2][2], gwc[2], acc[3];
  float rho0[2], scale[2], inv_scale[2];
  uint32_t qn[19];         // q * n: population q's offset inside a component (19 n < 2^32)
  // half storage, per component and weight class k of q (0 rest, 1 axis,
  // 2 diagonal: these constants depend on q only through w_q):
  float wrho[2][3];        // w_q * rho0_c (f_q = w_q rho0_c + w_q scale_c h)
  float wscale[2][3];      // w_q * scale_c
  float inv_wscale[2][3];  // 1 / (w_q * scale_c)
  float hoff[2][3];        // -w_q rho0_c / (w_q scale_c): half value = v / (w_q scale_c) + hoff
  // per (x, tile) of TY = 8 tiles: 1 if a site of the tile or of its ring
  // in plane x has a solid neighbour (or is solid); planes without run the
  // wall-free code.  nullptr: every plane of a walled lattice is walled.
  const uint8_t* tile_walls;
  // dynamic scheduling (single lattice): a zeroed counter and the run length
  // in planes; nullptr: static equal ranges
  int* work_counter;
  int32_t run_len;
  // plane range [x_begin, x_end) of the dynamically scheduled kernels (the
  // whole lattice: 0, nx)
  int32_t x_begin, x_end;
  // the single-lattice schedule: planes [x_begin, x_split) of every tile in
  // runs of run_len, then [x_split, x_end) in runs of tail_len
  int32_t x_split, tail_len;
  // the pair kernel: the solid sites are exactly the planes z = 0 and
  // z = nz - 1 (nz a multiple of the tile width, no wall force)
  int32_t zwall;
};

// The dynamic schedule of the single-lattice kernels (k_fused, k_pairs,
// k_fused2d): work item i of a counter is a run of planes [x0, x1) of one of
// ntl tiles.  The first items cover planes [x_begin, x_split) of every tile
// in runs of run_len, x-chunk-major (neighbouring tiles march over the same
// planes at the same time and share their ring sites through L2); the last
// cover [x_split, x_end) in the shorter runs of tail_len.  The CTAs take
// those last, so the step ends at nearly the same time on every CTA instead
// of waiting for the few that drew a last long run.
__host__ __device__ __forceinline__ int sched_units(const FusedParams& P, int ntl) {
  const int bulk = (P.x_split - P.x_begin) / P.run_len;
  const int tail = (P.x_end - P.x_split + P.tail_len - 1) / P.tail_len;
  return ntl * (bulk + tail);
}
__host__ __device__ __forceinline__ void sched_run(const FusedParams& P, int ntl, int item, int& tile, int& x0, int& x1) {
  const int ub = ntl * ((P.x_split - P.x_begin) / P.run_len);
  if (item < ub) {
    const int ch = item / ntl;
    tile = item - ch * ntl;
    x0 = P.x_begin + ch * P.run_len;
    x1 = x0 + P.run_len;
  } else {
    const int j = item - ub;
    const int ch = j / ntl;
    tile = j - ch * ntl;
    x0 = P.x_split + ch * P.tail_len;
    x1 = min(x0 + P.tail_len, P.x_end);
  }
}
// Run lengths for `tiles` tiles and `grid` resident CTAs: runs of 32 planes
// (halved while there would be fewer runs than CTAs; every run gathers two
// extra planes to warm up), and about two runs per CTA of a quarter of that
// length at the end of every tile.
inline void plan_runs(FusedParams& G, int64_t tiles, int64_t grid) {
  const int span = G.x_end - G.x_begin;
  int rl = 32;
  while (rl > 4 && tiles * ((span + rl - 1) / rl) < grid) rl /= 2;
  if (rl > span) rl = span;
  const int tl = rl >= 8 ? rl / 4 : rl;
  int tail = int((2 * grid * tl + tiles - 1) / tiles);
  tail = ((tail + tl - 1) / tl) * tl;
  if (tail > span / 2) tail = span / 2;
  G.run_len = rl;
  G.tail_len = tl;
  G.x_split = G.x_begin + ((span - tail) / rl) * rl;
}

// Storage of connectivity Q (D3Q19 or D2Q9): the half form's constants
// depend on q only through its weight class.
template <typename T, int Q = 19>
struct FStore;
template <int Q>
struct FStore<float, Q> {
  __device__ static __forceinline__ float load(const float* p, int, int, const FusedParams&) { return __ldg(p); }
  // population q or, bounced back, population b (q, b compile-time constants)
  __device__ static __forceinline__ float load2(const float* p, int, int, int, bool, const FusedParams&) {
    return __ldg(p);
  }
  __device__ static __forceinline__ void store(float* p, float v, int, int, const FusedParams&) { *p = v; }
};
template <int Q>
struct FStore<__half, Q> {
  __device__ static __forceinline__ float load(const __half* p, int c, int q, const FusedParams& P) {
    return fmaf(P.wscale[c][Conn<Q>::wclass(q)], __half2float(__ldg(p)), P.wrho[c][Conn<Q>::wclass(q)]);
  }
  // opposite populations have equal weights (w_b = w_q), so either decodes
  // with q's constants
  __device__ static __forceinline__ float load2(const __half* p, int c, int q, int, bool, const FusedParams& P) {
    return fmaf(P.wscale[c][Conn<Q>::wclass(q)], __half2float(__ldg(p)), P.wrho[c][Conn<Q>::wclass(q)]);
  }
  __device__ static __forceinline__ void store(__half* p, float v, int c, int q, const FusedParams& P) {
    *p = __float2half_rn(fmaf(v, P.inv_wscale[c][Conn<Q>::wclass(q)], P.hoff[c][Conn<Q>::wclass(q)]));
  }
};
// 16-bit fixed-point offsets (LBGPU_I16): the half form's constants, the
// offset rounded to the nearest integer (ties to even) and saturated to
// +-32767, as the pair kernel stores it
template <int Q>
struct FStore<int16_t, Q> {
  __device__ static __forceinline__ float load(const int16_t* p, int c, int q, const FusedParams& P) {
    return fmaf(P.wscale[c][Conn<Q>::wclass(q)], float(__ldg(p)), P.wrho[c][Conn<Q>::wclass(q)]);
  }
  __device__ static __forceinline__ float load2(const int16_t* p, int c, int q, int, bool, const FusedParams& P) {
    return load(p, c, q, P);
  }
  __device__ static __forceinline__ void store(int16_t* p, float v, int c, int q, const FusedParams& P) {
    store_h(p, fmaf(v, P.inv_wscale[c][Conn<Q>::wclass(q)], P.hoff[c][Conn<Q>::wclass(q)]));
  }
  // an offset already integral within +-32767
  __device__ static __forceinline__ void store_int(int16_t* p, float h) { *p = int16_t(__float2int_rz(h)); }
  // an offset in units of the scale, rounded and saturated
  __device__ static __forceinline__ void store_h(int16_t* p, float hf) {
    const int h = __float2int_rn(hf);
    *p = int16_t(h < -32767 ? -32767 : (h > 32767 ? 32767 : h));
  }
};

// NP = 19: the tile's populations; NP = 3: its momentum per component (the
// populations-free collision), which leaves room for more CTAs per SM
template <int TY, int NP = 19>
struct FusedShared {
  float pops[2][2][NP][TY * kFusedTZ];  // [buffer][c][q][site in tile]
  float psi[3][2][TY + 2][kFusedRZ];    // [plane slot][c][y+1][z+1]
  float rho[3][2][TY + 2][kFusedRZ];
};

// shared-memory address of a generic pointer into shared memory
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ int wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// acc += v * c for a lattice velocity c with components in {-1, 0, 1}
__device__ __forceinline__ void stencil_acc(float (&acc)[3], int cx, int cy, int cz, float v) {
  if (cx > 0) acc[0] += v;
  if (cx < 0) acc[0] -= v;
  if (cy > 0) acc[1] += v;
  if (cy < 0) acc[1] -= v;
  if (cz > 0) acc[2] += v;
  if (cz < 0) acc[2] -= v;
}

// Float arithmetic of the fused kernels.  Their translation units are
// compiled without FMA contraction and every fused multiply-add is written
// out with fmaf, so the same source expression gives the same bits in every
// kernel variant (single lattice, batch, populations-free).

// S = w_axis * sum_axis + w_diag * sum_diag (w = 1/18, 1/36)
__device__ __forceinline__ float stencil_weigh(float axis, float diag) {
  return fmaf(1.0f / 18.0f, axis, (1.0f / 36.0f) * diag);
}

// dv = tau (F / rho + a) + w, or with tau = 1: F / rho + a + w
__device__ __forceinline__ float shifted_velocity(float Fc, float rden, float acc, float wv, float tau, bool unit) {
  const float u = fmaf(Fc, rden, acc);
  return unit ? u + wv : fmaf(tau, u, wv);
}

// BGK relaxation pop (1 - omega) + omega eq
__device__ __forceinline__ float relax(float pop, float omo, float omega, float eq) {
  return fmaf(pop, omo, omega * eq);
}

// The BDist2 D3Q19 equilibrium (eqdist.d:102-184) in float, the density
// folded into the pair constants: with u' = 3 dv and cst = 1 - 3/2 dv.dv,
// a pair +-c with weight w (1/36, twice that on the axes) gets
// rho w (cst + (c.u')^2 / 2) +- rho w (cst c.u' + (c.u')^3 / 6), the rest
// population rho/3 cst.  The same mathematical values as the reference's
// expression, in fewer operations (about 75 instead of 120).
__device__ __forceinline__ void eq_bdist2_f(const float (&dv)[3], float rho, float (&dist)[19]) {
  const float ux = 3.0f * dv[0], uy = 3.0f * dv[1], uz = 3.0f * dv[2];
  const float uu = fmaf(dv[2], uz, fmaf(dv[1], uy, dv[0] * ux));
  const float cst = fmaf(-0.5f, uu, 1.0f);
  const float r1 = (rho * (1.0f / 36.0f)) * cst;   // rho aN1 cst
  const float rh = rho * (1.0f / 72.0f);           // rho aN1 / 2
  const float r6 = rho * (1.0f / 216.0f);          // rho aN1 / 6
  const float a1 = 2.0f * r1, ah = 2.0f * rh, a6 = 2.0f * r6;
  auto pair = [&](float cu, float k1, float kh, float k6, int ip, int im) {
    const float cu2 = cu * cu;
    const float even = fmaf(kh, cu2, k1);
    const float odd = fmaf(k6, cu2, k1) * cu;
    dist[ip] = even + odd;
    dist[im] = even - odd;
  };
  pair(ux, a1, ah, a6, 1, 2);
  pair(uy, a1, ah, a6, 3, 4);
  pair(uz, a1, ah, a6, 5, 6);
  pair(ux + uy, r1, rh, r6, 7, 14);
  pair(ux - uy, r1, rh, r6, 13, 8);
  pair(ux + uz, r1, rh, r6, 11, 18);
  pair(ux - uz, r1, rh, r6, 12, 17);
  pair(uy + uz, r1, rh, r6, 9, 16);
  pair(uy - uz, r1, rh, r6, 15, 10);
  dist[0] = (rho * (1.0f / 3.0f)) * cst;
}

// (y, z) offsets of a site and its 8 in-plane neighbours: off[cy+1][cz+1]
struct YZ {
  int off[3][3];
};

__device__ __forceinline__ YZ make_yz(int y, int z, const FusedParams& P) {
  YZ r;
  const int ys[3] = {wrap(y - 1, P.ny), y, wrap(y + 1, P.ny)};
  const int zs[3] = {wrap(z - 1, P.nz), z, wrap(z + 1, P.nz)};
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) r.off[a][b] = ys[a] * P.nz + zs[b];
  return r;
}

// Pull-gather one site; planes[0..2] are the offsets of planes xg-1, xg,
// xg+1 of the gathered plane xg; nbm is the site's neighbour mask.
// For the I16 form mass[c] accumulates the gathered mass in units of s/36,
// 12 h_0 + 2 sum_axis h + sum_diag h, exactly (an integer held in float).
template <typename T, bool WALLS, int C>
__device__ __forceinline__ void fused_gather(const T* const (&fc)[2], const FusedParams& P,
                                             const uint32_t (&planes)[3], const YZ& yz, uint32_t nbm,
                                             float (&pop)[C][19], float (&mass)[C]) {
  const uint32_t s = planes[1] + uint32_t(yz.off[1][1]);
  const bool solid = WALLS && (nbm & 1u);
  // branch-free (warps straddling a wall must not run two code paths):
  // a solid site keeps its own populations, a fluid site pulls from x - c_q
  // or, when that site is solid, bounces back its own opposite population
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    const int cx = Conn<19>::cx(q), cy = Conn<19>::cy(q), cz = Conn<19>::cz(q);
    const uint32_t nb = planes[1 - cx] + uint32_t(yz.off[1 - cy][1 - cz]);
    const int b = Conn<19>::bounce(q);
    bool bb = false;
    if (WALLS && q > 0) bb = ((nbm >> b) & 1u) && !solid;  // x - c_q = x + c_b is solid
    const uint32_t off = (bb ? P.qn[b] : P.qn[q]) + ((WALLS && (solid || bb)) ? s : nb);
#pragma unroll
    for (int c = 0; c < C; ++c) {
      if constexpr (std::is_same<T, int16_t>::value) {
        const float h = float(__ldg(fc[c] + off));
        const int k = Conn<19>::wclass(q);
        pop[c][q] = fmaf(P.wscale[c][k], h, P.wrho[c][k]);  // FStore<int16_t>::load2
        mass[c] = fmaf(k == 0 ? 12.f : (k == 1 ? 2.f : 1.f), h, mass[c]);
      } else {
        pop[c][q] = FStore<T>::load2(fc[c] + off, c, q, b, bb, P);
      }
    }
  }
}

// Shared-memory slots per component and site of the tile's kept state: the
// momenta (MOM) or the populations, and for the I16 form the gathered mass
template <typename T, bool MOM>
constexpr int fused_np() {
  return (MOM ? 3 : 19) + (std::is_same<T, int16_t>::value ? 1 : 0);
}

// Process plane-tiles [w0, w1) of one lattice (tile-major: w = tile*nx + x).
// P may live in the constant bank (single lattice) or in shared memory
// (batches); every thread of the CTA calls this with the same range.
//
// MOM: every tau is 1 and the equilibrium is BDist2, so the collision needs
// only the density and momentum of each component, not the populations: the
// gather keeps the three momentum components per component in the population
// buffer instead of the 19 populations.
template <typename T, int C, bool WALLS, int TY, bool MOM = false>
__device__ __forceinline__ void fused_body(const FusedParams& P, const T* __restrict__ f, T* __restrict__ fout,
                                           const uint32_t* __restrict__ nbmask, double* __restrict__ force_out,
                                           int64_t w0, int64_t w1, FusedShared<TY, fused_np<T, MOM>()>& sh) {
  constexpr int kFusedTY = TY;
  // the I16 form conserves every site's mass exactly (see the collision)
  constexpr bool EXACT = std::is_same<T, int16_t>::value;
  constexpr int NP = fused_np<T, MOM>();
  const int t = threadIdx.x;
  const int ty = t / kFusedTZ, tz = t % kFusedTZ;
  const uint32_t plane_sz = uint32_t(P.ny) * uint32_t(P.nz);
  const T* const fc[2] = {f, f + size_t(19) * size_t(P.n)};
  T* const fo[2] = {fout, fout + size_t(19) * size_t(P.n)};
  const bool unit = MOM || P.unit_tau != 0;
  const int ntiles = P.tiles_y * P.tiles_z;
  int64_t w = w0;
  while (w < w1) {
    const int tile = int(w / P.nx);
    const int xs = int(w - int64_t(tile) * P.nx);
    const int run = int(min(w1 - w, int64_t(P.nx - xs)));
    const int y0 = (tile / P.tiles_z) * kFusedTY, z0 = (tile % P.tiles_z) * kFusedTZ;
    const int tyv = min(kFusedTY, P.ny - y0), tzv = min(kFusedTZ, P.nz - z0);
    const bool active = ty < tyv && tz < tzv;
    // interior site offsets and this thread's ring site (if any)
    const YZ yz_in = make_yz(y0 + ty, z0 + tz, P);
    // this thread's ring site: the row above, the row below, then the left
    // and right columns
    const int ring = 2 * (tzv + 2) + 2 * tyv;
    int rry = 0, rrz = 0;
    const bool has_ring = t < ring;
    if (has_ring) {
      if (t < tzv + 2) {
        rry = -1;
        rrz = t - 1;
      } else if (t < 2 * (tzv + 2)) {
        rry = tyv;
        rrz = t - (tzv + 2) - 1;
      } else {
        const int k = t - 2 * (tzv + 2);
        rry = k >> 1;
        rrz = (k & 1) ? tzv : -1;
      }
    }
    const YZ yz_ring = make_yz(wrap(y0 + rry, P.ny), wrap(z0 + rrz, P.nz), P);
    // neighbour masks of this thread's interior site at the gathered plane
    // (nbm_next) and at the plane being collided (nbm_cur)
    uint32_t nbm_next = 0, nbm_cur = 0;
    bool pw_next = WALLS, pw_cur = WALLS;
    // whether plane xg of this tile needs the wall code (uniform in the CTA)
    auto walled = [&](int xg) -> bool {
      return WALLS && (P.tile_walls == nullptr || __ldg(P.tile_walls + size_t(xg) * ntiles + tile) != 0);
    };
    // the wall flag and neighbour masks of the next gathered plane are
    // loaded one plane ahead, so that the population loads, whose addresses
    // depend on them, do not wait for them
    bool pw_pre = false;
    uint32_t nbm_pre_in = 0, nbm_pre_ring = 0;
    auto prefetch = [&](int xg) {
      if (!WALLS) return;
      pw_pre = walled(xg);
      const uint32_t pb = uint32_t(xg) * plane_sz;
      nbm_pre_in = (active && nbmask) ? __ldg(nbmask + pb + uint32_t(yz_in.off[1][1])) : 0u;
      nbm_pre_ring = (has_ring && nbmask) ? __ldg(nbmask + pb + uint32_t(yz_ring.off[1][1])) : 0u;
    };

    // rho/psi of plane xg into psi slot ps (and the tile's populations into
    // buffer keep, unless keep < 0); prefetches plane xn's flag and masks
    auto gather_plane = [&](int ps, int xg, int keep, int xn) {
      const uint32_t planes[3] = {uint32_t(wrap(xg - 1, P.nx)) * plane_sz, uint32_t(xg) * plane_sz,
                                  uint32_t(wrap(xg + 1, P.nx)) * plane_sz};
      const bool pw = WALLS && pw_pre;
      const uint32_t nbm_in = nbm_pre_in, nbm_ring = nbm_pre_ring;
      prefetch(xn);
      pw_next = pw;
      if (active) {
        const uint32_t nbm = pw ? nbm_in : 0u;
        nbm_next = nbm;
        float pop[C][19], mass[C];
#pragma unroll
        for (int c = 0; c < C; ++c) mass[c] = 0.f;
        if (pw)
          fused_gather<T, WALLS, C>(fc, P, planes, yz_in, nbm, pop, mass);
        else
          fused_gather<T, false, C>(fc, P, planes, yz_in, 0u, pop, mass);
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const float den = density<19, float>(pop[c]);
          sh.rho[ps][c][ty + 1][tz + 1] = den;
          sh.psi[ps][c][ty + 1][tz + 1] = P.psi_form ? 1.0f - __expf(-den) : den;
          if (keep >= 0) {
            if (EXACT) sh.pops[keep][c][NP - 1][t] = mass[c];
            if (MOM) {
#pragma unroll
              for (int vd = 0; vd < 3; ++vd) sh.pops[keep][c][vd][t] = moment<19, float>(pop[c], vd);
            } else {
#pragma unroll
              for (int q = 0; q < 19; ++q) sh.pops[keep][c][q][t] = pop[c][q];
            }
          }
        }
      }
      if (has_ring) {
        const uint32_t nbm = pw ? nbm_ring : 0u;
        float pop[C][19], mass[C];  // (the ring sites' mass is not needed)
#pragma unroll
        for (int c = 0; c < C; ++c) mass[c] = 0.f;
        if (pw)
          fused_gather<T, WALLS, C>(fc, P, planes, yz_ring, nbm, pop, mass);
        else
          fused_gather<T, false, C>(fc, P, planes, yz_ring, 0u, pop, mass);
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const float den = density<19, float>(pop[c]);
          sh.rho[ps][c][rry + 1][rrz + 1] = den;
          sh.psi[ps][c][rry + 1][rrz + 1] = P.psi_form ? 1.0f - __expf(-den) : den;
        }
      }
    };

    // warm-up: rho/psi of xs-1; rho/psi + populations of xs
    __syncthreads();
    prefetch(wrap(xs - 1, P.nx));
    gather_plane(0, wrap(xs - 1, P.nx), -1, xs);
    gather_plane(1, xs, 0, wrap(xs + 1, P.nx));
    int cur = 0;
    for (int k = 0; k < run; ++k) {
      const int x = xs + k;
      const int sm = k % 3, s0 = (k + 1) % 3, sp = (k + 2) % 3;  // psi slots of x-1, x, x+1
      nbm_cur = nbm_next;
      pw_cur = pw_next;
      __syncthreads();  // psi slot sp and pops buffer 1-cur are free
      gather_plane(sp, wrap(x + 1, P.nx), 1 - cur, wrap(x + 2, P.nx));
      __syncthreads();
      // the collision of plane x, with or without the wall code
      auto collide = [&](auto wtag) {
        constexpr bool W = decltype(wtag)::value;
        const uint32_t s = uint32_t(x) * plane_sz + uint32_t(yz_in.off[1][1]);
        const int c1y = ty + 1, c1z = tz + 1;
        // branch-free: solid sites compute like fluid ones but store nothing
        // (both population buffers hold their constant populations; warps
        // straddling a wall run one code path)
        const bool solid = W && (nbm_cur & 1u);
        float den[C];
#pragma unroll
        for (int c = 0; c < C; ++c) den[c] = sh.rho[s0][c][c1y][c1z];
        const int pslot[3] = {sm, s0, sp};  // by cx + 1
        // --- Shan-Chen force: S_c = sum_q w_q psi_c(x + c_q) c_q, a solid
        // neighbour contributing the site's own psi (force.d:273)
        float F[C][3];
#pragma unroll
        for (int c = 0; c < C; ++c) F[c][0] = F[c][1] = F[c][2] = 0.f;
        if (P.shan_chen) {
          float S[C][3];
          float own[C];
#pragma unroll
          for (int c = 0; c < C; ++c) {
            own[c] = sh.psi[s0][c][c1y][c1z];
            float a[3] = {0.f, 0.f, 0.f}, d[3] = {0.f, 0.f, 0.f};  // axis and diagonal sums
#pragma unroll
            for (int q = 1; q < 19; ++q) {
              const int cx = Conn<19>::cx(q), cy = Conn<19>::cy(q), cz = Conn<19>::cz(q);
              float v = sh.psi[pslot[cx + 1]][c][c1y + cy][c1z + cz];
              if (W && ((nbm_cur >> q) & 1u)) v = own[c];
              if (Conn<19>::wclass(q) == 1)
                stencil_acc(a, cx, cy, cz, v);
              else
                stencil_acc(d, cx, cy, cz, v);
            }
#pragma unroll
            for (int vd = 0; vd < 3; ++vd) S[c][vd] = stencil_weigh(a[vd], d[vd]);
          }
#pragma unroll
          for (int f1 = 0; f1 < C; ++f1) {
            float g[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int f2 = 0; f2 < C; ++f2) {
              const float cc = P.gcc[f1][f2];
#pragma unroll
              for (int vd = 0; vd < 3; ++vd) g[vd] = fmaf(cc, S[f2][vd], g[vd]);
            }
#pragma unroll
            for (int vd = 0; vd < 3; ++vd) F[f1][vd] = -own[f1] * g[vd];
            if (W) {
              const float wc = P.gwc[f1];
              if (wc != 0.f) {
                float a[3] = {0.f, 0.f, 0.f}, d[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int q = 1; q < 19; ++q) {
                  const int cx = Conn<19>::cx(q), cy = Conn<19>::cy(q), cz = Conn<19>::cz(q);
                  const float v = ((nbm_cur >> q) & 1u) ? sh.rho[pslot[cx + 1]][f1][c1y + cy][c1z + cz] : 0.f;
                  if (Conn<19>::wclass(q) == 1)
                    stencil_acc(a, cx, cy, cz, v);
                  else
                    stencil_acc(d, cx, cy, cz, v);
                }
#pragma unroll
                for (int vd = 0; vd < 3; ++vd) F[f1][vd] -= own[f1] * wc * stencil_weigh(a[vd], d[vd]);
              }
            }
          }
        }
        float tot = den[0];
        if (C > 1) tot = tot + den[1];
#pragma unroll
        for (int c = 0; c < C; ++c) {
          // distributeForce with no distributed force: only its NaN cases matter
          const bool bad = tot == 0.f || isnan(tot) || isinf(den[c]) || isnan(den[c]);
          if (bad) F[c][0] = F[c][1] = F[c][2] = NAN;
          if (solid && !bad) F[c][0] = F[c][1] = F[c][2] = 0.f;
        }
        if (P.record_force) {
#pragma unroll
          for (int c = 0; c < C; ++c)
#pragma unroll
            for (int vd = 0; vd < 3; ++vd) force_out[(size_t(c) * P.n + s) * 3 + vd] = double(F[c][vd]);
        }
        // --- BDist2 weighted velocity (collision.d:156-196); the populations
        // of the last component stay in registers for its collision
        float pop[19];
        float wv[3] = {0.f, 0.f, 0.f};
        if (MOM || P.eq_form == 2) {
          float a[3] = {0.f, 0.f, 0.f};
#pragma unroll
          for (int c = 0; c < C; ++c) {
            if (MOM) {
#pragma unroll
              for (int vd = 0; vd < 3; ++vd) a[vd] += sh.pops[cur][c][vd][t];
              continue;
            }
#pragma unroll
            for (int q = 0; q < 19; ++q) pop[q] = sh.pops[cur][c][q][t];
            if (unit) {
#pragma unroll
              for (int vd = 0; vd < 3; ++vd) a[vd] += moment<19, float>(pop, vd);
            } else {
#pragma unroll
              for (int vd = 0; vd < 3; ++vd) a[vd] = fmaf(moment<19, float>(pop, vd), P.inv_tau[c], a[vd]);
            }
          }
          const float rtot = __frcp_rn(tot);
#pragma unroll
          for (int vd = 0; vd < 3; ++vd) wv[vd] = a[vd] * rtot;
        }
        // --- collision; solid sites store nothing.  With tau == 1 the new
        // populations are the equilibrium (pop*0 + 1*eq)
#pragma unroll
        for (int cc = 0; cc < C; ++cc) {
          const int c = C - 1 - cc;  // last component first: its populations are loaded
          if (!MOM && !(P.eq_form == 2 && cc == 0)) {
#pragma unroll
            for (int q = 0; q < 19; ++q) pop[q] = sh.pops[cur][c][q][t];
          }
          const float rden = __frcp_rn(den[c]);
          float dv[3];
#pragma unroll
          for (int vd = 0; vd < 3; ++vd) dv[vd] = shifted_velocity(F[c][vd], rden, P.acc[vd], wv[vd], P.tau[c], unit);
          float eq[19];
          if (MOM || P.eq_form == 2)
            eq_bdist2_f(dv, den[c], eq);
          else
            eq_poly<19, float>(pop, dv, den[c], P.eq_form == 1, eq);
          const float omega = P.omega[c], omo = P.one_minus_omega[c];
          if constexpr (EXACT) {
            // Exact mass conservation (the pair kernel's rule): the new
            // values rounded to integers and saturated, their mass 12 h_0 +
            // 2 sum_axis h + sum_diag h made equal to the gathered one, the
            // difference to h_0 in multiples of 12 and the rest to the
            // opposite pair h_7, h_14 (half each, an odd unit to h_7)
            float m_out = 0.f;
#pragma unroll
            for (int q = 0; q < 19; ++q) {
              const float v = (MOM || unit) ? eq[q] : relax(pop[q], omo, omega, eq[q]);
              const int k = Conn<19>::wclass(q);
              eq[q] = fminf(fmaxf(rintf(fmaf(v, P.inv_wscale[c][k], P.hoff[c][k])), -32767.f), 32767.f);
              m_out = fmaf(k == 0 ? 12.f : (k == 1 ? 2.f : 1.f), eq[q], m_out);
            }
            const int d = __float2int_rz(sh.pops[cur][c][NP - 1][t] - m_out);
            const int d0 = d / 12, r = d - 12 * d0, hr = r / 2;
            eq[0] += float(d0);
            eq[7] += float(r - hr);
            eq[14] += float(hr);
            if (!solid) {
#pragma unroll
              for (int q = 0; q < 19; ++q) {
                if (q == 0 || q == 7 || q == 14)
                  FStore<int16_t>::store_h(fo[c] + (P.qn[q] + s), eq[q]);
                else
                  FStore<int16_t>::store_int(fo[c] + (P.qn[q] + s), eq[q]);
              }
            }
            continue;
          }
          if (!solid) {
#pragma unroll
            for (int q = 0; q < 19; ++q) {
              const float v = (MOM || unit) ? eq[q] : relax(pop[q], omo, omega, eq[q]);
              FStore<T>::store(fo[c] + (P.qn[q] + s), v, c, q, P);
            }
          }
        }
      };
      // (a wall-free plane of a walled lattice has zero neighbour masks: the
      // wall code computes the same there, so only the gather is specialised)
      if (active) collide(std::integral_constant<bool, WALLS>{});
      cur = 1 - cur;
    }
    w += run;
  }
}

// (the populations-free variant needs 28 KB of shared memory instead of 94,
// which leaves L1 room for the ring re-reads and allows 3-4 CTAs per SM)
template <typename T, int C, bool WALLS, int TY, bool MOM = false>
__global__ void __launch_bounds__(TY * kFusedTZ, MOM ? (8 / TY) * mom_ctas<WALLS>() : (8 / TY * 2 > 4 ? 4 : 8 / TY * 2))
    k_fused(const T* __restrict__ f, T* __restrict__ fout, const uint32_t* __restrict__ nbmask,
            double* __restrict__ force_out, FusedParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FusedShared<TY, fused_np<T, MOM>()>& sh = *reinterpret_cast<FusedShared<TY, fused_np<T, MOM>()>*>(smem_raw);
  if (!P.work_counter) {
    const int64_t w0 = P.work * blockIdx.x / gridDim.x;
    const int64_t w1 = P.work * (blockIdx.x + 1) / gridDim.x;
    fused_body<T, C, WALLS, TY, MOM>(P, f, fout, nbmask, force_out, w0, w1, sh);
    return;
  }
  // dynamic: runs of planes of one tile taken from a counter (sched_run),
  // so that CTAs on cheap (wall-free) tiles take more runs; x-chunk-major
  // (8-12 % faster than tile-major order)
  __shared__ int s_item;
  const int ntl = P.tiles_y * P.tiles_z;
  const int units = sched_units(P, ntl);
  for (;;) {
    __syncthreads();  // every thread has read the previous item
    if (threadIdx.x == 0) s_item = atomicAdd(P.work_counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= units) break;
    int tile, x0, x1;
    sched_run(P, ntl, item, tile, x0, x1);
    const int64_t w0 = int64_t(tile) * P.nx + x0;
    fused_body<T, C, WALLS, TY, MOM>(P, f, fout, nbmask, force_out, w0, w0 + (x1 - x0), sh);
  }
}

// One simulation of a batch.  The step reads populations f[(parity + phase)
// & 1] and writes the other buffer.
struct FusedSim {
  FusedParams P;
  const void* f[2];
  const uint32_t* nbmask;  // neighbour masks; nullptr: no solid site
  double* force_out;       // nullptr unless recording
  int64_t work_begin;      // first plane-tile of this simulation in the batch
  int64_t unit_begin;      // first run of this simulation (dynamic scheduling)
  int32_t phase;
  int32_t nchunks;         // runs per tile: ceil(nx / P.run_len)
};

// Many independent lattices of any sizes in one persistent launch.  With
// `counters`, CTAs take runs of at most run_len planes of one tile (all
// simulations' runs concatenated) from counters[parity] and zero the other
// counter for the next launch; without, the concatenated plane-tile work is
// split into equal contiguous ranges, one per CTA.
template <typename T, int C, bool WALLS, int TY>
__global__ void __launch_bounds__(TY * kFusedTZ, 8 / TY * 2 > 4 ? 4 : 8 / TY * 2)
    k_fused_batch(const FusedSim* __restrict__ sims, int nsims, int64_t total_work, int parity,
                  int64_t total_units, int* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FusedShared<TY, fused_np<T, false>()>& sh = *reinterpret_cast<FusedShared<TY, fused_np<T, false>()>*>(smem_raw);
  __shared__ FusedParams Ps;
  __shared__ int s_idx;
  __shared__ long long s_w[2];
  if (counters && blockIdx.x == 0 && threadIdx.x == 0) counters[1 - parity] = 0;
  // static: this CTA's equal share [w, wend) of the plane-tiles; dynamic:
  // runs taken from the counter
  long long w = total_work * blockIdx.x / gridDim.x;
  const long long wend = total_work * (blockIdx.x + 1) / gridDim.x;
  for (;;) {
    __syncthreads();  // every thread has used the previous range and Ps
    if (threadIdx.x == 0) {
      long long r0 = 0, r1 = 0;
      int idx = 0;
      const long long key = counters ? (long long)atomicAdd(counters + parity, 1) : w;
      if (counters ? key < total_units : key < wend) {
        int lo = 0, hi = nsims - 1;  // last simulation starting at or before key
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if ((counters ? sims[mid].unit_begin : sims[mid].work_begin) <= key)
            lo = mid;
          else
            hi = mid - 1;
        }
        idx = lo;
        if (counters) {
          const long long local = key - sims[lo].unit_begin;
          const int ntl = sims[lo].P.tiles_y * sims[lo].P.tiles_z;
          const long long ch = local / ntl, tile = local - ch * ntl;  // x-chunk-major, as k_fused
          const int nx = sims[lo].P.nx, rl = sims[lo].P.run_len;
          r0 = sims[lo].work_begin + tile * nx + ch * rl;
          const long long tile_end = sims[lo].work_begin + (tile + 1) * nx;
          r1 = r0 + rl < tile_end ? r0 + rl : tile_end;
        } else {
          const long long sim_end = sims[lo].work_begin + sims[lo].P.work;
          r0 = key;
          r1 = wend < sim_end ? wend : sim_end;
        }
      }
      s_w[0] = r0;
      s_w[1] = r1;
      s_idx = idx;
    }
    __syncthreads();
    if (s_w[0] >= s_w[1]) break;
    const int i = s_idx;
    // stage this simulation's parameters (FusedParams is a multiple of 4 bytes)
    const int* src = reinterpret_cast<const int*>(&sims[i].P);
    int* dst = reinterpret_cast<int*>(&Ps);
    for (int k = threadIdx.x; k < int(sizeof(FusedParams) / 4); k += blockDim.x) dst[k] = src[k];
    const long long wb = sims[i].work_begin;
    const int par = (parity + sims[i].phase) & 1;
    const T* fin = static_cast<const T*>(sims[i].f[par]);
    T* fout = const_cast<T*>(static_cast<const T*>(sims[i].f[1 - par]));
    const long long r0 = s_w[0], r1 = s_w[1];
    __syncthreads();
    // tau = 1 BDist2 members take the populations-free collision (the same
    // bits as the general body, with fewer instructions)
    if (C == 2 && Ps.unit_tau && Ps.eq_form == 2)
      fused_body<T, C, WALLS, TY, true>(Ps, fin, fout, sims[i].nbmask, sims[i].force_out, r0 - wb, r1 - wb,
                                               *reinterpret_cast<FusedShared<TY, fused_np<T, true>()>*>(smem_raw));
    else
      fused_body<T, C, WALLS, TY>(Ps, fin, fout, sims[i].nbmask, sims[i].force_out, r0 - wb, r1 - wb, sh);
    w = r1;
  }
}

}  // namespace lbk
