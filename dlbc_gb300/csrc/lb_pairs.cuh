// Fused single-pass D3Q19 timestep, two z-adjacent sites per thread (the
// bandwidth forms: float arithmetic on float, half-offset or 16-bit
// fixed-point storage).
//
// Layout of the work.  A CTA owns a tile of TY rows (y) x 64 sites (z) and
// marches along x (TY = pair_ty: 8, or 14 for half offsets).  TY + 2 warps:
// warp w < TY owns row y0 + w, lane l
// the sites z0 + 2l and z0 + 2l + 1 (one 4-byte or 8-byte word of every
// population array); the two ring warps gather the rows y0 - 1 and
// y0 + TY and the sites z0 - 1 / z0 + 64 of every row, whose psi the
// stencil needs but which other tiles own.  Per plane:
//
//   1. every warp pull-gathers its row of plane x+1 with one aligned word
//      load per population and component; the populations that stream
//      along z (c_z = +-1) take their neighbour from the adjacent lane with
//      a warp shuffle, the warp's edge lane from one extra load;
//   2. it sums them into density and momentum (and, for tau != 1, keeps the
//      gathered words in shared memory), and writes psi of its sites into a
//      shared ring of plane slots;
//   3. after a barrier the row warps collide plane x: the 18-point psi
//      stencil from the ring, Shan-Chen force, BDist2 weighted velocity and
//      equilibrium, relaxation, one word store per population; meanwhile
//      the ring warps gather the scalar ring sites of plane x+2.
//
// Density and momentum of the plane being collided stay in registers from
// the gather one plane earlier (a warp gathers and collides the same row).
// With every tau = 1 (MOM) the collision needs nothing else; otherwise the
// gathered words come back from shared memory for the relaxation.  All
// per-site float arithmetic runs on Blackwell's packed two-lane FP32
// instructions (__fadd2_rn, __fmul2_rn, __ffma2_rn: one instruction for the
// two sites of a thread); every operation is IEEE single precision rounded
// to nearest, so a site's result does not depend on which lane or tile
// computes it (the ring warps' scalar gathers give the same bits as the
// pair gathers of the owning tile).
//
// Storage.  FP32 holds f_q.  FP16 holds h_q = (f_q / w_q - rho0) / scale as
// half (the format of the other kernels), I16 the same offset rounded to a
// 16-bit integer; the kernel works on h directly: rho = rho0 + scale/36
// (12 h_0 + 2 sum_axis h + sum_diag h), the momentum likewise, and the
// equilibrium goes straight to h space, h_eq = (rho / scale) g_q(u) -
// rho0 / scale (the weight cancels).
//
// Requirements: nz even (aligned words), the BDist2 equilibrium and no solid
// site; the launcher runs the one-site-per-thread kernel (lb_fused.cuh)
// otherwise.  (Walled rows with per-site bounce-back addresses were slower
// here than the one-site kernel's wall code: a word covers two sites whose
// sources differ next to a wall.)
//
// The arithmetic restates the reference (advectFieldsKernel
// advection.d:61-89, psi force.d:320-333, addShanChenForcePsi
// force.d:238-309, distributeForce force.d:179-197,
// precalculateWeightedVelocity collision.d:156-196, collideFieldsKernel
// collision.d:90-119, eqDist BDist2 eqdist.d:102-184) in float, with sums
// regrouped by weight class and the density folded into the equilibrium's
// constants.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "lb_fused.cuh"
#include "lb_fused_launch.cuh"
#include "lb_launch.h"

namespace lbk {

// (kPairTZ = 64 sites per tile row, 32 lanes x 2: lb_launch.h)
constexpr int kPairRZ = kPairTZ + 4;        // shared row: [1] left ring, [2, 2 + tzv) tile, [2 + tzv] right ring
// the storage kind, tile height, threads (row warps + the two ring warps)
// and resident CTAs per SM of the pair kernel for storage T
template <typename T>
constexpr int pair_kind() {
  return std::is_same<T, __half>::value ? kStoreF16 : (std::is_same<T, int16_t>::value ? kStoreI16 : kStoreF32);
}
template <typename T>
constexpr int pair_ty_of() {
  return pair_ty(pair_kind<T>());
}
template <typename T>
constexpr int pair_threads() {
  return (pair_ty_of<T>() + 2) * 32;
}

// ---------------------------------------------------------------------------
// float and float2 arithmetic with the same per-lane rounding
// ---------------------------------------------------------------------------
__device__ __forceinline__ float vadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float vsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float vmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 vsub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 vmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 vfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
template <typename V>
__device__ __forceinline__ V splat(float a);
template <>
__device__ __forceinline__ float splat<float>(float a) {
  return a;
}
template <>
__device__ __forceinline__ float2 splat<float2>(float a) {
  return make_float2(a, a);
}

// ---------------------------------------------------------------------------
// Storage words: two z-adjacent sites of one population array
// ---------------------------------------------------------------------------
template <typename T>
struct PairIO;

template <>
struct PairIO<float> {
  using W = float2;
  static constexpr bool kOffsets = false;
  // element offset of the left edge load relative to the neighbour site:
  // FP32 loads the neighbour's value itself
  static constexpr int kLeftEdge = 0;
  __device__ static __forceinline__ W ld(const float* p) { return __ldg(reinterpret_cast<const float2*>(p)); }
  __device__ static __forceinline__ float ld1(const float* p) { return __ldg(p); }
  // (f(z-1), f(z)) from the pair (f(z), f(z+1)): the lane below's upper site,
  // or at the warp's left edge one load at edge_p (the site z0 - 1)
  __device__ static __forceinline__ W up(W w, bool lane0, const float* edge_p) {
    float prev = __shfl_up_sync(0xffffffffu, w.y, 1);
    if (lane0) prev = __ldg(edge_p);
    return make_float2(prev, w.x);
  }
  // (f(z+1), f(z+2)): the lane above's lower site, or at the right edge one
  // load at edge_p (the site z0 + tzv)
  __device__ static __forceinline__ W down(W w, bool lastl, const float* edge_p) {
    float next = __shfl_down_sync(0xffffffffu, w.x, 1);
    if (lastl) next = __ldg(edge_p);
    return make_float2(w.y, next);
  }
  __device__ static __forceinline__ float2 val(W w) { return w; }
  __device__ static __forceinline__ W enc(float2 v) { return v; }
  // evict-first (streaming) stores: the new populations are not read again
  // in this step, and the L2 keeps the ring rows that a neighbouring tile
  // gathers again (measured at 512^3: 16 570 -> 16 950 MLUPS; the 16-bit
  // forms were not faster with them)
  __device__ static __forceinline__ void st(float* p, W w) { __stcs(reinterpret_cast<float2*>(p), w); }
  // planar z-walls: one site of the pair replaced, or stored, alone (the
  // wall code compiles for every storage; FP16 runs it)
  __device__ static __forceinline__ W with_lo(W w, W b) { return make_float2(b.x, w.y); }
  __device__ static __forceinline__ W with_hi(W w, W b) { return make_float2(w.x, b.y); }
  __device__ static __forceinline__ void st_lo(float* p, W w) { __stcs(p, w.x); }
  __device__ static __forceinline__ void st_hi(float* p, W w) { __stcs(p + 1, w.y); }
};

// The 16-bit storages share their word handling: site z in the low half,
// z + 1 in the high half.  Edge loads fetch the aligned word holding the
// neighbour: at the left edge the word (z0 - 2, z0 - 1), whose high half is
// the neighbour; at the right edge (z0 + tzv, z0 + tzv + 1).
template <typename T>
struct PairIO16 {
  using W = uint32_t;
  static constexpr bool kOffsets = true;
  static constexpr int kLeftEdge = -1;
  __device__ static __forceinline__ W ld(const T* p) { return __ldg(reinterpret_cast<const unsigned int*>(p)); }
  __device__ static __forceinline__ W up(W w, bool lane0, const T* edge_p) {
    W prev = __shfl_up_sync(0xffffffffu, w, 1);
    if (lane0) prev = __ldg(reinterpret_cast<const unsigned int*>(edge_p));
    return __byte_perm(prev, w, 0x5432);  // (prev.hi, w.lo)
  }
  __device__ static __forceinline__ W down(W w, bool lastl, const T* edge_p) {
    W next = __shfl_down_sync(0xffffffffu, w, 1);
    if (lastl) next = __ldg(reinterpret_cast<const unsigned int*>(edge_p));
    return __byte_perm(w, next, 0x5432);  // (w.hi, next.lo)
  }
  __device__ static __forceinline__ void st(T* p, W w) { *reinterpret_cast<unsigned int*>(p) = w; }
  // planar z-walls: one site of the pair replaced, or stored, alone
  __device__ static __forceinline__ W with_lo(W w, W b) { return (b & 0xffffu) | (w & 0xffff0000u); }
  __device__ static __forceinline__ W with_hi(W w, W b) { return (w & 0xffffu) | (b & 0xffff0000u); }
  __device__ static __forceinline__ void st_lo(T* p, W w) {
    *reinterpret_cast<unsigned short*>(p) = static_cast<unsigned short>(w & 0xffffu);
  }
  __device__ static __forceinline__ void st_hi(T* p, W w) {
    *reinterpret_cast<unsigned short*>(p + 1) = static_cast<unsigned short>(w >> 16);
  }
};

template <>
struct PairIO<__half> : PairIO16<__half> {
  __device__ static __forceinline__ float ld1(const __half* p) { return __half2float(__ldg(p)); }
  __device__ static __forceinline__ float2 val(W w) {
    __half2 h;
    *reinterpret_cast<W*>(&h) = w;
    return __half22float2(h);
  }
  __device__ static __forceinline__ W enc(float2 v) {
    const __half2 h = __float22half2_rn(v);
    return *reinterpret_cast<const W*>(&h);
  }
};

// 16-bit fixed point (the I16 form): h rounded to nearest, saturated to
// +-32767
__device__ __forceinline__ uint32_t pack_s16x2(float a, float b) {
  uint32_t r;
  asm("{\n\t.reg .s16 lo, hi;\n\tcvt.rni.sat.s16.f32 lo, %1;\n\tcvt.rni.sat.s16.f32 hi, %2;\n\t"
      "max.s16 lo, lo, -32767;\n\tmax.s16 hi, hi, -32767;\n\tmov.b32 %0, {lo, hi};\n\t}"
      : "=r"(r)
      : "f"(a), "f"(b));
  return r;
}

template <>
struct PairIO<int16_t> : PairIO16<int16_t> {
  __device__ static __forceinline__ float ld1(const int16_t* p) { return float(__ldg(p)); }
  __device__ static __forceinline__ float2 val(W w) {
    return make_float2(float(int16_t(w & 0xffffu)), float(int16_t(w >> 16)));
  }
  __device__ static __forceinline__ W enc(float2 v) { return pack_s16x2(v.x, v.y); }
  // v already integral within +-32767 (the exact-mass collision rounds and
  // saturates before it accounts the mass): the conversion needs no
  // rounding or saturation (measured at 512^3: 18 760 -> 20 540 MLUPS
  // against enc)
  __device__ static __forceinline__ W enc_int(float2 v) {
    return __byte_perm(uint32_t(__float2int_rz(v.x)), uint32_t(__float2int_rz(v.y)), 0x5410);
  }
};

// ---------------------------------------------------------------------------
// Per-site moments of one component from its 19 gathered values (FP32: the
// populations; FP16/I16: the stored offsets h), in one fixed order for every
// kernel variant and for float and float2 alike
// ---------------------------------------------------------------------------
template <typename V>
struct PairMom {
  V rho, j[3];
  // offsets: the mass in units of s/36, 12 h_0 + 2 sum_axis h + sum_diag h
  // (an integer for the I16 form, held exactly in float)
  V mass;
};

template <bool OFFSETS, typename V>
__device__ __forceinline__ PairMom<V> pair_moments(const V (&v)[19], float s36, float rho0) {
  const V A = vadd(vadd(vadd(v[1], v[2]), vadd(v[3], v[4])), vadd(v[5], v[6]));
  const V Ax = vsub(v[1], v[2]), Ay = vsub(v[3], v[4]), Az = vsub(v[5], v[6]);
  const V xp = vadd(vadd(v[7], v[11]), vadd(v[12], v[13]));  // c_x = +1
  const V xm = vadd(vadd(v[8], v[14]), vadd(v[17], v[18]));  // c_x = -1
  const V y0p = vadd(v[9], v[15]), y0m = vadd(v[10], v[16]);  // c_x = 0, c_y = +-1
  const V Dx = vsub(xp, xm);
  const V D = vadd(vadd(xp, xm), vadd(y0p, y0m));
  const V Dy = vsub(vadd(vadd(v[7], v[8]), y0p), vadd(vadd(v[13], v[14]), y0m));
  const V Dz = vsub(vadd(vadd(v[9], v[10]), vadd(v[11], v[17])), vadd(vadd(v[12], v[15]), vadd(v[16], v[18])));
  PairMom<V> m;
  if (OFFSETS) {
    // f_q = w_q (rho0 + s h_q), w = 12/36, 2/36, 1/36
    const V two = splat<V>(2.f);
    m.mass = vfma(splat<V>(12.f), v[0], vfma(two, A, D));
    m.rho = vfma(splat<V>(s36), m.mass, splat<V>(rho0));
    m.j[0] = vmul(splat<V>(s36), vfma(two, Ax, Dx));
    m.j[1] = vmul(splat<V>(s36), vfma(two, Ay, Dy));
    m.j[2] = vmul(splat<V>(s36), vfma(two, Az, Dz));
  } else {
    m.rho = vadd(vadd(v[0], A), D);
    m.mass = m.rho;
    m.j[0] = vadd(Ax, Dx);
    m.j[1] = vadd(Ay, Dy);
    m.j[2] = vadd(Az, Dz);
  }
  return m;
}

__device__ __forceinline__ float pair_psi(float rho, int psi_form) { return psi_form ? 1.0f - __expf(-rho) : rho; }

// ---------------------------------------------------------------------------
// Shared memory and equilibrium constants
// ---------------------------------------------------------------------------
template <int C, bool MOM, typename T>
struct PairShared {
  // four plane slots: the ring warps gather the z-ring of plane x + 2 while
  // the row warps collide plane x with the slots of x - 1, x, x + 1
  float psi[4][C][pair_ty_of<T>() + 2][kPairRZ];
  // tau != 1: the row warps' gathered words of the next plane, [buffer][c][q][row][lane]
  typename PairIO<T>::W pops[MOM ? 1 : 2][C][MOM ? 1 : 19][MOM ? 1 : pair_ty_of<T>()][32];
  // tau = 1: the row warps' density and momentum of the next plane,
  // [buffer][c][rho, jx, jy, jz][row][lane] (kept here rather than in
  // registers across the gather of the following plane)
  float2 mom[MOM ? 2 : 1][C][4][MOM ? pair_ty_of<T>() : 1][32];
};

// BDist2 equilibrium constants of one component for one pair: value_q =
// k1 + kh (c.u')^2 +- (kc + k6 (c.u')^2) (c.u') with u' = 3 dv for a
// diagonal pair, twice that for an axis pair in FP32 storage (w = 2/36; the
// doubling is exact), the same for both classes in the offset storages (the
// weight cancels); rest value e0
struct PairEq {
  float2 k1, kh, k6, kc, e0;
};

template <bool OFFSETS>
__device__ __forceinline__ PairEq pair_eq_constants(float2 rho, float2 cst, float rho0_s, float inv_s, float2 scale) {
  PairEq e;
  if (OFFSETS) {
    // h_eq = (rho/s) g - rho0/s
    const float2 R = vmul(rho, splat<float2>(inv_s));
    e.k1 = vmul(vfma(R, cst, splat<float2>(-rho0_s)), scale);
    e.kh = vmul(vmul(R, splat<float2>(0.5f)), scale);
    e.k6 = vmul(vmul(R, splat<float2>(1.0f / 6.0f)), scale);
    e.kc = vmul(vmul(R, cst), scale);
    e.e0 = e.k1;
  } else {
    // f_eq = rho w g: diagonal w = 1/36, rest rho/3 cst
    e.k1 = vmul(vmul(vmul(rho, splat<float2>(1.0f / 36.0f)), cst), scale);
    e.kh = vmul(vmul(rho, splat<float2>(1.0f / 72.0f)), scale);
    e.k6 = vmul(vmul(rho, splat<float2>(1.0f / 216.0f)), scale);
    e.kc = e.k1;
    e.e0 = vmul(vmul(vmul(rho, splat<float2>(1.0f / 3.0f)), cst), scale);
  }
  return e;
}

// Process plane-tiles [w0, w1) of one lattice (tile-major: w = tile*nx + x).
// Every thread of the CTA calls this with the same range.  ZW: the solid
// sites are exactly the planes z = 0 and z = nz - 1 (P.zwall; nz a multiple
// of the tile width, no wall force): the lane holding z = 0 and 1 and the
// one holding nz - 2 and nz - 1 take the bounce-back of the populations
// pulled from the wall (advectFieldsKernel, advection.d:61-89: the site's
// own opposite population), the site's own psi for a wall neighbour
// (addShanChenForcePsi, force.d:273) and store their fluid site alone.
template <typename T, int C, bool MOM, bool ZW = false>
__device__ __forceinline__ void pair_body(const FusedParams& P, const T* __restrict__ f, T* __restrict__ fout,
                                          double* __restrict__ force_out, int64_t w0, int64_t w1,
                                          PairShared<C, MOM, T>& sh) {
  using IO = PairIO<T>;
  using W = typename IO::W;
  constexpr bool OFF = IO::kOffsets;
  // the I16 form conserves every site's mass exactly (see the collision)
  constexpr bool EXACT = std::is_same<T, int16_t>::value;
  constexpr int TY = pair_ty_of<T>();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t plane_sz = uint32_t(P.ny) * uint32_t(P.nz);
  const T* fc[C];
  T* fo[C];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    fc[c] = f + size_t(c) * 19 * size_t(P.n);
    fo[c] = fout + size_t(c) * 19 * size_t(P.n);
  }
  const bool unit = MOM || P.unit_tau != 0;
  float s36[C];
#pragma unroll
  for (int c = 0; c < C; ++c) s36[c] = P.scale[c] * (1.0f / 36.0f);

  int64_t w = w0;
  while (w < w1) {
    const int tile = int(w / P.nx);
    const int xs = int(w - int64_t(tile) * P.nx);
    const int run = int(min(w1 - w, int64_t(P.nx - xs)));
    const int y0 = (tile / P.tiles_z) * TY, z0 = (tile % P.tiles_z) * kPairTZ;
    const int tyv = min(TY, P.ny - y0), tzv = min(kPairTZ, P.nz - z0);
    // this warp's gathered row: r (shared row index) and y; ring warps take
    // rows 0 and tyv + 1
    const bool ring_warp = warp >= TY;
    const int r = ring_warp ? (warp == TY ? 0 : tyv + 1) : warp + 1;
    const bool row_on = ring_warp || warp < tyv;
    const int y = wrap(y0 + r - 1, P.ny);
    // this lane's pair; idle lanes (beyond the row's end) repeat the first
    // pair so that their loads stay in bounds
    const bool active = row_on && 2 * lane < tzv;
    const int zl = z0 + (active ? 2 * lane : 0);
    const bool lane0 = lane == 0;
    const bool lastl = 2 * lane == tzv - 2;
    const bool wlo = ZW && active && z0 == 0 && lane == 0;
    const bool whi = ZW && active && lastl && z0 + tzv == P.nz;
    // a word of new populations: both sites, or the wall lanes' fluid site
    auto put = [&](T* p, W wv) {
      if (ZW && wlo)
        IO::st_hi(p, wv);
      else if (ZW && whi)
        IO::st_lo(p, wv);
      else
        IO::st(p, wv);
    };
    const int zleft = z0 > 0 ? z0 - 1 : P.nz - 1;
    const int zright = z0 + tzv < P.nz ? z0 + tzv : 0;
    const int dl = zleft + IO::kLeftEdge - zl, dr = zright - zl;
    const uint32_t r3[3] = {uint32_t(wrap(y - 1, P.ny)) * uint32_t(P.nz) + uint32_t(zl),
                            uint32_t(y) * uint32_t(P.nz) + uint32_t(zl),
                            uint32_t(wrap(y + 1, P.ny)) * uint32_t(P.nz) + uint32_t(zl)};
    // ring warps' scalar sites: warp TY the left column (z0 - 1), the
    // other the right column (z0 + tzv), lane = shared row
    const bool has_zring = ring_warp && lane < tyv + 2;
    const int zr = warp == TY ? zleft : zright;
    const int zr_i = warp == TY ? 1 : 2 + tzv;  // shared column
    const int yr = wrap(y0 + lane - 1, P.ny);
    int yrs[3], zrs[3];
    yrs[0] = wrap(yr - 1, P.ny);
    yrs[1] = yr;
    yrs[2] = wrap(yr + 1, P.ny);
    zrs[0] = zr > 0 ? zr - 1 : P.nz - 1;
    zrs[1] = zr;
    zrs[2] = zr + 1 < P.nz ? zr + 1 : 0;

    // moments of the plane the row warp collides next (cur) and of the plane
    // it gathers (nxt)
    PairMom<float2> m_cur[C], m_nxt[C];

    // gather the warp's row of plane xg into psi slot ps (and, for the row
    // warps, the moments/words for its collision: keep >= 0 selects the
    // words buffer)
    auto gather_rows = [&](int ps, int xg, int keep) {
      const uint32_t p3[3] = {uint32_t(wrap(xg - 1, P.nx)) * plane_sz, uint32_t(xg) * plane_sz,
                              uint32_t(wrap(xg + 1, P.nx)) * plane_sz};
      if (!row_on) return;
      PairMom<float2> m[C];
      float2 ps2[C];
#pragma unroll
      for (int c = 0; c < C; ++c) {
        float2 v[19];
#pragma unroll
        for (int q = 0; q < 19; ++q) {
          const int cx = Conn<19>::cx(q), cy = Conn<19>::cy(q), cz = Conn<19>::cz(q);
          const uint32_t off = p3[1 - cx] + r3[1 - cy] + P.qn[q];
          W word = IO::ld(fc[c] + off);
          if (cz == 1) word = IO::up(word, lane0, fc[c] + (off + uint32_t(dl)));
          if (cz == -1) word = IO::down(word, lastl, fc[c] + (off + uint32_t(dr)));
          if (ZW && cz == 1 && wlo)
            word = IO::with_hi(word, IO::ld(fc[c] + (p3[1] + r3[1] + P.qn[Conn<19>::bounce(q)])));
          if (ZW && cz == -1 && whi)
            word = IO::with_lo(word, IO::ld(fc[c] + (p3[1] + r3[1] + P.qn[Conn<19>::bounce(q)])));
          if (!MOM && keep >= 0 && !ring_warp) sh.pops[keep][c][q][warp][lane] = word;
          v[q] = IO::val(word);
        }
        m[c] = pair_moments<OFF>(v, s36[c], P.rho0[c]);
        ps2[c] = make_float2(pair_psi(m[c].rho.x, P.psi_form), pair_psi(m[c].rho.y, P.psi_form));
        if (active) *reinterpret_cast<float2*>(&sh.psi[ps][c][r][2 + 2 * lane]) = ps2[c];
        // one component's loads in flight at a time: the next component's
        // loads are not hoisted above this point, which bounds the live
        // registers (two components' 38 words would spill)
        __syncwarp();
      }
      if (keep >= 0 && !ring_warp) {
#pragma unroll
        for (int c = 0; c < C; ++c) {
          if (MOM) {
            // (I16: the exact mass, from which the collision recomputes rho
            // with the same operation)
            sh.mom[keep][c][0][warp][lane] = EXACT ? m[c].mass : m[c].rho;
#pragma unroll
            for (int vd = 0; vd < 3; ++vd) sh.mom[keep][c][1 + vd][warp][lane] = m[c].j[vd];
          } else {
            m_nxt[c] = m[c];
          }
        }
      }
    };
    // the ring warps' scalar sites of plane xg (z0 - 1 and z0 + tzv of each
    // row) into psi slot ps
    auto gather_zring = [&](int ps, int xg) {
      if (!has_zring) return;
      const uint32_t p3[3] = {uint32_t(wrap(xg - 1, P.nx)) * plane_sz, uint32_t(xg) * plane_sz,
                              uint32_t(wrap(xg + 1, P.nx)) * plane_sz};
#pragma unroll
      for (int c = 0; c < C; ++c) {
        float v[19];
#pragma unroll
        for (int q = 0; q < 19; ++q) {
          const int cx = Conn<19>::cx(q), cy = Conn<19>::cy(q), cz = Conn<19>::cz(q);
          const uint32_t off = p3[1 - cx] + uint32_t(yrs[1 - cy]) * uint32_t(P.nz) + uint32_t(zrs[1 - cz]) + P.qn[q];
          v[q] = IO::ld1(fc[c] + off);
        }
        const PairMom<float> m = pair_moments<OFF>(v, s36[c], P.rho0[c]);
        sh.psi[ps][c][lane][zr_i] = pair_psi(m.rho, P.psi_form);
      }
    };

    // warm-up: psi of xs - 1; psi and moments of xs; the z-ring of xs + 1.
    // Plane xs - 1 + j lives in psi slot j % 4.
    __syncthreads();
    gather_rows(0, wrap(xs - 1, P.nx), -1);
    gather_zring(0, wrap(xs - 1, P.nx));
    gather_rows(1, xs, 0);
    gather_zring(1, xs);
    gather_zring(2, wrap(xs + 1, P.nx));
    int cur = 0;
    for (int k = 0; k < run; ++k) {
      const int x = xs + k;
      const int sm = k % 4, s0 = (k + 1) % 4, sp = (k + 2) % 4;  // psi slots of x-1, x, x+1
      if (!MOM) {
#pragma unroll
        for (int c = 0; c < C; ++c) m_cur[c] = m_nxt[c];
      }
      __syncthreads();  // psi slot sp (plane x - 3) and words buffer 1 - cur are free
      gather_rows(sp, wrap(x + 1, P.nx), 1 - cur);
      __syncthreads();
      // the ring warps, idle in the collision: the z-ring of plane x + 2 into
      // slot (k + 3) % 4 (plane x - 2, last read by the previous collision)
      if (ring_warp && k + 1 < run) gather_zring((k + 3) % 4, wrap(x + 2, P.nx));
      if (!ring_warp && active) {
        // ------------------------------------------------------------------
        // collision of plane x at this lane's two sites
        // ------------------------------------------------------------------
        const uint32_t own = uint32_t(x) * plane_sz + r3[1];
        const int zi = 2 + 2 * lane;
        if (MOM) {
#pragma unroll
          for (int c = 0; c < C; ++c) {
            if (EXACT) {
              m_cur[c].mass = sh.mom[cur][c][0][warp][lane];
              m_cur[c].rho = vfma(splat<float2>(s36[c]), m_cur[c].mass, splat<float2>(P.rho0[c]));
            } else {
              m_cur[c].rho = sh.mom[cur][c][0][warp][lane];
            }
#pragma unroll
            for (int vd = 0; vd < 3; ++vd) m_cur[c].j[vd] = sh.mom[cur][c][1 + vd][warp][lane];
          }
        }
        const int slot[3] = {sm, s0, sp};  // by c_x + 1
        // psi of this lane's own sites (written by its own gather of plane x)
        auto psi_own = [&](int c) { return *reinterpret_cast<const float2*>(&sh.psi[s0][c][r][zi]); };
        // --- Shan-Chen: S_c = sum_q w_q psi_c(x + c_q) c_q
        float2 F[C][3];
#pragma unroll
        for (int c = 0; c < C; ++c) F[c][0] = F[c][1] = F[c][2] = make_float2(0.f, 0.f);
        if (P.shan_chen) {
          float2 S[C][3];
#pragma unroll
          for (int c = 0; c < C; ++c) {
            // psi of the 3x3 (x, y) rows around the pair: z-1, (z, z+1), z+2
            auto M = [&](int dx, int dy) {
              return *reinterpret_cast<const float2*>(&sh.psi[slot[dx + 1]][c][r + dy][zi]);
            };
            auto Lv = [&](int dx, int dy) { return sh.psi[slot[dx + 1]][c][r + dy][zi - 1]; };
            auto Rv = [&](int dx, int dy) { return sh.psi[slot[dx + 1]][c][r + dy][zi + 2]; };
            // psi_c(x + c_q) at both sites (planar z-walls: a wall neighbour
            // contributes the site's own psi)
            const float2 ownp = ZW ? psi_own(c) : make_float2(0.f, 0.f);
            auto nbv = [&](int q) -> float2 {
              const int cx = Conn<19>::cx(q), cy = Conn<19>::cy(q), cz = Conn<19>::cz(q);
              float2 v;
              if (cz == 0) {
                v = M(cx, cy);
              } else if (cz == 1) {
                const float2 m = M(cx, cy);
                v = make_float2(m.y, Rv(cx, cy));
                if (ZW && whi) v.x = ownp.x;
              } else {
                const float2 m = M(cx, cy);
                v = make_float2(Lv(cx, cy), m.x);
                if (ZW && wlo) v.y = ownp.y;
              }
              return v;
            };
            // axis and diagonal sums per direction, in a fixed order
            const float2 ax = vsub(nbv(1), nbv(2)), ay = vsub(nbv(3), nbv(4)), az = vsub(nbv(5), nbv(6));
            const float2 dx = vsub(vadd(vadd(nbv(7), nbv(11)), vadd(nbv(12), nbv(13))),
                                   vadd(vadd(nbv(8), nbv(14)), vadd(nbv(17), nbv(18))));
            const float2 dy = vsub(vadd(vadd(nbv(7), nbv(8)), vadd(nbv(9), nbv(15))),
                                   vadd(vadd(nbv(10), nbv(13)), vadd(nbv(14), nbv(16))));
            const float2 dz = vsub(vadd(vadd(nbv(9), nbv(10)), vadd(nbv(11), nbv(17))),
                                   vadd(vadd(nbv(12), nbv(15)), vadd(nbv(16), nbv(18))));
            // S = (2 axis + diag) / 36
            const float2 w36 = splat<float2>(1.0f / 36.0f), two = splat<float2>(2.f);
            S[c][0] = vmul(w36, vfma(two, ax, dx));
            S[c][1] = vmul(w36, vfma(two, ay, dy));
            S[c][2] = vmul(w36, vfma(two, az, dz));
          }
#pragma unroll
          for (int f1 = 0; f1 < C; ++f1) {
            float2 g[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
            for (int f2 = 0; f2 < C; ++f2) {
              const float2 cc = splat<float2>(P.gcc[f1][f2]);
#pragma unroll
              for (int vd = 0; vd < 3; ++vd) g[vd] = vfma(cc, S[f2][vd], g[vd]);
            }
            const float2 own_psi = psi_own(f1);
            const float2 mp = make_float2(-own_psi.x, -own_psi.y);
#pragma unroll
            for (int vd = 0; vd < 3; ++vd) F[f1][vd] = vmul(mp, g[vd]);
          }
        }
        float2 tot = m_cur[0].rho;
        if (C > 1) tot = vadd(tot, m_cur[1].rho);
#pragma unroll
        for (int c = 0; c < C; ++c) {
          // distributeForce with no distributed force: only its NaN cases
          // matter
          const bool bad0 = tot.x == 0.f || isnan(tot.x) || isinf(m_cur[c].rho.x) || isnan(m_cur[c].rho.x);
          const bool bad1 = tot.y == 0.f || isnan(tot.y) || isinf(m_cur[c].rho.y) || isnan(m_cur[c].rho.y);
#pragma unroll
          for (int vd = 0; vd < 3; ++vd) {
            if (bad0) F[c][vd].x = NAN;
            if (bad1) F[c][vd].y = NAN;
          }
        }
        if (P.record_force) {
#pragma unroll
          for (int c = 0; c < C; ++c)
#pragma unroll
            for (int vd = 0; vd < 3; ++vd) {
              // (planar z-walls: no force on the wall sites)
              force_out[(size_t(c) * P.n + own) * 3 + vd] = (ZW && wlo) ? 0.0 : double(F[c][vd].x);
              force_out[(size_t(c) * P.n + own + 1) * 3 + vd] = (ZW && whi) ? 0.0 : double(F[c][vd].y);
            }
        }
        // --- BDist2 weighted velocity: sum_c j_c / tau_c / sum_c rho_c
        float2 wv[3];
        {
          const float2 rt = make_float2(__frcp_rn(tot.x), __frcp_rn(tot.y));
#pragma unroll
          for (int vd = 0; vd < 3; ++vd) {
            float2 a;
            if (unit) {
              a = m_cur[0].j[vd];
              if (C > 1) a = vadd(a, m_cur[1].j[vd]);
            } else {
              a = vmul(m_cur[0].j[vd], splat<float2>(P.inv_tau[0]));
              if (C > 1) a = vfma(m_cur[1].j[vd], splat<float2>(P.inv_tau[1]), a);
            }
            wv[vd] = vmul(a, rt);
          }
        }
        // --- collision: equilibrium (and relaxation) of every population,
        // one word store per population
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const float2 rd = make_float2(__frcp_rn(m_cur[c].rho.x), __frcp_rn(m_cur[c].rho.y));
          float2 dv[3];
#pragma unroll
          for (int vd = 0; vd < 3; ++vd) {
            const float2 u = vfma(F[c][vd], rd, splat<float2>(P.acc[vd]));
            dv[vd] = unit ? vadd(u, wv[vd]) : vfma(splat<float2>(P.tau[c]), u, wv[vd]);
          }
          const float2 three = splat<float2>(3.f);
          const float2 ux = vmul(three, dv[0]), uy = vmul(three, dv[1]), uz = vmul(three, dv[2]);
          const float2 uu = vfma(dv[2], uz, vfma(dv[1], uy, vmul(dv[0], ux)));
          const float2 cst = vfma(splat<float2>(-0.5f), uu, splat<float2>(1.f));
          const float2 scale = splat<float2>(unit ? 1.f : P.omega[c]);
          const PairEq e = pair_eq_constants<OFF>(m_cur[c].rho, cst, P.rho0[c] * P.inv_scale[c], P.inv_scale[c], scale);
          const float2 omo = splat<float2>(P.one_minus_omega[c]);
          // the new value of every population (equilibrium, relaxed for
          // tau != 1), handed to sink(q, value) pair by pair
          auto emit_all = [&](auto&& sink) {
            auto val = [&](int q, float2 v) {
              if (!unit) v = vfma(IO::val(sh.pops[cur][c][q][warp][lane]), omo, v);
              sink(q, v);
            };
            auto pair = [&](float2 cu, int axis, int ip, int im) {
              const float2 cu2 = vmul(cu, cu);
              const float2 even = vfma(e.kh, cu2, e.k1);
              const float2 odd = vmul(vfma(e.k6, cu2, e.kc), cu);
              float2 vp = vadd(even, odd), vm = vsub(even, odd);
              if (!OFF && axis) {
                vp = vmul(splat<float2>(2.f), vp);
                vm = vmul(splat<float2>(2.f), vm);
              }
              val(ip, vp);
              val(im, vm);
            };
            val(0, e.e0);
            pair(ux, 1, 1, 2);
            pair(uy, 1, 3, 4);
            pair(uz, 1, 5, 6);
            pair(vadd(ux, uy), 0, 7, 14);
            pair(vsub(ux, uy), 0, 13, 8);
            pair(vadd(ux, uz), 0, 11, 18);
            pair(vsub(ux, uz), 0, 12, 17);
            pair(vadd(uy, uz), 0, 9, 16);
            pair(vsub(uy, uz), 0, 15, 10);
          };
          if constexpr (EXACT) {
            // Exact mass conservation: rounded to integers (and saturated to
            // +-32767), the new values' mass 12 h_0 + 2 sum_axis h +
            // sum_diag h differs from the gathered one (which the collision
            // conserves in real arithmetic) by a few units, more where a
            // value saturated.  The difference goes to h_0 in multiples of
            // 12 and the rest to the opposite pair h_7, h_14 (half each, an
            // odd unit to h_7: no momentum but that unit), which are stored
            // last; the other 16 are stored as they are formed.  Streaming
            // and bounce-back move stored values, so every lattice's total
            // mass stays exactly what it was uploaded with (unless one of
            // the three adjusted values saturates).
            auto rnd = [](float v) { return fminf(fmaxf(rintf(v), -32767.f), 32767.f); };
            float2 mout = make_float2(0.f, 0.f), h0, h7, h14;
            emit_all([&](int q, float2 v) {
              const float2 r = make_float2(rnd(v.x), rnd(v.y));
              const float k = Conn<19>::wclass(q) == 0 ? 12.f : (Conn<19>::wclass(q) == 1 ? 2.f : 1.f);
              mout = vfma(splat<float2>(k), r, mout);
              if (q == 0)
                h0 = r;
              else if (q == 7)
                h7 = r;
              else if (q == 14)
                h14 = r;
              else
                put(fo[c] + (P.qn[q] + own), IO::enc_int(r));
            });
            const int dx = __float2int_rz(m_cur[c].mass.x - mout.x), dy = __float2int_rz(m_cur[c].mass.y - mout.y);
            const int d0x = dx / 12, d0y = dy / 12;
            const int rx = dx - 12 * d0x, ry = dy - 12 * d0y;
            const int hx = rx / 2, hy = ry / 2;
            h0 = vadd(h0, make_float2(float(d0x), float(d0y)));
            h7 = vadd(h7, make_float2(float(rx - hx), float(ry - hy)));
            h14 = vadd(h14, make_float2(float(hx), float(hy)));
            put(fo[c] + (P.qn[0] + own), IO::enc(h0));
            put(fo[c] + (P.qn[7] + own), IO::enc(h7));
            put(fo[c] + (P.qn[14] + own), IO::enc(h14));
          } else {
            emit_all([&](int q, float2 v) { put(fo[c] + (P.qn[q] + own), IO::enc(v)); });
          }
        }
      }
      cur = 1 - cur;
    }
    w += run;
  }
}

// resident CTAs per SM the kernels are compiled for: two of 10 warps at up
// to 96 registers, one of 16 warps for half offsets (14 rows)
template <typename T>
constexpr int pair_minb() {
  return pair_ty_of<T>() > 8 ? 1 : 2;
}

// The variants that run: every tau = 1 (MOM) for FP32 and FP16, and for the
// I16 form also tau != 1 (pairs_eligible: FP32 and FP16 lattices with a
// tau != 1 run the one-site kernel).
template <typename T>
constexpr bool pairs_general() {
  return std::is_same<T, int16_t>::value;
}

// The single-lattice kernel: persistent CTAs take runs of run_len planes of
// one tile from the counter, x-chunk-major (neighbouring tiles march over
// the same planes together and share their ring rows through L2), over the
// planes [x_begin, x_end) of every tile.  ZW: planar z-walls (pair_body).
template <typename T, int C, bool MOM, bool ZW = false>
__global__ void __launch_bounds__(pair_threads<T>(), pair_minb<T>())
    k_pairs(const T* __restrict__ f, T* __restrict__ fout, double* __restrict__ force_out, FusedParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& sh = *reinterpret_cast<PairShared<C, MOM, T>*>(smem_raw);
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
    pair_body<T, C, MOM, ZW>(P, f, fout, force_out, w0, w0 + (x1 - x0), sh);
  }
}

// One simulation of a batch for the pair kernel.  The step reads
// populations f[(parity + phase) & 1] and writes the other buffer.
struct PairSim {
  FusedParams P;           // pair tiling (pair_ty x 64), run_len set
  const void* f[2];
  double* force_out;       // nullptr unless recording
  int64_t unit_begin;      // first run of this simulation in the batch
  int32_t phase;
  int32_t nchunks;         // runs per tile: ceil(nx / P.run_len)
};

// Many independent lattices of any (even nz) sizes in one persistent
// launch: CTAs take runs of at most run_len planes of one tile (all
// simulations' runs concatenated) from counters[parity] and zero the other
// counter for the next launch.  Each member runs pair_body with its own
// parameters (staged in shared memory), so it computes exactly what its
// lone lattice computes.
template <typename T>
__global__ void __launch_bounds__(pair_threads<T>(), pair_minb<T>())
    k_pairs_batch(const PairSim* __restrict__ sims, int nsims, int parity, int64_t total_units,
                  int* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ FusedParams Ps;
  __shared__ int s_idx;
  __shared__ long long s_w[2];
  if (blockIdx.x == 0 && threadIdx.x == 0) counters[1 - parity] = 0;
  for (;;) {
    __syncthreads();  // every thread has used the previous range and Ps
    if (threadIdx.x == 0) {
      long long r0 = 0, r1 = 0;
      int idx = 0;
      const long long key = (long long)atomicAdd(counters + parity, 1);
      if (key < total_units) {
        int lo = 0, hi = nsims - 1;  // last simulation starting at or before key
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (sims[mid].unit_begin <= key)
            lo = mid;
          else
            hi = mid - 1;
        }
        idx = lo;
        const long long local = key - sims[lo].unit_begin;
        const int ntl = sims[lo].P.tiles_y * sims[lo].P.tiles_z;
        const long long ch = local / ntl, tile = local - ch * ntl;  // x-chunk-major, as k_pairs
        const int nx = sims[lo].P.nx, rl = sims[lo].P.run_len;
        r0 = tile * nx + ch * rl;
        const long long tile_end = (tile + 1) * nx;
        r1 = r0 + rl < tile_end ? r0 + rl : tile_end;
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
    const int par = (parity + sims[i].phase) & 1;
    const T* fin = static_cast<const T*>(sims[i].f[par]);
    T* fout = const_cast<T*>(static_cast<const T*>(sims[i].f[1 - par]));
    const long long r0 = s_w[0], r1 = s_w[1];
    __syncthreads();
    if (!pairs_general<T>() || Ps.unit_tau) {
      pair_body<T, 2, true>(Ps, fin, fout, sims[i].force_out, r0, r1,
                            *reinterpret_cast<PairShared<2, true, T>*>(smem_raw));
    } else if constexpr (pairs_general<T>()) {
      pair_body<T, 2, false>(Ps, fin, fout, sims[i].force_out, r0, r1,
                             *reinterpret_cast<PairShared<2, false, T>*>(smem_raw));
    }
  }
}

// Host side: one persistent launch of k_pairs (F holds the pair tiling, the
// plane range and the zeroed work counter).
template <typename T, int C, bool MOM, bool ZW = false>
cudaError_t go_pairs(const StepBuffers& b, const FusedParams& F, cudaStream_t st, int device) {
  static KernelInfo info;
  auto kern = k_pairs<T, C, MOM, ZW>;
  const int smem = int(sizeof(PairShared<C, MOM, T>));
  int per_sm = 0;
  cudaError_t e = kernel_setup(kern, smem, pair_threads<T>(), device, info, &per_sm);
  if (e != cudaSuccess) return e;
  int64_t grid = int64_t(per_sm) * sm_count(device);
  FusedParams G = F;
  const int64_t tiles = int64_t(G.tiles_y) * G.tiles_z;
  plan_runs(G, tiles, grid);
  const int64_t units = sched_units(G, int(tiles));
  if (grid > units) grid = units;
  kern<<<unsigned(grid), pair_threads<T>(), smem, st>>>(static_cast<const T*>(b.f), static_cast<T*>(b.fout), b.force,
                                                        G);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_pairs(int c, bool mom, const StepBuffers& b, const FusedParams& F, cudaStream_t st, int device) {
  if (b.mask) {
    // planar z-walls in FP16 (two components, every tau = 1, nz a multiple
    // of the tile width); other solid sites run the one-site kernel
    if (!F.zwall || c != 2 || !mom || F.nz % kPairTZ != 0) return cudaErrorInvalidValue;
    if constexpr (std::is_same<T, __half>::value) return go_pairs<T, 2, true, true>(b, F, st, device);
    return cudaErrorInvalidValue;
  }
  if constexpr (pairs_general<T>()) {
    if (c == 2) return mom ? go_pairs<T, 2, true>(b, F, st, device) : go_pairs<T, 2, false>(b, F, st, device);
    return mom ? go_pairs<T, 1, true>(b, F, st, device) : go_pairs<T, 1, false>(b, F, st, device);
  } else {
    if (!mom) return cudaErrorInvalidValue;  // tau != 1: the one-site kernel
    return c == 2 ? go_pairs<T, 2, true>(b, F, st, device) : go_pairs<T, 1, true>(b, F, st, device);
  }
}

}  // namespace lbk
