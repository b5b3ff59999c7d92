// Fused single-pass D2Q9 timestep, two y-adjacent sites per thread: the
// two-dimensional counterpart of lb_pairs.cuh, for the float-arithmetic
// forms (float or half-offset storage) of lattices with every tau = 1, the
// BDist2 equilibrium, two components, an even ny and no solid site (the
// others run the one-site-per-thread k_fused2d, lb_fused2d.cuh).  The
// launcher runs it for the half-offset form, where it is the faster kernel.
//
// Sites are x * ny + y (y contiguous).  A CTA of kP2Threads threads owns a
// tile of kF2W consecutive y and marches along x; thread t the sites
// y0 + 2t and y0 + 2t + 1, one aligned 8-byte (float) or 4-byte (half)
// word of every population array.  Per row x + 1 it pull-gathers its word of
// every population (the populations streaming along y, c_y = +-1, take their
// neighbour from the adjacent lane by a warp shuffle, a warp's edge lanes
// from one extra load), sums density and momentum (in half storage directly
// on the stored offsets, the weights factored out), writes psi into a
// three-row shared ring and the momenta into shared memory; threads 0 and 1
// also gather the tile's two ring sites y0 - 1 and y0 + tv.  After a barrier
// the row x is collided from the ring: the 8-point psi stencil, the
// Shan-Chen force, the BDist2 weighted velocity and equilibrium, one word
// store per population.  All per-site float arithmetic runs on the packed
// two-lane FP32 instructions (__fadd2_rn, __fmul2_rn, __ffma2_rn), rounded
// to nearest like the scalar ring gathers, so a site's result does not
// depend on which lane computes it.
//
// The arithmetic restates the reference (advectFieldsKernel
// advection.d:61-89, psi force.d:320-333, addShanChenForcePsi
// force.d:238-309, distributeForce force.d:179-197,
// precalculateWeightedVelocity collision.d:156-196, collideFieldsKernel
// collision.d:90-119, eqDist for D2Q9 eqdist.d:185-235) in float, with sums
// regrouped by weight class and the density folded into the equilibrium's
// constants; it agrees with the one-site kernel to rounding, not bit for
// bit.
#pragma once

#include "lb_fused2d.cuh"
#include "lb_pairs.cuh"

namespace lbk {

constexpr int kP2Threads = kF2W / 2;  // one thread per two sites of the tile

struct Pair2Shared {
  float psi[3][2][kF2W + 4];          // [row slot][c][y - y0 + 2]: [1] left ring, [2, 2 + tv) tile, [2 + tv] right ring
  float2 mom[2][2][3][kP2Threads];    // [buffer][c][rho, jx, jy][thread]
};

// Density and momentum of one component from its 9 gathered values (float:
// the populations; half: the stored offsets h with f_q = w_q (rho0 + s h_q),
// w = 16/36, 4/36, 1/36), in one fixed order for float and float2 alike.
template <bool OFFSETS, typename V>
__device__ __forceinline__ void pair2_moments(const V (&v)[9], float s36, float rho0, V& rho, V& jx, V& jy) {
  const V A = vadd(vadd(v[1], v[2]), vadd(v[3], v[4]));
  const V Ax = vsub(v[1], v[2]), Ay = vsub(v[3], v[4]);
  const V D = vadd(vadd(v[5], v[8]), vadd(v[6], v[7]));
  const V Dx = vsub(vadd(v[5], v[6]), vadd(v[7], v[8]));  // c_x = +1: 5, 6
  const V Dy = vsub(vadd(v[5], v[7]), vadd(v[6], v[8]));  // c_y = +1: 5, 7
  if (OFFSETS) {
    const V four = splat<V>(4.f);
    rho = vfma(splat<V>(s36), vfma(splat<V>(16.f), v[0], vfma(four, A, D)), splat<V>(rho0));
    jx = vmul(splat<V>(s36), vfma(four, Ax, Dx));
    jy = vmul(splat<V>(s36), vfma(four, Ay, Dy));
  } else {
    rho = vadd(vadd(v[0], A), D);
    jx = vadd(Ax, Dx);
    jy = vadd(Ay, Dy);
  }
}

// one run: rows [xa, xb) of tile `tile`
template <typename T>
__device__ __forceinline__ void pair2_run(const FusedParams& P, const T* __restrict__ f, T* __restrict__ fout,
                                          double* __restrict__ force_out, int tile, int xa, int xb,
                                          Pair2Shared& sh) {
  using IO = PairIO<T>;
  using W = typename IO::W;
  constexpr bool OFF = IO::kOffsets;
  const int t = threadIdx.x, lane = t & 31;
  const int ny = P.ny;
  const int y0 = tile * kF2W;
  const int tv = min(kF2W, ny - y0);
  // this thread's pair; idle threads (beyond the tile's end) repeat the
  // first pair so that their loads stay in bounds
  const bool active = 2 * t < tv;
  const int y = y0 + (active ? 2 * t : 0);
  // edge lanes load the neighbour the shuffle cannot reach: y - 1 (the
  // word holding it, for half) and y + 2, periodic
  const bool lane0 = lane == 0;
  const bool lastl = lane == 31 || 2 * t == tv - 2;
  const int yl = y > 0 ? y - 1 : ny - 1, yr = y + 2 < ny ? y + 2 : 0;
  const int dl = yl + IO::kLeftEdge - y, dr = yr - y;
  const T* const fc[2] = {f, f + size_t(9) * size_t(P.n)};
  T* const fo[2] = {fout, fout + size_t(9) * size_t(P.n)};
  float s36[2];
  s36[0] = P.scale[0] * (1.0f / 36.0f);
  s36[1] = P.scale[1] * (1.0f / 36.0f);
  // threads 0 and 1: the ring sites y0 - 1 and y0 + tv
  const bool has_ring = t < 2;
  const int ry = t == 0 ? wrap(y0 - 1, ny) : wrap(y0 + tv, ny);
  const int rslot = t == 0 ? 1 : 2 + tv;
  const int rys[3] = {wrap(ry - 1, ny), ry, wrap(ry + 1, ny)};

  // psi of row xg into slot ps and, unless keep < 0, the momenta into
  // buffer keep
  auto gather_row = [&](int ps, int xg, int keep) {
    const uint32_t rows[3] = {uint32_t(wrap(xg - 1, P.nx)) * uint32_t(ny), uint32_t(xg) * uint32_t(ny),
                              uint32_t(wrap(xg + 1, P.nx)) * uint32_t(ny)};
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      float2 v[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        const int cx = Conn<9>::cx(q), cy = Conn<9>::cy(q);
        const uint32_t off = rows[1 - cx] + uint32_t(y) + P.qn[q];
        W word = IO::ld(fc[c] + off);
        if (cy == 1) word = IO::up(word, lane0, fc[c] + (off + uint32_t(dl)));
        if (cy == -1) word = IO::down(word, lastl, fc[c] + (off + uint32_t(dr)));
        v[q] = IO::val(word);
      }
      float2 rho, jx, jy;
      pair2_moments<OFF>(v, s36[c], P.rho0[c], rho, jx, jy);
      if (active) {
        *reinterpret_cast<float2*>(&sh.psi[ps][c][2 + 2 * t]) =
            make_float2(pair_psi(rho.x, P.psi_form), pair_psi(rho.y, P.psi_form));
        if (keep >= 0) {
          sh.mom[keep][c][0][t] = rho;
          sh.mom[keep][c][1][t] = jx;
          sh.mom[keep][c][2][t] = jy;
        }
      }
      // one component's loads in flight at a time (bounds the registers)
      __syncwarp();
    }
    if (has_ring) {
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        float v[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
          const int cx = Conn<9>::cx(q), cy = Conn<9>::cy(q);
          v[q] = IO::ld1(fc[c] + (rows[1 - cx] + uint32_t(rys[1 - cy]) + P.qn[q]));
        }
        float rho, jx, jy;
        pair2_moments<OFF>(v, s36[c], P.rho0[c], rho, jx, jy);
        sh.psi[ps][c][rslot] = pair_psi(rho, P.psi_form);
      }
    }
  };

  gather_row(0, wrap(xa - 1, P.nx), -1);
  gather_row(1, xa, 0);
  int cur = 0;
  for (int k = 0; k < xb - xa; ++k) {
    const int x = xa + k;
    const int sm = k % 3, s0 = (k + 1) % 3, sp = (k + 2) % 3;  // row slots of x-1, x, x+1
    __syncthreads();  // row slot sp and momenta buffer 1-cur are free
    gather_row(sp, wrap(x + 1, P.nx), 1 - cur);
    __syncthreads();
    if (active) {
      const uint32_t own = uint32_t(x) * uint32_t(ny) + uint32_t(y);
      const int zi = 2 + 2 * t;
      const int slot[3] = {sm, s0, sp};  // by c_x + 1
      float2 rho[2], j[2][2];
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        rho[c] = sh.mom[cur][c][0][t];
        j[c][0] = sh.mom[cur][c][1][t];
        j[c][1] = sh.mom[cur][c][2][t];
      }
      // --- Shan-Chen: S_c = sum_q w_q psi_c(x + c_q) c_q (w = 4/36 axis,
      // 1/36 diagonal)
      float2 F[2][2];
#pragma unroll
      for (int c = 0; c < 2; ++c) F[c][0] = F[c][1] = make_float2(0.f, 0.f);
      if (P.shan_chen) {
        float2 S[2][2];
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          auto M = [&](int dx) { return *reinterpret_cast<const float2*>(&sh.psi[slot[dx + 1]][c][zi]); };
          auto Lv = [&](int dx) { return sh.psi[slot[dx + 1]][c][zi - 1]; };
          auto Rv = [&](int dx) { return sh.psi[slot[dx + 1]][c][zi + 2]; };
          // psi_c(x + c_q) at both sites
          auto nbv = [&](int q) -> float2 {
            const int cx = Conn<9>::cx(q), cy = Conn<9>::cy(q);
            const float2 m = M(cx);
            if (cy == 0) return m;
            if (cy == 1) return make_float2(m.y, Rv(cx));
            return make_float2(Lv(cx), m.x);
          };
          const float2 ax = vsub(nbv(1), nbv(2)), ay = vsub(nbv(3), nbv(4));
          const float2 dx = vsub(vadd(nbv(5), nbv(6)), vadd(nbv(7), nbv(8)));
          const float2 dy = vsub(vadd(nbv(5), nbv(7)), vadd(nbv(6), nbv(8)));
          // S = (4 axis + diag) / 36
          const float2 w36 = splat<float2>(1.0f / 36.0f), four = splat<float2>(4.f);
          S[c][0] = vmul(w36, vfma(four, ax, dx));
          S[c][1] = vmul(w36, vfma(four, ay, dy));
        }
#pragma unroll
        for (int f1 = 0; f1 < 2; ++f1) {
          float2 g[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
          for (int f2 = 0; f2 < 2; ++f2) {
            const float2 cc = splat<float2>(P.gcc[f1][f2]);
#pragma unroll
            for (int vd = 0; vd < 2; ++vd) g[vd] = vfma(cc, S[f2][vd], g[vd]);
          }
          const float2 own_psi = *reinterpret_cast<const float2*>(&sh.psi[s0][f1][zi]);
          const float2 mp = make_float2(-own_psi.x, -own_psi.y);
#pragma unroll
          for (int vd = 0; vd < 2; ++vd) F[f1][vd] = vmul(mp, g[vd]);
        }
      }
      const float2 tot = vadd(rho[0], rho[1]);
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        // distributeForce with no distributed force: only its NaN cases
        // matter
        const bool bad0 = tot.x == 0.f || isnan(tot.x) || isinf(rho[c].x) || isnan(rho[c].x);
        const bool bad1 = tot.y == 0.f || isnan(tot.y) || isinf(rho[c].y) || isnan(rho[c].y);
#pragma unroll
        for (int vd = 0; vd < 2; ++vd) {
          if (bad0) F[c][vd].x = NAN;
          if (bad1) F[c][vd].y = NAN;
        }
      }
      if (P.record_force) {
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
          for (int vd = 0; vd < 2; ++vd) {
            force_out[(size_t(c) * P.n + own) * 2 + vd] = double(F[c][vd].x);
            force_out[(size_t(c) * P.n + own + 1) * 2 + vd] = double(F[c][vd].y);
          }
      }
      // --- BDist2 weighted velocity (every tau = 1): sum_c j_c / sum_c rho_c
      const float2 rt = make_float2(__frcp_rn(tot.x), __frcp_rn(tot.y));
      const float2 wvx = vmul(vadd(j[0][0], j[1][0]), rt), wvy = vmul(vadd(j[0][1], j[1][1]), rt);
      // --- collision: the equilibrium of every population, one word store
      // per population
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const float2 rd = make_float2(__frcp_rn(rho[c].x), __frcp_rn(rho[c].y));
        const float2 dvx = vadd(vfma(F[c][0], rd, splat<float2>(P.acc[0])), wvx);
        const float2 dvy = vadd(vfma(F[c][1], rd, splat<float2>(P.acc[1])), wvy);
        const float2 three = splat<float2>(3.f);
        const float2 ux = vmul(three, dvx), uy = vmul(three, dvy);
        const float2 uu = vfma(dvy, uy, vmul(dvx, ux));
        const float2 cst = vfma(splat<float2>(-0.5f), uu, splat<float2>(1.f));
        // pair values k1 + kh (c.u')^2 +- (kc + k6 (c.u')^2) (c.u'), rest e0;
        // float: f_eq (axis pairs twice the diagonal constants); half: the
        // offset h_eq = (f_eq / w_q - rho0) / s, whose class factors
        // (aN / w: rest 9/8, axis 3/4, diagonal 3/2 of the rho/24 scale)
        // differ per weight class
        float2 k1[2], kh[2], k6[2], kc[2], e0;
        if (OFF) {
          const float2 R = vmul(rho[c], splat<float2>(P.inv_scale[c]));
          const float2 r0 = splat<float2>(-P.rho0[c] * P.inv_scale[c]);
          const float fac[2] = {0.75f, 1.5f};  // axis, diagonal
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            const float2 Rf = vmul(R, splat<float2>(fac[k]));
            kc[k] = vmul(Rf, cst);
            k1[k] = vadd(kc[k], r0);
            kh[k] = vmul(Rf, splat<float2>(0.5f));
            k6[k] = vmul(Rf, splat<float2>(1.0f / 6.0f));
          }
          e0 = vfma(vmul(R, splat<float2>(1.125f)), cst, r0);
        } else {
          const float2 r1 = vmul(vmul(rho[c], splat<float2>(1.0f / 24.0f)), cst);
          const float2 rh = vmul(rho[c], splat<float2>(1.0f / 48.0f));
          const float2 r6 = vmul(rho[c], splat<float2>(1.0f / 144.0f));
          const float2 two = splat<float2>(2.f);
          k1[0] = vmul(two, r1);
          kh[0] = vmul(two, rh);
          k6[0] = vmul(two, r6);
          kc[0] = k1[0];
          k1[1] = r1;
          kh[1] = rh;
          k6[1] = r6;
          kc[1] = r1;
          e0 = vmul(vmul(rho[c], splat<float2>(0.5f)), cst);
        }
        auto put = [&](int q, float2 val) { IO::st(fo[c] + (P.qn[q] + own), IO::enc(val)); };
        auto pair = [&](float2 cu, int k, int ip, int im) {
          const float2 cu2 = vmul(cu, cu);
          const float2 even = vfma(kh[k], cu2, k1[k]);
          const float2 odd = vmul(vfma(k6[k], cu2, kc[k]), cu);
          put(ip, vadd(even, odd));
          put(im, vsub(even, odd));
        };
        put(0, e0);
        pair(ux, 0, 1, 2);
        pair(uy, 0, 3, 4);
        pair(vadd(ux, uy), 1, 5, 8);
        pair(vsub(ux, uy), 1, 6, 7);
      }
    }
    cur = 1 - cur;
  }
}

// resident CTAs per SM the kernel is compiled for (eight: 32 warps at up
// to 64 registers)
#ifndef LB_P2_MINB
#define LB_P2_MINB 8
#endif

// P.tiles_z tiles of kF2W y per row; rows in the runs of sched_run
template <typename T>
__global__ void __launch_bounds__(kP2Threads, LB_P2_MINB)
    k_pairs2d(const T* __restrict__ f, T* __restrict__ fout, double* __restrict__ force_out, FusedParams P) {
  __shared__ Pair2Shared sh;
  __shared__ int s_item;
  const int tiles = P.tiles_z;
  const int units = sched_units(P, tiles);
  for (;;) {
    __syncthreads();  // every thread has read the previous item
    if (threadIdx.x == 0) s_item = atomicAdd(P.work_counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= units) break;
    int tile, xa, xb;
    sched_run(P, tiles, item, tile, xa, xb);
    pair2_run<T>(P, f, fout, force_out, tile, xa, xb, sh);
  }
}

}  // namespace lbk
