// Fused single-pass D2Q9 timestep for the bandwidth forms (float arithmetic;
// float or half-offset storage): the two-dimensional counterpart of
// lb_fused.cuh.
//
// Sites are x * ny + y (y contiguous).  A CTA of kF2W threads owns a segment
// of kF2W consecutive y (a tile) and marches along x.  For each row x + 1 it
// pull-gathers the tile's populations and those of its two ring sites
// (y0 - 1 and y0 + kF2W), computes rho and psi there and keeps them in a
// three-row shared-memory ring, and keeps the tile's momenta (every tau = 1
// with BDist2: the collision needs nothing else) or its populations (the
// other collisions) for one row; then row x is collided with the 8-point psi
// stencil read from shared memory and written out.  A row's populations are
// read from HBM once and written once; the two ring sites per row are read
// again by the neighbouring tile.  With walls, the 32-bit neighbour mask of
// every site (bit 0: solid; bit q: the site x + c_q is solid) selects the
// bounce-back source of the gather, the stencil's wall substitution and the
// wall force, as in the D3Q19 kernel; solid sites are not written (both
// population buffers hold them).
//
// Scheduling: runs of consecutive rows of one tile taken from an atomic
// counter (sched_run: x-chunk-major, shorter runs last), or, without a
// counter, run items strided over the CTAs.  Every run starts with two
// warm-up rows.
//
// Per-site arithmetic restates the reference (addShanChenForcePsi
// force.d:238-309, distributeForce force.d:179-197,
// precalculateWeightedVelocity collision.d:156-196, collideFieldsKernel
// collision.d:90-119, eqDist for D2Q9 eqdist.d:185-235) in float, with the
// Shan-Chen sum re-associated as in lb_fused.cuh: -psi_c1 * sum_c2 g_c1c2 *
// S_c2 with S_c2 = sum_q w_q psi_c2(x + c_q) c_q.
#pragma once

#include "lb_fused.cuh"

namespace lbk {

// sites of a tile = threads of a CTA
constexpr int kF2W = 256;

// NP = 9: the tile's populations; NP = 2: its momentum per component
template <int NP>
struct Fused2Shared {
  float pops[2][2][NP][kF2W];   // [buffer][c][q or vd][site in tile]
  float psi[3][2][kF2W + 2];    // [row slot][c][y - y0 + 1]
  float rho[3][2][kF2W + 2];
};

// S = w_axis * sum_axis + w_diag * sum_diag (D2Q9: w = 1/9, 1/36)
__device__ __forceinline__ float stencil_weigh9(float axis, float diag) {
  return fmaf(1.0f / 9.0f, axis, (1.0f / 36.0f) * diag);
}

// The BDist2 D2Q9 equilibrium (eqdist.d:185-235) in float, the density
// folded into the pair constants as in eq_bdist2_f: with u' = 3 dv and
// cst = 1 - 3/2 dv.dv, a pair +-c with weight w (1/24, twice that on the
// axes) gets rho w (cst + (c.u')^2 / 2) +- rho w (cst c.u' + (c.u')^3 / 6),
// the rest population rho/2 cst.
__device__ __forceinline__ void eq_bdist2_f9(const float (&dv)[3], float rho, float (&dist)[9]) {
  const float ux = 3.0f * dv[0], uy = 3.0f * dv[1];
  const float uu = fmaf(dv[1], uy, dv[0] * ux);
  const float cst = fmaf(-0.5f, uu, 1.0f);
  const float r1 = (rho * (1.0f / 24.0f)) * cst;  // rho aN1 cst
  const float rh = rho * (1.0f / 48.0f);          // rho aN1 / 2
  const float r6 = rho * (1.0f / 144.0f);         // rho aN1 / 6
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
  pair(ux + uy, r1, rh, r6, 5, 8);
  pair(ux - uy, r1, rh, r6, 6, 7);
  dist[0] = (rho * 0.5f) * cst;
}

// Pull-gather one site of row xg; rows[0..2] are the offsets of rows xg-1,
// xg, xg+1, yo[0..2] of y-1, y, y+1; nbm is the site's neighbour mask.
template <typename T, bool WALLS, int C>
__device__ __forceinline__ void gather9(const T* const (&fc)[2], const FusedParams& P, const uint32_t (&rows)[3],
                                        const int (&yo)[3], uint32_t nbm, float (&pop)[C][9]) {
  const uint32_t s = rows[1] + uint32_t(yo[1]);
  const bool solid = WALLS && (nbm & 1u);
  // branch-free: a solid site keeps its own populations, a fluid site pulls
  // from x - c_q or, when that site is solid, bounces back its own opposite
  // population (x - c_q = x + c_b)
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const int cx = Conn<9>::cx(q), cy = Conn<9>::cy(q);
    const uint32_t nb = rows[1 - cx] + uint32_t(yo[1 - cy]);
    const int b = Conn<9>::bounce(q);
    bool bb = false;
    if (WALLS && q > 0) bb = ((nbm >> b) & 1u) && !solid;
    const uint32_t off = (bb ? P.qn[b] : P.qn[q]) + ((WALLS && (solid || bb)) ? s : nb);
#pragma unroll
    for (int c = 0; c < C; ++c) pop[c][q] = FStore<T, 9>::load2(fc[c] + off, c, q, b, bb, P);
  }
}

// One run: rows [xa, xb) of tile `tile`.
template <typename T, int C, bool WALLS, bool MOM>
__device__ __forceinline__ void fused2d_run(const FusedParams& P, const T* __restrict__ f, T* __restrict__ fout,
                                            const uint32_t* __restrict__ nbmask, double* __restrict__ force_out,
                                            int tile, int xa, int xb, Fused2Shared<MOM ? 2 : 9>& sh) {
  const int t = threadIdx.x;
  const int ny = P.ny;
  const int y0 = tile * kF2W;
  const int tv = min(kF2W, ny - y0);
  const bool active = t < tv;
  const T* const fc[2] = {f, f + size_t(9) * size_t(P.n)};
  T* const fo[2] = {fout, fout + size_t(9) * size_t(P.n)};
  const bool unit = MOM || P.unit_tau != 0;
  const int y = y0 + (active ? t : 0);
  const int yo_in[3] = {wrap(y - 1, ny), y, wrap(y + 1, ny)};
  // threads 0 and 1 also gather the ring sites y0 - 1 and y0 + tv
  const bool has_ring = t < 2;
  const int ry = t == 0 ? wrap(y0 - 1, ny) : wrap(y0 + tv, ny);
  const int rslot = t == 0 ? 0 : tv + 1;
  const int yo_ring[3] = {wrap(ry - 1, ny), ry, wrap(ry + 1, ny)};

  // rho/psi of row xg into slot ps (and the tile's momenta or populations
  // into buffer keep, unless keep < 0); returns the site's neighbour mask
  auto gather_row = [&](int ps, int xg, int keep) -> uint32_t {
    const uint32_t rows[3] = {uint32_t(wrap(xg - 1, P.nx)) * uint32_t(ny), uint32_t(xg) * uint32_t(ny),
                              uint32_t(wrap(xg + 1, P.nx)) * uint32_t(ny)};
    uint32_t nbm_in = 0;
    if (active) {
      if (WALLS) nbm_in = __ldg(nbmask + rows[1] + uint32_t(y));
      float pop[C][9];
      gather9<T, WALLS, C>(fc, P, rows, yo_in, nbm_in, pop);
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const float den = density<9, float>(pop[c]);
        sh.rho[ps][c][t + 1] = den;
        sh.psi[ps][c][t + 1] = P.psi_form ? 1.0f - __expf(-den) : den;
        if (keep >= 0) {
          if (MOM) {
#pragma unroll
            for (int vd = 0; vd < 2; ++vd) sh.pops[keep][c][vd][t] = moment<9, float>(pop[c], vd);
          } else {
#pragma unroll
            for (int q = 0; q < 9; ++q) sh.pops[keep][c][q][t] = pop[c][q];
          }
        }
      }
    }
    if (has_ring) {
      const uint32_t nbm = WALLS ? __ldg(nbmask + rows[1] + uint32_t(ry)) : 0u;
      float pop[C][9];
      gather9<T, WALLS, C>(fc, P, rows, yo_ring, nbm, pop);
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const float den = density<9, float>(pop[c]);
        sh.rho[ps][c][rslot] = den;
        sh.psi[ps][c][rslot] = P.psi_form ? 1.0f - __expf(-den) : den;
      }
    }
    return nbm_in;
  };

  gather_row(0, wrap(xa - 1, P.nx), -1);
  uint32_t nbm_next = gather_row(1, xa, 0);
  int cur = 0;
  for (int k = 0; k < xb - xa; ++k) {
    const int x = xa + k;
    const int sm = k % 3, s0 = (k + 1) % 3, sp = (k + 2) % 3;  // row slots of x-1, x, x+1
    const uint32_t nbm_cur = nbm_next;
    __syncthreads();  // row slot sp and buffer 1-cur are free
    nbm_next = gather_row(sp, wrap(x + 1, P.nx), 1 - cur);
    __syncthreads();
    if (active) {
      const uint32_t s = uint32_t(x) * uint32_t(ny) + uint32_t(y);
      const int cy1 = t + 1;
      // branch-free: solid sites compute like fluid ones but store nothing
      const bool solid = WALLS && (nbm_cur & 1u);
      const int pslot[3] = {sm, s0, sp};  // by cx + 1
      float den[C];
#pragma unroll
      for (int c = 0; c < C; ++c) den[c] = sh.rho[s0][c][cy1];
      // --- Shan-Chen force, a solid neighbour contributing the site's own
      // psi (force.d:273), and the wall force from the solid neighbours'
      // densities
      float F[C][3];
#pragma unroll
      for (int c = 0; c < C; ++c) F[c][0] = F[c][1] = F[c][2] = 0.f;
      if (P.shan_chen) {
        float S[C][2], own[C];
#pragma unroll
        for (int c = 0; c < C; ++c) {
          own[c] = sh.psi[s0][c][cy1];
          float acc[3] = {0.f, 0.f, 0.f}, dacc[3] = {0.f, 0.f, 0.f};  // axis and diagonal sums
#pragma unroll
          for (int q = 1; q < 9; ++q) {
            const int cx = Conn<9>::cx(q), cy = Conn<9>::cy(q);
            float v = sh.psi[pslot[cx + 1]][c][cy1 + cy];
            if (WALLS && ((nbm_cur >> q) & 1u)) v = own[c];
            if (Conn<9>::wclass(q) == 1)
              stencil_acc(acc, cx, cy, 0, v);
            else
              stencil_acc(dacc, cx, cy, 0, v);
          }
#pragma unroll
          for (int vd = 0; vd < 2; ++vd) S[c][vd] = stencil_weigh9(acc[vd], dacc[vd]);
        }
#pragma unroll
        for (int f1 = 0; f1 < C; ++f1) {
          float g[2] = {0.f, 0.f};
#pragma unroll
          for (int f2 = 0; f2 < C; ++f2) {
            const float cc = P.gcc[f1][f2];
#pragma unroll
            for (int vd = 0; vd < 2; ++vd) g[vd] = fmaf(cc, S[f2][vd], g[vd]);
          }
#pragma unroll
          for (int vd = 0; vd < 2; ++vd) F[f1][vd] = -own[f1] * g[vd];
          if (WALLS) {
            const float wc = P.gwc[f1];
            if (wc != 0.f) {
              float acc[3] = {0.f, 0.f, 0.f}, dacc[3] = {0.f, 0.f, 0.f};
#pragma unroll
              for (int q = 1; q < 9; ++q) {
                const int cx = Conn<9>::cx(q), cy = Conn<9>::cy(q);
                const float v = ((nbm_cur >> q) & 1u) ? sh.rho[pslot[cx + 1]][f1][cy1 + cy] : 0.f;
                if (Conn<9>::wclass(q) == 1)
                  stencil_acc(acc, cx, cy, 0, v);
                else
                  stencil_acc(dacc, cx, cy, 0, v);
              }
#pragma unroll
              for (int vd = 0; vd < 2; ++vd) F[f1][vd] -= own[f1] * wc * stencil_weigh9(acc[vd], dacc[vd]);
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
        if (bad) F[c][0] = F[c][1] = NAN;
        if (solid && !bad) F[c][0] = F[c][1] = 0.f;
      }
      if (P.record_force) {
#pragma unroll
        for (int c = 0; c < C; ++c)
#pragma unroll
          for (int vd = 0; vd < 2; ++vd) force_out[(size_t(c) * P.n + s) * 2 + vd] = double(F[c][vd]);
      }
      // --- BDist2 weighted velocity (collision.d:156-196)
      float wv[3] = {0.f, 0.f, 0.f};
      if (MOM || P.eq_form == 2) {
        float a[2] = {0.f, 0.f};
#pragma unroll
        for (int c = 0; c < C; ++c) {
          float pc[9];
          if (!MOM) {
#pragma unroll
            for (int q = 0; q < 9; ++q) pc[q] = sh.pops[cur][c][q][t];
          }
#pragma unroll
          for (int vd = 0; vd < 2; ++vd) {
            const float m = MOM ? sh.pops[cur][c][vd][t] : moment<9, float>(pc, vd);
            a[vd] = unit ? a[vd] + m : fmaf(m, P.inv_tau[c], a[vd]);
          }
        }
        const float rtot = __frcp_rn(tot);
#pragma unroll
        for (int vd = 0; vd < 2; ++vd) wv[vd] = a[vd] * rtot;
      }
      // --- collision; solid sites store nothing.  With tau == 1 the new
      // populations are the equilibrium
#pragma unroll
      for (int c = 0; c < C; ++c) {
        float pop[9];
        if (!MOM) {
#pragma unroll
          for (int q = 0; q < 9; ++q) pop[q] = sh.pops[cur][c][q][t];
        }
        const float rden = __frcp_rn(den[c]);
        float dv[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int vd = 0; vd < 2; ++vd) dv[vd] = shifted_velocity(F[c][vd], rden, P.acc[vd], wv[vd], P.tau[c], unit);
        float eq[9];
        if (MOM || P.eq_form == 2)
          eq_bdist2_f9(dv, den[c], eq);
        else
          eq_poly<9, float>(pop, dv, den[c], P.eq_form == 1, eq);
        const float omega = P.omega[c], omo = P.one_minus_omega[c];
        if (!solid) {
#pragma unroll
          for (int q = 0; q < 9; ++q) {
            const float v = (MOM || unit) ? eq[q] : relax(pop[q], omo, omega, eq[q]);
            FStore<T, 9>::store(fo[c] + (P.qn[q] + s), v, c, q, P);
          }
        }
      }
    }
    cur = 1 - cur;
  }
}

// P.tiles_z y-segments of kF2W sites per row (P.tiles_y = 1); rows
// [P.x_begin, P.x_end) in the runs of sched_run
template <typename T, int C, bool WALLS, bool MOM>
__global__ void __launch_bounds__(kF2W, MOM ? 4 : 3)
    k_fused2d(const T* __restrict__ f, T* __restrict__ fout, const uint32_t* __restrict__ nbmask,
              double* __restrict__ force_out, FusedParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Fused2Shared<MOM ? 2 : 9>& sh = *reinterpret_cast<Fused2Shared<MOM ? 2 : 9>*>(smem_raw);
  __shared__ int s_item;
  const int tiles = P.tiles_z;
  const int units = sched_units(P, tiles);
  int next = blockIdx.x;
  for (;;) {
    __syncthreads();  // every thread has read the previous item
    if (threadIdx.x == 0) s_item = P.work_counter ? atomicAdd(P.work_counter, 1) : next;
    __syncthreads();
    const int item = s_item;
    next += gridDim.x;
    if (item >= units) break;
    int tile, xa, xb;
    sched_run(P, tiles, item, tile, xa, xb);
    fused2d_run<T, C, WALLS, MOM>(P, f, fout, nbmask, force_out, tile, xa, xb, sh);
  }
}

}  // namespace lbk
