// Fused D3Q19 step with the populations staged in shared memory by
// asynchronous copies (cp.async), for the half-offset storage form.
//
// Same per-site arithmetic as k_fused (lb_fused.cuh); what changes is how the
// populations reach the threads.  A CTA owns a TY x 32 tile of the (y, z)
// plane and marches along x.  For every plane d whose densities it needs, it
// stages "the slabs of d": for each component c and population q the rows
// y0-2 .. y0+TY+1, columns z0-8 .. z0+39 of source plane d - c_q,x (the
// plane population q streams from), copied in 16-byte pieces with
// cp.async.cg into shared memory.  Pull streaming then reads slab (c, q) at
// the in-plane offset (-c_q,y, -c_q,z): shared-memory loads at constant
// offsets, with the global-memory latency hidden behind two iterations of
// work.  Rows wrap periodically in y and columns in z: a 16-byte piece never
// straddles the z boundary because nz is a multiple of 8.
//
// Three slab buffers rotate: the slabs of plane x (collided in this
// iteration, re-gathered from shared memory), of plane x+1 (its densities and
// psi are computed in this iteration) and of plane x+2 (in flight); the
// copies for plane x+3 are issued as soon as plane x has been collided.
// Every thread commits exactly one copy group per staged plane, so
// cp.async.wait_group counts planes.
//
// Bounce-back needs the site's own opposite population; for populations that
// move along y or z only, that value is in the slab of the same plane, for
// the others it is read from global memory (sites next to a wall only).
//
// Scheduling: every CTA processes one or more (tile, x-chunk) units; the
// chunks split x evenly so that CTAs on neighbouring tiles march in lockstep
// and the staged halo rows, which neighbouring tiles share, come from L2.
#pragma once

#include "lb_fused.cuh"

namespace lbk {

constexpr int kStagedZH = 8;                          // halves per 16 bytes
constexpr int kStagedZW = kFusedTZ + 2 * kStagedZH;   // 48 staged columns
constexpr int kStagedPieces = kStagedZW / kStagedZH;  // 16-byte pieces per row
constexpr int kStagedMaxRows = 2;                     // staged rows per thread

template <int TY>
struct StagedShared {
  static constexpr int ROWS = TY + 4;
  __half slab[3][2][19][ROWS][kStagedZW];  // [buffer][c][q][row][col]
  float psi[3][2][TY + 2][kFusedRZ];       // [plane slot][c][y+1][z+1]
  float rho[3][2][TY + 2][kFusedRZ];
};

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ int cx_of(int q) {
  return (q == 1 || q == 7 || q == 11 || q == 12 || q == 13) ? 1
         : (q == 2 || q == 8 || q == 14 || q == 17 || q == 18) ? -1 : 0;
}

__device__ __forceinline__ int wrap_any(int v, int n) {
  v %= n;
  return v < 0 ? v + n : v;
}

__device__ __forceinline__ float dec_half(__half h, int c, int q, const FusedParams& P) {
  return fmaf(P.wscale[c][Conn<19>::wclass(q)], __half2float(h), P.wrho[c][Conn<19>::wclass(q)]);
}

// own population `src` of the site at (row, col) in plane d: in the slab
// when it does not move along x, else from global memory
template <int TY>
__device__ __forceinline__ float staged_own(const StagedShared<TY>& sh, int buf, const __half* fc,
                                            const FusedParams& P, int c, int src, int row, int col, uint32_t s) {
  if (cx_of(src) == 0) return dec_half(sh.slab[buf][c][src][row][col], c, src, P);
  return dec_half(__ldg(fc + P.qn[src] + s), c, src, P);
}

// Pull-gathered populations of component c at tile position (row, col) of
// the slabs in `buf` (plane d); s is the site's global index in plane d.
// Every site takes the plain shared-memory path; the few next to or inside a
// wall (nbm != 0) then replace the populations that bounce back (the
// opposite own population) or, for a solid site, take all their own.
template <bool WALLS, int TY>
__device__ __forceinline__ void staged_gather_c(const StagedShared<TY>& sh, int buf, const __half* fc,
                                                const FusedParams& P, int c, int row, int col, uint32_t s,
                                                uint32_t nbm, float (&pop)[19]) {
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    const int cy = Conn<19>::cy(q), cz = Conn<19>::cz(q);
    pop[q] = dec_half(sh.slab[buf][c][q][row - cy][col - cz], c, q, P);
  }
  if (WALLS && nbm != 0u) {
    const bool solid = nbm & 1u;
#pragma unroll
    for (int q = 1; q < 19; ++q) {
      const int b = Conn<19>::bounce(q);
      if (solid)
        pop[q] = staged_own(sh, buf, fc, P, c, q, row, col, s);
      else if ((nbm >> b) & 1u)
        pop[q] = staged_own(sh, buf, fc, P, c, b, row, col, s);
    }
  }
}

template <int C, bool WALLS, int TY>
__global__ void __launch_bounds__(TY * kFusedTZ, 1)
    k_staged(const __half* __restrict__ f, __half* __restrict__ fout, const uint32_t* __restrict__ nbmask,
             double* __restrict__ force_out, FusedParams P, int chunks) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  StagedShared<TY>& sh = *reinterpret_cast<StagedShared<TY>*>(smem_raw);
  constexpr int ROWS = TY + 4;
  constexpr int kRows = C * 19 * ROWS;  // staged rows per plane
  static_assert(kRows <= kStagedMaxRows * TY * kFusedTZ, "too many staged rows per thread");
  const int t = threadIdx.x;
  const int ty = t / kFusedTZ, tz = t % kFusedTZ;
  const uint32_t plane_sz = uint32_t(P.ny) * uint32_t(P.nz);
  const __half* const fc[2] = {f, f + size_t(19) * size_t(P.n)};
  __half* const fo[2] = {fout, fout + size_t(19) * size_t(P.n)};
  const bool unit = P.unit_tau != 0;
  const int tiles = P.tiles_y * P.tiles_z;
  const int units = tiles * chunks;

  for (int u = blockIdx.x; u < units; u += gridDim.x) {
    const int tile = u % tiles;
    const int chunk = u / tiles;
    const int xs = int(int64_t(chunk) * P.nx / chunks);
    const int run = int(int64_t(chunk + 1) * P.nx / chunks) - xs;
    if (run <= 0) continue;
    const int y0 = (tile / P.tiles_z) * TY, z0 = (tile % P.tiles_z) * kFusedTZ;
    const int tyv = min(TY, P.ny - y0), tzv = min(kFusedTZ, P.nz - z0);
    const bool active = ty < tyv && tz < tzv;
    const YZ yz_in = make_yz(y0 + ty, z0 + tz, P);
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
    uint32_t nbm_next = 0, nbm_cur = 0;

    // this thread's staged rows (fixed for the tile): global row start
    // without the plane, c_q,x (2: no row), and the shared-memory row in
    // buffer 0
    size_t row_base[kStagedMaxRows];
    int row_cx[kStagedMaxRows];
    uint32_t row_dst[kStagedMaxRows];
#pragma unroll
    for (int j = 0; j < kStagedMaxRows; ++j) {
      const int i = t + j * TY * kFusedTZ;
      const int ii = i < kRows ? i : 0;
      const int c = ii / (19 * ROWS);
      const int r = ii - c * (19 * ROWS);
      const int q = r / ROWS;
      const int row = r - q * ROWS;
      row_base[j] = (size_t(c) * 19 + q) * size_t(P.n) + size_t(wrap_any(y0 - 2 + row, P.ny)) * P.nz;
      row_cx[j] = i < kRows ? cx_of(q) : 2;
      row_dst[j] = smem_u32(&sh.slab[0][c][q][row][0]);
    }
    // the 16-byte pieces' columns, periodic in z
    int zoff[kStagedPieces];
#pragma unroll
    for (int k = 0; k < kStagedPieces; ++k) zoff[k] = wrap_any(z0 - kStagedZH + k * kStagedZH, P.nz);
    constexpr uint32_t kBufBytes = uint32_t(sizeof(__half)) * 2 * 19 * ROWS * kStagedZW;

    // plane p's slabs live in buffer (p - xs + 1) % 3, its psi in slot
    // (p - xs + 1) % 3; one copy group per call (empty when not needed)
    auto issue = [&](int p, bool needed) {
      if (needed) {
        const uint32_t boff = uint32_t((p - xs + 1) % 3) * kBufBytes;
#pragma unroll
        for (int j = 0; j < kStagedMaxRows; ++j) {
          if (row_cx[j] == 2) continue;
          const int plane = wrap_any(p - row_cx[j], P.nx);
          const __half* src = f + row_base[j] + size_t(plane) * plane_sz;
#pragma unroll
          for (int k = 0; k < kStagedPieces; ++k) cp_async16(row_dst[j] + boff + 16u * k, src + zoff[k]);
        }
      }
      cp_async_commit();
    };
    // densities and psi of plane p (interior and ring) from its slabs
    auto density_pass = [&](int p) {
      const int b = (p - xs + 1) % 3;
      const uint32_t pbase = uint32_t(wrap(p, P.nx)) * plane_sz;
      if (active) {
        const uint32_t s = pbase + uint32_t(yz_in.off[1][1]);
        const uint32_t nbm = (WALLS && nbmask) ? __ldg(nbmask + s) : 0u;
        nbm_next = nbm;
#pragma unroll
        for (int c = 0; c < C; ++c) {
          float pop[19];
          staged_gather_c<WALLS, TY>(sh, b, fc[c], P, c, ty + 2, tz + kStagedZH, s, nbm, pop);
          const float den = density<19, float>(pop);
          sh.rho[b][c][ty + 1][tz + 1] = den;
          sh.psi[b][c][ty + 1][tz + 1] = P.psi_form ? 1.0f - __expf(-den) : den;
        }
      }
      if (has_ring) {
        const uint32_t s = pbase + uint32_t(yz_ring.off[1][1]);
        const uint32_t nbm = (WALLS && nbmask) ? __ldg(nbmask + s) : 0u;
#pragma unroll
        for (int c = 0; c < C; ++c) {
          float pop[19];
          staged_gather_c<WALLS, TY>(sh, b, fc[c], P, c, rry + 2, rrz + kStagedZH, s, nbm, pop);
          const float den = density<19, float>(pop);
          sh.rho[b][c][rry + 1][rrz + 1] = den;
          sh.psi[b][c][rry + 1][rrz + 1] = P.psi_form ? 1.0f - __expf(-den) : den;
        }
      }
    };

    // warm-up: slabs of xs-1, xs, xs+1 (and xs+2) in flight; psi of xs-1 and xs
    __syncthreads();  // the previous unit's reads of every buffer are done
    issue(xs - 1, true);
    issue(xs, true);
    issue(xs + 1, true);
    cp_async_wait<2>();  // plane xs-1 has landed (this thread's copies)
    __syncthreads();     // ... and every thread's
    density_pass(xs - 1);
    __syncthreads();
    issue(xs + 2, run >= 2);
    cp_async_wait<2>();  // plane xs
    __syncthreads();
    density_pass(xs);

    for (int k = 0; k < run; ++k) {
      const int x = xs + k;
      const int bc = (k + 1) % 3;  // slabs / psi slot of x
      const int bn = (k + 2) % 3;  // of x+1
      const int bp = k % 3;        // psi slot of x-1
      cp_async_wait<1>();          // plane x+1 (only x+2 may still be in flight)
      __syncthreads();
      nbm_cur = nbm_next;
      density_pass(x + 1);
      __syncthreads();
      if (active) {
        const uint32_t s = uint32_t(x) * plane_sz + uint32_t(yz_in.off[1][1]);
        const int c1y = ty + 1, c1z = tz + 1;
        const bool solid = WALLS && (nbm_cur & 1u);
        float den[C];
#pragma unroll
        for (int c = 0; c < C; ++c) den[c] = sh.rho[bc][c][c1y][c1z];
        const int pslot[3] = {bp, bc, bn};  // by c_q,x + 1
        float F[C][3];
#pragma unroll
        for (int c = 0; c < C; ++c) F[c][0] = F[c][1] = F[c][2] = 0.f;
        if (P.shan_chen) {
          float S[C][3];
          float own[C];
#pragma unroll
          for (int c = 0; c < C; ++c) {
            own[c] = sh.psi[bc][c][c1y][c1z];
            float a[3] = {0.f, 0.f, 0.f}, dd[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int q = 1; q < 19; ++q) {
              const int cx = Conn<19>::cx(q), cy = Conn<19>::cy(q), cz = Conn<19>::cz(q);
              float v = sh.psi[pslot[cx + 1]][c][c1y + cy][c1z + cz];
              if (WALLS && ((nbm_cur >> q) & 1u)) v = own[c];
              if (Conn<19>::wclass(q) == 1)
                stencil_acc(a, cx, cy, cz, v);
              else
                stencil_acc(dd, cx, cy, cz, v);
            }
#pragma unroll
            for (int vd = 0; vd < 3; ++vd) S[c][vd] = stencil_weigh(a[vd], dd[vd]);
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
            if (WALLS) {
              const float wc = P.gwc[f1];
              if (wc != 0.f) {
                float a[3] = {0.f, 0.f, 0.f}, dd[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int q = 1; q < 19; ++q) {
                  const int cx = Conn<19>::cx(q), cy = Conn<19>::cy(q), cz = Conn<19>::cz(q);
                  const float v = ((nbm_cur >> q) & 1u) ? sh.rho[pslot[cx + 1]][f1][c1y + cy][c1z + cz] : 0.f;
                  if (Conn<19>::wclass(q) == 1)
                    stencil_acc(a, cx, cy, cz, v);
                  else
                    stencil_acc(dd, cx, cy, cz, v);
                }
#pragma unroll
                for (int vd = 0; vd < 3; ++vd) F[f1][vd] -= own[f1] * wc * stencil_weigh(a[vd], dd[vd]);
              }
            }
          }
        }
        float tot = den[0];
        if (C > 1) tot = tot + den[1];
#pragma unroll
        for (int c = 0; c < C; ++c) {
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
        float pop[19];
        float wv[3] = {0.f, 0.f, 0.f};
        if (P.eq_form == 2) {
          float a[3] = {0.f, 0.f, 0.f};
#pragma unroll
          for (int c = 0; c < C; ++c) {
            staged_gather_c<WALLS, TY>(sh, bc, fc[c], P, c, ty + 2, tz + kStagedZH, s, nbm_cur, pop);
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
#pragma unroll
        for (int cc = 0; cc < C; ++cc) {
          const int c = C - 1 - cc;  // last component first: its populations are loaded
          if (!(P.eq_form == 2 && cc == 0))
            staged_gather_c<WALLS, TY>(sh, bc, fc[c], P, c, ty + 2, tz + kStagedZH, s, nbm_cur, pop);
          const float rden = __frcp_rn(den[c]);
          float dv[3];
#pragma unroll
          for (int vd = 0; vd < 3; ++vd) dv[vd] = shifted_velocity(F[c][vd], rden, P.acc[vd], wv[vd], P.tau[c], unit);
          float eq[19];
          if (P.eq_form == 2)
            eq_bdist2_f(dv, den[c], eq);
          else
            eq_poly<19, float>(pop, dv, den[c], P.eq_form == 1, eq);
          const float omega = P.omega[c], omo = P.one_minus_omega[c];
          // solid sites store nothing: both buffers hold their populations
          if (!solid) {
#pragma unroll
            for (int q = 0; q < 19; ++q) {
              const float v = unit ? eq[q] : relax(pop[q], omo, omega, eq[q]);
              FStore<__half>::store(fo[c] + (P.qn[q] + s), v, c, q, P);
            }
          }
        }
      }
      __syncthreads();  // every read of the slabs of x and of psi slot x-1 is done
      issue(x + 3, x + 3 <= xs + run);
    }
  }
  cp_async_wait<0>();  // no copy may outlive the CTA
}

}  // namespace lbk
