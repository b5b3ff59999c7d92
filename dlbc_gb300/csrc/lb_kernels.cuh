// Two-kernel lattice-Boltzmann timestep, templated on storage type T and
// arithmetic type R.
//
//   k_density_psi : pull-stream (periodic wrap + mask bounce-back) -> rho, psi
//                   (advectFieldsKernel src/dlbc/lb/advection.d:61-89,
//                    densityField src/dlbc/lb/density.d:89-96,
//                    psiField src/dlbc/lb/force.d:360-367)
//   k_collide     : pull-stream again, Shan-Chen force from the psi stencil,
//                   BDist2 weighted velocity, BGK collision with force shift
//                   (addShanChenForcePsi force.d:238-309, distributeForce
//                    force.d:179-197, precalculateWeightedVelocity
//                    collision.d:156-196, collideFieldsKernel collision.d:90-119)
//
// Storage is SoA: f[c][q][site], site = (x*NY + y)*NZ + z, z contiguous.
// Solid sites are neither streamed nor collided: their populations are
// copied through unchanged.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "lb_core.cuh"

namespace lbk {

struct StepParams {
  int32_t nx, ny, nz;
  int64_t n;              // sites
  // sites [s_begin, s_end) of one launch of the two-kernel step (whole
  // x-planes, for host transfers that overlap the step); s_end == 0: all n
  int64_t s_begin;
  int64_t s_end;
  int32_t shan_chen;
  int32_t psi_form;
  int32_t eq_form;
  int32_t record_force;
  // every component has tau == 1: m/tau, tau*x and pop*(1-omega) + omega*eq
  // reduce exactly to m, x and eq (for finite populations), which saves
  // about a quarter of the FP64 work of k_collide
  int32_t unit_tau;
  double tau[2];
  double omega[2];        // 1/tau
  double one_minus_omega[2];
  double gcc[2][2];
  double gwc[2];
  double acc[3];
  // FP16 storage of weight-normalised offsets: f_q = w_q * (rho0 + scale*h)
  float rho0[2];
  float scale[2];
  float inv_scale[2];
};

// ---------------------------------------------------------------------------
// storage conversion
// ---------------------------------------------------------------------------
template <typename T, typename R, int Q>
struct Store;

template <typename R, int Q>
struct Store<double, R, Q> {
  __device__ static __forceinline__ R load(const double* p, int, int, const StepParams&) { return R(__ldg(p)); }
  __device__ static __forceinline__ void store(double* p, R v, int, int, const StepParams&) { *p = double(v); }
};

template <typename R, int Q>
struct Store<float, R, Q> {
  __device__ static __forceinline__ R load(const float* p, int, int, const StepParams&) { return R(__ldg(p)); }
  __device__ static __forceinline__ void store(float* p, R v, int, int, const StepParams&) { *p = float(v); }
};

template <typename R, int Q>
struct Store<__half, R, Q> {
  __device__ static __forceinline__ R load(const __half* p, int c, int q, const StepParams& P) {
    const float h = __half2float(__ldg(p));
    return R(weight<Q, float>(q) * fmaf(P.scale[c], h, P.rho0[c]));
  }
  __device__ static __forceinline__ void store(__half* p, R v, int c, int q, const StepParams& P) {
    *p = __float2half_rn((float(v) * (1.0f / weight<Q, float>(q)) - P.rho0[c]) * P.inv_scale[c]);
  }
};

// site coordinates and wrapped neighbour coordinates
struct Site {
  int x, y, z;
  int xs[5];                // x - 2 .. x + 2 (periodic; +-2 only for D1Q5)
  int ys[3], zs[3];         // coordinate - 1, coordinate, coordinate + 1 (periodic)
};

__device__ __forceinline__ Site make_site(int64_t s, const StepParams& P) {
  Site S;
  const int64_t t = s / P.nz;
  S.z = int(s - t * P.nz);
  S.x = int(t / P.ny);
  S.y = int(t - int64_t(S.x) * P.ny);
  S.xs[1] = S.x == 0 ? P.nx - 1 : S.x - 1;
  S.xs[2] = S.x;
  S.xs[3] = S.x == P.nx - 1 ? 0 : S.x + 1;
  S.xs[0] = S.xs[1] == 0 ? P.nx - 1 : S.xs[1] - 1;
  S.xs[4] = S.xs[3] == P.nx - 1 ? 0 : S.xs[3] + 1;
  S.ys[0] = S.y == 0 ? P.ny - 1 : S.y - 1;
  S.ys[1] = S.y;
  S.ys[2] = S.y == P.ny - 1 ? 0 : S.y + 1;
  S.zs[0] = S.z == 0 ? P.nz - 1 : S.z - 1;
  S.zs[1] = S.z;
  S.zs[2] = S.z == P.nz - 1 ? 0 : S.z + 1;
  return S;
}

// index of site + sign*c_q
template <int Q>
__device__ __forceinline__ int64_t nb_index(const Site& S, int q, int sign, const StepParams& P) {
  const int ix = S.xs[2 + sign * Conn<Q>::cx(q)];
  const int iy = S.ys[1 + sign * Conn<Q>::cy(q)];
  const int iz = S.zs[1 + sign * Conn<Q>::cz(q)];
  return (int64_t(ix) * P.ny + iy) * P.nz + iz;
}

// F -= prefactor * c for a velocity component c in {-2, ..., 2}, exactly as
// the reference's `force[vd] -= prefactor * cv[vq][vd]` (force.d:283, :304)
template <typename R>
__device__ __forceinline__ R force_sub(R F, R prefactor, int c) {
  if (c == 1) return F - prefactor;
  if (c == -1) return F + prefactor;
  if (c == 2) return F - prefactor * R(2);
  if (c == -2) return F + prefactor * R(2);
  return F;
}

// Solid tests around site s: from the 8-bit mask, one load per neighbour,
// or (NBM) from the site's 32-bit neighbour mask (bit 0: the site is solid;
// bit q: the site x + c_q is solid, periodic images included), one load per
// site.  The two give the same answers.
template <bool NBM>
struct Solids {
  const uint8_t* mask;
  uint32_t bits;
  __device__ __forceinline__ Solids(const uint8_t* m, const uint32_t* nbm, int64_t s)
      : mask(m), bits(NBM ? __ldg(nbm + s) : 0u) {}
  // the site itself
  __device__ __forceinline__ bool self(int64_t s) const { return NBM ? (bits & 1u) != 0 : mask[s] != 0; }
  // the site x + c_q, whose index is nb
  __device__ __forceinline__ bool at(int q, int64_t nb) const {
    return NBM ? ((bits >> q) & 1u) != 0 : __ldg(mask + nb) != 0;
  }
};

// Pull-streamed populations of one component at a fluid site.
template <typename T, typename R, int Q, bool WALLS, bool NBM>
__device__ __forceinline__ void gather(const T* __restrict__ f, const Solids<NBM>& W, const Site& S, int64_t s, int c,
                                       const StepParams& P, R* pop) {
  const T* fc = f + int64_t(c) * Q * P.n;
  pop[0] = Store<T, R, Q>::load(fc + s, c, 0, P);
#pragma unroll
  for (int q = 1; q < Q; ++q) {
    const int64_t nb = nb_index<Q>(S, q, -1, P);
    // the source x - c_q is x + c_b
    if (WALLS && W.at(Conn<Q>::bounce(q), nb)) {
      const int b = Conn<Q>::bounce(q);
      pop[q] = Store<T, R, Q>::load(fc + int64_t(b) * P.n + s, c, b, P);
    } else {
      pop[q] = Store<T, R, Q>::load(fc + int64_t(q) * P.n + nb, c, q, P);
    }
  }
}

template <typename T, typename R, int Q>
__device__ __forceinline__ void load_local(const T* __restrict__ f, int64_t s, int c, const StepParams& P, R* pop) {
  const T* fc = f + int64_t(c) * Q * P.n;
#pragma unroll
  for (int q = 0; q < Q; ++q) pop[q] = Store<T, R, Q>::load(fc + int64_t(q) * P.n + s, c, q, P);
}

// ---------------------------------------------------------------------------
// kernel 1: densities and psi after streaming, at every site
// ---------------------------------------------------------------------------
// (NBM: solid tests from the neighbour masks nbmask, else from mask)
template <typename T, typename R, int Q, int C, bool WALLS, bool STREAM = true, bool NBM = false>
__global__ void __launch_bounds__(128) k_density_psi(const T* __restrict__ f, const uint8_t* __restrict__ mask,
                                                     const uint32_t* __restrict__ nbmask, R* __restrict__ rho,
                                                     R* __restrict__ psi, StepParams P) {
  const int64_t s = P.s_begin + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= (P.s_end ? P.s_end : P.n)) return;
  const Site S = make_site(s, P);
  const Solids<WALLS && NBM> W(mask, nbmask, s);
  const bool solid = WALLS && W.self(s);
#pragma unroll
  for (int c = 0; c < C; ++c) {
    R pop[Q];
    if (solid || !STREAM)
      load_local<T, R, Q>(f, s, c, P, pop);
    else
      gather<T, R, Q, WALLS>(f, W, S, s, c, P, pop);
    const R den = density<Q, R>(pop);
    rho[int64_t(c) * P.n + s] = den;
    // psi of a solid site is never read (force.d:273 uses the site's own psi)
    psi[int64_t(c) * P.n + s] = solid ? den : psi_of<R>(den, P.psi_form);
  }
}

// ---------------------------------------------------------------------------
// kernel 2: force + collision, writes the new populations
// ---------------------------------------------------------------------------
// (at most 168 registers, three 128-thread CTAs per SM: the FP64 form is
// latency bound at two)
template <typename T, typename R, int Q, int C, bool WALLS, bool STREAM = true, bool NBM = false>
__global__ void __launch_bounds__(128, 3) k_collide(const T* __restrict__ f, T* __restrict__ fout,
                                                 const uint8_t* __restrict__ mask,
                                                 const uint32_t* __restrict__ nbmask, const R* __restrict__ rho,
                                                 const R* __restrict__ psi, double* __restrict__ force_out,
                                                 StepParams P) {
  constexpr int D = Conn<Q>::D;
  const int64_t s = P.s_begin + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= (P.s_end ? P.s_end : P.n)) return;
  const Solids<WALLS && NBM> W(mask, nbmask, s);
  const bool solid = WALLS && W.self(s);

  R den[C];
#pragma unroll
  for (int c = 0; c < C; ++c) den[c] = rho[int64_t(c) * P.n + s];

  if (solid) {
    // not advectable, not collidable: copy through
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const T* fc = f + int64_t(c) * Q * P.n;
      T* oc = fout + int64_t(c) * Q * P.n;
#pragma unroll
      for (int q = 0; q < Q; ++q) oc[int64_t(q) * P.n + s] = fc[int64_t(q) * P.n + s];
    }
    if (P.record_force) {
      R tot = den[0];
      if (C > 1) tot = tot + den[1];
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const bool bad = tot == R(0) || isnan(tot) || isinf(den[c]) || isnan(den[c]);
        for (int vd = 0; vd < D; ++vd) force_out[(int64_t(c) * P.n + s) * D + vd] = bad ? double(NAN) : 0.0;
      }
    }
    return;
  }
  const Site S = make_site(s, P);

  // --- Shan-Chen force (force.d:253-308), per component in f2 order
  R F[C][3];
#pragma unroll
  for (int c = 0; c < C; ++c) F[c][0] = F[c][1] = F[c][2] = R(0);
  if (P.shan_chen) {
    R ps[C];
#pragma unroll
    for (int c = 0; c < C; ++c) ps[c] = psi[int64_t(c) * P.n + s];
#pragma unroll
    for (int f1 = 0; f1 < C; ++f1) {
      const R wpsi1 = weight<Q, R>(1) * ps[f1];  // cw[q] * psiden1, axis class
      const R wpsi2 = weight<Q, R>(Q - 1) * ps[f1];  // diagonal class
#pragma unroll
      for (int f2 = 0; f2 < C; ++f2) {
        const R cc = R(P.gcc[f1][f2]);
        if (cc == R(0)) continue;
        const R* p2 = psi + int64_t(f2) * P.n;
#pragma unroll
        for (int q = 1; q < Q; ++q) {
          const int64_t nb = nb_index<Q>(S, q, +1, P);
          const R psiden2 = (WALLS && W.at(q, nb)) ? ps[f2] : __ldg(p2 + nb);
          const R prefactor = (Conn<Q>::wclass(q) == 1 ? wpsi1 : wpsi2) * psiden2 * cc;
#pragma unroll
          for (int vd = 0; vd < D; ++vd) F[f1][vd] = force_sub(F[f1][vd], prefactor, cvel<Q>(q, vd));
        }
      }
      if (WALLS) {
        const R wc = R(P.gwc[f1]);
        if (wc != R(0)) {
          const R* r1 = rho + int64_t(f1) * P.n;
#pragma unroll
          for (int q = 1; q < Q; ++q) {
            const int64_t nb = nb_index<Q>(S, q, +1, P);
            if (W.at(q, nb)) {
              const R prefactor = (Conn<Q>::wclass(q) == 1 ? wpsi1 : wpsi2) * __ldg(r1 + nb) * wc;
#pragma unroll
              for (int vd = 0; vd < D; ++vd) F[f1][vd] = force_sub(F[f1][vd], prefactor, cvel<Q>(q, vd));
            }
          }
        }
      }
    }
  }
  // distributeForce with no distributed force: adds 0*(rho_f/rho_tot),
  // which only matters when that ratio is not finite
  {
    R tot = den[0];
    if (C > 1) tot = tot + den[1];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const bool bad = tot == R(0) || isnan(tot) || isinf(den[c]) || isnan(den[c]);
      if (bad) F[c][0] = F[c][1] = F[c][2] = R(NAN);
    }
  }
  if (P.record_force) {
#pragma unroll
    for (int c = 0; c < C; ++c)
#pragma unroll
      for (int vd = 0; vd < D; ++vd) force_out[(int64_t(c) * P.n + s) * D + vd] = double(F[c][vd]);
  }

  // --- populations after streaming
  R pop[C][Q];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    if (STREAM)
      gather<T, R, Q, WALLS>(f, W, S, s, c, P, pop[c]);
    else
      load_local<T, R, Q>(f, s, c, P, pop[c]);
  }

  // --- BDist2 weighted velocity (collision.d:156-196)
  R wv[3] = {R(0), R(0), R(0)};
  const bool unit = P.unit_tau != 0;
  if (P.eq_form == 2) {
#pragma unroll
    for (int vd = 0; vd < D; ++vd) {
      R acc = unit ? moment<Q, R>(pop[0], vd) : moment<Q, R>(pop[0], vd) / R(P.tau[0]);
      if (C > 1) acc = acc + (unit ? moment<Q, R>(pop[1], vd) : moment<Q, R>(pop[1], vd) / R(P.tau[1]));
      wv[vd] = acc;
    }
    R tot = den[0];
    if (C > 1) tot = tot + den[1];
    const Divisor<R> by_tot(tot);
#pragma unroll
    for (int vd = 0; vd < D; ++vd) wv[vd] = by_tot.div(wv[vd]);
  }

  // --- collision (collision.d:98-118)
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const R tau = R(P.tau[c]);
    const Divisor<R> by_den(den[c]);
    R dv[3];
#pragma unroll
    for (int vd = 0; vd < D; ++vd) {
      const R a = R(P.acc[vd]) + by_den.div(F[c][vd]);
      dv[vd] = unit ? a : tau * a;
      if (P.eq_form == 2) dv[vd] = dv[vd] + wv[vd];
    }
    R eq[Q];
    if (P.eq_form == 2) {
      if constexpr (Conn<Q>::D == 1) {
        // BDist2 is not implemented for 1D and returns the population
        // itself (eqdist.d:268-272)
#pragma unroll
        for (int q = 0; q < Q; ++q) eq[q] = pop[c][q];
      } else {
        eq_bdist2<Q, R>(dv, den[c], eq);
      }
    } else {
      eq_poly<Q, R>(pop[c], dv, den[c], P.eq_form == 1, eq);
    }
    const R omega = R(P.omega[c]);
    const R omo = R(P.one_minus_omega[c]);
    T* oc = fout + int64_t(c) * Q * P.n;
    if (unit) {
#pragma unroll
      for (int q = 0; q < Q; ++q) Store<T, R, Q>::store(oc + int64_t(q) * P.n + s, eq[q], c, q, P);
    } else {
#pragma unroll
      for (int q = 0; q < Q; ++q)
        Store<T, R, Q>::store(oc + int64_t(q) * P.n + s, pop[c][q] * omo + omega * eq[q], c, q, P);
    }
  }
}

// ---------------------------------------------------------------------------
// advection alone (advectFieldsKernel src/dlbc/lb/advection.d:61-89), for the
// phase-split timestep: fout = pull-streamed f at fluid sites (bounce-back
// from solid neighbours), f copied at solid sites.  The stored values move
// unconverted, so advection followed by k_density_psi/k_collide with
// STREAM = false is bit for bit the streamed two-kernel step.
// ---------------------------------------------------------------------------
template <typename T, int Q, int C, bool WALLS>
__global__ void __launch_bounds__(128) k_advect(const T* __restrict__ f, T* __restrict__ fout,
                                                const uint8_t* __restrict__ mask, StepParams P) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= P.n) return;
  const bool solid = WALLS && mask[s];
  const Site S = make_site(s, P);
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const T* fc = f + int64_t(c) * Q * P.n;
    T* oc = fout + int64_t(c) * Q * P.n;
    oc[s] = fc[s];
#pragma unroll
    for (int q = 1; q < Q; ++q) {
      T v;
      if (solid) {
        v = fc[int64_t(q) * P.n + s];
      } else {
        const int64_t nb = nb_index<Q>(S, q, -1, P);
        if (WALLS && __ldg(mask + nb))
          v = fc[int64_t(Conn<Q>::bounce(q)) * P.n + s];
        else
          v = fc[int64_t(q) * P.n + nb];
      }
      oc[int64_t(q) * P.n + s] = v;
    }
  }
}

}  // namespace lbk
