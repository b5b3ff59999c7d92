// Per-site lattice-Boltzmann arithmetic shared by every kernel form.
//
// The functions here restate the reference's per-site operations in its
// expression order, templated on the arithmetic type R:
//   R = double in lb_step_f64.cu, compiled with -fmad=false, so that the
//          FP64 form reproduces the reference's IEEE double results bit for
//          bit (the CPU oracle checks this);
//   R = float  in lb_step_lp.cu (FP32 and FP16-storage forms).
// Terms whose lattice velocity component is 0 are left out and terms with
// component -1 are subtracted instead of added: in IEEE arithmetic this
// changes at most the sign of a zero, which no later operation can observe
// in the populations.
#pragma once

#include <stdint.h>

#include "lb_math.h"

namespace lbk {

// ---------------------------------------------------------------------------
// Connectivities (src/dlbc/lb/connectivity.d:250-418).  Kernels index the
// lattice as [x][y][z] with z contiguous; D2Q9 runs with a z extent of 1,
// D1Q3 and D1Q5 with y and z extents of 1.  css is the speed of sound
// squared (generateSpeedOfSound, connectivity.d:213-245).
// ---------------------------------------------------------------------------
template <int Q>
struct Conn;

template <>
struct Conn<19> {
  static constexpr int D = 3;
  __host__ __device__ static constexpr int cx(int q) {
    return (q == 1 || q == 7 || q == 11 || q == 12 || q == 13) ? 1
           : (q == 2 || q == 8 || q == 14 || q == 17 || q == 18) ? -1 : 0;
  }
  __host__ __device__ static constexpr int cy(int q) {
    return (q == 3 || q == 7 || q == 8 || q == 9 || q == 15) ? 1
           : (q == 4 || q == 10 || q == 13 || q == 14 || q == 16) ? -1 : 0;
  }
  __host__ __device__ static constexpr int cz(int q) {
    return (q == 5 || q == 9 || q == 10 || q == 11 || q == 17) ? 1
           : (q == 6 || q == 12 || q == 15 || q == 16 || q == 18) ? -1 : 0;
  }
  __host__ __device__ static constexpr int bounce(int q) {
    return q == 0 ? 0 : q == 1 ? 2 : q == 2 ? 1 : q == 3 ? 4 : q == 4 ? 3 : q == 5 ? 6 : q == 6 ? 5
         : q == 7 ? 14 : q == 8 ? 13 : q == 9 ? 16 : q == 10 ? 15 : q == 11 ? 18 : q == 12 ? 17
         : q == 13 ? 8 : q == 14 ? 7 : q == 15 ? 10 : q == 16 ? 9 : q == 17 ? 12 : 11;
  }
  // weight class: 0 rest, 1 axis (1/18), 2 diagonal (1/36)
  __host__ __device__ static constexpr int wclass(int q) { return q == 0 ? 0 : (q < 7 ? 1 : 2); }
  __host__ __device__ static constexpr double css() { return 1.0 / 3.0; }
};

template <>
struct Conn<9> {
  static constexpr int D = 2;
  __host__ __device__ static constexpr int cx(int q) {
    return (q == 1 || q == 5 || q == 6) ? 1 : (q == 2 || q == 7 || q == 8) ? -1 : 0;
  }
  __host__ __device__ static constexpr int cy(int q) {
    return (q == 3 || q == 5 || q == 7) ? 1 : (q == 4 || q == 6 || q == 8) ? -1 : 0;
  }
  __host__ __device__ static constexpr int cz(int) { return 0; }
  __host__ __device__ static constexpr int bounce(int q) {
    return q == 0 ? 0 : q == 1 ? 2 : q == 2 ? 1 : q == 3 ? 4 : q == 4 ? 3 : q == 5 ? 8 : q == 6 ? 7 : q == 7 ? 6 : 5;
  }
  __host__ __device__ static constexpr int wclass(int q) { return q == 0 ? 0 : (q < 5 ? 1 : 2); }
  __host__ __device__ static constexpr double css() { return 1.0 / 3.0; }
};

// D1Q3 (generateD1Q3, connectivity.d:339-345): 0, +1, -1
template <>
struct Conn<3> {
  static constexpr int D = 1;
  __host__ __device__ static constexpr int cx(int q) { return q == 1 ? 1 : q == 2 ? -1 : 0; }
  __host__ __device__ static constexpr int cy(int) { return 0; }
  __host__ __device__ static constexpr int cz(int) { return 0; }
  __host__ __device__ static constexpr int bounce(int q) { return q == 1 ? 2 : q == 2 ? 1 : 0; }
  __host__ __device__ static constexpr int wclass(int q) { return q == 0 ? 0 : 1; }
  __host__ __device__ static constexpr double css() { return 1.0 / 3.0; }
};

// D1Q5 (generateD1Q5, connectivity.d:347-353): 0, +1, -1, +2, -2
template <>
struct Conn<5> {
  static constexpr int D = 1;
  __host__ __device__ static constexpr int cx(int q) {
    return q == 1 ? 1 : q == 2 ? -1 : q == 3 ? 2 : q == 4 ? -2 : 0;
  }
  __host__ __device__ static constexpr int cy(int) { return 0; }
  __host__ __device__ static constexpr int cz(int) { return 0; }
  __host__ __device__ static constexpr int bounce(int q) {
    return q == 1 ? 2 : q == 2 ? 1 : q == 3 ? 4 : q == 4 ? 3 : 0;
  }
  __host__ __device__ static constexpr int wclass(int q) { return q == 0 ? 0 : (q < 3 ? 1 : 2); }
  __host__ __device__ static constexpr double css() { return 1.0; }
};

template <int Q, typename R>
__host__ __device__ __forceinline__ R weight(int q) {
  // generateWeights (connectivity.d:250-295)
  if (Q == 19) return Conn<19>::wclass(q) == 0 ? R(1.0 / 3.0) : Conn<19>::wclass(q) == 1 ? R(1.0 / 18.0) : R(1.0 / 36.0);
  if (Q == 9) return Conn<9>::wclass(q) == 0 ? R(4.0 / 9.0) : Conn<9>::wclass(q) == 1 ? R(1.0 / 9.0) : R(1.0 / 36.0);
  if (Q == 3) return q == 0 ? R(4.0 / 6.0) : R(1.0 / 6.0);
  return q == 0 ? R(6.0 / 12.0) : q < 3 ? R(2.0 / 12.0) : R(1.0 / 12.0);
}

// weight of population q of connectivity Q (host and device, runtime Q)
__host__ __device__ __forceinline__ double weight_of(int Q, int q) {
  return Q == 19 ? weight<19, double>(q) : Q == 9 ? weight<9, double>(q) : Q == 3 ? weight<3, double>(q)
                                                                                    : weight<5, double>(q);
}

template <int Q>
__host__ __device__ __forceinline__ int cvel(int q, int vd) {
  return vd == 0 ? Conn<Q>::cx(q) : vd == 1 ? Conn<Q>::cy(q) : Conn<Q>::cz(q);
}

// ---------------------------------------------------------------------------
// density(): Phobos std.algorithm.sum of double[Q] = 0.0 + pairwise sum with
// recursive halving (src/dlbc/lb/density.d:37-39)
// ---------------------------------------------------------------------------
template <int Q, typename R>
__device__ __forceinline__ R density(const R* a) {
  if (Q == 19) {
    const R lo = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + (a[7] + a[8])));
    const R hi = ((a[9] + a[10]) + (a[11] + (a[12] + a[13]))) + ((a[14] + a[15]) + (a[16] + (a[17] + a[18])));
    return R(0) + (lo + hi);
  } else if (Q == 9) {
    return R(0) + (((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + (a[7] + a[8]))));
  } else if (Q == 5) {
    return R(0) + ((a[0] + a[1]) + (a[2] + (a[3] + a[4])));
  } else {
    return R(0) + (a[0] + (a[1] + a[2]));
  }
}

// sum_q a_q * c_q[vd] in q order, starting from 0 (velocity.d:37-48,
// collision.d:171-176)
template <int Q, typename R>
__device__ __forceinline__ R moment(const R* a, int vd) {
  R s = R(0);
#pragma unroll
  for (int q = 1; q < Q; ++q) {
    const int c = cvel<Q>(q, vd);
    if (c == 1) s = s + a[q];
    if (c == -1) s = s - a[q];
    if (c == 2) s = s + a[q] * R(2);   // D1Q5: a * c exactly
    if (c == -2) s = s - a[q] * R(2);
  }
  return s;
}

template <typename R>
__device__ __forceinline__ R psi_of(R rho, int psi_form);

template <>
__device__ __forceinline__ double psi_of<double>(double rho, int psi_form) {
  // psi (src/dlbc/lb/force.d:320-333)
  return psi_form ? 1.0 - lbmath::lb_exp(-rho) : rho;
}

template <>
__device__ __forceinline__ float psi_of<float>(float rho, int psi_form) {
  return psi_form ? 1.0f - expf(-rho) : rho;
}

// Division by one divisor b for several numerators: in double the integer
// IEEE division (lbmath::div_rn, the same bits as a / b for far fewer FP64
// operations), in float the plain division.
template <typename R>
struct Divisor;
template <>
struct Divisor<double> {
  lbmath::DivRecip r;
  __device__ __forceinline__ explicit Divisor(double b) : r(lbmath::div_recip(b)) {}
  __device__ __forceinline__ double div(double a) const { return lbmath::div_rn(a, r); }
};
template <>
struct Divisor<float> {
  float b;
  __device__ __forceinline__ explicit Divisor(float b_) : b(b_) {}
  __device__ __forceinline__ float div(float a) const { return a / b; }
};

// 2x and x/2 for the arithmetic type: exact scalings by a power of two, in
// double as an exponent step on the bits (integer operations; GB300 runs
// FP64 at a small fraction of its integer rate) where the operand and the
// result are normal numbers, else the multiplication
template <typename R>
__device__ __forceinline__ R twice(R x) {
  return R(2) * x;
}
template <>
__device__ __forceinline__ double twice<double>(double x) {
  const uint64_t u = lbmath::double_to_bits(x);
  const uint64_t e = (u >> 52) & 0x7ff;
  if (e != 0 && e < 0x7fe) return lbmath::bits_to_double(u + (uint64_t(1) << 52));
  return 2.0 * x;
}
template <typename R>
__device__ __forceinline__ R halve(R x) {
  return R(0.5) * x;
}
template <>
__device__ __forceinline__ double halve<double>(double x) {
  const uint64_t u = lbmath::double_to_bits(x);
  const uint64_t e = (u >> 52) & 0x7ff;
  if (e > 1 && e != 0x7ff) return lbmath::bits_to_double(u - (uint64_t(1) << 52));
  return 0.5 * x;
}

// ---------------------------------------------------------------------------
// Equilibria (src/dlbc/lb/eqdist.d:61-278).  `pop` is only read by the
// SecondOrder/ThirdOrder forms (their velocity is the population's own
// velocity plus dv).
// ---------------------------------------------------------------------------
template <int Q, typename R>
__device__ __forceinline__ void eq_bdist2(const R* dv, R rho0, R* dist) {
  if (Q == 19) {
    const R aN1 = R(1.0 / 36.0);
    const R aN0 = R(1.0 / 3.0);
    const R haN1 = R(0.5) * aN1;
    const R aN1_6 = aN1 / R(6.0);
    const R holdit = R(1.0) / R(1.0 / 3.0);
    const R tux = dv[0], tuy = dv[1], tuz = dv[2];
    const R tuxt = tux * holdit, tuyt = tuy * holdit, tuzt = tuz * holdit;
    const R uke = halve<R>(tux * tuxt + tuy * tuyt + tuz * tuzt);
    const R cst = R(1.0) - uke;
    const R const1 = aN1 * cst;
#define LB_PAIR(CD, IP, IM, TWO)                                         \
  {                                                                      \
    const R cdotu = (CD);                                                \
    const R even = const1 + haN1 * cdotu * cdotu;                        \
    const R odd = const1 * cdotu + aN1_6 * cdotu * cdotu * cdotu;        \
    if (TWO) {                                                           \
      dist[IP] = twice<R>(even + odd);                                   \
      dist[IM] = twice<R>(even - odd);                                   \
    } else {                                                             \
      dist[IP] = even + odd;                                             \
      dist[IM] = even - odd;                                             \
    }                                                                    \
  }
    LB_PAIR(tuxt, 1, 2, true)
    LB_PAIR(tuyt, 3, 4, true)
    LB_PAIR(tuzt, 5, 6, true)
    LB_PAIR(tuxt + tuyt, 7, 14, false)
    LB_PAIR(tuxt - tuyt, 13, 8, false)
    LB_PAIR(tuxt + tuzt, 11, 18, false)
    LB_PAIR(tuxt - tuzt, 12, 17, false)
    LB_PAIR(tuyt + tuzt, 9, 16, false)
    LB_PAIR(tuyt - tuzt, 15, 10, false)
    dist[0] = aN0 * cst;
  } else {
    const R aN1 = R(1.0 / 24.0);
    const R aN0 = R(1.0 / 2.0);
    const R haN1 = R(0.5) * aN1;
    const R aN1_6 = aN1 / R(6.0);
    const R holdit = R(1.0) / R(1.0 / 3.0);
    const R tux = dv[0], tuy = dv[1];
    const R tuxt = tux * holdit, tuyt = tuy * holdit;
    const R uke = halve<R>(tux * tuxt + tuy * tuyt);
    const R cst = R(1.0) - uke;
    const R const1 = aN1 * cst;
    LB_PAIR(tuxt, 1, 2, true)
    LB_PAIR(tuyt, 3, 4, true)
    LB_PAIR(tuxt + tuyt, 5, 8, false)
    LB_PAIR(tuxt - tuyt, 6, 7, false)
#undef LB_PAIR
    dist[0] = aN0 * cst;
  }
#pragma unroll
  for (int q = 0; q < Q; ++q) dist[q] *= rho0;
}

// SecondOrder (third == false) and ThirdOrder (third == true)
template <int Q, typename R>
__device__ __forceinline__ void eq_poly(const R* pop, const R* dv, R rho0, bool third, R* dist) {
  constexpr int D = Conn<Q>::D;
  const R css = R(Conn<Q>::css());
  const R css2 = R(2.0) * css;
  const R css2p2 = css2 * css;
  const R css6p3 = R(3.0) * css2p2 * css;
  // the divisions by these constants, exact (integer arithmetic in double)
  const Divisor<R> by_css(css), by_css2(css2), by_css2p2(css2p2), by_css6p3(css6p3);
  // rawVelocity(pop, rho0): sum_q pop_q c_q, then `vel[] /= density`, a D
  // array operation that druntime evaluates as a multiplication by 1/density
  const R recip = Divisor<R>(rho0).div(R(1.0));
  R v[3];
#pragma unroll
  for (int vd = 0; vd < D; ++vd) v[vd] = dv[vd] + moment<Q, R>(pop, vd) * recip;
  R vdotv = v[0] * v[0];
  if (D >= 2) vdotv = vdotv + v[1] * v[1];
  if (D == 3) vdotv = vdotv + v[2] * v[2];
  const R k2 = by_css2.div(vdotv);
  const R z1 = by_css.div(R(0)), z2 = by_css2p2.div(R(0) * R(0));  // v.c_0 = 0
  dist[0] = rho0 * weight<Q, R>(0) * ((R(1.0) + z1 + z2) - k2);
  if (third) dist[0] = rho0 * weight<Q, R>(0) * ((((R(1.0) + z1 + z2) - k2) + R(0)) - R(0));
#pragma unroll
  for (int q = 1; q < Q; ++q) {
    const int b = Conn<Q>::bounce(q);
    if (b < q) continue;  // handled with its partner
    // v . c_q in component order (range.d:57-67)
    R vdc = R(0);
    bool first = true;
#pragma unroll
    for (int vd = 0; vd < D; ++vd) {
      const int c = cvel<Q>(q, vd);
      if (c == 0) continue;
      // |c| = 1: +-v exactly; D1Q5's |c| = 2: v * c
      const R vc = (c == 1) ? v[vd] : (c == -1) ? -v[vd] : v[vd] * R(c);
      if (first) {
        vdc = vc;
        first = false;
      } else {
        vdc = vdc + vc;
      }
    }
    // v . c_b = -(v . c_q) exactly
    const R A = by_css.div(vdc);
    const R sq = vdc * vdc;
    const R B = by_css2p2.div(sq);
    const R w = weight<Q, R>(q);
    if (!third) {
      dist[q] = rho0 * w * (((R(1.0) + A) + B) - k2);
      dist[b] = rho0 * w * (((R(1.0) - A) + B) - k2);
    } else {
      const R T3 = by_css6p3.div(sq * vdc);
      const R T4 = by_css2p2.div(vdotv * vdc);
      dist[q] = rho0 * w * (((((R(1.0) + A) + B) - k2) + T3) - T4);
      dist[b] = rho0 * w * (((((R(1.0) - A) + B) - k2) - T3) + T4);
    }
  }
}

}  // namespace lbk
