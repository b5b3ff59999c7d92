// Double-precision exp for the Shan-Chen psi = 1 - exp(-rho).
//
// The reference evaluates psi with Phobos std.math.exp
// (src/dlbc/lb/force.d:320-333), which computes in 80-bit `real` and rounds
// to double, i.e. it is correctly rounded for practically every argument.
// CUDA's and glibc's exp differ from that (and from each other) in the last
// bit for some arguments.  Because spinodal decomposition amplifies
// last-bit differences, the GPU kernels and the CPU oracle both call this
// one function, compiled without FMA contraction, so that the two agree
// bit for bit on every machine.
//
// Method: P. T. P. Tang, "Table-driven implementation of the exponential
// function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989.
//   N  = nearest integer to x*32/ln2,   N = 32*M + J,  0 <= J < 32
//   R  = (x - N*L1) - N*L2,  |R| <= ln2/64   (L1 + L2 = ln2/32, L1 has
//        32 significant bits so N*L1 is exact)
//   exp(x) = 2^M * 2^(J/32) * exp(R)
//   exp(R) - 1 = R + R^2/2 + ... + R^8/8!  (truncation below 2^-76)
//   2^(J/32) = S_lead[J] + S_trail[J]  (S_lead has 46 significant bits)
// The table entries are the mathematical values 2^(J/32) rounded to the
// stated number of bits (computed with 200-bit arithmetic).  Unlike Tang's
// single-double evaluation (error up to ~0.54 ulp), R is carried as a
// double-double and the leading products and sums are formed exactly with
// fma and error-free additions (Dekker/Knuth TwoSum), so that the value
// before the final rounding is within about 2^-72 relative of exp(x): the
// result is the correctly rounded exp(x) except for arguments within that
// distance of a rounding boundary (a few in a million).  The reduction
// constants keep R's error below that bound for |x| < 2^10.
//
// lb_exp itself evaluates the common range 2^-83 <= |x| <= 707 in integer
// fixed-point arithmetic (no FP64 operations, ~2^-90 relative, then rounded
// to 64 and to 53 significant bits exactly as the 80-bit evaluation is;
// see its comment) and uses the FP64 routine above (lb_exp_fp64) elsewhere.
// Where the two differ (~1.4e-7 of arguments) the integer one is the exact
// double rounding.  The division helpers at the end (div_rn) serve the same
// purpose: IEEE division in integer arithmetic.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define LB_HD __host__ __device__ __forceinline__
#else
#define LB_HD static inline
#endif

namespace lbmath {

LB_HD double bits_to_double(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double d;
  memcpy(&d, &u, sizeof d);
  return d;
#endif
}

LB_HD uint64_t double_to_bits(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  memcpy(&u, &d, sizeof u);
  return u;
#endif
}

// 2^e for -1022 <= e <= 1023, exact.
LB_HD double pow2i(int e) { return bits_to_double((uint64_t)(e + 1023) << 52); }

#if defined(__CUDA_ARCH__)
#define LB_EXP_TABLE_QUAL __device__ __constant__
#else
#define LB_EXP_TABLE_QUAL static const
#endif

// the integer exp's table is read with divergent indices: global memory
#if defined(__CUDA_ARCH__)
#define LB_EXP256_QUAL __device__
#else
#define LB_EXP256_QUAL static const
#endif
}  // namespace lbmath
#include "lb_exp_table.h"
namespace lbmath {

// {S_lead, S_trail} for J = 0..31
LB_EXP_TABLE_QUAL double kExpTable[32][2] = {
    {0x1.0000000000000p+0, 0x0.0p+0},
    {0x1.059b0d3158580p+0, -0x1.78a30756e292ep-49},
    {0x1.0b5586cf98900p+0, 0x1.ec5317256e308p-49},
    {0x1.11301d0125b80p+0, -0x1.7ad8a20728936p-47},
    {0x1.172b83c7d5180p+0, -0x1.48c820dcebc54p-50},
    {0x1.1d4873168b980p+0, 0x1.53c02dc0144c8p-47},
    {0x1.2387a6e756200p+0, 0x1.c3360fd6d8e0bp-47},
    {0x1.29e9df51fdf00p+0, -0x1.ed3da2ea0a5dbp-48},
    {0x1.306fe0a31b700p+0, 0x1.52de8d5a46306p-48},
    {0x1.371a7373aaa00p+0, -0x1.aac75d57e85d6p-47},
    {0x1.3dea64c123400p+0, 0x1.11ada0911f09fp-47},
    {0x1.44e0860618900p+0, 0x1.68189b7a04ef8p-47},
    {0x1.4bfdad5362a00p+0, 0x1.38ea1cbd7f621p-47},
    {0x1.5342b569d4f80p+0, 0x1.df0a83c49d86ap-52},
    {0x1.5ab07dd485400p+0, 0x1.4ac64980a8c8fp-47},
    {0x1.6247eb03a5580p+0, 0x1.2c7c3e81bf4b7p-50},
    {0x1.6a09e667f3c00p+0, -0x1.9b7ba682764c9p-47},
    {0x1.71f75e8ec5f80p+0, -0x1.845b91e1a21eap-49},
    {0x1.7a11473eb0180p+0, 0x1.b5f54408fdb37p-50},
    {0x1.82589994cce00p+0, 0x1.28acf88afab35p-48},
    {0x1.8ace5422aa100p+0, -0x1.2522c1d52f36ap-47},
    {0x1.93737b0cdc600p+0, -0x1.b0bafe3c0dabfp-48},
    {0x1.9c49182a3f080p+0, 0x1.01c7c46b071f3p-48},
    {0x1.a5503b23e2580p+0, -0x1.1ba5eddb71a84p-47},
    {0x1.ae89f995ad380p+0, 0x1.6af439a68bb99p-47},
    {0x1.b7f76f2fb5e80p+0, -0x1.c8aac27bf2a56p-47},
    {0x1.c199bdd855280p+0, 0x1.c2220cb12a092p-48},
    {0x1.cb720dcef9080p+0, -0x1.6eafc342e16b6p-48},
    {0x1.d5818dcfba480p+0, 0x1.c976816bad9b8p-50},
    {0x1.dfc97337b9b80p+0, -0x1.0a34b9a9e3097p-47},
    {0x1.ea4afa2a49100p+0, -0x1.33d38462f3851p-47},
    {0x1.f50765b6e4580p+0, -0x1.fcc583da44ebdp-47},
};

// fused multiply-add with one rounding (IEEE fma on both sides)
LB_HD double fma_(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
  return __fma_rn(a, b, c);
#else
  return __builtin_fma(a, b, c);
#endif
}

// exp(x) in IEEE double, identical on host (compiled with
// -ffp-contract=off) and device (compiled with -fmad=false; the explicit
// fma_ calls are the only fused operations).
LB_HD uint64_t umulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

LB_HD double lb_exp_fp64(double x) {
  const double kInvL = 0x1.71547652b82fep+5;   // 32/ln2
  const double kL1 = 0x1.62e42ff000000p-6;     // ln2/32, leading 32 bits
  const double kL2 = -0x1.718432a1b0e26p-40;   // ln2/32 - kL1
  const double kShift = 0x1.8p52;              // round-to-nearest-integer shifter
  if (!(x == x)) return x + x;                 // NaN
  if (x > 709.782712893384) return bits_to_double(0x7ff0000000000000ull);
  if (x < -745.1332191019412) return 0.0;
  // N = rint(x*32/ln2) via the 1.5*2^52 shifter (round to nearest even)
  const double t = x * kInvL + kShift;         // contraction disabled: mul then add
  const double Nd = t - kShift;
  const int N = (int)Nd;
  const int J = N & 31;
  const int M = (N - J) / 32;
  // R = Rh + Rl: Rh is the rounded reduced argument, Rl its rounding error
  // plus the rounding error of Nd*kL2 (both exact through fma / Fast2Sum)
  const double R1 = x - Nd * kL1;               // exact
  const double T = Nd * kL2;
  const double Tl = fma_(Nd, kL2, -T);
  const double Rh = R1 - T;
  const double Rl = ((R1 - Rh) - T) - Tl;
  // exp(R) - 1 = Rh + H + small, with H = Rh^2/2 exact and small holding
  // the low part of Rh^2/2, the Rl cross term and R^3/6 + ... + R^8/8!
  const double R2h = Rh * Rh;
  const double R2l = fma_(Rh, Rh, -R2h);
  const double H = 0.5 * R2h;
  const double c3 = R2h * Rh * (0x1.5555555555555p-3 + Rh * (0x1.5555555555555p-5 +
                    Rh * (0x1.1111111111111p-7 + Rh * (0x1.6c16c16c16c17p-10 +
                    Rh * (0x1.a01a01a01a01ap-13 + Rh * 0x1.a01a01a01a01ap-16)))));
  const double small = (0.5 * R2l + Rh * Rl) + (Rl + c3);
  // 2^(J/32) * exp(R) = (Sl + St)(1 + Rh + H + small), summed so that only
  // the last addition rounds at the result's precision
  const double Sl = kExpTable[J][0];
  const double St = kExpTable[J][1];
  const double Ah = Sl * Rh;
  const double Al = fma_(Sl, Rh, -Ah);
  const double Bh = Sl * H;
  const double Bl = fma_(Sl, H, -Bh);
  const double s1 = Ah + Bh;                    // TwoSum(Ah, Bh)
  const double bv = s1 - Ah;
  const double e1 = (Ah - (s1 - bv)) + (Bh - bv);
  const double s = Sl + s1;                     // Fast2Sum: |Sl| >= 1 > |s1|
  const double e2 = (Sl - s) + s1;
  const double tail = e2 + (e1 + (Al + (Bl + (Sl * small + (St + St * ((Rh + H) + small))))));
  double y = s + tail;
  // The reference rounds twice: its exp works in the x87 80-bit format (64
  // significant bits) and the result is stored as a double.  RN53(RN64(v))
  // differs from RN53(v) = y only when RN64(v) is the midpoint between y and
  // its neighbour, i.e. when v lies within half a 64-bit ulp of that midpoint;
  // the midpoint then rounds to the even one of the two.
  const double rr = tail - (y - s);            // v = y + rr (Fast2Sum residual)
  const uint64_t yb = double_to_bits(y);
  const double ulp = bits_to_double(((yb >> 52) - 52) << 52);   // y in [0.98, 2.03]
  const double gap = 0.5 * ulp - (rr < 0.0 ? -rr : rr);
  if ((yb & 1) && gap <= ulp * 0x1p-12) y = bits_to_double(rr > 0.0 ? yb + 1 : yb - 1);
  if (M >= -1021) {
    if (M <= 1023) return y * pow2i(M);
    return (y * pow2i(M - 1)) * 2.0;
  }
  // subnormal result: first scale exactly, then round once
  return (y * pow2i(M + 600)) * pow2i(-600);
}

// ---------------------------------------------------------------------------
// The same exp in integer fixed-point arithmetic, for 2^-83 <= |x| <= 707
// (every other argument takes lb_exp_fp64).  GB300 executes FP64 at a small
// fraction of its integer rate and lb_exp_fp64 costs ~60 FP64 operations;
// this costs none.  It computes exp(x) to ~2^-90 relative and then rounds it
// exactly as the reference's 80-bit evaluation does: to a 64-bit
// significand, then to 53 bits (both round to nearest even).
//   N = round(|x| 256/ln2) (from |x|'s significand times 256/ln2 in 2^-55
//       units; a rare off-by-one only enlarges |R| negligibly), J = N mod
//       256, M = floor(N / 256) (signs applied)
//   R = x - N ln2/256 in units of 2^-136: |x| 2^136 and N ln2/256 2^136
//       agree above bit 127, so their difference mod 2^128 is R exactly
//       (up to ln2/256's rounding, < 2^-118)
//   exp(R) = 1 + R + R^2/2 + R^3 P(R), P(R) = sum_i R^i/(i+3)! (i < 6), in
//       units of 2^-126: R^2 from R's top 64 bits plus the cross term, P by
//       Horner in 2^-63 units (|R| <= ln2/512, truncation below 2^-104)
//   exp(x) = 2^M * (2^(J/256) in 2^-127 units, kExp256) * exp(R)
// ---------------------------------------------------------------------------
typedef unsigned __int128 lb_u128;
typedef __int128 lb_i128;

LB_HD int64_t mulhi64(int64_t a, int64_t b) {
#if defined(__CUDA_ARCH__)
  return __mul64hi(a, b);
#else
  return (int64_t)(((__int128)a * b) >> 64);
#endif
}

LB_HD uint64_t exp_table(int j, int w) {
#if defined(__CUDA_ARCH__)
  return __ldg(&kExp256[j][w]);
#else
  return kExp256[j][w];
#endif
}

LB_HD double lb_exp(double x) {
  const uint64_t ux = double_to_bits(x);
  const int ex = int((ux >> 52) & 0x7ff);
  const uint64_t ax = ux & 0x7fffffffffffffffull;
  // 2^-83 <= |x| <= 707 (0x408618 = 707's top bits)
  if (ex < 940 || ax > 0x4086180000000000ull) return lb_exp_fp64(x);
  const bool neg = (ux >> 63) != 0;
  const uint64_t mx = (ux & 0xfffffffffffffull) | (uint64_t(1) << 52);
  // N = round(|x| 256/ln2) = round(mx kExpK 2^(ex - 1130))
  const int sn = 1130 - 64 - 1 - ex;  // in [33, 125]
  const uint64_t n2 = sn >= 64 ? 0 : (umulhi64(mx, kExpK) >> sn);
  const int64_t nabs = (int64_t)((n2 + 1) >> 1);
  // R = |x| - nabs ln2/256 in 2^-136 units (mod 2^128), then the sign of x
  const lb_u128 X = (lb_u128)mx << (ex - 939);
  const lb_u128 L = ((lb_u128)kExpL136Hi << 64) | kExpL136Lo;
  lb_u128 Ru = X - (lb_u128)(uint64_t)nabs * L;
  if (neg) Ru = (lb_u128)0 - Ru;
  const lb_i128 R = (lb_i128)Ru;
  const int64_t N = neg ? -nabs : nabs;
  const bool rneg = R < 0;
  const lb_u128 A = rneg ? (lb_u128)0 - Ru : Ru;  // |R|
  const uint64_t a1 = (uint64_t)(A >> 64), a0 = (uint64_t)A;
  const int64_t r1 = (int64_t)(R >> 64);  // R 2^72
  // E = exp(R) in 2^-126 units
  lb_i128 E = (lb_i128)1 << 126;
  E += R >> 10;
  const lb_u128 a1sq = (lb_u128)a1 * a1;  // R^2 2^144
  E += (lb_i128)(a1sq >> 19) + (lb_i128)(umulhi64(a1, a0) >> 18);
  int64_t p = kExpP5;
  p = kExpP4 + (mulhi64(r1, p) >> 8);
  p = kExpP3 + (mulhi64(r1, p) >> 8);
  p = kExpP2 + (mulhi64(r1, p) >> 8);
  p = kExpP1 + (mulhi64(r1, p) >> 8);
  p = kExpP0 + (mulhi64(r1, p) >> 8);
  const uint64_t s2 = (uint64_t)(a1sq >> 62);       // R^2 2^82
  const uint64_t s3 = umulhi64(s2, a1);             // |R|^3 2^90
  const uint64_t t = umulhi64(s3, (uint64_t)p);     // |R|^3 P 2^89
  const lb_i128 T = (lb_i128)((lb_u128)t << 37);
  E += rneg ? -T : T;
  // V = E * 2^(J/256) in 2^-125 units (in [0.998, 1.998] 2^125)
  const int J = int(N & 255);
  const int64_t M = N >> 8;  // floor
  const uint64_t th = exp_table(J, 0), tl = exp_table(J, 1);
  const lb_u128 Eu = (lb_u128)E;
  const uint64_t eh = (uint64_t)(Eu >> 64), el = (uint64_t)Eu;
  const lb_u128 V = (lb_u128)eh * th + (lb_u128)umulhi64(eh, tl) + (lb_u128)umulhi64(el, th);
  // round to a 64-bit significand, then to 53 bits (nearest even both)
  int Lb = (V >> 125) != 0 ? 125 : 124;  // leading bit
  uint64_t m64 = (uint64_t)(V >> (Lb - 63));
  const bool rb = ((V >> (Lb - 64)) & 1) != 0;
  const bool st = (V & (((lb_u128)1 << (Lb - 64)) - 1)) != 0;
  if (rb && (st || (m64 & 1))) {
    m64 += 1;
    if (m64 == 0) {
      m64 = uint64_t(1) << 63;
      Lb += 1;
    }
  }
  uint64_t m53 = m64 >> 11;
  if (((m64 >> 10) & 1) && ((m64 & 0x3ff) != 0 || (m53 & 1))) {
    m53 += 1;
    if (m53 == (uint64_t(1) << 53)) {
      m53 >>= 1;
      Lb += 1;
    }
  }
  const int64_t e = int64_t(Lb) + M + 898;
  return bits_to_double((uint64_t(e) << 52) | (m53 & 0xfffffffffffffull));
}

// ---------------------------------------------------------------------------
// IEEE double division a / b (round to nearest even) in integer arithmetic.
//
// GB300 executes FP64 at a small fraction of its integer rate, and a
// hardware-sequence division costs about 14 FP64 operations.  The FP64
// timestep divides 9 times per site (F/rho per component, the weighted
// velocity by the total density), so it uses this instead for operands in
// the common range; IEEE division is exactly specified, so the result is
// the same bits as a / b (tested against the hardware division).
//
// For b = mb 2^(eb-1075) with mb in (2^52, 2^53), DivRecip holds
// v ~ 2^116 / mb within a few units: a correctly rounded float reciprocal
// of mb's top 24 bits (relative error < 2^-22) refined by two Newton steps
// v += v (2^116 - mb v) / 2^116 in 64/128-bit integer arithmetic.  For
// a = ma 2^(ea-1075) (ma scaled so that ma/mb is in [1, 2)),
// q = floor(ma 2^53 / mb) is floor(ma v / 2^63) or one more, fixed with the
// exact remainder ma 2^53 - q mb; q's 54 bits are the mantissa, the
// rounding bit and (with the remainder) the sticky bit.  Operands or
// results outside the normal range, and b a power of two, take a / b.
// ---------------------------------------------------------------------------
LB_HD float frcp_rn(float x) {
#if defined(__CUDA_ARCH__)
  return __frcp_rn(x);
#else
  return 1.0f / x;  // correctly rounded, as __frcp_rn
#endif
}

struct DivRecip {
  double b;      // the divisor
  uint64_t mb;   // its 53-bit significand
  uint64_t v;    // ~2^116 / mb
  int eb;        // its biased exponent
  uint64_t sb;   // its sign bit (bit 63)
  bool ok;       // normal, finite, not a power of two
};

// one Newton step for v ~ 2^116 / m; e = 2^116 - m v is taken >> sh
// (|e| < 2^(62 + sh)) and the correction v e / 2^116 as
// umulhi(v, |e| >> sh) >> (52 - sh)
LB_HD uint64_t recip_step(uint64_t m, uint64_t v, int sh) {
  const uint64_t pl = m * v, ph = umulhi64(m, v);  // m v < 2^117
  // e = 2^116 - (ph:pl) as a signed 128-bit value (hi:lo)
  const uint64_t lo = 0 - pl;
  const uint64_t hi = (uint64_t(1) << 52) - ph - (pl != 0 ? 1 : 0);
  const bool neg = (int64_t)hi < 0;
  // |e| (128-bit) >> sh, fits in 63 bits
  uint64_t ahi = hi, alo = lo;
  if (neg) {
    alo = 0 - lo;
    ahi = ~hi + (lo == 0 ? 1 : 0);
  }
  const uint64_t es = (ahi << (64 - sh)) | (alo >> sh);
  const uint64_t corr = umulhi64(v, es) >> (52 - sh);
  return neg ? v - corr : v + corr;
}

LB_HD DivRecip div_recip(double b) {
  DivRecip r;
  r.b = b;
  const uint64_t ub = double_to_bits(b);
  r.eb = int((ub >> 52) & 0x7ff);
  r.sb = ub & (uint64_t(1) << 63);
  const uint64_t fb = ub & ((uint64_t(1) << 52) - 1);
  r.mb = fb | (uint64_t(1) << 52);
  r.ok = r.eb != 0 && r.eb != 0x7ff && fb != 0;
  r.v = 0;
  if (!r.ok) return r;
  // v0 from the float reciprocal of mb's top 24 bits (mf exact, in (2^23, 2^24))
  const float mf = (float)(uint32_t)(r.mb >> 29);
  const float rf = frcp_rn(mf);  // in [2^-24, 2^-23]
  uint32_t rb;
  memcpy(&rb, &rf, sizeof rb);
  const uint64_t sig = (uint64_t)((rb & 0x7fffffu) | 0x800000u);
  const int e = int((rb >> 23) & 0xff);  // 103 for rf < 2^-23, 104 for rf = 2^-23
  uint64_t v = e == 103 ? sig << 40 : ~uint64_t(0);  // rf * 2^87
  v = recip_step(r.mb, v, 32);  // |e| < 2^94 before, relative error ~2^-45 after
  v = recip_step(r.mb, v, 10);  // |e| < 2^72 before, within a few units after
  r.v = v;
  return r;
}

LB_HD double div_rn(double a, const DivRecip& r) {
  const uint64_t ua = double_to_bits(a);
  const int ea = int((ua >> 52) & 0x7ff);
  const uint64_t sign = (ua & (uint64_t(1) << 63)) ^ r.sb;
  if (r.ok && (ua << 1) == 0) return bits_to_double(sign);  // +-0 / b
  if (!r.ok || ea == 0 || ea == 0x7ff) return a / r.b;
  uint64_t ma = (ua & ((uint64_t(1) << 52) - 1)) | (uint64_t(1) << 52);
  int e = ea - r.eb + 1023;
  if (ma < r.mb) {
    ma <<= 1;
    e -= 1;
  }
  if (e < 1 || e > 2045) return a / r.b;  // subnormal or overflowing quotient
  // q = floor(ma 2^53 / mb) in [2^53, 2^54), remainder rem in [0, mb)
  const uint64_t pl = ma * r.v, ph = umulhi64(ma, r.v);
  uint64_t q = (ph << 1) | (pl >> 63);
  uint64_t rem = (ma << 53) - q * r.mb;  // exact: the true value is < 2 mb < 2^54
  if ((int64_t)rem < 0) {
    q -= 1;
    rem += r.mb;
  }
  if (rem >= r.mb) {
    q += 1;
    rem -= r.mb;
  }
  uint64_t m53 = q >> 1;
  if ((q & 1) && (rem != 0 || (m53 & 1))) m53 += 1;
  if (m53 == (uint64_t(1) << 53)) {
    m53 >>= 1;
    e += 1;
  }
  return bits_to_double(sign | (uint64_t(e) << 52) | (m53 & ((uint64_t(1) << 52) - 1)));
}

LB_HD double div_rn(double a, double b) { return div_rn(a, div_recip(b)); }

}  // namespace lbmath
