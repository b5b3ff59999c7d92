// CPU oracle for the DLBC timestep (TEST INFRASTRUCTURE, see lb_oracle.h).
//
// Every function restates the D source it cites, in the same loop and
// expression order, in IEEE double without FMA contraction
// (built with -O2 -ffp-contract=off, no fast-math).
#include "lb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../dlbc_gb300/csrc/lb_math.h"

namespace {

// ---------------------------------------------------------------------------
// Connectivity: src/dlbc/lb/connectivity.d:250-418
// ---------------------------------------------------------------------------
struct Conn {
  int d, q;
  int c[19][3];
  double w[19];
  int bounce[19];
  double css;  // speed of sound squared (generateSpeedOfSound, connectivity.d:213-245)
};

Conn make_conn(int d, int q) {
  Conn k;
  memset(&k, 0, sizeof k);
  k.d = d;
  k.q = q;
  if (d == 3 && q == 19) {
    // generateD3Q19 (connectivity.d:401-418)
    static const int v[19][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                                 {0, 0, 1},  {0, 0, -1},  {1, 1, 0},  {-1, 1, 0}, {0, 1, 1},
                                 {0, -1, 1}, {1, 0, 1},   {1, 0, -1}, {1, -1, 0}, {-1, -1, 0},
                                 {0, 1, -1}, {0, -1, -1}, {-1, 0, 1}, {-1, 0, -1}};
    memcpy(k.c, v, sizeof v);
    // generateWeights (connectivity.d:253-256)
    k.w[0] = 1.0 / 3.0;
    for (int i = 1; i < 7; ++i) k.w[i] = 1.0 / 18.0;
    for (int i = 7; i < 19; ++i) k.w[i] = 1.0 / 36.0;
  } else if (d == 2 && q == 9) {
    // generateD2Q9 (connectivity.d:372-381)
    static const int v[9][3] = {{0, 0, 0},  {1, 0, 0}, {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                                {1, 1, 0},  {1, -1, 0}, {-1, 1, 0}, {-1, -1, 0}};
    memcpy(k.c, v, sizeof v);
    // connectivity.d:266-269
    k.w[0] = 4.0 / 9.0;
    for (int i = 1; i < 5; ++i) k.w[i] = 1.0 / 9.0;
    for (int i = 5; i < 9; ++i) k.w[i] = 1.0 / 36.0;
  } else if (d == 1 && q == 3) {
    // generateD1Q3 (connectivity.d:339-345): 0, +1, -1; weights 4/6, 1/6
    static const int v[3][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}};
    memcpy(k.c, v, sizeof v);
    k.w[0] = 4.0 / 6.0;
    k.w[1] = k.w[2] = 1.0 / 6.0;
  } else if (d == 1 && q == 5) {
    // generateD1Q5 (connectivity.d:347-353): 0, +1, -1, +2, -2; weights
    // 6/12, 2/12, 1/12
    static const int v[5][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {2, 0, 0}, {-2, 0, 0}};
    memcpy(k.c, v, sizeof v);
    k.w[0] = 6.0 / 12.0;
    k.w[1] = k.w[2] = 2.0 / 12.0;
    k.w[3] = k.w[4] = 1.0 / 12.0;
  } else {
    k.q = 0;
  }
  k.css = (d == 1 && q == 5) ? 1.0 : 1.0 / 3.0;
  // generateBounce (connectivity.d:198-212): first j with c_i + c_j == 0
  for (int i = 0; i < k.q; ++i)
    for (int j = 0; j < k.q; ++j)
      if (k.c[i][0] + k.c[j][0] == 0 && k.c[i][1] + k.c[j][1] == 0 && k.c[i][2] + k.c[j][2] == 0) {
        k.bounce[i] = j;
        break;
      }
  return k;
}

// Phobos std.algorithm.sum for a double[] slice, dmd 2.066-2.070:
//   sum(r) = 0.0 + sumPairwise(r), sumPairwise splitting at length/2.
double sum_pairwise(const double* a, size_t n) {
  switch (n) {
    case 0: return 0.0;
    case 1: return a[0];
    case 2: return a[0] + a[1];
    default: return sum_pairwise(a, n / 2) + sum_pairwise(a + n / 2, n - n / 2);
  }
}

// std.random.uniform!"[)"(a, b, Mt19937) for doubles
double uniform_ab(std::mt19937& g, double a, double b) {
  const double bb = nextafter(b, -INFINITY);
  const double u = (double)(uint32_t)g();
  return a + (bb - a) * u / 4294967295.0;
}

}  // namespace

struct or_lattice {
  or_config cfg;
  Conn k;
  int d, q, C, h;
  long n[3], nH[3];
  long sizeH;
  std::vector<std::vector<double>> fluids;   // C x sizeH x q
  std::vector<double> advection;             // sizeH x q
  std::vector<int32_t> mask;                 // sizeH (Mask.None = 0, Mask.Solid = 1)
  std::vector<std::vector<double>> density;  // C x sizeH
  std::vector<std::vector<double>> psi;      // C x sizeH
  std::vector<std::vector<double>> force;    // C x sizeH x d
  std::vector<double> wv;                    // sizeH x 3 (weightedVelocityBDist2)

  long idx(long x, long y, long z) const { return (x * nH[1] + y) * nH[2] + z; }
  bool solid(long i) const { return mask[i] != 0; }

  double density_of(const double* pop) const {
    if (cfg.sum_mode & 1) {
      double s = 0.0;
      for (int i = 0; i < q; ++i) s += pop[i];
      return s;
    }
    return 0.0 + sum_pairwise(pop, q);
  }

  double psi_of(double rho) const {
    // psi (src/dlbc/lb/force.d:320-333)
    if (cfg.psi_form == 0) return rho;
    double e;
    if (cfg.exp_mode == 1)
      e = lbmath::lb_exp(-rho);
    else
      e = (double)expl(-(long double)rho);
    return 1.0 - e;
  }
};

namespace {

template <typename F>
void for_physical(const or_lattice& L, F&& fn) {
  const long x0 = L.h, x1 = L.n[0] + L.h;
#pragma omp parallel for schedule(static) if (L.cfg.threads > 1) num_threads(L.cfg.threads > 1 ? L.cfg.threads : 1)
  for (long x = x0; x < x1; ++x) {
    const long yh = (L.d >= 2) ? L.h : 0;
    for (long y = yh; y < L.n[1] + yh; ++y) {
      const long zh = (L.d == 3) ? L.h : 0;
      for (long z = zh; z < L.n[2] + zh; ++z) fn(x, y, z, L.idx(x, y, z));
    }
  }
}

template <typename F>
void for_all(const or_lattice& L, F&& fn) {
#pragma omp parallel for schedule(static) if (L.cfg.threads > 1) num_threads(L.cfg.threads > 1 ? L.cfg.threads : 1)
  for (long x = 0; x < L.nH[0]; ++x)
    for (long y = 0; y < L.nH[1]; ++y)
      for (long z = 0; z < L.nH[2]; ++z) fn(x, y, z, L.idx(x, y, z));
}

// exchangeHalo for one rank on a periodic cartesian grid
// (src/dlbc/fields/parallel.d:40-143): per dimension, the top h physical
// layers go to the low halo and the bottom h physical layers to the high
// halo, over the full haloed extent of the other dimensions.
template <typename T>
void exchange_field(const or_lattice& L, T* a, int len) {
  const long h = L.h;
  for (int dim = 0; dim < L.d; ++dim) {
    const long n = L.n[dim];
    for (long x = 0; x < L.nH[0]; ++x)
      for (long y = 0; y < L.nH[1]; ++y)
        for (long z = 0; z < L.nH[2]; ++z) {
          long p[3] = {x, y, z};
          const long v = p[dim];
          long src;
          if (v < h)
            src = v + n;
          else if (v >= n + h)
            src = v - n;
          else
            continue;
          long s[3] = {x, y, z};
          s[dim] = src;
          const long di = L.idx(x, y, z), si = L.idx(s[0], s[1], s[2]);
          memcpy(a + di * len, a + si * len, sizeof(T) * len);
        }
  }
}

bool is_on_edge(const or_lattice& L, long x, long y, long z) {
  // isOnEdge (advection.d:91-99)
  const long p[3] = {x, y, z};
  for (int i = 0; i < L.d; ++i)
    if (p[i] == 0 || p[i] == L.nH[i] - 1) return true;
  return false;
}

// advectFieldsKernel (src/dlbc/lb/advection.d:61-89).  D1Q5's |c| = 2
// velocities would pull halo site 1 from outside the haloed array (the
// reference reads out of bounds there; its D1Q5 test is disabled): for D1Q5
// only physical sites are advected and the halo is refreshed with their
// periodic images afterwards, which is what the other connectivities' halo
// sites hold after advection anyway.
void advect(or_lattice& L) {
  const int q = L.q;
  const bool long_vel = L.d == 1 && q == 5;
  for (int f = 0; f < L.C; ++f) {
    const double* src = L.fluids[f].data();
    double* dst = L.advection.data();
    for_all(L, [&](long x, long y, long z, long i) {
      if (is_on_edge(L, x, y, z)) return;
      if (long_vel && (x < L.h || x >= L.n[0] + L.h)) return;
      double* pop = dst + i * q;
      if (!L.solid(i)) {  // isAdvectable
        for (int vq = 0; vq < q; ++vq) {
          const long nb = L.idx(x - L.k.c[vq][0], y - L.k.c[vq][1], z - L.k.c[vq][2]);
          if (L.solid(nb))  // isBounceBack
            pop[vq] = src[i * q + L.k.bounce[vq]];
          else
            pop[vq] = src[nb * q + vq];
        }
      } else {
        memcpy(pop, src + i * q, sizeof(double) * q);
      }
    });
    std::swap(L.fluids[f], L.advection);
    if (long_vel) exchange_field(L, L.fluids[f].data(), q);
  }
}

// precalculateDensities -> densityField over all sites incl. halo
// (src/dlbc/lb/density.d:89-96, :344-352), then psiField (force.d:360-367)
void densities_and_psi(or_lattice& L) {
  for (int f = 0; f < L.C; ++f) {
    const double* a = L.fluids[f].data();
    double* den = L.density[f].data();
    double* ps = L.psi[f].data();
    for_all(L, [&](long, long, long, long i) {
      den[i] = L.density_of(a + i * L.q);
      ps[i] = L.psi_of(den[i]);
    });
  }
}

// resetForce (force.d:165-170) + addShanChenForcePsi (force.d:238-309)
// + distributeForce (force.d:179-197) with a zero distributed force
void forces(or_lattice& L) {
  const int q = L.q, d = L.d, C = L.C;
  for (int f = 0; f < C; ++f) std::fill(L.force[f].begin(), L.force[f].end(), 0.0);
  if (L.cfg.shan_chen) {
    for (int f1 = 0; f1 < C; ++f1) {
      for (int f2 = 0; f2 < C; ++f2) {
        const double cc = L.cfg.gcc[f1][f2];
        if (cc == 0.0) continue;
        for_physical(L, [&](long x, long y, long z, long i) {
          if (L.solid(i)) return;  // isCollidable
          double* force = L.force[f1].data() + i * d;
          const double psiden1 = L.psi[f1][i];
          for (int vq = 1; vq < q; ++vq) {  // Iota!(1, q-1) = 1 .. q-1
            const long nb = L.idx(x + L.k.c[vq][0], y + L.k.c[vq][1], z + L.k.c[vq][2]);
            const double psiden2 = L.solid(nb) ? L.psi[f2][i] : L.psi[f2][nb];
            const double prefactor = L.k.w[vq] * psiden1 * psiden2 * cc;
            for (int vd = 0; vd < d; ++vd) force[vd] -= prefactor * (double)L.k.c[vq][vd];
          }
        });
      }
      const double wc = L.cfg.gwc[f1];
      if (wc == 0.0) continue;
      for_physical(L, [&](long x, long y, long z, long i) {
        if (L.solid(i)) return;
        double* force = L.force[f1].data() + i * d;
        const double psiden1 = L.psi[f1][i];
        for (int vq = 0; vq < q; ++vq) {
          const long nb = L.idx(x + L.k.c[vq][0], y + L.k.c[vq][1], z + L.k.c[vq][2]);
          if (L.solid(nb)) {
            const double prefactor = L.k.w[vq] * psiden1 * L.density[f1][nb] * wc;
            for (int vd = 0; vd < d; ++vd) force[vd] -= prefactor * (double)L.k.c[vq][vd];
          }
        }
      });
    }
  }
  // distributeForce: force += forceDistributed * (rho_f / rho_tot) with
  // forceDistributed == 0 (no elec); kept for its NaN/-0 semantics
  for_physical(L, [&](long, long, long, long i) {
    double totalDensity = 0.0;
    for (int f = 0; f < C; ++f) totalDensity += L.density[f][i];
    for (int f = 0; f < C; ++f)
      for (int vd = 0; vd < d; ++vd) L.force[f][i * d + vd] += 0.0 * (L.density[f][i] / totalDensity);
  });
}

// precalculateWeightedVelocity (src/dlbc/lb/collision.d:156-196)
void weighted_velocity(or_lattice& L) {
  const int q = L.q, d = L.d, C = L.C;
  for_physical(L, [&](long, long, long, long i) {
    double* wv = L.wv.data() + i * 3;
    for (int vd = 0; vd < 3; ++vd) wv[vd] = 0.0;
    for (int f = 0; f < C; ++f) {
      double perFluid[3] = {0.0, 0.0, 0.0};
      const double* pop = L.fluids[f].data() + i * q;
      for (int vq = 0; vq < q; ++vq)
        for (int vd = 0; vd < d; ++vd) perFluid[vd] += pop[vq] * (double)L.k.c[vq][vd];
      for (int vd = 0; vd < d; ++vd) wv[vd] += perFluid[vd] / L.cfg.tau[f];
    }
  });
  for_physical(L, [&](long, long, long, long i) {
    double* wv = L.wv.data() + i * 3;
    double totalDensity = 0.0;
    for (int f = 0; f < C; ++f) totalDensity += L.density[f][i];
    for (int vd = 0; vd < d; ++vd) wv[vd] /= totalDensity;
  });
}

// rawVelocity (src/dlbc/lb/velocity.d:37-48)
void raw_velocity(const or_lattice& L, const double* pop, double den, double* vel) {
  for (int j = 0; j < L.d; ++j) vel[j] = 0.0;
  for (int i = 0; i < L.q; ++i)
    for (int j = 0; j < L.d; ++j) vel[j] += pop[i] * (double)L.k.c[i][j];
  // `vel[] /= density` is a D array operation; druntime's array-op
  // routine for `a[] /= value` on doubles multiplies by the reciprocal,
  // which reproduces the SecondOrder/ThirdOrder goldens more closely than
  // a true division does.
  const double recip = 1.0 / den;
  for (int j = 0; j < L.d; ++j) vel[j] *= recip;
}

// dotProduct (src/dlbc/range.d:57-67)
double dot(const double* a, const double* b, int d) {
  double s = 0;
  for (int i = 0; i < d; ++i) s += a[i] * b[i];
  return s;
}

// eqDist (src/dlbc/lb/eqdist.d:61-278)
void eq_dist(const or_lattice& L, const double* pop, const double* dv, double rho0, double* dist) {
  const int q = L.q, d = L.d;
  const int form = L.cfg.eq_form;
  if (form == 0 || form == 1) {
    const double css = L.k.css;
    double pv[3];
    raw_velocity(L, pop, rho0, pv);
    double v[3] = {0, 0, 0};
    for (int vd = 0; vd < d; ++vd) v[vd] = dv[vd] + pv[vd];
    const double vdotv = dot(v, v, d);
    const double css2 = 2.0 * css;
    const double css2p2 = css2 * css;
    const double css6p3 = 3.0 * css2p2 * css;
    for (int vq = 0; vq < q; ++vq) {
      const double cv[3] = {(double)L.k.c[vq][0], (double)L.k.c[vq][1], (double)L.k.c[vq][2]};
      const double vdotcv = dot(v, cv, d);
      if (form == 0)
        dist[vq] = rho0 * L.k.w[vq] * (1.0 + (vdotcv / css) + (vdotcv * vdotcv / css2p2) - (vdotv / css2));
      else
        dist[vq] = rho0 * L.k.w[vq] *
                   (1.0 + (vdotcv / css) + (vdotcv * vdotcv / css2p2) - (vdotv / css2) +
                    (vdotcv * vdotcv * vdotcv / css6p3) - (vdotv * vdotcv / css2p2));
    }
    return;
  }
  // BDist2
  if (d == 3 && q == 19) {
    const double aN1 = 1.0 / 36.0;
    const double aN0 = 1.0 / 3.0;
    const double haN1 = 0.5 * aN1;
    const double aN1_6 = aN1 / 6.0;
    const double T = 1.0 / 3.0;
    const double holdit = 1.0 / T;
    const double tux = dv[0], tuy = dv[1], tuz = dv[2];
    const double tuxt = tux * holdit, tuyt = tuy * holdit, tuzt = tuz * holdit;
    const double uke = 0.5 * (tux * tuxt + tuy * tuyt + tuz * tuzt);
    const double cst = 1.0 - uke;
    const double const1 = aN1 * cst;
    double cdotu, even, odd;
#define OR_PAIR(CD, IP, IM, SCALE2)                                  \
  cdotu = (CD);                                                      \
  even = const1 + haN1 * cdotu * cdotu;                              \
  odd = const1 * cdotu + aN1_6 * cdotu * cdotu * cdotu;              \
  if (SCALE2) {                                                      \
    dist[IP] = 2.0 * (even + odd);                                   \
    dist[IM] = 2.0 * (even - odd);                                   \
  } else {                                                           \
    dist[IP] = even + odd;                                           \
    dist[IM] = even - odd;                                           \
  }
    OR_PAIR(tuxt, 1, 2, true)
    OR_PAIR(tuyt, 3, 4, true)
    OR_PAIR(tuzt, 5, 6, true)
    OR_PAIR(tuxt + tuyt, 7, 14, false)
    OR_PAIR(tuxt - tuyt, 13, 8, false)
    OR_PAIR(tuxt + tuzt, 11, 18, false)
    OR_PAIR(tuxt - tuzt, 12, 17, false)
    OR_PAIR(tuyt + tuzt, 9, 16, false)
    OR_PAIR(tuyt - tuzt, 15, 10, false)
    dist[0] = aN0 * cst;
    for (int vq = 0; vq < q; ++vq) dist[vq] *= rho0;
  } else if (d == 2 && q == 9) {
    const double aN1 = 1.0 / 24.0;
    const double aN0 = 1.0 / 2.0;
    const double haN1 = 0.5 * aN1;
    const double aN1_6 = aN1 / 6.0;
    const double T = 1.0 / 3.0;
    const double holdit = 1.0 / T;
    const double tux = dv[0], tuy = dv[1];
    const double tuxt = tux * holdit, tuyt = tuy * holdit;
    const double uke = 0.5 * (tux * tuxt + tuy * tuyt);
    const double cst = 1.0 - uke;
    const double const1 = aN1 * cst;
    double cdotu, even, odd;
    OR_PAIR(tuxt, 1, 2, true)
    OR_PAIR(tuyt, 3, 4, true)
    OR_PAIR(tuxt + tuyt, 5, 8, false)
    OR_PAIR(tuxt - tuyt, 6, 7, false)
#undef OR_PAIR
    dist[0] = aN0 * cst;
    for (int vq = 0; vq < q; ++vq) dist[vq] *= rho0;
  } else {
    // D1Q3 / D1Q5: BDist2 is not implemented and returns the population
    // itself (eqdist.d:268-272)
    for (int vq = 0; vq < q; ++vq) dist[vq] = pop[vq];
  }
}

// collideFieldsKernel (src/dlbc/lb/collision.d:90-119)
void collide(or_lattice& L) {
  const int q = L.q, d = L.d;
  for (int f = 0; f < L.C; ++f) {
    const double tau = L.cfg.tau[f];
    const double omega = 1.0 / tau;
    for_physical(L, [&](long, long, long, long i) {
      if (L.solid(i)) return;
      double* pop = L.fluids[f].data() + i * q;
      const double den = L.density[f][i];
      double dv[3] = {0, 0, 0};
      for (int vd = 0; vd < d; ++vd) {
        dv[vd] = tau * (L.cfg.global_acc[vd] + L.force[f][i * d + vd] / den);
        if (L.cfg.eq_form == 2) dv[vd] += L.wv[i * 3 + vd];
      }
      double eq[19];
      eq_dist(L, pop, dv, den, eq);
      for (int vq = 0; vq < q; ++vq) pop[vq] = pop[vq] * (1.0 - omega) + omega * eq[vq];
    });
  }
}

// eqDistUnity (eqdist.d:310-315)
void eq_unity(const or_lattice& L, double* out) {
  double pop0[19] = {0};
  pop0[0] = 1.0;
  double dv[3] = {0, 0, 0};
  const double rho0 = L.density_of(pop0);
  eq_dist(L, pop0, dv, rho0, out);
}

// symmetricLinearTransition (src/dlbc/fields/init.d:346-366)
double slt(double pos, double width, double negval, double posval) {
  if (width == 0.0) return (pos < 0) ? negval : posval;
  if (pos < -0.5 * width) return negval;
  if (pos > 0.5 * width) return posval;
  return (negval * (0.5 - pos / width) + posval * (0.5 + pos / width));
}

}  // namespace

extern "C" {

or_lattice* or_create(const or_config* cfg) {
  if (!cfg) return nullptr;
  if (!((cfg->d == 3 && cfg->q == 19) || (cfg->d == 2 && cfg->q == 9) || (cfg->d == 1 && (cfg->q == 3 || cfg->q == 5))))
    return nullptr;
  if (cfg->components < 1 || cfg->components > OR_MAXC) return nullptr;
  or_lattice* L = new or_lattice;
  L->cfg = *cfg;
  L->k = make_conn(cfg->d, cfg->q);
  L->d = cfg->d;
  L->q = cfg->q;
  L->C = cfg->components;
  L->h = 2;
  for (int i = 0; i < 3; ++i) {
    L->n[i] = (i < L->d) ? cfg->gn[i] : 1;
    L->nH[i] = (i < L->d) ? L->n[i] + 2 * L->h : 1;
  }
  L->sizeH = L->nH[0] * L->nH[1] * L->nH[2];
  L->fluids.assign(L->C, std::vector<double>(L->sizeH * L->q, 0.0));
  L->advection.assign(L->sizeH * L->q, 0.0);
  L->mask.assign(L->sizeH, 0);
  L->density.assign(L->C, std::vector<double>(L->sizeH, 0.0));
  L->psi.assign(L->C, std::vector<double>(L->sizeH, 0.0));
  L->force.assign(L->C, std::vector<double>(L->sizeH * L->d, 0.0));
  L->wv.assign(L->sizeH * 3, 0.0);
  return L;
}

void or_destroy(or_lattice* L) { delete L; }

void or_lengths_h(const or_lattice* L, int32_t out[3], int32_t* halo) {
  for (int i = 0; i < 3; ++i) out[i] = (int32_t)L->nH[i];
  *halo = L->h;
}

// initMask (src/dlbc/lb/mask.d:134-172) + initFluids (src/dlbc/lb/init.d:77-134)
// on every emulated rank's local haloed block, then assembly of the
// physical blocks into the global lattice and exchangeHalo.
int or_init_lattice(or_lattice* Lp, const or_init* ini) {
  or_lattice& L = *Lp;
  const int d = L.d, q = L.q, h = L.h;
  long nc[3], nl[3], nlH[3];
  for (int i = 0; i < 3; ++i) {
    nc[i] = (i < d && ini->nc[i] > 0) ? ini->nc[i] : 1;
    if (L.n[i] % nc[i]) return -1;
    nl[i] = L.n[i] / nc[i];
    nlH[i] = (i < d) ? nl[i] + 2 * h : 1;
  }
  const long sizeLH = nlH[0] * nlH[1] * nlH[2];
  double eqpop[19];
  eq_unity(L, eqpop);
  const long gsz[3] = {L.n[0], L.n[1], L.n[2]};
  long smallSize = gsz[0];
  for (int i = 0; i < d; ++i) smallSize = std::min(smallSize, gsz[i]);

  const int nranks = (int)(nc[0] * nc[1] * nc[2]);
  for (int rank = 0; rank < nranks; ++rank) {
    // MPI cartesian rank order: last dimension fastest
    const long cc[3] = {rank / (nc[1] * nc[2]), (rank / nc[2]) % nc[1], rank % nc[2]};
    std::vector<int32_t> lmask(sizeLH, 0);
    std::vector<std::vector<double>> lf(L.C, std::vector<double>(sizeLH * q, NAN));
    auto lidx = [&](long x, long y, long z) { return (x * nlH[1] + y) * nlH[2] + z; };
    // global integer coordinate of a local haloed index
    auto gcoord = [&](int dim, long p) -> long { return p + cc[dim] * nl[dim] - ((dim < d) ? h : 0); };

    // --- initMask
    for (long x = 0; x < nlH[0]; ++x)
      for (long y = 0; y < nlH[1]; ++y)
        for (long z = 0; z < nlH[2]; ++z) {
          const long p[3] = {x, y, z};
          int32_t e = 0;
          switch (ini->mask_init) {
            case 0: e = 0; break;
            case 2: {  // initPlates (fields/init.d:425-436)
              const int ax = ini->mask_axis;
              const long gp = gcoord(ax, p[ax]);
              e = (gp == ini->wall_offset || gp == (nl[ax] * nc[ax] - 1 - ini->wall_offset)) ? 1 : 0;
              break;
            }
            case 3:    // initTube (fields/init.d:400-412)
            case 4: {  // initBox (fields/init.d:377-388)
              for (int vd = 0; vd < d; ++vd) {
                const long g = gcoord(vd, p[vd]);
                if (ini->mask_init == 3 && vd == ini->mask_axis) continue;
                if (g == 0 || g == nl[vd] * nc[vd] - 1) e = 1;
              }
              break;
            }
            case 5: {  // initWalls (fields/init.d:449-467)
              for (int vd = 0; vd < d; ++vd) {
                const long g = gcoord(vd, p[vd]);
                if (ini->dimension_has_wall[vd][0] && g < ini->wall_thickness) e = 1;
                if (ini->dimension_has_wall[vd][1] && g >= nl[vd] * nc[vd] - ini->wall_thickness) e = 1;
              }
              break;
            }
            default: return -2;  // File: not supported by the oracle
          }
          lmask[lidx(x, y, z)] = e;
        }

    // --- initFluids: RNG seeded per rank (random.d:43-53, init.d:109-122)
    std::mt19937 grng((uint32_t)(ini->seed + (ini->shift_seed_by_rank ? rank : 0)));
    for (int f = 0; f < L.C; ++f) {
      std::mt19937 lrng_own;
      std::mt19937* lrng = &grng;
      if (ini->random_reseed[f]) {
        lrng_own.seed((uint32_t)(ini->random_seed[f] + (ini->shift_seed_by_rank ? rank : 0)));
        lrng = &lrng_own;
      }
      double* a = lf[f].data();
      const double* dens = ini->densities[f];
      const int fi = ini->fluid_init[f];
      // FluidInit values (init.d:139-253)
      enum { None, File, Const, EqDist, EqDistPerturb, EqDistPerturbFrac, ConstRandom, EqDistRandom,
             EqDistSphere, EqDistSphereFrac, EqDistCylinder, EqDistCylinderFrac, EqDistTwoSpheres,
             EqDistTwoSpheresFrac, EqDistLamellae, EqDistLamellaeFrac };
      double R = ini->init_radius;
      double off[3] = {ini->init_offset[0], ini->init_offset[1], ini->init_offset[2]};
      double sep[3] = {ini->init_separation[0], ini->init_separation[1], ini->init_separation[2]};
      if (fi == EqDistSphereFrac || fi == EqDistTwoSpheresFrac) {
        R = ini->init_radius * (double)smallSize;
        for (int vd = 0; vd < d; ++vd) {
          off[vd] = ini->init_offset[vd] * (double)gsz[vd];
          sep[vd] = ini->init_separation[vd] * (double)gsz[vd];
        }
      }
      if (fi == EqDistCylinderFrac) {
        long ss = 0;
        for (int vd = 0; vd < d; ++vd)
          if (vd != ini->init_axis && (gsz[vd] < ss || ss == 0)) ss = gsz[vd];
        R = ini->init_radius * (double)ss;
        for (int vd = 0; vd < d; ++vd) off[vd] = ini->init_offset[vd] * (double)gsz[vd];
      }
      std::vector<double> interfaces;
      if (fi == EqDistLamellae || fi == EqDistLamellaeFrac) {
        // calculateInterfaces (fields/init.d:335-344)
        interfaces.push_back(0.0);
        for (int i = 0; i < ini->n_lamellae; ++i) {
          double w = ini->lamellae_widths[i];
          if (fi == EqDistLamellaeFrac) w = ini->lamellae_widths[i] * (double)gsz[ini->init_axis];
          interfaces.push_back(w);
        }
        for (size_t i = 1; i < interfaces.size(); ++i) interfaces[i] += interfaces[i - 1];
        for (auto& v : interfaces) v -= 0.5;
      }
      for (long x = 0; x < nlH[0]; ++x)
        for (long y = 0; y < nlH[1]; ++y)
          for (long z = 0; z < nlH[2]; ++z) {
            const long p[3] = {x, y, z};
            double* e = a + lidx(x, y, z) * q;
            double val = 0.0;
            switch (fi) {
              case None:
              case File: continue;
              case Const:
                for (int vq = 0; vq < q; ++vq) e[vq] = dens[0];
                continue;
              case ConstRandom:
                for (int vq = 0; vq < q; ++vq) e[vq] = dens[0] * uniform_ab(*lrng, 0.0, 2.0);
                continue;
              case EqDist: {
                for (int vq = 0; vq < q; ++vq) e[vq] = dens[0] * eqpop[vq];
                continue;
              }
              case EqDistRandom: val = dens[0] * uniform_ab(*lrng, 0.0, 2.0); break;
              case EqDistPerturb: val = dens[0] + uniform_ab(*lrng, -ini->perturb[f], ini->perturb[f]); break;
              case EqDistPerturbFrac:
                val = dens[0] * (1.0 + uniform_ab(*lrng, -ini->perturb[f], ini->perturb[f]));
                break;
              case EqDistSphere:
              case EqDistSphereFrac: {
                double offset[3];
                for (int i = 0; i < d; ++i) {
                  const double g = (double)(p[i] + cc[i] * nl[i]) - (double)h;
                  offset[i] = g - ((double)(nc[i] * nl[i]) * 0.5 + off[i]) + 0.5;
                }
                const double relpos = sqrt(dot(offset, offset, d)) - R;
                val = slt(relpos, ini->interface_thickness, dens[0], dens[1]);
                break;
              }
              case EqDistCylinder:
              case EqDistCylinderFrac: {
                double offset[3] = {0, 0, 0};
                for (int i = 0; i < d; ++i) {
                  if (i == ini->init_axis) {
                    offset[i] = 0.0;
                  } else {
                    const double g = (double)(p[i] + cc[i] * nl[i]) - (double)h;
                    offset[i] = g - ((double)(nc[i] * nl[i]) * 0.5 + off[i]) + 0.5;
                  }
                }
                const double relpos = sqrt(dot(offset, offset, d)) - R;
                val = slt(relpos, ini->interface_thickness, dens[0], dens[1]);
                break;
              }
              case EqDistTwoSpheres:
              case EqDistTwoSpheresFrac: {
                double o1[3], o2[3];
                for (int i = 0; i < d; ++i) {
                  const double g = (double)(p[i] + cc[i] * nl[i]) - (double)h;
                  o1[i] = g - ((double)(nc[i] * nl[i]) * 0.5 + off[i] - 0.5 * sep[i]) + 0.5;
                  o2[i] = g - ((double)(nc[i] * nl[i]) * 0.5 + off[i] + 0.5 * sep[i]) + 0.5;
                }
                const double r1 = sqrt(dot(o1, o1, d)) - R;
                const double r2 = sqrt(dot(o2, o2, d)) - R;
                val = slt(std::min(r1, r2), ini->interface_thickness, dens[0], dens[1]);
                break;
              }
              case EqDistLamellae:
              case EqDistLamellaeFrac: {
                const int ax = ini->init_axis;
                const double gp = (double)(p[ax] + cc[ax] * nl[ax]) - (double)h;
                // findClosestInterface (fields/init.d:315-333)
                size_t ci = 0;
                double minD = fabs(interfaces[0] - gp);
                for (size_t i = 1; i < interfaces.size(); ++i) {
                  const double df = fabs(interfaces[i] - gp);
                  if (df < minD) {
                    minD = df;
                    ci = i;
                  }
                }
                const double minDiff = gp - interfaces[ci];
                const int nv = ini->n_dens[f];
                if (ci == 0)
                  val = slt(minDiff, ini->interface_thickness, dens[nv - 1], dens[ci]);
                else if ((int)ci == nv)
                  val = slt(minDiff, ini->interface_thickness, dens[ci - 1], dens[0]);
                else
                  val = slt(minDiff, ini->interface_thickness, dens[ci - 1], dens[ci]);
                break;
              }
              default: return -3;
            }
            for (int vq = 0; vq < q; ++vq) e[vq] = val * eqpop[vq];
          }
      // initEqDistWall (fields/init.d:469-477)
      for (long i = 0; i < sizeLH; ++i)
        if (lmask[i] == 1) {
          for (int vq = 0; vq < q; ++vq) a[i * q + vq] = 0.0;
          a[i * q] = 1.0;
        }
    }
    // copy the physical block into the global lattice
    for (long x = 0; x < nl[0]; ++x)
      for (long y = 0; y < nl[1]; ++y)
        for (long z = 0; z < nl[2]; ++z) {
          const long lx = x + h, ly = (d >= 2) ? y + h : y, lz = (d == 3) ? z + h : z;
          const long gx = x + cc[0] * nl[0] + h, gy = (d >= 2) ? y + cc[1] * nl[1] + h : y;
          const long gz = (d == 3) ? z + cc[2] * nl[2] + h : z;
          const long gi = L.idx(gx, gy, gz), li = lidx(lx, ly, lz);
          L.mask[gi] = lmask[li];
          for (int f = 0; f < L.C; ++f) memcpy(&L.fluids[f][gi * q], &lf[f][li * q], sizeof(double) * q);
        }
  }
  or_exchange_halo(Lp);
  return 0;
}

void or_get_fluid(const or_lattice* L, int c, double* out) {
  memcpy(out, L->fluids[c].data(), sizeof(double) * L->fluids[c].size());
}
void or_set_fluid(or_lattice* L, int c, const double* in) {
  memcpy(L->fluids[c].data(), in, sizeof(double) * L->fluids[c].size());
}
void or_get_mask(const or_lattice* L, int32_t* out) { memcpy(out, L->mask.data(), sizeof(int32_t) * L->sizeH); }
void or_set_mask(or_lattice* L, const int32_t* in) { memcpy(L->mask.data(), in, sizeof(int32_t) * L->sizeH); }

void or_exchange_halo(or_lattice* L) {
  for (int f = 0; f < L->C; ++f) exchange_field(*L, L->fluids[f].data(), L->q);
  exchange_field(*L, L->mask.data(), 1);
}

void or_run(or_lattice* L, int nsteps) {
  for (int t = 0; t < nsteps; ++t) {
    or_exchange_halo(L);         // main.d:179
    advect(*L);                  // main.d:182
    densities_and_psi(*L);       // precalculatePsi inside addShanChenForcePsi (force.d:250)
    forces(*L);                  // main.d:188-191
    if (L->cfg.eq_form == 2) weighted_velocity(*L);  // prepareToCollide (collision.d:41-51)
    collide(*L);                 // main.d:195
  }
}

static void phys_copy(const or_lattice* L, const double* src, int len, double* out) {
  long o = 0;
  const long zh = (L->d == 3) ? L->h : 0, yh = (L->d >= 2) ? L->h : 0;
  for (long x = L->h; x < L->n[0] + L->h; ++x)
    for (long y = yh; y < L->n[1] + yh; ++y)
      for (long z = zh; z < L->n[2] + zh; ++z) {
        memcpy(out + o * len, src + L->idx(x, y, z) * len, sizeof(double) * len);
        ++o;
      }
}

void or_population(const or_lattice* L, int c, double* out) { phys_copy(L, L->fluids[c].data(), L->q, out); }

void or_density(const or_lattice* L, int c, double* out) {
  std::vector<double> den(L->sizeH);
  for (long i = 0; i < L->sizeH; ++i) den[i] = L->density_of(&L->fluids[c][i * L->q]);
  phys_copy(L, den.data(), 1, out);
}

void or_colour(const or_lattice* L, int c1, int c2, double* out) {
  // colourField (density.d:284-295)
  std::vector<double> col(L->sizeH);
  for (long i = 0; i < L->sizeH; ++i)
    col[i] = L->solid(i) ? 0.0
                         : L->density_of(&L->fluids[c1][i * L->q]) - L->density_of(&L->fluids[c2][i * L->q]);
  phys_copy(L, col.data(), 1, out);
}

void or_velocity(const or_lattice* L, int c, double* out) {
  // rawVelocityField (velocity.d:106-117)
  std::vector<double> v(L->sizeH * L->d, 0.0);
  for (long i = 0; i < L->sizeH; ++i) {
    if (L->solid(i)) continue;
    const double* pop = &L->fluids[c][i * L->q];
    raw_velocity(*L, pop, L->density_of(pop), &v[i * L->d]);
  }
  phys_copy(L, v.data(), L->d, out);
}

void or_force(const or_lattice* L, int c, double* out) { phys_copy(L, L->force[c].data(), L->d, out); }

void or_mask_phys(const or_lattice* L, int32_t* out) {
  long o = 0;
  const long zh = (L->d == 3) ? L->h : 0, yh = (L->d >= 2) ? L->h : 0;
  for (long x = L->h; x < L->n[0] + L->h; ++x)
    for (long y = yh; y < L->n[1] + yh; ++y)
      for (long z = zh; z < L->n[2] + zh; ++z) out[o++] = L->mask[L->idx(x, y, z)];
}

double or_total_mass(const or_lattice* L, int c) {
  // localTotalMass (density.d:136-147): fluid physical sites, sequential
  double mass = 0.0;
  const long zh = (L->d == 3) ? L->h : 0, yh = (L->d >= 2) ? L->h : 0;
  for (long x = L->h; x < L->n[0] + L->h; ++x)
    for (long y = yh; y < L->n[1] + yh; ++y)
      for (long z = zh; z < L->n[2] + zh; ++z) {
        const long i = L->idx(x, y, z);
        if (!L->solid(i)) mass += L->density_of(&L->fluids[c][i * L->q]);
      }
  return mass;
}

double or_uniform_sequence(uint32_t seed, double a, double b, int n, double* out) {
  std::mt19937 g(seed);
  for (int i = 0; i < n; ++i) out[i] = uniform_ab(g, a, b);
  return n > 0 ? out[n - 1] : 0.0;
}

void or_exp(int mode, int n, const double* x, double* out) {
  for (int i = 0; i < n; ++i)
    out[i] = mode == 1 ? lbmath::lb_exp(x[i]) : mode == 2 ? lbmath::lb_exp_fp64(x[i]) : (double)expl((long double)x[i]);
}

void or_div(int n, const double* a, const double* b, double* out) {
  for (int i = 0; i < n; ++i) out[i] = lbmath::div_rn(a[i], b[i]);
}

}  // extern "C"
