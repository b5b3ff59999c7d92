// The reference's random draws for the initial fields (host code).
//
// initFluids (src/dlbc/lb/init.d:105-125) draws on each rank of the process
// grid nc (ranks numbered with the last dimension fastest) from Mt19937
// seeded with seed (+ rank with shiftSeedByRank; src/dlbc/random.d:43-53;
// the standard 32-bit Mersenne Twister, as std::mt19937): one uniform draw
// per haloed site of the rank's block in row-major order (z fastest),
// ConstRandom one per population of each site (src/dlbc/fields/init.d),
// component 0's draws before component 1's from the one generator unless
// randomReseed gives a component a generator of its own seeded with
// randomSeed (+ rank).  The draws of halo sites only advance the generator
// (exchangeHalo overwrites those sites with periodic images).
#pragma once

#include <stdint.h>

#include <random>
#include <vector>

namespace lbk {

struct DrawSpec {
  int64_t n[3] = {1, 1, 1};     // lattice extents (1 beyond the dimension)
  int64_t halo[3] = {2, 2, 2};  // halo width per axis (0 beyond the dimension)
  int64_t nc[3] = {1, 1, 1};    // process grid
  uint32_t seed = 0;            // random.seed
  bool shift_seed_by_rank = true;
  int components = 2;
  int64_t per_site[2] = {0, 0};  // draws per site of component c (0: none)
  bool reseed[2] = {false, false};
  uint32_t random_seed[2] = {0, 0};
};

// out[c]: component c's draws of the physical sites in the lattice's site
// order ([x][y][z], per_site draws per site); false if the lattice does not
// divide over the process grid
inline bool reference_draws(const DrawSpec& S, std::vector<uint32_t> (&out)[2]) {
  int64_t nl[3], nlh[3];
  for (int i = 0; i < 3; ++i) {
    if (S.nc[i] < 1 || S.n[i] % S.nc[i] != 0) return false;
    nl[i] = S.n[i] / S.nc[i];
    nlh[i] = nl[i] + 2 * S.halo[i];
  }
  const int64_t sites = S.n[0] * S.n[1] * S.n[2];
  for (int c = 0; c < S.components && c < 2; ++c) out[c].assign(size_t(sites * S.per_site[c]), 0u);
  const int64_t nranks = S.nc[0] * S.nc[1] * S.nc[2];
  for (int64_t rank = 0; rank < nranks; ++rank) {
    const int64_t cc[3] = {rank / (S.nc[1] * S.nc[2]), (rank / S.nc[2]) % S.nc[1], rank % S.nc[2]};
    const uint32_t shift = S.shift_seed_by_rank ? uint32_t(rank) : 0u;
    std::mt19937 global(S.seed + shift);
    for (int c = 0; c < S.components && c < 2; ++c) {
      const int64_t m = S.per_site[c];
      if (m == 0) continue;
      std::mt19937 own(S.random_seed[c] + shift);
      std::mt19937& gen = S.reseed[c] ? own : global;
      uint32_t* dst = out[c].data();
      for (int64_t hx = 0; hx < nlh[0]; ++hx) {
        const int64_t gx = cc[0] * nl[0] + hx - S.halo[0];
        const bool px = hx >= S.halo[0] && hx < S.halo[0] + nl[0];
        for (int64_t hy = 0; hy < nlh[1]; ++hy) {
          const int64_t gy = cc[1] * nl[1] + hy - S.halo[1];
          const bool py = px && hy >= S.halo[1] && hy < S.halo[1] + nl[1];
          for (int64_t hz = 0; hz < nlh[2]; ++hz) {
            const int64_t gz = cc[2] * nl[2] + hz - S.halo[2];
            const bool pz = py && hz >= S.halo[2] && hz < S.halo[2] + nl[2];
            const int64_t site = (gx * S.n[1] + gy) * S.n[2] + gz;
            for (int64_t q = 0; q < m; ++q) {
              const uint32_t u = uint32_t(gen());
              if (pz) dst[site * m + q] = u;
            }
          }
        }
      }
    }
  }
  return true;
}

}  // namespace lbk
