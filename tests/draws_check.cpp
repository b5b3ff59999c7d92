// Host harness for lb_draws.h: writes one component's reference draws as
// raw uint32 to a file.  Arguments: out nx ny nz hx hy hz ncx ncy ncz seed
// shift per_site0 per_site1 reseed0 reseed1 rseed0 rseed1 component
#include <stdio.h>
#include <stdlib.h>

#include "../dlbc_gb300/csrc/lb_draws.h"

int main(int argc, char** argv) {
  if (argc != 20) return 2;
  lbk::DrawSpec S;
  for (int i = 0; i < 3; ++i) {
    S.n[i] = atoll(argv[2 + i]);
    S.halo[i] = atoll(argv[5 + i]);
    S.nc[i] = atoll(argv[8 + i]);
  }
  S.seed = uint32_t(strtoll(argv[11], nullptr, 10));
  S.shift_seed_by_rank = atoi(argv[12]) != 0;
  for (int c = 0; c < 2; ++c) {
    S.per_site[c] = atoll(argv[13 + c]);
    S.reseed[c] = atoi(argv[15 + c]) != 0;
    S.random_seed[c] = uint32_t(strtoll(argv[17 + c], nullptr, 10));
  }
  std::vector<uint32_t> out[2];
  if (!lbk::reference_draws(S, out)) return 3;
  const int c = atoi(argv[19]);
  FILE* f = fopen(argv[1], "wb");
  if (!f) return 4;
  fwrite(out[c].data(), sizeof(uint32_t), out[c].size(), f);
  fclose(f);
  return 0;
}
