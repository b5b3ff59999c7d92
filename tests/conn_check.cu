// Host dump of the kernels' connectivity tables (Conn<Q> and weight_of in
// lb_core.cuh): one line per population, "Q q cx cy cz bounce weight".
#include <cstdio>

#include "../dlbc_gb300/csrc/lb_core.cuh"

template <int Q>
void dump() {
  using C = lbk::Conn<Q>;
  for (int q = 0; q < Q; ++q)
    std::printf("%d %d %d %d %d %d %.17g %.17g\n", Q, q, C::cx(q), C::cy(q), C::cz(q), C::bounce(q),
                lbk::weight_of(Q, q), C::css());
}

int main() {
  dump<19>();
  dump<9>();
  dump<5>();
  dump<3>();
  return 0;
}
