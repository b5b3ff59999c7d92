// Host check of the fused kernels' run schedule (plan_runs, sched_units,
// sched_run in lb_fused.cuh): for many plane ranges, tile counts and grid
// sizes, the runs cover every plane of every tile exactly once, no run is
// longer than run_len, and the long runs come before the short ones.
// Prints "OK <cases>" or the first failing case.
#include <cstdio>
#include <vector>

#include "../dlbc_gb300/csrc/lb_fused.cuh"

int main() {
  using lbk::FusedParams;
  long cases = 0;
  const int nxs[] = {1, 2, 3, 5, 8, 16, 31, 64, 100, 128, 256, 511, 512, 1000};
  const int tiles_list[] = {1, 2, 7, 16, 64, 100, 1024};
  const int grids[] = {1, 3, 152, 304, 456, 608, 1216};
  for (int nx : nxs)
    for (int x0 = 0; x0 < nx; x0 += (nx > 8 ? nx / 3 + 1 : 1))
      for (int x1 = x0 + 1; x1 <= nx; x1 += (nx > 8 ? nx / 4 + 1 : 1))
        for (int tiles : tiles_list)
          for (int grid : grids) {
            FusedParams G{};
            G.nx = nx;
            G.x_begin = x0;
            G.x_end = x1;
            lbk::plan_runs(G, tiles, grid);
            const int units = lbk::sched_units(G, tiles);
            std::vector<int> seen(size_t(tiles) * nx, 0);
            int last_len = 1 << 30;
            bool ok = G.run_len >= 1 && G.tail_len >= 1 && G.x_split >= x0 && G.x_split <= x1;
            for (int i = 0; ok && i < units; ++i) {
              int tile, a, b;
              lbk::sched_run(G, tiles, i, tile, a, b);
              if (tile < 0 || tile >= tiles || a < x0 || b > x1 || b <= a || b - a > G.run_len) ok = false;
              if (ok && b - a > last_len && a < G.x_split) ok = false;  // bulk runs first
              for (int x = a; ok && x < b; ++x) seen[size_t(tile) * nx + x]++;
              if (a >= G.x_split) last_len = 0;  // the tail has started
            }
            for (int t = 0; ok && t < tiles; ++t)
              for (int x = 0; x < nx; ++x) {
                const int want = (x >= x0 && x < x1) ? 1 : 0;
                if (seen[size_t(t) * nx + x] != want) {
                  ok = false;
                  break;
                }
              }
            ++cases;
            if (!ok) {
              std::printf("FAIL nx=%d x=[%d,%d) tiles=%d grid=%d run_len=%d tail_len=%d x_split=%d\n", nx, x0, x1,
                          tiles, grid, G.run_len, G.tail_len, G.x_split);
              return 1;
            }
          }
  std::printf("OK %ld\n", cases);
  return 0;
}
