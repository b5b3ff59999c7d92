// The single-lattice fused D2Q9 step (lb_fused2d.cuh), float and half-offset
// storage.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lb_fused2d.cuh"
#include "lb_fused_launch.cuh"
#include "lb_launch.h"

namespace lbk {

namespace {

template <typename T, int C, bool W, bool MOM>
cudaError_t go2d(const StepBuffers& b, const FusedParams& F, cudaStream_t st, int device) {
  static KernelInfo info;
  auto kern = k_fused2d<T, C, W, MOM>;
  const int smem = int(sizeof(Fused2Shared<MOM ? 2 : 9>));
  int per_sm = 0;
  cudaError_t e = kernel_setup(kern, smem, kF2W, device, info, &per_sm);
  if (e != cudaSuccess) return e;
  int64_t grid = int64_t(per_sm) * sm_count(device);
  FusedParams G = F;
  G.tiles_y = 1;
  G.tiles_z = (G.ny + kF2W - 1) / kF2W;
  plan_runs(G, G.tiles_z, grid);
  const int64_t units = sched_units(G, G.tiles_z);
  if (grid > units) grid = units;
  kern<<<unsigned(grid), kF2W, smem, st>>>(static_cast<const T*>(b.f), static_cast<T*>(b.fout), b.nbmask, b.force,
                                            G);
  return cudaGetLastError();
}

template <typename T>
cudaError_t go2d_any(int c, bool w, bool mom, const StepBuffers& b, const FusedParams& F, cudaStream_t st,
                     int device) {
  if (mom) return w ? go2d<T, 2, true, true>(b, F, st, device) : go2d<T, 2, false, true>(b, F, st, device);
  if (c == 2) return w ? go2d<T, 2, true, false>(b, F, st, device) : go2d<T, 2, false, false>(b, F, st, device);
  return w ? go2d<T, 1, true, false>(b, F, st, device) : go2d<T, 1, false, false>(b, F, st, device);
}

}  // namespace

cudaError_t launch_fused2d(int kind, int c, bool walls, bool mom, const StepBuffers& b, const FusedParams& F,
                           cudaStream_t st, int device) {
  if (kind == kStoreF16) return go2d_any<__half>(c, walls, mom, b, F, st, device);
  if (kind == kStoreF32) return go2d_any<float>(c, walls, mom, b, F, st, device);
  return cudaErrorInvalidValue;
}

}  // namespace lbk
