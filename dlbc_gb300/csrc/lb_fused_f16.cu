// The single-lattice fused step with half-offset populations, and the pair
// step with half or 16-bit fixed-point offsets.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lb_fused.cuh"
#include "lb_fused_launch.cuh"
#include "lb_launch.h"
#include "lb_pairs.cuh"

namespace lbk {

namespace {

template <typename T, int C, bool W, int TY, bool MOM = false>
cudaError_t go_single(const StepBuffers& b, const FusedParams& F, cudaStream_t st, int device) {
  static KernelInfo info;
  auto kern = k_fused<T, C, W, TY, MOM>;
  const int smem = int(sizeof(FusedShared<TY, fused_np<T, MOM>()>));
  int per_sm = 0;
  cudaError_t e = kernel_setup(kern, smem, TY * kFusedTZ, device, info, &per_sm);
  if (e != cudaSuccess) return e;
  int64_t grid = int64_t(per_sm) * sm_count(device);
  FusedParams G = F;
  if (G.work_counter) {
    const int64_t tiles = int64_t(G.tiles_y) * G.tiles_z;
    plan_runs(G, tiles, grid);
    const int64_t units = sched_units(G, int(tiles));
    if (grid > units) grid = units;
  }
  if (grid > G.work) grid = G.work;
  kern<<<unsigned(grid), TY * kFusedTZ, smem, st>>>(static_cast<const T*>(b.f), static_cast<T*>(b.fout), b.nbmask,
                                                    b.force, G);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_fused_single_f16(int c, bool w, bool mom, const StepBuffers& b, const FusedParams& F, cudaStream_t st,
                   int device) {
  if (mom)
    return w ? go_single<__half, 2, true, 8, true>(b, F, st, device) : go_single<__half, 2, false, 8, true>(b, F, st, device);
  if (c == 2) return w ? go_single<__half, 2, true, 8>(b, F, st, device) : go_single<__half, 2, false, 8>(b, F, st, device);
  return w ? go_single<__half, 1, true, 8>(b, F, st, device) : go_single<__half, 1, false, 8>(b, F, st, device);
}

// I16 lattices with solid sites (the pair kernel's walled rows are slower)
cudaError_t launch_fused_single_i16(int c, bool w, bool mom, const StepBuffers& b, const FusedParams& F,
                                   cudaStream_t st, int device) {
  if (mom)
    return w ? go_single<int16_t, 2, true, 8, true>(b, F, st, device)
             : go_single<int16_t, 2, false, 8, true>(b, F, st, device);
  if (c == 2)
    return w ? go_single<int16_t, 2, true, 8>(b, F, st, device) : go_single<int16_t, 2, false, 8>(b, F, st, device);
  return w ? go_single<int16_t, 1, true, 8>(b, F, st, device) : go_single<int16_t, 1, false, 8>(b, F, st, device);
}

cudaError_t launch_pairs_single_f16(int c, bool mom, const StepBuffers& b, const FusedParams& F, cudaStream_t st,
                                    int device) {
  return launch_pairs<__half>(c, mom, b, F, st, device);
}

cudaError_t launch_pairs_single_i16(int c, bool mom, const StepBuffers& b, const FusedParams& F, cudaStream_t st,
                                    int device) {
  return launch_pairs<int16_t>(c, mom, b, F, st, device);
}

}  // namespace lbk
