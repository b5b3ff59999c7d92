// The single-lattice fused D2Q9 step (lb_fused2d.cuh), float and half-offset
// storage.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lb_fused2d.cuh"
#include "lb_fused_launch.cuh"
#include "lb_launch.h"
#include "lb_pairs2d.cuh"

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

template <typename T>
cudaError_t go_pairs2d(const StepBuffers& b, const FusedParams& F, cudaStream_t st, int device) {
  static KernelInfo info;
  auto kern = k_pairs2d<T>;
  int per_sm = 0;
  cudaError_t e = kernel_setup(kern, 0, kP2Threads, device, info, &per_sm);
  if (e != cudaSuccess) return e;
  int64_t grid = int64_t(per_sm) * sm_count(device);
  FusedParams G = F;
  G.tiles_y = 1;
  G.tiles_z = (G.ny + kF2W - 1) / kF2W;
  plan_runs(G, G.tiles_z, grid);
  const int64_t units = sched_units(G, G.tiles_z);
  if (grid > units) grid = units;
  kern<<<unsigned(grid), kP2Threads, 0, st>>>(static_cast<const T*>(b.f), static_cast<T*>(b.fout), b.force, G);
  return cudaGetLastError();
}

}  // namespace

bool pairs2d_eligible(int kind, int c, const StepParams& P, const StepBuffers& b) {
  // aligned two-site words need an even y extent; every tau = 1, BDist2,
  // two components, no solid site, the work counter.  FP16 only: measured
  // on GB300 at 4096^2 the pair kernel runs FP16 at 48 950 MLUPS against the
  // one-site kernel's 42 610, FP32 at 37 150 against 38 590.
  return kind == kStoreF16 && c == 2 && P.ny % 2 == 0 && P.unit_tau != 0 && P.eq_form == 2 &&
         b.mask == nullptr && b.work_counter != nullptr;
}

cudaError_t launch_pairs2d(int kind, const StepBuffers& b, const FusedParams& F, cudaStream_t st, int device) {
  if (kind == kStoreF16) return go_pairs2d<__half>(b, F, st, device);
  if (kind == kStoreF32) return go_pairs2d<float>(b, F, st, device);
  return cudaErrorInvalidValue;
}

cudaError_t launch_fused2d(int kind, int c, bool walls, bool mom, const StepBuffers& b, const FusedParams& F,
                           cudaStream_t st, int device) {
  if (kind == kStoreF16) return go2d_any<__half>(c, walls, mom, b, F, st, device);
  if (kind == kStoreF32) return go2d_any<float>(c, walls, mom, b, F, st, device);
  return cudaErrorInvalidValue;
}

}  // namespace lbk
