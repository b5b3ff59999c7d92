// The batched fused step: many lattices in one persistent launch.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lb_fused.cuh"
#include "lb_fused_launch.cuh"
#include "lb_launch.h"
#include "lb_pairs.cuh"

namespace lbk {

namespace {

template <typename T, bool W, int TY>
cudaError_t go_batch(const FusedSim* sims, int nsims, int64_t total, int parity, int ctas_per_sm, cudaStream_t st,
                     int device, int64_t total_units, int* counters) {
  static KernelInfo info;
  auto kern = k_fused_batch<T, 2, W, TY>;
  const int smem = int(sizeof(FusedShared<TY, fused_np<T, false>()>));
  int per_sm = 0;
  cudaError_t e = kernel_setup(kern, smem, TY * kFusedTZ, device, info, &per_sm);
  if (e != cudaSuccess) return e;
  if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
  int64_t grid = int64_t(per_sm) * sm_count(device);
  if (grid > total) grid = total;
  if (grid < 1) return cudaSuccess;
  kern<<<unsigned(grid), TY * kFusedTZ, smem, st>>>(sims, nsims, total, parity, total_units, counters);
  return cudaGetLastError();
}

template <typename T>
cudaError_t go_pairs_batch(const PairSim* sims, int nsims, int parity, int ctas_per_sm, cudaStream_t st, int device,
                           int64_t total_units, int* counters) {
  static KernelInfo info;
  auto kern = k_pairs_batch<T>;
  // (FP32 and FP16 members all have tau = 1: the smaller layout)
  const int smem = int(sizeof(PairShared<2, !pairs_general<T>(), T>));
  int per_sm = 0;
  cudaError_t e = kernel_setup(kern, smem, pair_threads<T>(), device, info, &per_sm);
  if (e != cudaSuccess) return e;
  if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
  int64_t grid = int64_t(per_sm) * sm_count(device);
  if (grid > total_units) grid = total_units;
  if (grid < 1) return cudaSuccess;
  kern<<<unsigned(grid), pair_threads<T>(), smem, st>>>(sims, nsims, parity, total_units, counters);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_pairs_batch(int kind, const PairSim* sims, int nsims, int parity, int ctas_per_sm,
                               cudaStream_t st, int device, int64_t total_units, int* counters) {
#define LB_PBATCH(T) go_pairs_batch<T>(sims, nsims, parity, ctas_per_sm, st, device, total_units, counters)
  if (kind == kStoreF16) return LB_PBATCH(__half);
  if (kind == kStoreI16) return LB_PBATCH(int16_t);
  return LB_PBATCH(float);
#undef LB_PBATCH
}

cudaError_t launch_fused_batch(int kind, int ty, bool walls, const FusedSim* sims, int nsims,
                               int64_t total_work, int parity, int ctas_per_sm, cudaStream_t st, int device,
                               int64_t total_units, int* counters) {
#define LB_BATCH(T, W, TYV) \
  go_batch<T, W, TYV>(sims, nsims, total_work, parity, ctas_per_sm, st, device, total_units, counters)
  if (kind == kStoreF16) {
    if (ty == 4) return walls ? LB_BATCH(__half, true, 4) : LB_BATCH(__half, false, 4);
    return walls ? LB_BATCH(__half, true, 8) : LB_BATCH(__half, false, 8);
  }
  if (kind == kStoreI16) {
    // I16 members here have solid sites (the rest run the pair batch)
    if (!walls) return cudaErrorInvalidValue;
    if (ty == 4) return LB_BATCH(int16_t, true, 4);
    return LB_BATCH(int16_t, true, 8);
  }
  if (ty == 4) return walls ? LB_BATCH(float, true, 4) : LB_BATCH(float, false, 4);
  return walls ? LB_BATCH(float, true, 8) : LB_BATCH(float, false, 8);
#undef LB_BATCH
}

}  // namespace lbk
