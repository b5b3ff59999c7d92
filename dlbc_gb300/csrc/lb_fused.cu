// The fused single-pass step (lb_fused.cuh): parameters, the single-lattice
// dispatch (kernels in lb_fused_f32.cu / lb_fused_f16.cu) and the opt-in
// variants (cp.async staging, thread-block clusters).
#include <cuda_runtime.h>

#include <stdlib.h>

#include <mutex>

#include "lb_fused.cuh"
#include "lb_fused_launch.cuh"
#include "lb_launch.h"
#include "lb_staged.cuh"

namespace lbk {

FusedParams make_fused_params(const StepParams& P, int ty) {
  FusedParams F{};
  F.nx = P.nx;
  F.ny = P.ny;
  F.nz = P.nz;
  F.n = P.n;
  F.tiles_y = (P.ny + ty - 1) / ty;
  F.tiles_z = (P.nz + kFusedTZ - 1) / kFusedTZ;
  F.work = int64_t(F.tiles_y) * F.tiles_z * P.nx;
  F.shan_chen = P.shan_chen;
  F.psi_form = P.psi_form;
  F.eq_form = P.eq_form;
  F.record_force = P.record_force;
  F.unit_tau = P.unit_tau;
  F.tile_walls = nullptr;
  F.work_counter = nullptr;
  F.run_len = P.nx;
  for (int c = 0; c < 2; ++c) {
    F.tau[c] = float(P.tau[c]);
    F.inv_tau[c] = float(1.0 / P.tau[c]);
    F.omega[c] = float(P.omega[c]);
    F.one_minus_omega[c] = float(P.one_minus_omega[c]);
    F.gwc[c] = float(P.gwc[c]);
    for (int c2 = 0; c2 < 2; ++c2) F.gcc[c][c2] = float(P.gcc[c][c2]);
    F.rho0[c] = P.rho0[c];
    F.scale[c] = P.scale[c];
    F.inv_scale[c] = P.inv_scale[c];
  }
  for (int i = 0; i < 3; ++i) F.acc[i] = float(P.acc[i]);
  for (int q = 0; q < 19; ++q) {
    F.qn[q] = uint32_t(int64_t(q) * P.n);
    for (int c = 0; c < 2; ++c) {
      // one value per weight class (q = 0, 1..6, 7..18)
      const int k = Conn<19>::wclass(q);
      F.wrho[c][k] = weight<19, float>(q) * P.rho0[c];
      F.wscale[c][k] = weight<19, float>(q) * P.scale[c];
      F.inv_wscale[c][k] = 1.0f / F.wscale[c][k];
      F.hoff[c][k] = -F.wrho[c][k] * F.inv_wscale[c][k];
    }
  }
  return F;
}


namespace {

template <int C, bool W>
cudaError_t go_staged(const StepBuffers& b, const FusedParams& F, cudaStream_t st, int device) {
  static KernelInfo info;
  auto kern = k_staged<C, W, 8>;
  const int smem = int(sizeof(StagedShared<8>));
  int per_sm = 0;
  cudaError_t e = kernel_setup(kern, smem, 8 * kFusedTZ, device, info, &per_sm);
  if (e != cudaSuccess) return e;
  // (tile, x-chunk) units: as many chunks per tile as keep every CTA slot
  // busy in lockstep
  const int64_t slots = int64_t(per_sm) * sm_count(device);
  const int64_t tiles = int64_t(F.tiles_y) * F.tiles_z;
  int chunks = tiles >= slots ? 1 : int(slots / tiles);
  if (chunks > F.nx) chunks = F.nx;
  const int64_t units = tiles * chunks;
  const int64_t grid = units < slots ? units : slots;
  kern<<<unsigned(grid), 8 * kFusedTZ, smem, st>>>(static_cast<const __half*>(b.f), static_cast<__half*>(b.fout),
                                                   b.nbmask, b.force, F, chunks);
  return cudaGetLastError();
}

template <typename T, int C, bool W>
cudaError_t go_cluster(const StepBuffers& b, const FusedParams& F, cudaStream_t st, int device) {
  static KernelInfo info;
  auto kern = k_fused_cluster<T, C, W>;
  const int smem = int(sizeof(FusedShared<8>));
  int per_sm = 0;
  cudaError_t e = kernel_setup(kern, smem, 8 * kFusedTZ, device, info, &per_sm);
  if (e != cudaSuccess) return e;
  static int max_clusters[64] = {0};
  if (!max_clusters[device & 63]) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(4 * 64, 1, 1);
    cfg.blockDim = dim3(8 * kFusedTZ, 1, 1);
    cfg.dynamicSmemBytes = size_t(smem);
    int n = 0;
    e = cudaOccupancyMaxActiveClusters(&n, kern, &cfg);
    if (e != cudaSuccess) return e;
    max_clusters[device & 63] = n > 0 ? n : 1;
  }
  const int clusters = max_clusters[device & 63];
  FusedParams G = F;
  const int64_t ctiles = int64_t(G.tiles_y / 2) * (G.tiles_z / 2);
  int rl = 32;
  while (rl > 4 && ctiles * ((G.nx + rl - 1) / rl) < 2 * clusters) rl /= 2;
  G.run_len = rl < G.nx ? rl : G.nx;
  const int64_t units = ctiles * ((G.nx + G.run_len - 1) / G.run_len);
  const int64_t grid = 4 * (units < clusters ? units : clusters);
  kern<<<unsigned(grid), 8 * kFusedTZ, smem, st>>>(static_cast<const T*>(b.f), static_cast<T*>(b.fout), b.nbmask,
                                                   b.force, G, b.work_counter);
  return cudaGetLastError();
}

}  // namespace

bool staged_eligible(const StepParams& P, int c, bool half_storage) {
  return half_storage && (c == 1 || c == 2) && P.nz % kStagedZH == 0 && P.nz >= kStagedZH &&
         19 * P.n < (int64_t(1) << 32);
}

cudaError_t launch_fused(bool half_storage, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                         int64_t* launches, const StepEvents* ev, int device, bool staged) {
  FusedParams F = make_fused_params(P, 8);
  F.tile_walls = b.tile_walls;
  if (b.work_counter && !(staged && staged_eligible(P, c, half_storage))) {
    // dynamic runs (length chosen at launch)
    F.work_counter = b.work_counter;
    F.run_len = 32;
    cudaMemsetAsync(b.work_counter, 0, sizeof(int), st);
  }
  const bool w = b.mask != nullptr;
  if (w && !b.nbmask) return cudaErrorInvalidValue;  // walls need the neighbour masks
  if (ev) {
    cudaEventRecord(ev->ev[0], st);
    cudaEventRecord(ev->ev[1], st);
  }
  cudaError_t e;
  // LBGPU_CLUSTER=1: 2 x 2 clusters of tiles where the lattice is a whole
  // number of 16 x 64 cluster tiles (bit-identical, slower on GB300: the
  // per-plane cluster barrier costs more than the halved ring saves)
  static const bool kCluster = [] {
    const char* s = getenv("LBGPU_CLUSTER");
    return s && s[0] == '1';
  }();
  const bool cluster = kCluster && F.work_counter && c == 2 && P.ny % 16 == 0 && P.nz % 64 == 0 &&
                       !(staged && staged_eligible(P, c, half_storage));
  const bool mom = c == 2 && P.unit_tau && P.eq_form == 2;
  if (cluster) {
    if (half_storage)
      e = w ? go_cluster<__half, 2, true>(b, F, st, device) : go_cluster<__half, 2, false>(b, F, st, device);
    else
      e = w ? go_cluster<float, 2, true>(b, F, st, device) : go_cluster<float, 2, false>(b, F, st, device);
  } else if (staged && staged_eligible(P, c, half_storage)) {
    if (c == 2)
      e = w ? go_staged<2, true>(b, F, st, device) : go_staged<2, false>(b, F, st, device);
    else
      e = w ? go_staged<1, true>(b, F, st, device) : go_staged<1, false>(b, F, st, device);
  } else if (half_storage) {
    e = launch_fused_single_f16(c, w, mom, b, F, st, device);
  } else {
    e = launch_fused_single_f32(c, w, mom, b, F, st, device);
  }
  if (ev) cudaEventRecord(ev->ev[2], st);
  *launches += 1;
  return e;
}

}  // namespace lbk
