// Launcher of the fused single-pass step (lb_fused.cuh).
#include <cuda_runtime.h>

#include <mutex>

#include "lb_fused.cuh"
#include "lb_launch.h"

namespace lbk {

namespace {

FusedParams to_fused(const StepParams& P) {
  FusedParams F{};
  F.nx = P.nx;
  F.ny = P.ny;
  F.nz = P.nz;
  F.n = P.n;
  F.tiles_y = (P.ny + kFusedTY - 1) / kFusedTY;
  F.tiles_z = (P.nz + kFusedTZ - 1) / kFusedTZ;
  F.work = int64_t(F.tiles_y) * F.tiles_z * P.nx;
  F.shan_chen = P.shan_chen;
  F.psi_form = P.psi_form;
  F.eq_form = P.eq_form;
  F.record_force = P.record_force;
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
    for (int c = 0; c < 2; ++c) F.wrho[c][q] = weight<19, float>(q) * P.rho0[c];
  }
  return F;
}

template <typename T, int C, bool W>
cudaError_t go(const StepBuffers& b, const FusedParams& F, cudaStream_t st, int device) {
  auto kern = k_fused<T, C, W>;
  const int smem = int(sizeof(FusedShared));
  static std::mutex mu;
  static int configured[64] = {0};
  static int grid_for[64] = {0};
  int grid;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!configured[device & 63]) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (e != cudaSuccess) return e;
      int per_sm = 0, sms = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFusedThreads, smem);
      if (e != cudaSuccess) return e;
      e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
      if (e != cudaSuccess) return e;
      grid_for[device & 63] = (per_sm > 0 ? per_sm : 1) * sms;
      configured[device & 63] = 1;
    }
    grid = grid_for[device & 63];
  }
  if (int64_t(grid) > F.work) grid = int(F.work);
  kern<<<grid, kFusedThreads, smem, st>>>(static_cast<const T*>(b.f), static_cast<T*>(b.fout), b.mask, b.force, F);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_fused(bool half_storage, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                         int64_t* launches, const StepEvents* ev, int device) {
  const FusedParams F = to_fused(P);
  const bool w = b.mask != nullptr;
  if (ev) {
    cudaEventRecord(ev->ev[0], st);
    cudaEventRecord(ev->ev[1], st);
  }
  cudaError_t e;
  if (half_storage) {
    if (c == 2)
      e = w ? go<__half, 2, true>(b, F, st, device) : go<__half, 2, false>(b, F, st, device);
    else
      e = w ? go<__half, 1, true>(b, F, st, device) : go<__half, 1, false>(b, F, st, device);
  } else {
    if (c == 2)
      e = w ? go<float, 2, true>(b, F, st, device) : go<float, 2, false>(b, F, st, device);
    else
      e = w ? go<float, 1, true>(b, F, st, device) : go<float, 1, false>(b, F, st, device);
  }
  if (ev) cudaEventRecord(ev->ev[2], st);
  *launches += 1;
  return e;
}

}  // namespace lbk
