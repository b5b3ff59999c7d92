// Launch helpers shared by the fused-step translation units (lb_fused*.cu).
#pragma once

#include <cuda_runtime.h>

#include <mutex>

namespace lbk {

// per (kernel, device): shared-memory opt-in done and resident CTAs per SM
struct KernelInfo {
  std::mutex mu;
  int per_sm[64] = {0};
};

template <typename K>
inline cudaError_t kernel_setup(K kern, int smem, int threads, int device, KernelInfo& info, int* per_sm) {
  std::lock_guard<std::mutex> lock(info.mu);
  if (!info.per_sm[device & 63]) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, threads, smem);
    if (e != cudaSuccess) return e;
    info.per_sm[device & 63] = n > 0 ? n : 1;
  }
  *per_sm = info.per_sm[device & 63];
  return cudaSuccess;
}

inline int sm_count(int device) {
  static int cache[64] = {0};
  if (!cache[device & 63]) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cache[device & 63] = sms > 0 ? sms : 1;
  }
  return cache[device & 63];
}

// The single-lattice fused step for one storage type (lb_fused_f32.cu,
// lb_fused_f16.cu): C components, walls or not, the populations-free
// collision (mom) or not.
struct StepBuffers;
struct FusedParams;
cudaError_t launch_fused_single_f32(int c, bool walls, bool mom, const StepBuffers& b, const FusedParams& F,
                                    cudaStream_t st, int device);
cudaError_t launch_fused_single_f16(int c, bool walls, bool mom, const StepBuffers& b, const FusedParams& F,
                                    cudaStream_t st, int device);
cudaError_t launch_fused_single_i16(int c, bool walls, bool mom, const StepBuffers& b, const FusedParams& F,
                                    cudaStream_t st, int device);
// The single-lattice pair step (lb_pairs.cuh), lattices without solid
// sites: F holds the pair tiling (pair_ty x 64); mom: every tau = 1 (the gathered
// populations are not kept).
cudaError_t launch_pairs_single_f32(int c, bool mom, const StepBuffers& b, const FusedParams& F, cudaStream_t st,
                                    int device);
cudaError_t launch_pairs_single_f16(int c, bool mom, const StepBuffers& b, const FusedParams& F, cudaStream_t st,
                                    int device);
cudaError_t launch_pairs_single_i16(int c, bool mom, const StepBuffers& b, const FusedParams& F, cudaStream_t st,
                                    int device);
// The single-lattice D2Q9 step (lb_fused2d.cuh), F from make_fused_params
// with q = 9; kind kStoreF32 or kStoreF16.
cudaError_t launch_fused2d(int kind, int c, bool walls, bool mom, const StepBuffers& b, const FusedParams& F,
                           cudaStream_t st, int device);
// The D2Q9 pair step (lb_pairs2d.cuh) and the lattices it runs: FP32/FP16,
// two components, every tau = 1, BDist2, even ny, no solid site.
bool pairs2d_eligible(int kind, int c, const StepParams& P, const StepBuffers& b);
cudaError_t launch_pairs2d(int kind, const StepBuffers& b, const FusedParams& F, cudaStream_t st, int device);

}  // namespace lbk
