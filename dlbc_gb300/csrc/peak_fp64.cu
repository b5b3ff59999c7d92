// FP64 instruction-rate microbenchmark: the measured ceiling for the FP64
// form's collision kernel, which is limited by the FP64 pipe, not by HBM.
//
// Every thread runs kChains independent dependency chains of one FP64
// operation (DADD, DMUL or DFMA, written with the _rn intrinsics so the
// compiler neither contracts nor reassociates them) for `iters` iterations;
// a full grid of CTAs keeps every SM's FP64 pipe busy.  The kernel is timed
// with CUDA events on its own stream after a warm-up launch; the result is
// warp-level FP64 instructions per second x 32 (thread operations per
// second), the unit in which a kernel's FP64 instruction count divided by its
// duration is compared against it.  Nothing about the GPU is changed (no
// clock or power settings); the inputs come from the host so that no chain
// can be folded at compile time, and every chain's value is stored.
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

template <int OP>
__global__ void __launch_bounds__(kThreads) k_fp64_chain(double a, double b, int iters, double* __restrict__ out) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) x[k] = b + double(threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) {
      if (OP == 0) x[k] = __dadd_rn(x[k], a);
      if (OP == 1) x[k] = __dmul_rn(x[k], a);
      if (OP == 2) x[k] = __fma_rn(x[k], a, b);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s = __dadd_rn(s, x[k]);
  out[size_t(blockIdx.x) * blockDim.x + threadIdx.x] = s;
}

template <int OP>
int time_op(int blocks, int iters, double* out, cudaStream_t st, double a, double b, double* ops_per_s) {
  k_fp64_chain<OP><<<blocks, kThreads, 0, st>>>(a, b, iters / 8, out);  // warm-up
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return -1;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return -1;
  }
  cudaEventRecord(e0, st);
  k_fp64_chain<OP><<<blocks, kThreads, 0, st>>>(a, b, iters, out);
  cudaEventRecord(e1, st);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess || ms <= 0.f) return -1;
  *ops_per_s = double(blocks) * kThreads * double(iters) * kChains / (double(ms) * 1e-3);
  return 0;
}

}  // namespace

// rates[0..2]: DADD, DMUL, DFMA thread operations per second on `device`
// (a DFMA counted once).  Returns 0 on success, -1 on a CUDA error.
extern "C" int peak_fp64_rates(int device, int iters, double* rates) {
  if (!rates || iters < 8) return -1;
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess) return -1;
  if (cudaSetDevice(device) != cudaSuccess) return -1;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = (sms > 0 ? sms : 1) * 8;
  double* out = nullptr;
  cudaStream_t st = nullptr;
  int rc = -1;
  if (cudaMalloc(&out, size_t(blocks) * kThreads * sizeof(double)) == cudaSuccess &&
      cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess) {
    const double a = 1.0 + 1.0 / 1048576.0, b = 0.5;
    rc = 0;
    rc |= time_op<0>(blocks, iters, out, st, a, b, &rates[0]);
    rc |= time_op<1>(blocks, iters, out, st, a, b, &rates[1]);
    rc |= time_op<2>(blocks, iters, out, st, a, b, &rates[2]);
  }
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  cudaSetDevice(prev);
  return rc;
}
