// FP64 timestep: IEEE double, compiled with -fmad=false so that every
// product and sum is rounded as in the reference's x86-64 builds.
#include "lb_step_dispatch.cuh"

namespace lbk {
cudaError_t launch_step_f64(int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                            int64_t* launches, const StepEvents* ev) {
  return dispatch_step<double, double>(q, c, b, P, st, launches, ev);
}
cudaError_t launch_part_f64(int part, int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                            int64_t* launches) {
  return dispatch_part<double, double>(part, q, c, b, P, st, launches);
}
cudaError_t launch_phase_f64(int phase, int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                             int64_t* launches) {
  return dispatch_phase<double, double>(phase, q, c, b, P, st, launches);
}
}  // namespace lbk
