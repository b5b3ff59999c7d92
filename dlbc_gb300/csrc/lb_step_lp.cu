// Reduced-precision timestep forms: float storage + float arithmetic, and
// half storage of the offsets f_q - w_q*rho0 (scaled) + float arithmetic.
#include "lb_step_dispatch.cuh"

namespace lbk {
cudaError_t launch_step_f32(int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                            int64_t* launches, const StepEvents* ev) {
  return dispatch_step<float, float>(q, c, b, P, st, launches, ev);
}
cudaError_t launch_step_f16(int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                            int64_t* launches, const StepEvents* ev) {
  return dispatch_step<__half, float>(q, c, b, P, st, launches, ev);
}
cudaError_t launch_phase_f32(int phase, int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                             int64_t* launches) {
  return dispatch_phase<float, float>(phase, q, c, b, P, st, launches);
}
cudaError_t launch_phase_f16(int phase, int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                             int64_t* launches) {
  return dispatch_phase<__half, float>(phase, q, c, b, P, st, launches);
}
}  // namespace lbk
