// Template dispatch shared by the per-form launch units.
#pragma once

#include "lb_launch.h"

namespace lbk {

constexpr int kStepThreads = 128;

// (NBM: the solid tests read the neighbour masks b.nbmask)
template <typename T, typename R, int Q, int C, bool W, bool NBM = false>
cudaError_t launch_step_t(const StepBuffers& b, const StepParams& P, cudaStream_t st, int64_t* launches,
                          const StepEvents* ev) {
  const unsigned blocks = unsigned((P.n + kStepThreads - 1) / kStepThreads);
  if (ev) cudaEventRecord(ev->ev[0], st);
  k_density_psi<T, R, Q, C, W, true, NBM><<<blocks, kStepThreads, 0, st>>>(
      static_cast<const T*>(b.f), b.mask, b.nbmask, static_cast<R*>(b.rho), static_cast<R*>(b.psi), P);
  if (ev) cudaEventRecord(ev->ev[1], st);
  k_collide<T, R, Q, C, W, true, NBM><<<blocks, kStepThreads, 0, st>>>(
      static_cast<const T*>(b.f), static_cast<T*>(b.fout), b.mask, b.nbmask, static_cast<const R*>(b.rho),
      static_cast<const R*>(b.psi), b.force, P);
  if (ev) cudaEventRecord(ev->ev[2], st);
  *launches += 2;
  return cudaGetLastError();
}

template <typename T, typename R>
cudaError_t dispatch_step(int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                          int64_t* launches, const StepEvents* ev) {
  const bool w = b.mask != nullptr;
  const bool nbm = w && b.nbmask != nullptr;
#define LB_CASE(QQ, CC)                                                               \
  if (q == QQ && c == CC)                                                             \
    return nbm ? launch_step_t<T, R, QQ, CC, true, true>(b, P, st, launches, ev)      \
           : w ? launch_step_t<T, R, QQ, CC, true>(b, P, st, launches, ev)            \
               : launch_step_t<T, R, QQ, CC, false>(b, P, st, launches, ev);
  LB_CASE(19, 2)
  LB_CASE(19, 1)
  LB_CASE(9, 2)
  LB_CASE(9, 1)
  LB_CASE(3, 2)
  LB_CASE(3, 1)
  LB_CASE(5, 2)
  LB_CASE(5, 1)
#undef LB_CASE
  return cudaErrorInvalidValue;
}

// One kernel of the timestep over the sites [P.s_begin, P.s_end) (whole
// x-planes): part kPartDensityPsi queues k_density_psi, kPartCollide
// k_collide.  The per-site arithmetic is that of launch_step_t.
template <typename T, typename R, int Q, int C, bool W, bool NBM = false>
cudaError_t launch_part_t(int part, const StepBuffers& b, const StepParams& P, cudaStream_t st, int64_t* launches) {
  const int64_t count = P.s_end - P.s_begin;
  if (P.s_end <= 0 || count <= 0 || P.s_begin < 0 || P.s_end > P.n) return cudaErrorInvalidValue;
  const unsigned blocks = unsigned((count + kStepThreads - 1) / kStepThreads);
  if (part == kPartDensityPsi)
    k_density_psi<T, R, Q, C, W, true, NBM><<<blocks, kStepThreads, 0, st>>>(
        static_cast<const T*>(b.f), b.mask, b.nbmask, static_cast<R*>(b.rho), static_cast<R*>(b.psi), P);
  else if (part == kPartCollide)
    k_collide<T, R, Q, C, W, true, NBM><<<blocks, kStepThreads, 0, st>>>(
        static_cast<const T*>(b.f), static_cast<T*>(b.fout), b.mask, b.nbmask, static_cast<const R*>(b.rho),
        static_cast<const R*>(b.psi), b.force, P);
  else
    return cudaErrorInvalidValue;
  *launches += 1;
  return cudaGetLastError();
}

template <typename T, typename R>
cudaError_t dispatch_part(int part, int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                          int64_t* launches) {
  const bool w = b.mask != nullptr;
  const bool nbm = w && b.nbmask != nullptr;
#define LB_CASE(QQ, CC)                                                           \
  if (q == QQ && c == CC)                                                         \
    return nbm ? launch_part_t<T, R, QQ, CC, true, true>(part, b, P, st, launches) \
           : w ? launch_part_t<T, R, QQ, CC, true>(part, b, P, st, launches)       \
               : launch_part_t<T, R, QQ, CC, false>(part, b, P, st, launches);
  LB_CASE(19, 2)
  LB_CASE(19, 1)
  LB_CASE(9, 2)
  LB_CASE(9, 1)
  LB_CASE(3, 2)
  LB_CASE(3, 1)
  LB_CASE(5, 2)
  LB_CASE(5, 1)
#undef LB_CASE
  return cudaErrorInvalidValue;
}

// One phase of the split timestep: kPhaseAdvect queues k_advect (f -> fout),
// kPhaseCollide the two kernels without streaming (f is already advected).
template <typename T, typename R, int Q, int C, bool W>
cudaError_t launch_phase_t(int phase, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                           int64_t* launches) {
  const unsigned blocks = unsigned((P.n + kStepThreads - 1) / kStepThreads);
  if (phase == kPhaseAdvect) {
    k_advect<T, Q, C, W><<<blocks, kStepThreads, 0, st>>>(static_cast<const T*>(b.f), static_cast<T*>(b.fout),
                                                          b.mask, P);
    *launches += 1;
  } else {
    k_density_psi<T, R, Q, C, W, false><<<blocks, kStepThreads, 0, st>>>(
        static_cast<const T*>(b.f), b.mask, nullptr, static_cast<R*>(b.rho), static_cast<R*>(b.psi), P);
    k_collide<T, R, Q, C, W, false><<<blocks, kStepThreads, 0, st>>>(
        static_cast<const T*>(b.f), static_cast<T*>(b.fout), b.mask, nullptr, static_cast<const R*>(b.rho),
        static_cast<const R*>(b.psi), b.force, P);
    *launches += 2;
  }
  return cudaGetLastError();
}

template <typename T, typename R>
cudaError_t dispatch_phase(int phase, int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                           int64_t* launches) {
  if (phase != kPhaseAdvect && phase != kPhaseCollide) return cudaErrorInvalidValue;
  const bool w = b.mask != nullptr;
#define LB_CASE(QQ, CC)                                                      \
  if (q == QQ && c == CC)                                                    \
    return w ? launch_phase_t<T, R, QQ, CC, true>(phase, b, P, st, launches) \
             : launch_phase_t<T, R, QQ, CC, false>(phase, b, P, st, launches);
  LB_CASE(19, 2)
  LB_CASE(19, 1)
  LB_CASE(9, 2)
  LB_CASE(9, 1)
  LB_CASE(3, 2)
  LB_CASE(3, 1)
  LB_CASE(5, 2)
  LB_CASE(5, 1)
#undef LB_CASE
  return cudaErrorInvalidValue;
}

}  // namespace lbk
