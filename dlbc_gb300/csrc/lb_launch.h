// Launchers for the timestep kernels, one translation unit per arithmetic
// form (lb_step_f64.cu is compiled without FMA contraction).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lb_kernels.cuh"

namespace lbk {

// Optional events recorded around each kernel (profiling): ev[0] before the
// first kernel, ev[1] between the kernels, ev[2] after the second.
struct StepEvents {
  cudaEvent_t ev[3];
};

// z sites per tile row of the pair step (lb_pairs.cuh): 32 lanes x 2
constexpr int kPairTZ = 64;

// storage of the float-arithmetic forms
constexpr int kStoreF32 = 0;  // float populations
constexpr int kStoreF16 = 1;  // half offsets (LBGPU_FP16)
constexpr int kStoreI16 = 2;  // 16-bit fixed-point offsets (LBGPU_I16)

// rows (y) of a pair-kernel tile for a storage kind: 14 for half offsets
// (one CTA of 16 warps per SM: 3.6 % faster at 512^3 than two of 10, which
// spill), 8 otherwise (two CTAs of 10 warps per SM)
constexpr int pair_ty(int kind) { return kind == kStoreF16 ? 14 : 8; }

struct StepBuffers {
  const void* f;        // populations in
  void* fout;           // populations out
  const uint8_t* mask;  // nullptr: no walls
  const uint32_t* nbmask = nullptr;  // neighbour masks (fused step; set iff mask is)
  const uint8_t* tile_walls = nullptr;  // per (x, 8x32 tile) wall flags (fused step)
  int zwall = 0;                        // the solid sites are exactly the planes z = 0 and nz - 1
  int* work_counter = nullptr;          // dynamic scheduling counter (fused step)
  void* rho;            // C*N (double for FP64, float otherwise)
  void* psi;            // C*N
  double* force;        // C*N*D when P.record_force
};

// Queue one timestep (two kernels) on `stream`.  Returns cudaSuccess or the
// launch error; *launches is incremented by the number of kernels queued.
cudaError_t launch_step_f64(int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t stream,
                            int64_t* launches, const StepEvents* ev);
cudaError_t launch_step_f32(int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t stream,
                            int64_t* launches, const StepEvents* ev);
cudaError_t launch_step_f16(int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t stream,
                            int64_t* launches, const StepEvents* ev);

// One kernel of the FP64 timestep over the x-planes whose sites are
// [P.s_begin, P.s_end): the step as a wavefront over plane ranges, for host
// transfers that overlap it.  A plane range of k_density_psi needs the
// populations of its planes and R planes either side (R = the largest |c_x|,
// periodic); one of k_collide needs those and the densities/psi of R planes
// either side.
constexpr int kPartDensityPsi = 1;
constexpr int kPartCollide = 2;
cudaError_t launch_part_f64(int part, int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t stream,
                            int64_t* launches);

// The timestep split at the reference's hook points (advection, then
// density/force/collision), for host code that runs hooks in between.
constexpr int kPhaseAdvect = 1;
constexpr int kPhaseCollide = 2;
cudaError_t launch_phase_f64(int phase, int q, int c, const StepBuffers& b, const StepParams& P,
                             cudaStream_t stream, int64_t* launches);
cudaError_t launch_phase_f32(int phase, int q, int c, const StepBuffers& b, const StepParams& P,
                             cudaStream_t stream, int64_t* launches);
cudaError_t launch_phase_f16(int phase, int q, int c, const StepBuffers& b, const StepParams& P,
                             cudaStream_t stream, int64_t* launches);

}  // namespace lbk

namespace lbk {

// Fused single-pass step for the float-arithmetic forms: D3Q19
// (lb_fused.cuh, lb_pairs.cuh; q = 19) or D2Q9 (lb_fused2d.cuh; q = 9);
// `kind` is the storage (kStoreF32 / kStoreF16 / kStoreI16; I16 runs on the
// D3Q19 pair kernel only).
cudaError_t launch_fused(int kind, int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t stream,
                         int64_t* launches, const StepEvents* ev, int device);
// whether launch_fused runs the pair kernel (lb_pairs.cuh) for this lattice
bool pairs_eligible(int kind, int c, const StepParams& P, const StepBuffers& b);
// the fused step over the planes [x0, x1) only (every tile), for the host
// transfers' wavefront; it reads the populations of planes x0 - 2 .. x1 + 1
cudaError_t launch_fused_range(int kind, int q, int c, const StepBuffers& b, const StepParams& P, int x0, int x1,
                               cudaStream_t stream, int64_t* launches, int device);

}  // namespace lbk

namespace lbk {

struct FusedParams;
struct FusedSim;
struct PairSim;

// float parameters of the fused kernel for tiles of height ty (4 or 8) and
// connectivity q (19, or 9 for the D2Q9 kernel)
FusedParams make_fused_params(const StepParams& P, int ty, int q = 19);

// One timestep of every simulation in `sims` (device array, two-component,
// D3Q19) in one persistent launch.  ctas_per_sm <= 0: as many as fit.
// counters (two ints, zero before the first launch): dynamic scheduling of
// total_units runs; nullptr: static equal ranges of total_work plane-tiles.
cudaError_t launch_fused_batch(int kind, int ty, bool walls, const FusedSim* sims, int nsims,
                               int64_t total_work, int parity, int ctas_per_sm, cudaStream_t stream, int device,
                               int64_t total_units, int* counters);
// The pair-kernel batch (lb_pairs.cuh): members with an even z extent, the
// BDist2 equilibrium and no solid site; counters as above (required).
cudaError_t launch_pairs_batch(int kind, const PairSim* sims, int nsims, int parity, int ctas_per_sm,
                               cudaStream_t stream, int device, int64_t total_units, int* counters);

}  // namespace lbk
