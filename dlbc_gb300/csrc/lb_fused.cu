// The fused single-pass step (lb_fused.cuh): parameters and the single-lattice
// dispatch (kernels in lb_fused_f32.cu / lb_fused_f16.cu).
#include <cuda_runtime.h>

#include "lb_fused.cuh"
#include "lb_fused_launch.cuh"
#include "lb_launch.h"

namespace lbk {

FusedParams make_fused_params(const StepParams& P, int ty, int q) {
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
  F.x_begin = 0;
  F.x_end = P.nx;
  F.x_split = P.nx;
  F.tail_len = 1;
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
  for (int i = 0; i < 19; ++i) F.qn[i] = i < q ? uint32_t(int64_t(i) * P.n) : 0u;
  for (int i = 0; i < q; ++i) {
    for (int c = 0; c < 2; ++c) {
      // one value per weight class (rest, axis, diagonal)
      const int k = q == 9 ? Conn<9>::wclass(i) : Conn<19>::wclass(i);
      const float w = q == 9 ? weight<9, float>(i) : weight<19, float>(i);
      F.wrho[c][k] = w * P.rho0[c];
      F.wscale[c][k] = w * P.scale[c];
      F.inv_wscale[c][k] = 1.0f / F.wscale[c][k];
      F.hoff[c][k] = -F.wrho[c][k] * F.inv_wscale[c][k];
    }
  }
  return F;
}


// solid sites the pair kernel handles: none, or (FP16) exactly the planes
// z = 0 and z = nz - 1 of a two-component lattice whose z extent is a
// multiple of the tile width, with no wall force and every tau = 1 (the
// edge lanes of the first and last z-tile take the bounce-back and the
// wall's psi).  Measured on the 256x128x128 droplet channel: FP16 12 530 ->
// 13 660 MLUPS; FP32 and I16 walled lattices stay on the one-site kernel.
bool pairs_walls_ok(int kind, int c, const StepParams& P, const StepBuffers& b) {
  if (b.mask == nullptr) return true;
  return kind == kStoreF16 && b.zwall != 0 && c == 2 && P.nz % kPairTZ == 0 && P.gwc[0] == 0.0 &&
         P.gwc[1] == 0.0 && P.unit_tau != 0;
}

bool pairs_eligible(int kind, int c, const StepParams& P, const StepBuffers& b) {
  // aligned two-site words need an even z extent; the pair kernel computes
  // the BDist2 equilibrium and schedules through the work counter
  if (!(P.nz % 2 == 0 && P.eq_form == 2 && b.work_counter != nullptr)) return false;
  // where it is the faster kernel (measured on GB300): no solid site (FP16:
  // or planar z-walls), and every tau = 1 or the I16 storage (general
  // walls, and for FP32/FP16 the relaxation's shared-memory populations,
  // favour one site per thread)
  return pairs_walls_ok(kind, c, P, b) && (kind == kStoreI16 || P.unit_tau != 0);
}

// the fused step over planes [x0, x1) of every tile (the host transfers
// wavefront; the pair kernel or the one-site-per-thread kernel, whichever
// launch_fused would run): reads the populations of planes x0 - 2 .. x1 + 1
// (periodic)
cudaError_t launch_fused_range(int kind, int q, int c, const StepBuffers& b, const StepParams& P, int x0, int x1,
                               cudaStream_t st, int64_t* launches, int device) {
  if (x1 <= x0) return cudaSuccess;
  if (!b.work_counter) return cudaErrorInvalidValue;
  FusedParams G = make_fused_params(P, 8, q);
  G.tile_walls = b.tile_walls;
  G.work_counter = b.work_counter;
  G.x_begin = x0;
  G.x_end = x1;
  cudaMemsetAsync(b.work_counter, 0, sizeof(int), st);
  const bool w = b.mask != nullptr;
  if (w && !b.nbmask) return cudaErrorInvalidValue;
  *launches += 1;
  if (q == 9)
    return pairs2d_eligible(kind, c, P, b) ? launch_pairs2d(kind, b, G, st, device)
                                           : launch_fused2d(kind, c, w, c == 2 && P.unit_tau && P.eq_form == 2, b, G,
                                                            st, device);
  if (pairs_eligible(kind, c, P, b)) {
    G.zwall = b.mask != nullptr;
    G.tiles_y = (P.ny + pair_ty(kind) - 1) / pair_ty(kind);
    G.tiles_z = (P.nz + kPairTZ - 1) / kPairTZ;
    G.work = int64_t(G.tiles_y) * G.tiles_z * P.nx;
    const bool mom = P.unit_tau != 0;
    return kind == kStoreF16   ? launch_pairs_single_f16(c, mom, b, G, st, device)
           : kind == kStoreI16 ? launch_pairs_single_i16(c, mom, b, G, st, device)
                               : launch_pairs_single_f32(c, mom, b, G, st, device);
  }
  const bool mom = c == 2 && P.unit_tau && P.eq_form == 2;
  return kind == kStoreF16   ? launch_fused_single_f16(c, w, mom, b, G, st, device)
         : kind == kStoreI16 ? launch_fused_single_i16(c, w, mom, b, G, st, device)
                             : launch_fused_single_f32(c, w, mom, b, G, st, device);
}

cudaError_t launch_fused(int kind, int q, int c, const StepBuffers& b, const StepParams& P, cudaStream_t st,
                         int64_t* launches, const StepEvents* ev, int device) {
  FusedParams F = make_fused_params(P, 8, q);
  F.tile_walls = b.tile_walls;
  if (b.work_counter) {
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
  if (q == 9) {
    e = pairs2d_eligible(kind, c, P, b)
            ? launch_pairs2d(kind, b, F, st, device)
            : launch_fused2d(kind, c, w, c == 2 && P.unit_tau && P.eq_form == 2, b, F, st, device);
  } else if (pairs_eligible(kind, c, P, b)) {
    // two z-adjacent sites per thread (lb_pairs.cuh): pair_ty x 64 tiles
    FusedParams G = F;
    G.zwall = b.mask != nullptr;
    G.tiles_y = (P.ny + pair_ty(kind) - 1) / pair_ty(kind);
    G.tiles_z = (P.nz + kPairTZ - 1) / kPairTZ;
    G.work = int64_t(G.tiles_y) * G.tiles_z * P.nx;
    const bool mom = P.unit_tau != 0;
    e = kind == kStoreF16   ? launch_pairs_single_f16(c, mom, b, G, st, device)
        : kind == kStoreI16 ? launch_pairs_single_i16(c, mom, b, G, st, device)
                            : launch_pairs_single_f32(c, mom, b, G, st, device);
  } else {
    const bool mom = c == 2 && P.unit_tau && P.eq_form == 2;
    e = kind == kStoreF16   ? launch_fused_single_f16(c, w, mom, b, F, st, device)
        : kind == kStoreI16 ? launch_fused_single_i16(c, w, mom, b, F, st, device)
                            : launch_fused_single_f32(c, w, mom, b, F, st, device);
  }
  if (ev) cudaEventRecord(ev->ev[2], st);
  *launches += 1;
  return e;
}

}  // namespace lbk
