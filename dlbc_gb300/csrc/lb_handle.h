// Internal definition of the lattice handle behind include/lbgpu.h, shared
// by the single-lattice entry points (lb_api.cu) and batches (lb_batch.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/lbgpu.h"
#include "lb_launch.h"

constexpr int kHalo = 2;
using lbk::StepParams;

struct lbgpu_handle {
  lbgpu_config cfg;
  int d = 3, Q = 19, C = 2;
  int nx = 1, ny = 1, nz = 1;       // kernel extents (nz = 1 for D2Q9)
  int nxh = 1, nyh = 1, nzh = 1;    // haloed host extents
  int hy = kHalo;                   // halo in y (0 for D1Q3/D1Q5)
  int hz = kHalo;                   // halo in z (0 for D2Q9, D1Q3, D1Q5)
  int64_t n = 0;
  cudaStream_t stream = nullptr;       // where work is queued
  cudaStream_t own_stream = nullptr;   // created with the handle
  void* f[2] = {nullptr, nullptr};
  size_t fbytes = 0;                // bytes of one population buffer
  int cur = 0;
  uint8_t* mask = nullptr;
  uint32_t* nbmask = nullptr;       // neighbour masks for the fused step (walls only)
  uint8_t* tile_walls = nullptr;    // per (x, 8x32 tile) wall flags for the fused step
  bool zwall = false;               // the solid sites are exactly the planes z = 0 and z = nz - 1
  int* work_counter = nullptr;      // the fused step's dynamic scheduling counter
  void* rho = nullptr;
  void* psi = nullptr;
  double* force = nullptr;
  int record_force = 0;
  int force_valid = 0;
  double* staging = nullptr;
  size_t staging_bytes = 0;
  // host transfers: copies on copy_stream into alternating halves of the
  // staging buffer, overlapping the transposes of the other half on stream
  // (events: [0..1] half filled, [2..3] half free again)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t xfer_ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // lbgpu_step_host: device-to-host copies on their own stream, so that both
  // directions of the host link carry data at once; events of its wavefront
  // (created on first use)
  cudaStream_t copy_stream2 = nullptr;
  cudaEvent_t pipe_ev[9] = {};
  bool owns_staging = true;         // false: borrowed from a batch
  bool lite = false;                // batch member: no rho/psi scratch (fused step only)
  double* moments = nullptr;        // device scratch for lbgpu_moments / lbgpu_reduce
  size_t moments_bytes = 0;
  StepParams P{};
  bool uploaded = false;
  bool advected = false;            // between lbgpu_advect and lbgpu_collide
  // FP32/FP16 D3Q19 run the fused single-pass kernel; LBGPU_TWO_KERNEL=1 in
  // the environment at lbgpu_create selects the two-kernel step instead
  bool fused = false;
  // The fused step does not write solid sites, so both population buffers
  // must hold their (constant) populations: false after an upload, a device
  // initialisation or a mask change, until lb_sync_solids copies the
  // current buffer over the other one.
  bool solids_synced = false;
  // FP16 / I16: rest density and scale of the stored offsets fixed by
  // lbgpu_set_storage_scale (uploads keep them instead of deriving them
  // from the input)
  bool scale_pinned = false;
  // per-kernel event timing (lbgpu_profile)
  bool profiling = false;
  std::vector<lbk::StepEvents> ev_pending, ev_pool;
  double kernel_ms[2] = {0.0, 0.0};
  int64_t kernel_n[2] = {0, 0};
  int64_t launches = 0;
  int64_t device_bytes = 0;
  std::string err;

  int fail(int code, const std::string& msg) {
    err = msg;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return LBGPU_E_CUDA;
  }
};

// Create a handle.  lite: allocate only the two population buffers, borrow
// `staging` (staging_bytes) for host transfers and queue work on `stream`
// (batch members); otherwise own everything.
int lb_handle_create(const lbgpu_config* cfg, bool lite, double* staging, size_t staging_bytes,
                     cudaStream_t stream, lbgpu_handle** out, std::string* err);
// bytes of device memory a lattice of this configuration needs as a batch member
int64_t lb_member_bytes(const lbgpu_config* cfg);
// scratch for lbgpu_moments / lbgpu_reduce, allocated on first use
int lb_ensure_moments(lbgpu_handle* h);
// (re)build or drop the neighbour masks after the mask changed
int lb_update_nbmask(lbgpu_handle* h);
// scale of the I16 form's fixed point for a component with rest density
// rho0 and largest initial |f_q / w_q - rho0| maxdev
double i16_scale(double rho0, double maxdev);
// copy buffer cur over the other one when the fused step needs the solid
// sites in both (see solids_synced)
int lb_sync_solids(lbgpu_handle* h, int cur, cudaStream_t st);
