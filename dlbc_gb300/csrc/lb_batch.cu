// Batches: many independent D3Q19 two-component lattices (FP32 or FP16
// offset storage) advanced together, one persistent launch per timestep.
//
// Members are lattice handles (lb_handle.h) that own only their population
// buffers and mask; the batch owns the stream and a shared staging buffer for
// host transfers, and admits members against a fixed device-memory budget.
// Members run the kernel their lone lattice would run: those with an even z
// extent and the BDist2 equilibrium the pair kernel (a device table of
// PairSim descriptors drives k_pairs_batch), the others the
// one-site-per-thread fused kernel (FusedSim descriptors, k_fused_batch);
// the tables are rebuilt when members join or leave.  Steps are replayed as
// a captured CUDA graph of two steps (the two buffer parities).  The launch
// shape (the fused kernel's tile height and CTAs per SM, the pair kernel's
// run length and CTAs per SM) is chosen by timing the candidates on the
// batch itself: every candidate computes the same per-site arithmetic, so
// tuning steps are ordinary steps.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/lbgpu.h"
#include "lb_fused.cuh"
#include "lb_handle.h"
#include "lb_pairs.cuh"

namespace {

constexpr size_t kBatchStaging = size_t(256) << 20;

struct Shape {
  int ty;           // fused kernel: tile height
  int ctas_per_sm;  // fused kernel: resident CTAs per SM (0: as many as fit)
  int prun;         // pair kernel: run length in planes
  int pctas;        // pair kernel: resident CTAs per SM (0: as many as fit)
};

const Shape kCandidates[] = {{8, 2, 32, 0}, {8, 1, 16, 0}, {4, 4, 32, 1}, {4, 2, 8, 0}};

std::mutex g_tune_mu;
std::map<std::string, Shape> g_tuned;  // member-size signature -> best shape

thread_local std::string g_batch_create_error;

}  // namespace

struct lbgpu_batch {
  int device = 0;
  int precision = LBGPU_FP16;
  int64_t budget = 0;
  int64_t used = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  double* staging = nullptr;
  std::vector<lbgpu_handle*> sims;   // by member id; nullptr once removed
  std::vector<int64_t> bytes;
  // descriptor table
  lbk::FusedSim* d_table = nullptr;
  int table_cap = 0;
  int table_n = 0;
  int64_t total_work = 0;
  int64_t total_units = 0;
  int* d_counters = nullptr;  // dynamic scheduling, one per buffer parity
  bool walls = false;
  // pair-kernel members
  lbk::PairSim* d_ptable = nullptr;
  int ptable_cap = 0;
  int ptable_n = 0;
  int64_t ptotal_units = 0;
  int* d_pcounters = nullptr;
  bool dirty = true;
  int64_t steps_since_build = 0;
  std::vector<int> table_ids;
  std::vector<int> table_phase;
  // launch shape
  Shape shape{8, 0, 32, 0};
  int autotune = 1;
  bool shape_fixed = false;
  int use_graph = 1;
  cudaGraphExec_t graph = nullptr;
  int64_t launches = 0;
  std::string err;

  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return LBGPU_E_CUDA;
  }
};

namespace {

void drop_graph(lbgpu_batch* b) {
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
}

std::string signature(const lbgpu_batch* b) {
  std::string s = std::to_string(b->precision);
  for (auto* h : b->sims)
    if (h) s += "|" + std::to_string(h->nx) + "x" + std::to_string(h->ny) + "x" + std::to_string(h->nz);
  return s;
}

// whether a member runs the pair kernel (the rule launch_fused applies to a
// lone lattice, lbk::pairs_eligible)
bool pair_member(const lbgpu_handle* h) {
  if (!(h->nz % 2 == 0 && h->P.eq_form == 2)) return false;
  return h->mask == nullptr && (h->cfg.precision == LBGPU_I16 || h->P.unit_tau != 0);
}

template <typename D>
int upload_table(lbgpu_batch* b, const std::vector<D>& tab, D** d_tab, int* cap) {
  if (int(tab.size()) > *cap) {
    if (*d_tab) cudaFree(*d_tab);
    *d_tab = nullptr;
    const int c = int(tab.size()) * 2;
    cudaError_t e = cudaMalloc(d_tab, sizeof(D) * size_t(c));
    if (e != cudaSuccess) {
      cudaGetLastError();
      *d_tab = nullptr;
      *cap = 0;
      return b->fail(LBGPU_E_NOMEM, "batch descriptor table allocation failed");
    }
    *cap = c;
  }
  if (!tab.empty()) {
    cudaError_t e = cudaMemcpyAsync(*d_tab, tab.data(), sizeof(D) * tab.size(), cudaMemcpyHostToDevice, b->stream);
    if (e != cudaSuccess) return b->cuda_fail(e, "batch table upload");
  }
  return LBGPU_OK;
}

// (re)build the descriptor tables for launch shape `sh`, with every member's
// current input buffer as parity 0
int build_table(lbgpu_batch* b, const Shape& sh) {
  std::vector<lbk::FusedSim> tab;
  std::vector<lbk::PairSim> ptab;
  b->table_ids.clear();
  b->table_phase.clear();
  b->total_work = 0;
  b->total_units = 0;
  b->ptotal_units = 0;
  b->walls = false;
  for (size_t id = 0; id < b->sims.size(); ++id) {
    lbgpu_handle* h = b->sims[id];
    if (!h) continue;
    if (pair_member(h)) {
      lbk::PairSim ps;
      memset(&ps, 0, sizeof ps);
      ps.P = lbk::make_fused_params(h->P, 8);
      const int pty = lbk::pair_ty(b->precision == LBGPU_FP16  ? lbk::kStoreF16
                                   : b->precision == LBGPU_I16 ? lbk::kStoreI16
                                                               : lbk::kStoreF32);
      ps.P.tiles_y = (h->ny + pty - 1) / pty;
      ps.P.tiles_z = (h->nz + lbk::kPairTZ - 1) / lbk::kPairTZ;
      ps.P.work = int64_t(ps.P.tiles_y) * ps.P.tiles_z * h->nx;
      ps.P.run_len = h->nx < sh.prun ? h->nx : sh.prun;
      ps.f[0] = h->f[0];
      ps.f[1] = h->f[1];
      ps.force_out = nullptr;
      ps.phase = h->cur;
      ps.nchunks = (h->nx + ps.P.run_len - 1) / ps.P.run_len;
      ps.unit_begin = b->ptotal_units;
      b->ptotal_units += int64_t(ps.P.tiles_y) * ps.P.tiles_z * ps.nchunks;
      ptab.push_back(ps);
    } else {
      lbk::FusedSim fs;
      memset(&fs, 0, sizeof fs);
      fs.P = lbk::make_fused_params(h->P, sh.ty);
      fs.f[0] = h->f[0];
      fs.f[1] = h->f[1];
      fs.nbmask = h->nbmask;
      fs.force_out = nullptr;
      fs.work_begin = b->total_work;
      fs.phase = h->cur;
      fs.P.run_len = h->nx < 64 ? h->nx : 32;
      fs.nchunks = (h->nx + fs.P.run_len - 1) / fs.P.run_len;
      fs.unit_begin = b->total_units;
      b->total_units += int64_t(fs.P.tiles_y) * fs.P.tiles_z * fs.nchunks;
      b->total_work += fs.P.work;
      b->walls = b->walls || h->mask != nullptr;
      tab.push_back(fs);
    }
    b->table_ids.push_back(int(id));
    b->table_phase.push_back(h->cur);
  }
  b->table_n = int(tab.size());
  b->ptable_n = int(ptab.size());
  if (int rc = upload_table(b, tab, &b->d_table, &b->table_cap)) return rc;
  if (int rc = upload_table(b, ptab, &b->d_ptable, &b->ptable_cap)) return rc;
  if (!b->d_counters) {
    cudaError_t e = cudaMalloc(&b->d_counters, 2 * sizeof(int));
    if (e != cudaSuccess) {
      cudaGetLastError();
      b->d_counters = nullptr;  // static scheduling
    }
  }
  if (b->d_counters) cudaMemsetAsync(b->d_counters, 0, 2 * sizeof(int), b->stream);
  if (b->ptable_n) {
    if (!b->d_pcounters) {
      cudaError_t e = cudaMalloc(&b->d_pcounters, 2 * sizeof(int));
      if (e != cudaSuccess) {
        cudaGetLastError();
        b->d_pcounters = nullptr;
        return b->fail(LBGPU_E_NOMEM, "batch counter allocation failed");
      }
    }
    if (b->ptotal_units >= (int64_t(1) << 31)) return b->fail(LBGPU_E_INVALID, "batch too large for its work counter");
    cudaMemsetAsync(b->d_pcounters, 0, 2 * sizeof(int), b->stream);
  }
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return b->cuda_fail(e, "batch table upload");
  b->steps_since_build = 0;
  b->dirty = false;
  drop_graph(b);
  return LBGPU_OK;
}

// kernel launches per batch step
int kernels_per_step(const lbgpu_batch* b) { return (b->table_n > 0 ? 1 : 0) + (b->ptable_n > 0 ? 1 : 0); }

// members' current-buffer index after the steps since the last build
void sync_members(lbgpu_batch* b) {
  for (size_t i = 0; i < b->table_ids.size(); ++i) {
    lbgpu_handle* h = b->sims[b->table_ids[i]];
    if (h) h->cur = int((b->table_phase[i] + b->steps_since_build) & 1);
  }
}

cudaError_t launch_one(lbgpu_batch* b, int parity) {
  // LBGPU_BATCH_STATIC=1: equal static shares instead of dynamic runs
  static const bool kStatic = [] {
    const char* s = getenv("LBGPU_BATCH_STATIC");
    return s && s[0] == '1';
  }();
  if (b->ptable_n) {
    b->launches++;
    const int kind = b->precision == LBGPU_FP16  ? lbk::kStoreF16
                     : b->precision == LBGPU_I16 ? lbk::kStoreI16
                                                 : lbk::kStoreF32;
    cudaError_t e = lbk::launch_pairs_batch(kind, b->d_ptable, b->ptable_n, parity, b->shape.pctas,
                                            b->stream, b->device, b->ptotal_units, b->d_pcounters);
    if (e != cudaSuccess) return e;
  }
  if (!b->table_n) return cudaSuccess;
  b->launches++;
  const int kind = b->precision == LBGPU_FP16  ? lbk::kStoreF16
                   : b->precision == LBGPU_I16 ? lbk::kStoreI16
                                               : lbk::kStoreF32;
  return lbk::launch_fused_batch(kind, b->shape.ty, b->walls, b->d_table, b->table_n,
                                 b->total_work, parity, b->shape.ctas_per_sm, b->stream, b->device,
                                 b->total_units,
                                 (!kStatic && b->total_units < (int64_t(1) << 31)) ? b->d_counters : nullptr);
}

// advance n steps with the current table and shape
int run_steps(lbgpu_batch* b, int n) {
  if ((b->table_n == 0 && b->ptable_n == 0) || n <= 0) return LBGPU_OK;
  // members with walls whose buffers do not both hold the solid sites yet
  for (size_t i = 0; i < b->table_ids.size(); ++i) {
    lbgpu_handle* h = b->sims[b->table_ids[i]];
    if (h && h->mask && !h->solids_synced) {
      const int cur = int((b->table_phase[i] + b->steps_since_build) & 1);
      if (int rc = lb_sync_solids(h, cur, b->stream)) return b->fail(rc, h->err);
    }
  }
  cudaError_t e;
  int done = 0;
  // a direct launch first: it makes the parity even for the graph and sets
  // up the kernel (attributes, occupancy) outside any capture
  if ((b->steps_since_build & 1) || !b->graph || !b->use_graph) {
    e = launch_one(b, int(b->steps_since_build & 1));
    if (e != cudaSuccess) return b->cuda_fail(e, "batch step launch");
    b->steps_since_build++;
    done++;
  }
  if (b->use_graph && n - done >= 2) {
    if ((b->steps_since_build & 1) == 1) {
      e = launch_one(b, 1);
      if (e != cudaSuccess) return b->cuda_fail(e, "batch step launch");
      b->steps_since_build++;
      done++;
    }
    if (!b->graph) {
      cudaGraph_t g = nullptr;
      e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        const int64_t before = b->launches;
        cudaError_t e0 = launch_one(b, 0);
        cudaError_t e1 = launch_one(b, 1);
        b->launches = before;  // counted when replayed
        e = cudaStreamEndCapture(b->stream, &g);
        if (e == cudaSuccess && e0 == cudaSuccess && e1 == cudaSuccess)
          e = cudaGraphInstantiate(&b->graph, g, 0);
        else if (e == cudaSuccess)
          e = e0 != cudaSuccess ? e0 : e1;
        if (g) cudaGraphDestroy(g);
      }
      if (e != cudaSuccess) {
        cudaGetLastError();
        b->graph = nullptr;
        b->use_graph = 0;  // fall back to direct launches
      }
    }
    while (b->graph && n - done >= 2) {
      e = cudaGraphLaunch(b->graph, b->stream);
      if (e != cudaSuccess) return b->cuda_fail(e, "batch graph launch");
      b->launches += 2 * kernels_per_step(b);
      b->steps_since_build += 2;
      done += 2;
    }
  }
  while (done < n) {
    e = launch_one(b, int(b->steps_since_build & 1));
    if (e != cudaSuccess) return b->cuda_fail(e, "batch step launch");
    b->steps_since_build++;
    done++;
  }
  return LBGPU_OK;
}

// time 2 steps of each candidate shape (real steps), keep the fastest;
// returns the number of steps taken
int autotune(lbgpu_batch* b, int budget_steps, int* rc) {
  *rc = LBGPU_OK;
  const std::string sig = signature(b);
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tuned.find(sig);
    if (it != g_tuned.end()) {
      const Shape& t = it->second;
      if (t.ty != b->shape.ty || t.ctas_per_sm != b->shape.ctas_per_sm || t.prun != b->shape.prun ||
          t.pctas != b->shape.pctas) {
        sync_members(b);
        b->shape = t;
        *rc = build_table(b, b->shape);
      }
      return 0;
    }
  }
  const int per = 2;
  const int ncand = int(sizeof(kCandidates) / sizeof(kCandidates[0]));
  if (budget_steps < per * ncand) return 0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  Shape best_shape = b->shape;
  int taken = 0;
  const int use_graph = b->use_graph;
  b->use_graph = 0;
  for (int i = 0; i < ncand; ++i) {
    sync_members(b);
    b->shape = kCandidates[i];
    if ((*rc = build_table(b, b->shape))) break;
    cudaEventRecord(e0, b->stream);
    if ((*rc = run_steps(b, per))) break;
    cudaEventRecord(e1, b->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    taken += per;
    if (ms < best) {
      best = ms;
      best_shape = kCandidates[i];
    }
  }
  b->use_graph = use_graph;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (*rc) return taken;
  sync_members(b);
  b->shape = best_shape;
  *rc = build_table(b, b->shape);
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tuned[sig] = best_shape;
  return taken;
}

}  // namespace

extern "C" {

int lbgpu_batch_create(int32_t device, int32_t precision, int64_t hbm_budget_bytes, lbgpu_batch** out) {
  if (!out) return LBGPU_E_INVALID;
  *out = nullptr;
  if (precision != LBGPU_FP32 && precision != LBGPU_FP16 && precision != LBGPU_I16) {
    g_batch_create_error = "batches run the FP32, FP16 or I16 forms";
    return LBGPU_E_INVALID;
  }
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    g_batch_create_error = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
    return LBGPU_E_CUDA;
  }
  lbgpu_batch* b = new lbgpu_batch;
  b->device = device;
  b->precision = precision;
  b->budget = hbm_budget_bytes > 0 ? hbm_budget_bytes : INT64_MAX;
  e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&b->staging, kBatchStaging);
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    g_batch_create_error = std::string("batch set-up failed: ") + cudaGetErrorString(e);
    delete b;
    return LBGPU_E_NOMEM;
  }
  b->stream = b->own_stream;
  *out = b;
  return LBGPU_OK;
}

void lbgpu_batch_destroy(lbgpu_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  for (auto* h : b->sims)
    if (h) lbgpu_destroy(h);
  drop_graph(b);
  if (b->d_table) cudaFree(b->d_table);
  if (b->d_counters) cudaFree(b->d_counters);
  if (b->d_ptable) cudaFree(b->d_ptable);
  if (b->d_pcounters) cudaFree(b->d_pcounters);
  cudaFree(b->staging);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
}

const char* lbgpu_batch_last_error(const lbgpu_batch* b) { return b ? b->err.c_str() : g_batch_create_error.c_str(); }

}  // extern "C"

namespace {

// admit a member whose fields are filled by `fill` (upload or device init)
template <typename Fill>
int batch_admit(lbgpu_batch* b, const lbgpu_config* cfg, int32_t* sim_id, Fill fill) {
  if (cfg->precision != b->precision) return b->fail(LBGPU_E_INVALID, "member precision differs from the batch's");
  if (cfg->q != 19 || cfg->components != 2)
    return b->fail(LBGPU_E_INVALID, "batch members are two-component D3Q19 lattices");
  if (cfg->device != b->device) return b->fail(LBGPU_E_INVALID, "member device differs from the batch's");
  const int64_t need = lb_member_bytes(cfg);
  if (b->used + need > b->budget)
    return b->fail(LBGPU_E_BUDGET, "admission refused: " + std::to_string(need) + " bytes over the budget (" +
                                       std::to_string(b->budget - b->used) + " left)");
  cudaSetDevice(b->device);
  std::string why;
  lbgpu_handle* h = nullptr;
  int rc = lb_handle_create(cfg, true, b->staging, kBatchStaging, b->stream, &h, &why);
  if (rc) return b->fail(rc, why);
  rc = fill(h);
  if (rc) {
    b->err = lbgpu_last_error(h);
    lbgpu_destroy(h);
    return rc;
  }
  sync_members(b);
  b->sims.push_back(h);
  b->bytes.push_back(h->device_bytes);
  b->used += b->bytes.back();
  b->dirty = true;
  *sim_id = int32_t(b->sims.size() - 1);
  return LBGPU_OK;
}

}  // namespace

extern "C" {

int lbgpu_batch_add(lbgpu_batch* b, const lbgpu_config* cfg, const double* const* fluids, const int32_t* mask,
                    int32_t* sim_id) {
  if (!b || !cfg || !fluids || !sim_id) return LBGPU_E_INVALID;
  return batch_admit(b, cfg, sim_id, [&](lbgpu_handle* h) { return lbgpu_upload(h, fluids, mask); });
}

int lbgpu_batch_add_init(lbgpu_batch* b, const lbgpu_config* cfg, const lbgpu_init* ini, int32_t* sim_id) {
  if (!b || !cfg || !ini || !sim_id) return LBGPU_E_INVALID;
  return batch_admit(b, cfg, sim_id, [&](lbgpu_handle* h) { return lbgpu_init_fields(h, ini); });
}

int lbgpu_batch_remove(lbgpu_batch* b, int32_t sim_id) {
  if (!b || sim_id < 0 || size_t(sim_id) >= b->sims.size() || !b->sims[sim_id]) return LBGPU_E_INVALID;
  cudaSetDevice(b->device);
  sync_members(b);
  cudaStreamSynchronize(b->stream);
  lbgpu_destroy(b->sims[sim_id]);
  b->sims[sim_id] = nullptr;
  b->used -= b->bytes[sim_id];
  b->dirty = true;
  return LBGPU_OK;
}

int lbgpu_batch_step(lbgpu_batch* b, int32_t nsteps) {
  if (!b || nsteps < 0) return LBGPU_E_INVALID;
  cudaSetDevice(b->device);
  if (b->dirty) {
    sync_members(b);
    int rc = build_table(b, b->shape);
    if (rc) return rc;
  }
  int remaining = nsteps;
  if (b->autotune && !b->shape_fixed) {
    int rc = LBGPU_OK;
    remaining -= autotune(b, remaining, &rc);
    if (rc) return rc;
  }
  int rc = run_steps(b, remaining);
  sync_members(b);
  return rc;
}

lbgpu_handle* lbgpu_batch_member(lbgpu_batch* b, int32_t sim_id) {
  if (!b || sim_id < 0 || size_t(sim_id) >= b->sims.size()) return nullptr;
  return b->sims[sim_id];
}

int lbgpu_batch_set_stream(lbgpu_batch* b, void* stream) {
  if (!b) return LBGPU_E_INVALID;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  b->stream = stream ? static_cast<cudaStream_t>(stream) : b->own_stream;
  for (auto* h : b->sims)
    if (h) h->stream = b->stream;
  drop_graph(b);
  return LBGPU_OK;
}

int lbgpu_batch_synchronize(lbgpu_batch* b) {
  if (!b) return LBGPU_E_INVALID;
  cudaSetDevice(b->device);
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return b->cuda_fail(e, "batch synchronize");
  return LBGPU_OK;
}

int64_t lbgpu_batch_device_bytes(const lbgpu_batch* b) { return b ? b->used : 0; }

int64_t lbgpu_batch_launch_count(const lbgpu_batch* b) { return b ? b->launches : 0; }

int lbgpu_batch_set_tuning(lbgpu_batch* b, int32_t autotune, int32_t tile_height, int32_t ctas_per_sm,
                           int32_t use_graph) {
  if (!b) return LBGPU_E_INVALID;
  if (tile_height != 0 && tile_height != 4 && tile_height != 8) return b->fail(LBGPU_E_INVALID, "tile height 4 or 8");
  b->autotune = autotune;
  b->use_graph = use_graph;
  if (tile_height) {
    sync_members(b);
    b->shape = Shape{tile_height, ctas_per_sm, 32, ctas_per_sm};
    b->shape_fixed = true;
    b->dirty = true;
  } else {
    b->shape_fixed = false;
  }
  drop_graph(b);
  return LBGPU_OK;
}

int lbgpu_batch_launch_shape(const lbgpu_batch* b, int32_t* tile_height, int32_t* ctas_per_sm) {
  if (!b) return LBGPU_E_INVALID;
  if (tile_height) *tile_height = b->shape.ty;
  if (ctas_per_sm) *ctas_per_sm = b->shape.ctas_per_sm;
  return LBGPU_OK;
}

}  // extern "C"
