/* lbgpu: GB300 (sm_103a) lattice-Boltzmann timestep behind a C ABI.
 *
 * This is the drop-in boundary for the DLBC time loop.  In the reference,
 * one timestep is (src/main.d:174-199):
 *
 *   L.exchangeHalo();        // src/dlbc/fields/parallel.d:40
 *   L.advectFields();        // src/dlbc/lb/advection.d:35
 *   L.resetForce();          // src/dlbc/lb/force.d:165
 *   L.addShanChenForce();    // src/dlbc/lb/force.d:223
 *   L.distributeForce();     // src/dlbc/lb/force.d:179
 *   L.prepareToCollide();    // src/dlbc/lb/collision.d:41
 *   L.collideFields(tau, globalAcc);   // src/dlbc/lb/collision.d:61
 *
 * lbgpu_step() replaces that whole sequence (halo exchange becomes periodic
 * index wrap on one in-GPU domain).  The lattice fields stay resident on the
 * device between calls; the host exchanges them in the reference's own layout
 * (Field.arr of src/dlbc/fields/field.d:114-125: row-major [x][y][z] over the
 * haloed lattice, halo width 2, the Q populations of a site contiguous), so a
 * D program passes `L.fluids[i].arr._data.ptr` and `L.mask.arr._data.ptr`
 * unchanged.
 *
 * Conventions: every entry point returns 0 on success or a negative
 * LBGPU_E_* code; nothing throws or exits across the ABI.  A handle is used
 * from one host thread at a time; work is ordered on the handle's stream.
 * Host buffers are borrowed for the duration of a call only.
 */
#ifndef LBGPU_H
#define LBGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBGPU_ABI_VERSION 2  /* 2: lbgpu_init gained rng, random_reseed, nc, shift_seed_by_rank, random_seed */
#define LBGPU_MAX_COMPONENTS 2

/* status codes */
#define LBGPU_OK 0
#define LBGPU_E_INVALID (-1)     /* bad argument or unsupported configuration */
#define LBGPU_E_NOMEM (-2)       /* device or pinned-host allocation failed */
#define LBGPU_E_CUDA (-3)        /* CUDA runtime error (see lbgpu_last_error) */
#define LBGPU_E_BUDGET (-4)      /* request exceeds the configured HBM budget */
#define LBGPU_E_NOTREADY (-5)    /* no state uploaded yet */
#define LBGPU_E_NONFINITE (-6)   /* a non-finite value was detected on the device */

/* lb.eqdist.eqDistForm (src/dlbc/lb/eqdist.d:23-36) */
#define LBGPU_EQ_SECOND_ORDER 0
#define LBGPU_EQ_THIRD_ORDER 1
#define LBGPU_EQ_BDIST2 2
/* lb.force.psiForm (src/dlbc/lb/force.d:48-57) */
#define LBGPU_PSI_LINEAR 0
#define LBGPU_PSI_EXPONENTIAL 1
/* storage/arithmetic forms */
#define LBGPU_FP64 0        /* double storage + double arithmetic: the reference's numbers */
#define LBGPU_FP32 1        /* float storage + float arithmetic */
#define LBGPU_FP16 2        /* half storage of f - w_q*rho0 (scaled) + float arithmetic */
#define LBGPU_I16 3         /* 16-bit fixed-point storage of f/w_q - rho0 (scaled) + float arithmetic;
                             * D3Q19 with an even z extent and the BDist2 equilibrium only; every
                             * collision conserves the site's stored (integer) mass exactly */

typedef struct lbgpu_config {
  int32_t d, q;               /* 3/19 (D3Q19), 2/9 (D2Q9), 1/3 (D1Q3) or 1/5 (D1Q5): gconn
                               * (src/dlbc/lb/connectivity.d) */
  int32_t gn[3];              /* lattice.gn (gn[2] ignored when d == 2); each >= 2 */
  int32_t components;         /* lb.components, 1 or 2 */
  int32_t shan_chen;          /* lb.force.enableShanChen */
  int32_t psi_form;           /* lb.force.psiForm */
  int32_t eq_form;            /* lb.eqdist.eqDistForm */
  int32_t precision;          /* LBGPU_FP64 / LBGPU_FP32 / LBGPU_FP16 / LBGPU_I16 */
  int32_t device;             /* CUDA device ordinal */
  double tau[LBGPU_MAX_COMPONENTS];                        /* lb.tau */
  double gcc[LBGPU_MAX_COMPONENTS][LBGPU_MAX_COMPONENTS];  /* lb.force.gcc */
  double gwc[LBGPU_MAX_COMPONENTS];                        /* lb.force.gwc */
  double global_acc[3];                                    /* lb.force.globalAcc */
  double rho0[LBGPU_MAX_COMPONENTS];  /* LBGPU_FP16 / LBGPU_I16: rest density of the stored
                                         offsets f_q - w_q*rho0 (0: use the mean density at upload) */
} lbgpu_config;

typedef struct lbgpu_handle lbgpu_handle;

/* Create a lattice on cfg->device.  No field data yet: call lbgpu_upload.
 * Replaces the allocation in prepareLBFields/prepareForce
 * (src/dlbc/lb/init.d:60-72, src/dlbc/lb/force.d:67-107). */
int lbgpu_create(const lbgpu_config* cfg, lbgpu_handle** out);
void lbgpu_destroy(lbgpu_handle* h);

/* Copy the host fields to the device.  fluids[c] points at component c's
 * haloed AoS array ((gn+4)^d sites x q doubles, i.e. Field.arr._data of
 * L.fluids[c]); mask points at the haloed Mask array (int32: 0 None, 1 Solid),
 * or is NULL for an all-fluid lattice.  Halo entries are ignored: the device
 * uses periodic images, which is what exchangeHalo (src/dlbc/fields/parallel.d:40)
 * puts there on one process. */
int lbgpu_upload(lbgpu_handle* h, const double* const* fluids, const int32_t* mask);

/* Advance nsteps timesteps (one call = nsteps iterations of runTimeloop's
 * body, src/main.d:175-199, without dumpData). */
int lbgpu_step(lbgpu_handle* h, int32_t nsteps);

/* One timestep in two phases, for a host that runs hooks between advection
 * and collision (postAdvectionHooks / preCollisionHooks, executed by
 * src/dlbc/lb/advection.d:53 and src/dlbc/lb/collision.d:70 and registered
 * through src/dlbc/hooks.d:57-118).  lbgpu_advect streams the populations
 * (advectFields, src/dlbc/lb/advection.d:35-55); lbgpu_collide does the
 * densities, psi, forces and collision without streaming
 * (src/dlbc/lb/force.d:165-309, src/dlbc/lb/collision.d:60-119).  Between
 * the two, lbgpu_download returns the advected populations and lbgpu_upload
 * may replace them.  lbgpu_advect then lbgpu_collide compute bit for bit
 * what lbgpu_step(h, 1) computes in the FP64 form; the FP32 and FP16 D3Q19
 * forms of lbgpu_step use the fused single-pass kernel, which rounds
 * differently (within the forms' documented error).  Calling lbgpu_collide
 * twice in a row, or lbgpu_step between the phases, is LBGPU_E_NOTREADY. */
int lbgpu_advect(lbgpu_handle* h);
int lbgpu_collide(lbgpu_handle* h);

/* Initial fields computed on the device (no host arrays cross the bus): the
 * deterministic initialisers of initFluids/initMask (src/dlbc/lb/init.d:139-339,
 * src/dlbc/fields/init.d) for one process.  Sphere, cylinder, two-sphere and
 * lamellae initialisers (and their Frac forms), EqDist, Const and every mask
 * but File give exactly the values the reference computes.  The random
 * initialisers (EqDistPerturb, EqDistPerturbFrac, EqDistRandom, ConstRandom)
 * with rng = 1 draw the reference's sequences: on each rank of the process
 * grid `nc`, Mt19937 seeded with `seed` (random.seed, plus the rank with
 * shift_seed_by_rank; src/dlbc/random.d:43-53), one draw per haloed site of
 * the rank's block in row-major order (ConstRandom: per population),
 * component 0 before component 1 unless random_reseed
 * (src/dlbc/lb/init.d:105-125); the draws are generated on the host, the
 * fields on the device, and the result equals the reference's bit for bit.  With rng = 0 they draw from a
 * counter-based generator keyed by `seed`, component and site (nothing
 * generated on the host; same distribution, different numbers).  rng = 1
 * holds the draws of the random components on the device during the call
 * (4 bytes per site, ConstRandom 4 per population).  FluidInit/MaskInit codes are the
 * reference's enum orders (FluidInit: None 0, File 1, Const 2, EqDist 3,
 * EqDistPerturb 4, EqDistPerturbFrac 5, ConstRandom 6, EqDistRandom 7,
 * EqDistSphere 8, EqDistSphereFrac 9, EqDistCylinder 10, EqDistCylinderFrac 11,
 * EqDistTwoSpheres 12, EqDistTwoSpheresFrac 13, EqDistLamellae 14,
 * EqDistLamellaeFrac 15; MaskInit: None 0, File 1, Plates 2, Tube 3, Box 4,
 * Walls 5). */
typedef struct lbgpu_init {
  int32_t fluid_init[LBGPU_MAX_COMPONENTS];      /* lb.init.fluidInit */
  int32_t n_densities[LBGPU_MAX_COMPONENTS];
  double densities[LBGPU_MAX_COMPONENTS][8];     /* lb.init.fluidDensities */
  double perturb[LBGPU_MAX_COMPONENTS];          /* lb.init.fluidPerturb */
  uint64_t seed;
  double init_radius;                            /* lb.init.initRadius */
  double init_offset[3];                         /* lb.init.initOffset */
  double init_separation[3];                     /* lb.init.initSeparation */
  int32_t init_axis;                             /* lb.init.initAxis (0 X, 1 Y, 2 Z) */
  double interface_thickness;                    /* lb.init.interfaceThickness */
  int32_t n_lamellae;
  double lamellae_widths[8];                     /* lb.init.lamellaeWidths */
  int32_t mask_init;                             /* lb.mask.maskInit */
  int32_t mask_axis;                             /* lb.mask.initAxis */
  int32_t wall_offset;                           /* lb.mask.wallOffset */
  int32_t wall_thickness;                        /* lb.mask.wallThickness */
  int32_t dimension_has_wall[3][2];              /* lb.mask.dimensionHasWall */
  int32_t rng;                                   /* 0: counter-based draws; 1: the reference's Mt19937 sequence */
  int32_t random_reseed[LBGPU_MAX_COMPONENTS];   /* lb.init.randomReseed (rng = 1) */
  int32_t nc[3];                                 /* parallel.nc whose per-rank sequences are drawn (rng = 1; 0 = 1) */
  int32_t shift_seed_by_rank;                    /* random.shiftSeedByRank (rng = 1) */
  uint64_t random_seed[LBGPU_MAX_COMPONENTS];    /* lb.init.randomSeed (rng = 1) */
} lbgpu_init;

int lbgpu_init_fields(lbgpu_handle* h, const lbgpu_init* ini);

/* Copy the current populations back into haloed AoS host arrays (halo sites
 * are filled with their periodic images, as after exchangeHalo). */
int lbgpu_download(lbgpu_handle* h, double* const* fluids);

/* One timestep with the fields on the host on both sides: the same result as
 * lbgpu_upload(h, fluids_in, mask), lbgpu_step(h, 1), lbgpu_download(h,
 * fluids_out), bit for bit, for a host that keeps L.fluids as the state and
 * runs hooks on it between steps (runTimeloop's body, src/main.d:179-195,
 * with pre/postAdvection and pre/postCollision hooks registered through
 * src/dlbc/hooks.d:57-118).  The input copies, the kernels and the output
 * copies run as a wavefront over chunks of x-planes, so both directions of
 * the host link carry data at once: in the FP64 form, in FP32, and in FP16 /
 * I16 once lbgpu_set_storage_scale has pinned their offsets' scale (for
 * D3Q19 lattices with an even z extent and BDist2; other lattices run the
 * three calls in turn).  fluids_out may alias fluids_in; a NULL
 * fluids_out[c] skips component c's output. */
int lbgpu_step_host(lbgpu_handle* h, const double* const* fluids_in, const int32_t* mask,
                    double* const* fluids_out);

/* FP16 / I16 forms: fix the rest density rho0[c] and the scale[c] of the
 * stored offsets (f_q = w_q (rho0 + scale h_q), h the stored half or 16-bit
 * integer) instead of deriving them from each upload's input (mean density,
 * largest offset).  Call before the first upload or device initialisation;
 * NULL arrays unpin.  With the scale pinned, lbgpu_upload skips its scan of
 * the input and lbgpu_step_host of these forms runs as the same wavefront
 * as FP32 and FP64.  No counterpart in the reference (its fields are double).
 * LBGPU_E_INVALID for other forms, non-positive scales, or after an upload. */
int lbgpu_set_storage_scale(lbgpu_handle* h, const double* rho0, const double* scale);

/* Fields as dumpLBData writes them (src/dlbc/lb/io.d:56-101), over the
 * physical lattice, row-major [x][y][z] (+ vector component fastest):
 *   density[c]   N doubles  (densityField, src/dlbc/lb/density.d:89)
 *   velocity[c]  N*d doubles (rawVelocityField, src/dlbc/lb/velocity.d:106; 0 on solids)
 *   colour       N doubles  (colourField of components 0 and 1, src/dlbc/lb/density.d:284)
 * Any pointer may be NULL to skip that field. */
int lbgpu_moments(lbgpu_handle* h, double* const* density, double* const* velocity, double* colour);

/* Force field of the last step (L.force, dumped as force-<name>), N*d
 * doubles per component; requires lbgpu_set_record_force(h, 1) before the
 * step. */
int lbgpu_set_record_force(lbgpu_handle* h, int32_t enable);
int lbgpu_force(lbgpu_handle* h, double* const* force);

/* Global mass and momentum over fluid sites (globalTotalMass,
 * src/dlbc/lb/density.d:172; globalTotalMomentum, src/dlbc/lb/momentum.d:172),
 * reduced in a fixed order in double precision.  mass: components doubles;
 * momentum: components*d doubles.  Either may be NULL. */
int lbgpu_reduce(lbgpu_handle* h, double* mass, double* momentum);

/* Wait for all work queued on the handle's stream. */
int lbgpu_synchronize(lbgpu_handle* h);

/* Queue the handle's work on a caller-owned cudaStream_t (passed as void*;
 * NULL restores the handle's own stream).  The caller keeps the stream alive
 * while the handle uses it. */
int lbgpu_set_stream(lbgpu_handle* h, void* stream);

/* Per-kernel timing with CUDA events on the handle's stream.  While enabled,
 * lbgpu_step brackets each timestep kernel with events; lbgpu_kernel_time
 * returns the accumulated milliseconds and launch count of kernel `which`
 * (LBGPU_KERNEL_*) since the last reset (it synchronizes the stream). */
#define LBGPU_KERNEL_DENSITY_PSI 0
#define LBGPU_KERNEL_COLLIDE 1
int lbgpu_profile(lbgpu_handle* h, int32_t enable);
int lbgpu_kernel_time(lbgpu_handle* h, int32_t which, double* total_ms, int64_t* launches);

/* One timestep on caller-owned device buffers, allocating no device memory.
 * It has no counterpart in the reference: it exists for callers that cannot
 * let a library call cudaMalloc (a host framework whose memory pool already
 * owns the GPU, or a caller that cannot take cudaMalloc's implicit device
 * synchronisation while its other streams run).  The caller passes device
 * pointers: f_in and f_out hold the populations in the kernels' SoA layout,
 * element [c][q][site] with site = (x*gn[1] + y)*gn[2] + z (D3Q19) or
 * x*gn[1] + y (D2Q9; the only two connectivities accepted), as doubles
 * (LBGPU_FP64) or floats (LBGPU_FP32); mask is uint8 [site] (nonzero =
 * solid) or NULL.  FP64 gives lbgpu_step's populations bit for bit; FP32 runs
 * the two-kernel float step, so it agrees with lbgpu_step's fused FP32 step
 * within the FP32 form's rounding, not bit for bit.  The work is queued on `stream` (a cudaStream_t,
 * NULL for the legacy default stream) and `cfg->device` is used.
 * The psi/density scratch is a 64 MiB static device array that every GPU
 * loading this library holds until exit, so at most 64 MiB /
 * (components * 2 * sizeof(arithmetic type)) sites are accepted (2,097,152
 * two-component FP64 sites); larger lattices return LBGPU_E_INVALID.  The
 * first call on a device looks up the array's address (make it before any
 * stream capture).  All calls share the array: calls that overlap on the GPU
 * race.  Error text goes to errbuf (may be NULL). */
int lbgpu_step_noalloc(const lbgpu_config* cfg, const void* f_in, void* f_out, const uint8_t* mask,
                       void* stream, char* errbuf, size_t errbuf_len);

/* ------------------------------------------------------------------------
 * Batches: many independent two-component D3Q19 lattices (LBGPU_FP32 or
 * LBGPU_FP16, any sizes) advanced together, one persistent launch per
 * timestep over all members, replayed as a CUDA graph.  No counterpart in the
 * reference (one lattice per process there): each member is exactly the
 * lattice lbgpu_create would hold and steps bit-identically to it.  A batch
 * is used from one host thread; its members are owned by it.
 * ---------------------------------------------------------------------- */
typedef struct lbgpu_batch lbgpu_batch;

/* hbm_budget_bytes <= 0: no budget.  Members are admitted while the device
 * memory they need (lbgpu_batch_add) fits in the budget. */
int lbgpu_batch_create(int32_t device, int32_t precision, int64_t hbm_budget_bytes, lbgpu_batch** out);
void lbgpu_batch_destroy(lbgpu_batch* b);
/* Admit a lattice (same arguments as lbgpu_create + lbgpu_upload); returns
 * LBGPU_E_BUDGET, leaving the batch unchanged, when it does not fit. */
int lbgpu_batch_add(lbgpu_batch* b, const lbgpu_config* cfg, const double* const* fluids, const int32_t* mask,
                    int32_t* sim_id);
/* lbgpu_batch_add with device-side initial fields (lbgpu_init_fields) */
int lbgpu_batch_add_init(lbgpu_batch* b, const lbgpu_config* cfg, const lbgpu_init* ini, int32_t* sim_id);
int lbgpu_batch_remove(lbgpu_batch* b, int32_t sim_id);
/* Advance every member nsteps timesteps. */
int lbgpu_batch_step(lbgpu_batch* b, int32_t nsteps);
/* The member's handle, for lbgpu_download / lbgpu_moments / lbgpu_reduce /
 * lbgpu_force (do not destroy or step it directly); NULL if removed. */
lbgpu_handle* lbgpu_batch_member(lbgpu_batch* b, int32_t sim_id);
int lbgpu_batch_set_stream(lbgpu_batch* b, void* stream);
int lbgpu_batch_synchronize(lbgpu_batch* b);
int64_t lbgpu_batch_device_bytes(const lbgpu_batch* b);
int64_t lbgpu_batch_launch_count(const lbgpu_batch* b);
/* Launch shape: autotune (1: time the candidate shapes on the batch's first
 * steps and cache the choice per set of member sizes), or a fixed tile height
 * (4 or 8 sites along y; 0 = keep tuning) and resident CTAs per SM (0 = as
 * many as fit); use_graph 0 launches every step directly. */
int lbgpu_batch_set_tuning(lbgpu_batch* b, int32_t autotune, int32_t tile_height, int32_t ctas_per_sm,
                           int32_t use_graph);
int lbgpu_batch_launch_shape(const lbgpu_batch* b, int32_t* tile_height, int32_t* ctas_per_sm);
const char* lbgpu_batch_last_error(const lbgpu_batch* b);

/* Number of kernel launches issued by this handle since creation. */
int64_t lbgpu_launch_count(const lbgpu_handle* h);

/* Device bytes held by the handle. */
int64_t lbgpu_device_bytes(const lbgpu_handle* h);

/* Message for the last failed call on h (or on lbgpu_create when h is NULL). */
const char* lbgpu_last_error(const lbgpu_handle* h);

/* ABI version of the loaded library (LBGPU_ABI_VERSION). */
int32_t lbgpu_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* LBGPU_H */
