// Written in the D programming language.

/**
   extern(C) binding of include/lbgpu.h (liblbgpu.so), for the D host of
   DLBC.  Declarations only: every type and function mirrors the C header
   one for one (same names, argument order and meaning), so that the GPU
   timestep can be called from the reference's time loop
   (src/main.d:174-200) without any wrapper library.

   Link with: -L-L<dir of liblbgpu.so> -L-llbgpu -L-rpath=<dir>.

   Output arrays (C `double* const*`) are `double**` here: D's const is
   transitive and cannot express a constant pointer to mutable data.

   This file is not compiled in this repository (there is no D toolchain
   here); the same interface is exercised from Python through ctypes.
*/
module dlbc.gpu.lbgpu;

extern(C) nothrow @nogc:

enum int LBGPU_ABI_VERSION = 2;
enum int LBGPU_MAX_COMPONENTS = 2;

enum int LBGPU_OK = 0;
enum int LBGPU_E_INVALID = -1;
enum int LBGPU_E_NOMEM = -2;
enum int LBGPU_E_CUDA = -3;
enum int LBGPU_E_BUDGET = -4;
enum int LBGPU_E_NOTREADY = -5;
enum int LBGPU_E_NONFINITE = -6;

enum int LBGPU_EQ_SECOND_ORDER = 0;
enum int LBGPU_EQ_THIRD_ORDER = 1;
enum int LBGPU_EQ_BDIST2 = 2;
enum int LBGPU_PSI_LINEAR = 0;
enum int LBGPU_PSI_EXPONENTIAL = 1;

enum int LBGPU_FP64 = 0;
enum int LBGPU_FP32 = 1;
enum int LBGPU_FP16 = 2;
enum int LBGPU_I16 = 3;

enum int LBGPU_KERNEL_DENSITY_PSI = 0;
enum int LBGPU_KERNEL_COLLIDE = 1;

/// C: lbgpu_config (D static arrays have C array layout)
struct lbgpu_config {
  int d, q;
  int[3] gn;
  int components;
  int shan_chen;
  int psi_form;
  int eq_form;
  int precision;
  int device;
  double[LBGPU_MAX_COMPONENTS] tau;
  double[LBGPU_MAX_COMPONENTS][LBGPU_MAX_COMPONENTS] gcc;
  double[LBGPU_MAX_COMPONENTS] gwc;
  double[3] global_acc;
  double[LBGPU_MAX_COMPONENTS] rho0;
}

/// C: lbgpu_init
struct lbgpu_init {
  int[LBGPU_MAX_COMPONENTS] fluid_init;
  int[LBGPU_MAX_COMPONENTS] n_densities;
  double[8][LBGPU_MAX_COMPONENTS] densities;
  double[LBGPU_MAX_COMPONENTS] perturb;
  ulong seed;
  double init_radius;
  double[3] init_offset;
  double[3] init_separation;
  int init_axis;
  double interface_thickness;
  int n_lamellae;
  double[8] lamellae_widths;
  int mask_init;
  int mask_axis;
  int wall_offset;
  int wall_thickness;
  int[2][3] dimension_has_wall;
  int rng;
  int[LBGPU_MAX_COMPONENTS] random_reseed;
  int[3] nc;
  int shift_seed_by_rank;
  ulong[LBGPU_MAX_COMPONENTS] random_seed;
}

struct lbgpu_handle;
struct lbgpu_batch;

int lbgpu_create(const(lbgpu_config)* cfg, lbgpu_handle** out_);
void lbgpu_destroy(lbgpu_handle* h);
int lbgpu_upload(lbgpu_handle* h, const(double*)* fluids, const(int)* mask);
int lbgpu_step(lbgpu_handle* h, int nsteps);
int lbgpu_advect(lbgpu_handle* h);
int lbgpu_collide(lbgpu_handle* h);
int lbgpu_init_fields(lbgpu_handle* h, const(lbgpu_init)* ini);
int lbgpu_download(lbgpu_handle* h, double** fluids);
int lbgpu_step_host(lbgpu_handle* h, const(double*)* fluidsIn, const(int)* mask, double** fluidsOut);
int lbgpu_set_storage_scale(lbgpu_handle* h, const(double)* rho0, const(double)* scale);
int lbgpu_moments(lbgpu_handle* h, double** density, double** velocity, double* colour);
int lbgpu_set_record_force(lbgpu_handle* h, int enable);
int lbgpu_force(lbgpu_handle* h, double** force);
int lbgpu_reduce(lbgpu_handle* h, double* mass, double* momentum);
int lbgpu_synchronize(lbgpu_handle* h);
int lbgpu_set_stream(lbgpu_handle* h, void* stream);
int lbgpu_profile(lbgpu_handle* h, int enable);
int lbgpu_kernel_time(lbgpu_handle* h, int which, double* total_ms, long* launches);
int lbgpu_step_noalloc(const(lbgpu_config)* cfg, const(void)* f_in, void* f_out, const(ubyte)* mask,
                       void* stream, char* errbuf, size_t errbuf_len);

int lbgpu_batch_create(int device, int precision, long hbm_budget_bytes, lbgpu_batch** out_);
void lbgpu_batch_destroy(lbgpu_batch* b);
int lbgpu_batch_add(lbgpu_batch* b, const(lbgpu_config)* cfg, const(double*)* fluids, const(int)* mask,
                    int* sim_id);
int lbgpu_batch_add_init(lbgpu_batch* b, const(lbgpu_config)* cfg, const(lbgpu_init)* ini, int* sim_id);
int lbgpu_batch_remove(lbgpu_batch* b, int sim_id);
int lbgpu_batch_step(lbgpu_batch* b, int nsteps);
lbgpu_handle* lbgpu_batch_member(lbgpu_batch* b, int sim_id);
int lbgpu_batch_set_stream(lbgpu_batch* b, void* stream);
int lbgpu_batch_synchronize(lbgpu_batch* b);
long lbgpu_batch_device_bytes(const(lbgpu_batch)* b);
long lbgpu_batch_launch_count(const(lbgpu_batch)* b);
int lbgpu_batch_set_tuning(lbgpu_batch* b, int autotune, int tile_height, int ctas_per_sm, int use_graph);
int lbgpu_batch_launch_shape(const(lbgpu_batch)* b, int* tile_height, int* ctas_per_sm);
const(char)* lbgpu_batch_last_error(const(lbgpu_batch)* b);

long lbgpu_launch_count(const(lbgpu_handle)* h);
long lbgpu_device_bytes(const(lbgpu_handle)* h);
const(char)* lbgpu_last_error(const(lbgpu_handle)* h);
int lbgpu_abi_version();
