/* CPU oracle for the DLBC lattice-Boltzmann timestep (TEST INFRASTRUCTURE).
 *
 * This library restates, operation for operation and in the reference's own
 * haloed array-of-structures layout, the D code of SFrijters/DLBC for one
 * timestep (src/main.d:174-199) and for the initialisers the tests need.
 * It is the checker for the CUDA path: only tests/, the smoke test and the
 * CPU-baseline leg of bench.py may load it.  Nothing in the product links it.
 *
 * Layout (as Field.arr in src/dlbc/fields/field.d:114-125): per component a
 * row-major array over the haloed lattice [x][y][z] (halo 2 on every side of
 * every lattice dimension), Q doubles per site, z fastest.  For D2Q9 the
 * z extent is 1 and carries no halo.
 */
#ifndef LB_ORACLE_H
#define LB_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define OR_MAXC 4

typedef struct {
  int32_t d, q;            /* 3/19 (D3Q19) or 2/9 (D2Q9) */
  int32_t gn[3];           /* lattice.gn; gn[2] ignored for d == 2 */
  int32_t components;      /* lb.components */
  int32_t shan_chen;       /* lb.force.enableShanChen */
  int32_t psi_form;        /* lb.force.psiForm: 0 Linear, 1 Exponential */
  int32_t eq_form;         /* lb.eqdist.eqDistForm: 0 SecondOrder, 1 ThirdOrder, 2 BDist2 */
  int32_t exp_mode;        /* 0: expl in long double rounded to double (as Phobos
                              std.math.exp on x86-64, where long double is the x87
                              80-bit format; other hosts' long double differs);
                              1: lbmath::lb_exp (the kernels' exp, which emulates
                              that double rounding on every host) */
  int32_t sum_mode;        /* density(): 0 Phobos pairwise (recursive halving), 1 sequential (negative control) */
  int32_t threads;         /* OpenMP threads for the sweeps (<= 1: serial) */
  double tau[OR_MAXC];
  double gcc[OR_MAXC][OR_MAXC];
  double gwc[OR_MAXC];
  double global_acc[3];
} or_config;

typedef struct {
  int32_t fluid_init[OR_MAXC];    /* FluidInit (src/dlbc/lb/init.d:139-253) */
  int32_t n_dens[OR_MAXC];
  double densities[OR_MAXC][8];   /* lb.init.fluidDensities */
  double perturb[OR_MAXC];        /* lb.init.fluidPerturb */
  int32_t random_reseed[OR_MAXC];
  int32_t random_seed[OR_MAXC];
  int32_t seed;                   /* random.seed */
  int32_t shift_seed_by_rank;     /* random.shiftSeedByRank */
  double init_radius;
  double init_offset[3];
  double init_separation[3];
  int32_t init_axis;              /* lb.init.initAxis: 0 X, 1 Y, 2 Z */
  double interface_thickness;
  int32_t n_lamellae;
  double lamellae_widths[8];
  int32_t mask_init;              /* MaskInit: 0 None, 1 File, 2 Plates, 3 Tube, 4 Box, 5 Walls */
  int32_t mask_axis;              /* lb.mask.initAxis */
  int32_t wall_offset;
  int32_t wall_thickness;
  int32_t dimension_has_wall[3][2];
  int32_t nc[3];                  /* process grid emulated for the initialisers (0 -> 1) */
} or_init;

typedef struct or_lattice or_lattice;

or_lattice* or_create(const or_config* cfg);
void or_destroy(or_lattice* L);
/* haloed lengths (n + 2h per dim) and the halo width */
void or_lengths_h(const or_lattice* L, int32_t out[3], int32_t* halo);

/* initMask + initFluids + exchangeHalo (src/main.d:138-142) */
int or_init_lattice(or_lattice* L, const or_init* ini);

/* whole haloed arrays in the reference layout */
void or_get_fluid(const or_lattice* L, int c, double* out);
void or_set_fluid(or_lattice* L, int c, const double* in);
void or_get_mask(const or_lattice* L, int32_t* out);
void or_set_mask(or_lattice* L, const int32_t* in);

void or_exchange_halo(or_lattice* L);
/* n iterations of runTimeloop (src/main.d:174-199) */
void or_run(or_lattice* L, int nsteps);

/* Physical-site outputs as written by dumpLBData (src/dlbc/lb/io.d:56-101);
 * arrays are [x][y][z](+vector) over the unhaloed lattice. */
void or_population(const or_lattice* L, int c, double* out);   /* N*Q */
void or_density(const or_lattice* L, int c, double* out);      /* N */
void or_colour(const or_lattice* L, int c1, int c2, double* out);
void or_velocity(const or_lattice* L, int c, double* out);     /* N*d */
void or_force(const or_lattice* L, int c, double* out);        /* N*d, last step's force */
void or_mask_phys(const or_lattice* L, int32_t* out);          /* N */
double or_total_mass(const or_lattice* L, int c);               /* fluid sites, sequential */

/* Mt19937 uniform(a, b) as Phobos std.random (src/dlbc/random.d:55-89) */
double or_uniform_sequence(uint32_t seed, double a, double b, int n, double* out);

/* exp of n arguments with exp_mode `mode` (see or_config); mode 2: the
 * kernels' FP64 fallback routine (lbmath::lb_exp_fp64) */
void or_exp(int mode, int n, const double* x, double* out);

/* a[i] / b[i] by the kernels' integer IEEE division (lbmath::div_rn), so
 * that tests can hold it against the hardware division */
void or_div(int n, const double* a, const double* b, double* out);

#ifdef __cplusplus
}
#endif
#endif
