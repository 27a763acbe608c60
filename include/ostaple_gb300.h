/* ostaple_gb300.h -- C ABI of the GB300 (sm_103a) staggered-fermion hot path.
 *
 * Drop-in for the reference's OpenACC hot path: the functions below carry the
 * reference's own names, argument order, argument meaning and return codes,
 * so that the reference's unmodified C host code can link against this
 * library instead of fermion_matrix.o, fermionic_utilities.o, inverter_*.o,
 * stouting.o and fermion_force*.o.  Each declaration cites the reference
 * declaration it replaces (paths relative to the reference source tree).
 *
 * Differences a host program must know about:
 *   - The lattice size is given at run time by ostaple_init() instead of the
 *     compile-time LOC_N0..3 macros (geometry_multidev.h:78-85).  Buffers keep
 *     the reference's layouts, sized by that lattice.
 *   - OpenACC `enter data create` / `update device|host` / `exit data`
 *     become ostaple_enter_data / ostaple_update_device / ostaple_update_host
 *     / ostaple_exit_data.  A pointer passed to a hot-path function must
 *     either be registered that way (the host address is then translated to
 *     its device mirror, like OpenACC's `present`) or be a device pointer.
 *   - Work is queued on one library stream (ostaple_set_stream() to share a
 *     caller stream).  Functions that return a scalar synchronise;
 *     ostaple_update_host synchronises; ostaple_synchronize() waits for all.
 *   - Errors are recorded (ostaple_get_error / ostaple_last_error); functions
 *     whose reference signature returns a status return the reference's
 *     INVERTER_SUCCESS / INVERTER_FAILURE.
 */
#ifndef OSTAPLE_GB300_H_
#define OSTAPLE_GB300_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- reference types --------------------------------------------------- */
/* SoA field types are opaque here: their size follows the run-time lattice.
 * The struct tags match the reference's (struct_c_def.h:16-60), so a host
 * that also includes the reference's struct_c_def.h sees compatible types. */
typedef struct vec3_soa_t vec3_soa;       /* c0,c1,c2 [sizeh] double complex */
typedef struct su3_soa_t su3_soa;         /* r0,r1,r2 vec3_soa               */
typedef struct double_soa_t double_soa;   /* d[sizeh]                        */
typedef struct tamat_soa_t tamat_soa;     /* c01,c02,c12 complex; ic00,ic11  */
typedef struct thmat_soa_t thmat_soa;     /* c01,c02,c12 complex; rc00,rc11  */
typedef struct vec3_soa_f_t vec3_soa_f;   /* float twins (generated sp_ types) */
typedef struct su3_soa_f_t su3_soa_f;
typedef struct float_soa_t float_soa;
typedef struct dcomplex_soa_t dcomplex_soa; /* c[sizeh] double complex     */
typedef struct global_su3_soa_t global_su3_soa; /* su3_soa of the whole lattice */

#define INVERTER_SUCCESS 1                /* inverter_full.h:12 */
#define INVERTER_FAILURE 0                /* inverter_full.h:13 */
#define MAX_APPROX_ORDER 25               /* rationalapprox.h:8 */
#define CONVERGENCE_CRITICAL 1            /* inverter_wrappers.h:11 */
#define CONVERGENCE_NONCRITICAL 0         /* inverter_wrappers.h:12 */

/* Plain structs whose layout must equal the reference's.  Define
 * OSTAPLE_HAVE_REFERENCE_TYPES when the reference's own headers are included
 * in the same translation unit. */
#ifndef OSTAPLE_HAVE_REFERENCE_TYPES
typedef struct RationalApprox_t {          /* rationalapprox.h:15-26 */
  int exponent_num;
  int exponent_den;
  int approx_order;
  double lambda_min;
  double lambda_max;
  int gmp_remez_precision;
  double error;
  double RA_a0;
  double RA_a[MAX_APPROX_ORDER];
  double RA_b[MAX_APPROX_ORDER];
} RationalApprox;

typedef struct ferm_param_t {             /* Include/fermion_parameters.h:9-41 */
  double ferm_mass;
  int degeneracy;
  int number_of_ps;
  char name[30];
  double ferm_charge;
  double ferm_im_chem_pot;
  int index_of_the_first_ps;
  int index_of_the_first_shift;
  double_soa *phases;
  double_soa *mag_re;
  double_soa *mag_im;
  int printed_bf_dbg_info;
  float_soa *phases_f;
  RationalApprox approx_fi_mother;
  RationalApprox approx_md_mother;
  RationalApprox approx_li_mother;
  RationalApprox approx_fi;
  RationalApprox approx_md;
  RationalApprox approx_li;
} ferm_param;

typedef struct inv_tricks_t {             /* Include/inverter_tricks.h:4-11 */
  int singlePInvAccelMultiInv;
  int useMixedPrecision;
  double mixedPrecisionDelta;
  int restartingEvery;
} inv_tricks;

typedef struct inverter_package_t {       /* OpenAcc/inverter_package.h:13-31 */
  const su3_soa *u;
  const su3_soa_f *u_f;
  vec3_soa *ferm_shift_temp;
  vec3_soa_f *ferm_shift_temp_f;
  int nshifts;
  vec3_soa *loc_r;
  vec3_soa *loc_h;
  vec3_soa *loc_s;
  vec3_soa *loc_p;
  vec3_soa_f *loc_r_f;
  vec3_soa_f *loc_h_f;
  vec3_soa_f *loc_s_f;
  vec3_soa_f *loc_p_f;
  vec3_soa_f *out_f;
} inverter_package;
#endif

#ifndef OSTAPLE_HAVE_REFERENCE_TYPES
typedef struct action_param_t {           /* OpenAcc/action.h:8-20 */
  double beta;
  int stout_steps;
  double stout_rho;
  int topo_action;
  double barrier;
  double width;
  char topo_file_path[20];
  int topo_stout_steps;
  double topo_rho;
} action_param;
#endif

#ifndef OSTAPLE_HAVE_REFERENCE_TYPES
typedef struct md_param_t {               /* OpenAcc/md_parameters.h:7-20 */
  int no_md;
  int gauge_scale;
  double t;
  double residue_metro;
  double expected_max_eigenvalue;
  int singlePrecMD;
  double residue_md;
  int max_cg_iterations;
  int recycleInvsForce;
  int extrapolateInvsForce;
} md_param;
#endif

/* Molecular-dynamics parameters and the integrator step sizes
 * (md_parameters.c:8-9, 57).  Weak library defaults; a host definition
 * overrides them. */
extern md_param md_parameters;
extern double deltas_Omelyan[7];

/* Stout parameters read by stout_wrapper / fermion_force_soloopenacc and the
 * stout kernels (action.h:22-23).  Weak library defaults: 2 steps of
 * rho = 0.15; a host definition overrides them. */
extern action_param act_params;
extern double gl_stout_rho, gl_topo_rho;

/* Inverter switches read by the dispatch wrappers.  The reference host
 * defines this global (Include/inverter_tricks.c); the library carries a
 * weak default {0, 0, 0.1, 10000} that a host definition overrides. */
extern inv_tricks inverter_tricks;

/* ---- runtime (replaces compile-time geometry and OpenACC data clauses) -- */
/* set_geom_glv (geometry.c:103-180) + select_init_acc_device (deviceinit.c:14-36).
 * Extents must be even.  Returns 0 on success. */
int ostaple_init(int n0, int n1, int n2, int n3);
int ostaple_finalize(void);
int ostaple_sizeh(void);
int ostaple_set_stream(void *cuda_stream);
int ostaple_synchronize(void);
int ostaple_get_error(void);
const char *ostaple_last_error(void);
void ostaple_clear_error(void);
/* `#pragma acc enter data create(p[0:bytes])` (alloc_vars.c:94-284) */
int ostaple_enter_data(const void *host, size_t bytes);
/* `#pragma acc exit data delete(p)` */
int ostaple_exit_data(const void *host);
/* `#pragma acc update device(p[0:bytes])` / `update host(...)` */
int ostaple_update_device(const void *host, size_t bytes);
int ostaple_update_host(void *host, size_t bytes);
/* acc_deviceptr(): device mirror of a registered host address, or NULL */
void *ostaple_deviceptr(const void *host);

/* Number of kernels the library has launched (graph replays count the
 * kernels they contain).  No reference counterpart. */
unsigned long long ostaple_kernel_launches(void);
/* Page-locks a host range so that update_device/update_host copies run at
 * full host-link bandwidth (cudaHostRegister).  No reference counterpart. */
int ostaple_pin_host(void *host, size_t bytes);
int ostaple_unpin_host(void *host);
/* Launch-shape autotuner of the FP32 D_oe hops (the mixed solver's block
 * size, the batched and multi-shift solvers' systems per thread).  Only
 * shapes that leave every result bit unchanged are tuned; each (kernel,
 * lattice) is timed once per process, before the solver captures its CUDA
 * graph.  enable = 0 keeps the default shapes (so does OSTAPLE_AUTOTUNE=0 in
 * the environment); enable = 2 + c forces candidate c of every tuned launch
 * (c past a kernel's candidate list means its default), which tests use to
 * check that each shape gives the same bits.  The report writes one line per tuned key (chosen
 * candidate and each candidate's microseconds) into buf (NUL-terminated,
 * truncated to len) and returns the full length.  No reference counterpart
 * (the reference's launch shapes are fixed at compile time). */
int ostaple_autotune(int enable);
/* 1 (default, unless OSTAPLE_DEVICE_LOOP=0 in the environment): the mixed
 * solver and the batched multi-shift CG run their iterations as one CUDA
 * graph launch whose loop and reliable-update decisions are taken on the
 * device (conditional graph nodes); 0: the host replays a captured chunk of
 * iterations and polls the solver's flags.  Both give the same bits.  No
 * reference counterpart. */
int ostaple_device_loop(int enable);
int ostaple_autotune_report(char *buf, int len);

/* ---- staggered Dirac operator (fermion_matrix.h:20-39) ----------------- */
/* out(even) = 1/2 sum_mu [ e^{i th} U_mu(x) in(x+mu) - e^{-i th} U_mu(x-mu)^+ in(x-mu) ] */
void acc_Deo(const su3_soa *u, vec3_soa *out, const vec3_soa *in, const double_soa *backfield);
/* the same with even and odd exchanged */
void acc_Doe(const su3_soa *u, vec3_soa *out, const vec3_soa *in, const double_soa *backfield);
/* without halo exchange (identical on one GPU) (fermion_matrix.h:29-39) */
void acc_Deo_unsafe(const su3_soa *u, vec3_soa *out, const vec3_soa *in, const double_soa *backfield);
void acc_Doe_unsafe(const su3_soa *u, vec3_soa *out, const vec3_soa *in, const double_soa *backfield);

/* out = m^2 in - D_eo D_oe in, temp1 receives D_oe in (fermion_matrix.h:95-99) */
void fermion_matrix_multiplication(const su3_soa *u, vec3_soa *out, const vec3_soa *in,
                                   vec3_soa *temp1, ferm_param *pars);
/* out = (m^2 + shift) in - D_eo D_oe in (fermion_matrix.h:101-106) */
void fermion_matrix_multiplication_shifted(const su3_soa *u, vec3_soa *out, const vec3_soa *in,
                                           vec3_soa *temp1, ferm_param *pars, double shift);

/* ---- fermion BLAS and global reductions (fermionic_utilities.h:38-123) - */
/* sum_x conj(a).b (fermionic_utilities.h:38-39).  The reference returns a
 * C99 `double complex`; a struct of two doubles is returned in the same
 * registers on x86-64 (SysV) and AArch64 (AAPCS64), so the symbol is
 * call-compatible with the reference's declaration. */
#ifndef OSTAPLE_HAVE_REFERENCE_TYPES
typedef struct ostaple_dcomplex_t { double re, im; } ostaple_dcomplex;
ostaple_dcomplex scal_prod_global(const vec3_soa *in_vect1, const vec3_soa *in_vect2);
#endif
/* the same, writing {re, im} to re_im (for FFI callers without complex types) */
void scal_prod_global_ri(const vec3_soa *in_vect1, const vec3_soa *in_vect2, double *re_im);
double real_scal_prod_global(const vec3_soa *in_vect1, const vec3_soa *in_vect2); /* :40 */
double l2norm2_global(const vec3_soa *in_vect1);                                  /* :42 */
/* real_scal_prod_global without any device allocation: its scratch (block
 * partials, ticket counter, result) is a fixed 33,920-byte static device
 * array, so it can be called where cudaMalloc cannot (in loops that must not
 * take cudaMalloc's implicit device synchronisation, or under a fixed
 * device-memory budget that forbids further allocations).  Limit: 3*sizeh <=
 * 8,388,608 complex numbers (sizeh <= 2,796,202); larger lattices get error
 * -14 and NAN.  The first call on a device looks up the array's address with
 * that device current, and should come before any stream capture.  Every
 * call shares the array: calls that overlap on the GPU race.  A NAN return
 * means this call failed (the error word says why).  No counterpart in the
 * reference. */
double ostaple_real_scal_prod_global_noalloc(const vec3_soa *in_vect1, const vec3_soa *in_vect2);
void combine_in1xfactor_plus_in2(const vec3_soa *in_vect1, const double factor,
                                 const vec3_soa *in_vect2, vec3_soa *out);        /* :48 */
void multiply_fermion_x_doublefactor(vec3_soa *in1, const double factor);         /* :55 */
void combine_add_factor_x_in2_to_in1(vec3_soa *in1, const vec3_soa *in2, double factor); /* :59 */
void combine_in1xferm_mass2_minus_in2_minus_in3(const vec3_soa *in_vect1, double ferm_mass,
                                                const vec3_soa *in_vect2, const vec3_soa *in_vect3,
                                                vec3_soa *out);                   /* :67 */
void combine_inside_loop(vec3_soa *vect_out, vec3_soa *vect_r, const vec3_soa *vect_s,
                         const vec3_soa *vect_p, const double omega);             /* :75 */
void combine_in1xferm_mass_minus_in2(const vec3_soa *in_vect1, double ferm_mass2,
                                     vec3_soa *in_vect2);                         /* :81 */
void combine_in1_minus_in2(const vec3_soa *in_vect1, const vec3_soa *in_vect2, vec3_soa *out); /* :86 */
void assign_in_to_out(const vec3_soa *in_vect1, vec3_soa *out);                   /* :90 */
void set_vec3_soa_to_zero(vec3_soa *fermion);                                     /* :94 */
void multiple_combine_in1_minus_in2x_factor_back_into_in1(vec3_soa *out, const vec3_soa *in,
                                                          const int maxiter, const int *flag,
                                                          const double *omegas);  /* :95 */
void multiple1_combine_in1_x_fact1_plus_in2_x_fact2_back_into_in1(
    vec3_soa *in1, int maxiter, const int *flag, const double *gammas, const vec3_soa *in2,
    const double *zeta_iii);                                                      /* :100 */
void combine_in1_x_fact1_minus_in2_back_into_in2(const vec3_soa *in1, double fact1,
                                                 vec3_soa *in2);                  /* :106 */
void combine_in1_minus_in2_allxfact(const vec3_soa *in1, const vec3_soa *in2, double fact,
                                    vec3_soa *out);                               /* :109 */

/* ---- single-precision twins (the reference's generated sp_*.c files) -----
 * Same meaning as the FP64 functions above on the float layouts su3_soa_f /
 * vec3_soa_f / float_soa (struct_c_def.h types with float complex elements,
 * sp_struct_c_def.h): FP32 links and vectors, FP64 scalars and FP64
 * accumulation in the global reductions; phases from ferm_param.phases_f.
 * The reference's benchmark drivers call them (deo_doe_test.c:311-342,
 * inverter_multishift_test.c:342). */
void acc_Deo_f(const su3_soa_f *u, vec3_soa_f *out, const vec3_soa_f *in, const float_soa *backfield);
void acc_Doe_f(const su3_soa_f *u, vec3_soa_f *out, const vec3_soa_f *in, const float_soa *backfield);
void acc_Deo_unsafe_f(const su3_soa_f *u, vec3_soa_f *out, const vec3_soa_f *in, const float_soa *backfield);
void acc_Doe_unsafe_f(const su3_soa_f *u, vec3_soa_f *out, const vec3_soa_f *in, const float_soa *backfield);
/* sp_fermion_matrix.c: the generator turns this file's `double` into `float` */
void fermion_matrix_multiplication_f(const su3_soa_f *u, vec3_soa_f *out, const vec3_soa_f *in,
                                     vec3_soa_f *temp1, ferm_param *pars);
void fermion_matrix_multiplication_shifted_f(const su3_soa_f *u, vec3_soa_f *out, const vec3_soa_f *in,
                                             vec3_soa_f *temp1, ferm_param *pars, float shift);
double l2norm2_global_f(const vec3_soa_f *in_vect1);
double real_scal_prod_global_f(const vec3_soa_f *in_vect1, const vec3_soa_f *in_vect2);
void set_vec3_soa_to_zero_f(vec3_soa_f *fermion);
void assign_in_to_out_f(const vec3_soa_f *in_vect1, vec3_soa_f *out);
void combine_in1xfactor_plus_in2_f(const vec3_soa_f *in_vect1, const double factor, const vec3_soa_f *in_vect2,
                                   vec3_soa_f *out);
void combine_add_factor_x_in2_to_in1_f(vec3_soa_f *in1, const vec3_soa_f *in2, double factor);
void combine_in1xferm_mass_minus_in2_f(const vec3_soa_f *in_vect1, double ferm_mass2, vec3_soa_f *in_vect2);
void combine_in1_minus_in2_f(const vec3_soa_f *in_vect1, const vec3_soa_f *in_vect2, vec3_soa_f *out);
void multiply_fermion_x_doublefactor_f(vec3_soa_f *in1, const double factor);
int ker_invert_openacc_f(const su3_soa_f *u, ferm_param *pars, vec3_soa_f *solution, const vec3_soa_f *in,
                         double res, vec3_soa_f *loc_r, vec3_soa_f *loc_h, vec3_soa_f *loc_s, vec3_soa_f *loc_p,
                         const int max_cg, double shift, int *cg_return);
int multishift_invert_f(const su3_soa_f *u, ferm_param *pars, RationalApprox *approx, vec3_soa_f *out,
                        const vec3_soa_f *in, double residuo, vec3_soa_f *loc_r, vec3_soa_f *loc_h,
                        vec3_soa_f *loc_s, vec3_soa_f *loc_p, vec3_soa_f *shiftferm, const int max_cg,
                        int *cg_return);
void recombine_shifted_vec3_to_vec3_f(const vec3_soa_f *in_shifted, const vec3_soa_f *in, vec3_soa_f *out,
                                      const RationalApprox *approx);
/* float <-> double conversions (float_double_conv.h:13-55): one vec3_soa,
 * one double_soa, or all 8 directions of a su3_soa (3 rows each) */
void convert_double_to_float_vec3_soa(const vec3_soa *d_var, vec3_soa_f *f_var);
void convert_float_to_double_vec3_soa(const vec3_soa_f *f_var, vec3_soa *d_var);
void convert_double_to_float_real_soa(const double_soa *d_var, float_soa *f_var);
void convert_float_to_double_real_soa(const float_soa *f_var, double_soa *d_var);
void convert_double_to_float_su3_soa(const su3_soa *d_var, su3_soa_f *f_var);
void convert_float_to_double_su3_soa(const su3_soa_f *f_var, su3_soa *d_var);

/* ---- solvers ------------------------------------------------------------ */
/* CG on (M^+M + shift) x = in, restarted every inverter_tricks.restartingEvery
 * iterations (inverter_full.h:20-31). */
int ker_invert_openacc(const su3_soa *u, ferm_param *pars, vec3_soa *solution, const vec3_soa *in,
                       double res, vec3_soa *loc_r, vec3_soa *loc_h, vec3_soa *loc_s,
                       vec3_soa *loc_p, const int max_cg, double shift, int *cg_return);
/* CG-M for all shifts of approx (inverter_multishift_full.h:15-27) */
int multishift_invert(const su3_soa *u, ferm_param *pars, RationalApprox *approx, vec3_soa *out,
                      const vec3_soa *in, double residuo, vec3_soa *loc_r, vec3_soa *loc_h,
                      vec3_soa *loc_s, vec3_soa *loc_p, vec3_soa *shiftferm, const int max_cg,
                      int *cg_return);
/* out = a0 in + sum_i a_i in_shifted[i] (inverter_multishift_full.h:30-33) */
/* Rational approximations r(x) = a0 + sum_i a_i/(x + b_i) (rationalapprox.h:29-53):
 * .REMEZ file names, reading and writing, rescaling of a mother
 * approximation on [lambda_min, 1] to the measured spectrum [min, max] of
 * M^+M (x -> x/(1.05 max)), the inverse renormalisation, and evaluation.
 * Host functions, exported as weak symbols so that a host program that
 * links the reference's rationalapprox.c keeps its own. */
char *rational_approx_filename(double error, int exponent_num, int exponent_den, double lambda_min);
char *rational_approx_filename_old(int approx_order, int exponent_num, int exponent_den, double lambda_min);
int rationalapprox_read(RationalApprox *rational_approx);
int rationalapprox_read_custom_nomefile(RationalApprox *rational_approx, char *nomefile);
void rationalapprox_save(const char *nomefile, RationalApprox *rational_approx);
void rescale_rational_approximation(RationalApprox *in, RationalApprox *out, double *minmax);
void renormalize_rational_approximation(RationalApprox *in, RationalApprox *out);
double rational_approx_evaluate(RationalApprox *in, double x);
/* The library's own generator of these approximations (host code, no GPU).
 * The reference generates .REMEZ files with a separate offline program over
 * GMP multiprecision (RationalApprox/rationalapprox_calc.cc:20-95,
 * Remez/alg_remez.cc); this is a new implementation in long double
 * arithmetic, with no counterpart as a library function.  It computes the
 * best relative-error approximation of x^|num/den| of order approx_order on
 * [lambda_min, 1] by the Remez exchange and writes RA_a0, RA_a, RA_b (the
 * partial fractions of r, or of 1/r for a negative exponent, poles
 * ascending), error and lambda_max = 1.  Needs 0 < |num/den| < 1.  Returns 0,
 * -3 for bad arguments, -15 when the exchange does not converge, -16 when
 * the order is so high that its error is near the rounding level. */
int ostaple_remez_approximation(RationalApprox *approx);
/* The reference driver's order loop around it: the order guessed as
 * log(goal) log(lambda_min)/19 + 2 (or fixed_order if > 0), raised by one
 * until error <= goal_error; exponent_num, exponent_den and lambda_min are
 * read from approx. */
int ostaple_remez_generate(RationalApprox *approx, double goal_error, int fixed_order);

void recombine_shifted_vec3_to_vec3(const vec3_soa *in_shifted, const vec3_soa *in, vec3_soa *out,
                                    const RationalApprox *approx);

/* Eigenvalue bounds of M^+M by power iteration (find_min_max.h:14-45):
 * loc_p / loc_p1 holds a Gaussian start vector on entry; the iteration stops
 * when the relative change of |p| is <= 1e-5.  find_min_max sets
 * minmax[0] = m^2 and minmax[1] = the largest eigenvalue. */
double ker_find_max_eigenvalue_openacc(su3_soa *u, ferm_param *pars, vec3_soa *loc_r, vec3_soa *loc_h,
                                       vec3_soa *loc_p);
double ker_find_min_eigenvalue_openacc(su3_soa *u, ferm_param *pars, vec3_soa *loc_r, vec3_soa *loc_h,
                                       vec3_soa *loc_p, double max);
void find_min_max_eigenvalue_soloopenacc(su3_soa *u, ferm_param *pars, vec3_soa *loc_r, vec3_soa *loc_h,
                                         vec3_soa *loc_p1, vec3_soa *loc_p2, double *minmax);

/* out = (m^2 + shift) in - D_eo D_oe in computed in double-float arithmetic
 * (FP32 pairs with error-free transformations, ~1e-14 relative): the
 * operator of the mixed solvers' intermediate reliable updates, exposed for
 * testing and for callers that want a near-FP64 M^+M at FP32 speed.  Needs
 * phases of 0 or pi.  No counterpart in the reference. */
int ostaple_mdagm_df(const su3_soa *u, const double_soa *phases, double mass, double shift, vec3_soa *out,
                     const vec3_soa *in);

/* Link format of the FP32 iteration of the mixed and batched solvers when
 * the library converts the FP64 links itself: fmt = 1 (default) the first
 * two rows in 16-bit fixed point (24 bytes per link, absolute error <= 2^-16;
 * the reliable updates and the FP64 closing residual keep every solution at
 * the requested FP64 residual), fmt = 0 two FP32 rows (48 bytes per link).
 * Returns the previous format.  Links passed by the caller as su3_soa_f
 * (inverter_package.u_f) are always used as given.  No reference
 * counterpart (the reference's sloppy links are FP32). */
int ostaple_set_sloppy_links(int fmt);
/* Host runs of the device-side link encoders, for tests without a GPU:
 * q[i] = the biased 16-bit word of h[i] (rint(32768 h) clamped to +-32767,
 * plus 32768); hi[i] = (float)x[i] and lo[i] = (float)(x[i] - (double)hi[i])
 * as the double-float links compute them.  No reference counterpart. */
int ostaple_q16_encode_host(const float *h, long n, unsigned *q);
int ostaple_df_split_host(const double *x, long n, float *hi, float *lo);
/* out = (m^2 + shift) in - D_eo D_oe in through the FP32 iteration kernels
 * with the current sloppy link format (FP32 in and out of the kernels, FP64
 * fields here): the operator of the FP32 iteration, exposed for testing.
 * No reference counterpart. */
int ostaple_mdagm_sloppy(const su3_soa *u, const double_soa *phases, double mass, double shift, vec3_soa *out,
                         const vec3_soa *in);

/* Mixed-precision CG: FP32 iteration, FP64 solution and reliable updates of
 * the residual when |r|^2 < inverter_tricks.mixedPrecisionDelta * max|r|^2
 * (inverter_mixedp.c:41-48).  FP32 links come from ip.u_f when set (the
 * reference's converted su3_soa_f), else from ip.u; ip's FP32/FP64 parking
 * vectors are used when set. */
int inverter_mixed_precision(inverter_package ip, ferm_param *pars, vec3_soa *solution, const vec3_soa *in,
                             double res, const int max_cg, double shift, int *cg_return);
/* Exits the process on a failure marked CONVERGENCE_CRITICAL
 * (inverter_wrappers.c:24-39). */
void convergence_messages(int conv_importance, int inverter_status);
/* Dispatches to inverter_mixed_precision or ker_invert_openacc by
 * inverter_tricks.useMixedPrecision; returns the iteration count
 * (inverter_wrappers.c:117-160). */
int inverter_wrapper(inverter_package ip, ferm_param *pars, vec3_soa *out, const vec3_soa *in, double res,
                     int max_cg, double shift, int convergence_importance);

/* ---- full-D inversion for the fermionic measurements (ferm_meas.h) ------ */
/* Solves the full staggered matrix D (out_e, out_o) = (in_e, in_o) by
 * even/odd reduction: phi_e = m in_e - D_eo in_o, out_e = (M^+M)^-1 phi_e
 * through inverter_wrapper (zero guess, CONVERGENCE_CRITICAL), out_o =
 * (in_o - D_oe out_e) / m.  phi_e and phi_o are work fields
 * (Meas/ferm_meas.c:50-71). */
void eo_inversion(inverter_package ip, ferm_param *tfermions_parameters, double res, int max_cg, vec3_soa *in_e,
                  vec3_soa *in_o, vec3_soa *out_e, vec3_soa *out_o, vec3_soa *phi_e, vec3_soa *phi_o);

/* ---- stout smearing (stouting.h:13-44) ---------------------------------- */
/* U' = exp(-Q_A) U with Q_A = rho/C_0 TA(U C), C the tree-level-Symanzik
 * weighted staples; writes uprime (rows 0,1), local_staples (if not NULL)
 * and tipdot = Q_A; rho = gl_stout_rho (gl_topo_rho if istopo). */
void stout_isotropic(const su3_soa *u, su3_soa *uprime, su3_soa *local_staples, su3_soa *auxiliary,
                     tamat_soa *tipdot, const int istopo);
/* act_params.stout_steps levels into tstout_conf_acc_arr[8*level] (stouting.c:27-72) */
void stout_wrapper(const su3_soa *tconf_acc, su3_soa *tstout_conf_acc_arr, const int istopo);
/* tu_out = exp(-QA) tu (stouting.c:136-165) */
void exp_minus_QA_times_conf(const su3_soa *tu, const tamat_soa *QA, su3_soa *tu_out, su3_soa *exp_aux);
/* Lambda of the stout chain rule (stouting.c:516-546) */
void compute_lambda(thmat_soa *L, const su3_soa *SP, const su3_soa *U, const tamat_soa *QA, su3_soa *TMP);
/* S: Sigma' in, Sigma out (stouting.c:1175-1302) */
void compute_sigma(const thmat_soa *L, const su3_soa *U, su3_soa *S, const tamat_soa *QA, su3_soa *TMP,
                   const int istopo);
/* staples, Q_A, Lambda and Sigma for one level (fermion_force.c:52-162) */
void compute_sigma_from_sigma_prime_backinto_sigma_prime(su3_soa *Sigma, thmat_soa *Lambda, tamat_soa *QA,
                                                         const su3_soa *U, su3_soa *TMP, const int istopo);
void set_su3_soa_to_zero(su3_soa *matrix);                    /* su3_utilities.c:43-55 */
void set_tamat_soa_to_zero(tamat_soa *matrix);                /* fermion_force_utilities.c:16-28 */

/* ---- rational fermion force (fermion_force_utilities.h:204-240) ---------- */
/* aux_u += RA_a[iter] (D_oe X)(x+mu) (x) X(x)^+ on even, the mirror on odd links */
void direct_product_of_fermions_into_auxmat(const vec3_soa *loc_s, const vec3_soa *loc_h, su3_soa *aux_u,
                                            const RationalApprox *approx, int iter);
/* the outer products of all approx_md shifts (fermion_force_utilities.c:183-201) */
void ker_openacc_compute_fermion_force(const su3_soa *u, su3_soa *aux_u, const vec3_soa *in_shiftmulti,
                                       vec3_soa *loc_s, vec3_soa *loc_h, ferm_param *tpars);
/* pseudo_ipdot += e^{i theta} auxmat (fermion_force_utilities.c:123-153) */
void multiply_backfield_times_force(ferm_param *tpars, const su3_soa *auxmat, su3_soa *pseudo_ipdot);
/* ipdot -= TA(U auxmat) (fermion_force_utilities.c:95-121) */
void multiply_conf_times_force_and_take_ta_nophase(const su3_soa *u, const su3_soa *auxmat, tamat_soa *ipdot);
/* the whole force of all flavours through the stout levels (fermion_force.h:23-36) */
void fermion_force_soloopenacc(su3_soa *tconf_acc, su3_soa *tstout_conf_acc_arr, su3_soa *gl3_aux,
                               tamat_soa *tipdot_acc, ferm_param *tfermion_parameters, int tNDiffFlavs,
                               const vec3_soa *ferm_in_acc, double res, su3_soa *taux_conf_acc,
                               vec3_soa *tferm_shiftmulti_acc, inverter_package ipt, const int max_cg);
/* multi-shift dispatch; with inverter_tricks.singlePInvAccelMultiInv every
 * shift is then refined by inverter_wrapper (inverter_wrappers.c:41-114) */
int inverter_multishift_wrapper(inverter_package ip, ferm_param *pars, RationalApprox *approx, vec3_soa *out,
                                const vec3_soa *in, double res, int max_cg, int convergence_importance);

/* ---- pure-gauge tree-level Symanzik HMC (ipdot_gauge.h, plaquettes.h,
 * rectangles.h, su3_utilities.h, su3_measurements.h, md_integrator.h,
 * md_parameters.h, random_assignement.h) ------------------------------------
 * Staples are dS/dU summed over the paths that close link (x, mu):
 * C_ZERO = 5/3 times the plaquette staples, C_ONE = -1/12 times the 2x1
 * rectangle staples of types A, B, C; each function ADDS its part. */
void calc_loc_staples_nnptrick_all(const su3_soa *u, su3_soa *loc_stap);                  /* plaquettes.h:16 */
void calc_loc_improved_staples_typeA_nnptrick_all(const su3_soa *u, su3_soa *loc_stap);   /* rectangles.h:40 */
void calc_loc_improved_staples_typeB_nnptrick_all(const su3_soa *u, su3_soa *loc_stap);   /* rectangles.h:42 */
void calc_loc_improved_staples_typeC_nnptrick_all(const su3_soa *u, su3_soa *loc_stap);   /* rectangles.h:44 */
/* tipdot = TA(U loc_stap) (su3_utilities.h:41) */
void conf_times_staples_ta_part(const su3_soa *u, const su3_soa *loc_stap, tamat_soa *tipdot);
/* the whole gauge force: local_staples = dS/dU (if not NULL), tipdot = TA(U dS/dU)
 * (ipdot_gauge.h, ipdot_gauge.c:361-426) */
void calc_ipdot_gauge_soloopenacc(const su3_soa *tconf_acc, su3_soa *local_staples, tamat_soa *tipdot);
/* sum over sites and planes mu < nu of Re tr of the plaquettes / of the 2x1
 * and 1x2 rectangles (su3_measurements.h:14, rectangles.h:80); the parking
 * arguments are not used */
double calc_plaquette_soloopenacc(su3_soa *tconf_acc, su3_soa *local_plaqs, dcomplex_soa *tr_local_plaqs);
double calc_rettangolo_soloopenacc(const su3_soa *tconf_acc, su3_soa *local_plaqs, dcomplex_soa *tr_local_plaqs);
/* sum over the links of direction mu (0..7) of 1/2 tr P^2 (su3_measurements.h:11) */
double calc_momenta_action(const thmat_soa *mom, double_soa *tr_local, const int mu);
/* mom -= i factor[id] ipdot (complex entries), += on the real diagonals (su3_utilities.h:53) */
void mom_sum_mult(thmat_soa *mom, const tamat_soa *ipdot, const double *factor, int id_factor);
/* U = exp(i tdelta[id] P) U, rows 0-1 reunitarised (su3_utilities.h:58) */
void mom_exp_times_conf_soloopenacc(su3_soa *tconf_acc, const thmat_soa *tmomenta, const double *tdelta,
                                    int id_delta);
/* deltas_Omelyan from md_params and act_params.beta (md_parameters.h:25) */
void initialize_md_global_variables(md_param md_params);
/* one gauge multistep of the 2MN integrator with md_parameters.gauge_scale
 * substeps and the steps in deltas_Omelyan (md_integrator.h:14) */
void multistep_2MN_gauge(su3_soa *tconf_acc, su3_soa *local_staples, tamat_soa *tipdot, thmat_soa *tmomenta);
/* Gaussian momenta into the HOST array mom8 (8 thmat_soa), as the
 * reference's (random_assignement.h:26); the deviates come from the
 * library's counter-based generator seeded by ostaple_set_momenta_seed (no
 * reference counterpart), not from the reference's dSFMT stream */
void generate_Momenta_gauss(thmat_soa *mom8);
void ostaple_set_momenta_seed(unsigned long long seed);

/* Link generator (no reference counterpart): ntraj pure-gauge tree-level
 * Symanzik HMC trajectories of length traj_len with the reference's
 * integrator (no_md steps, each two gauge multisteps of gauge_scale 2MN
 * substeps: md_integrator.c:347-376, 502-742 without fermions), Metropolis
 * on exp(-delta S) when metropolis != 0.  Momenta come from the counter-based
 * generator (seed, trajectory first_traj + k).  precision 0: FP64 molecular
 * dynamics; 1: FP32 molecular dynamics (force, kicks and link updates) from
 * the FP64 links, the result reunitarised in FP64, actions and Metropolis in
 * FP64.  plaquette[k] (<Re tr P>/3 after trajectory k) and delta_s[k] may be
 * NULL.  Returns 0 or an error code. */
int ostaple_pure_gauge_hmc(su3_soa *u, double beta, int ntraj, int no_md, int gauge_scale, double traj_len,
                           unsigned long long seed, int first_traj, int precision, int metropolis, int *accepted,
                           double *plaquette, double *delta_s);
/* Gaussian momenta on the device from (seed, stream); the same counter-based
 * generator the host field helpers use */
int ostaple_gauge_momenta(thmat_soa *mom, unsigned long long seed, unsigned long long stream);
/* Fills a vec3_soa on the device with Gaussian complex numbers (real and
 * imaginary parts of variance 1/2, as generate_vec3_soa_gauss,
 * random_assignement.c:58-92) from the counter-based generator (seed,
 * stream): element k takes the Box-Muller pair k, the same numbers as the
 * host field helpers.  No reference counterpart (the reference draws on the
 * host). */
int ostaple_gaussian_vec3(vec3_soa *v, unsigned long long seed, unsigned long long stream);
/* plaquette and rectangle sums and the action -beta/3 (C_ZERO P + C_ONE R) */
int ostaple_gauge_action(const su3_soa *u, double beta, double *plaq_sum, double *rect_sum, double *action);

/* ---- RHMC trajectory ------------------------------------------------------ */
/* the molecular dynamics with fermions (md_integrator.h:17-32):
 *   F(d0) [G F(d1) G F(d2)]^(no_md-1) G F(d1) G F(d0)
 * with F the fermion force of all flavours (fermion_force_soloopenacc, then
 * mom_sum_mult) and G multistep_2MN_gauge; steps from deltas_Omelyan and
 * md_parameters.  local_sums is not used. */
void multistep_2MN_SOLOOPENACC(tamat_soa *tipdot_acc, su3_soa *tconf_acc, su3_soa *tstout_conf_acc_arr,
                               su3_soa *tauxbis_conf_acc, su3_soa *taux_conf_acc, ferm_param *tfermions_parameters,
                               int tNDiffFlavs, vec3_soa *ferm_in_acc, vec3_soa *tferm_shiftmulti_acc,
                               inverter_package ip, thmat_soa *tmomenta, dcomplex_soa *local_sums, double res,
                               const int max_cg);
/* One RHMC update with explicit arguments (the reference's
 * UPDATE_SOLOACC_UNOSTEP_VERSATILE, update_versatile.c:44-665, reads them
 * from its globals): Gaussian momenta and pseudofermions phi from the
 * counter-based generator (seed, traj); eigenvalue bounds of M^+M on the
 * smeared links and approx_fi/md/li rescaled from the mothers in fpars;
 * chi = r_fi phi; 2MN molecular dynamics of no_md steps x gauge_scale
 * substeps over traj_len with beta; phi' = r_li chi; Metropolis on
 * dS = dH (when metropolis != 0; a rejected update restores u).  Solvers
 * follow inverter_tricks.  action[6] (may be NULL): -S_gauge, S_mom, S_ferm
 * before, then after.  No reference counterpart as a function. */
int ostaple_rhmc_trajectory(su3_soa *u, ferm_param *fpars, int nflavs, double beta, int no_md, int gauge_scale,
                            double traj_len, double res_metro, double res_md, int max_cg, unsigned long long seed,
                            int traj, int metropolis, int *accepted, double *delta_s, double *action);

/* ---- configuration files (io.h:17-89; host memory, no GPU needed) ---------
 * On one process the global lattice is the local one: conf is a host
 * su3_soa[8] of the lattice given to ostaple_init.  ASCII: a header line
 * "nx ny nz nt beta mass nflavs traj" (beta from act_params; mass and the
 * flavour count from ostaple_io_ferm_mass / ostaple_io_nflavs, 0 by
 * default), then every link as 3 rows of "(re, im)" pairs printed %.18lf, in
 * the order direction 2*mu+parity, half-lattice index; with back_phases the
 * links are written times the sign of their staggered phase, and reading
 * undoes a determinant of -1.  ILDG: LIME records "ildg-format" (XML with
 * lx..lt), "MD_traj", "input-file" (input_file_str), "ildg-binary-data"
 * (big-endian doubles, t z y x with x fastest, directions x y z t, 3x3
 * row-major complex) and "ildg-data-lfn".  Return 0 on success, 1 when the
 * file cannot be opened for reading, 2 on other errors. */
int print_su3_soa_ASCII(global_su3_soa *const conf, const char *nomefile, int conf_id_iter, double_soa *back_phases);
int read_su3_soa_ASCII(global_su3_soa *conf, const char *nomefile, int *conf_id_iter);
int print_su3_soa_ildg_binary(global_su3_soa *conf, const char *nomefile, int conf_id_iter);
int read_su3_soa_ildg_binary(global_su3_soa *conf, const char *nomefile, int *conf_id_iter);
extern char input_file_str[300 * 500];        /* setting_file_parser.h:11 */
extern double ostaple_io_ferm_mass;            /* no reference counterpart */
extern int ostaple_io_nflavs;                  /* no reference counterpart */

/* Mixed-precision CG that iterates until the FP64 true residual
 * sqrt(|b - (M^+M + shift) x|^2 / |b|^2) is <= res (or max_iter), with a
 * reliable update every `reliable_every` iterations, or (reliable_every = 0)
 * when |r|^2 < delta_frac * max|r|^2 since the last one (delta_frac <= 0:
 * inverter_tricks.mixedPrecisionDelta).  Reports iterations, the final FP64
 * true residual and the number of reliable updates.  Extends
 * inverter_mixed_precision; no reference counterpart. */
int ostaple_invert_mixed(const su3_soa *u, const double_soa *phases, double mass, double shift,
                         vec3_soa *solution, const vec3_soa *in, double res, int max_iter, int reliable_every,
                         double delta_frac, int *iters, double *true_res, int *n_reliable);

/* ---- batched solvers (no reference counterpart: the reference solves one
 * right-hand side at a time, update_versatile.c:258-275) --------------------- */
/* nsys solves (M^+M + shifts[k]) x_k = b_k sharing the links: every FP32
 * Dslash reads each link once for a batch of up to 8 systems; each system
 * keeps its own scalars and reliable updates and reaches its own FP64 true
 * residual <= res.  solutions/sources: nsys consecutive vec3_soa; shifts may
 * be NULL (all zero).  delta_frac <= 0 selects 1e-4. */
int ostaple_invert_mixed_batch(const su3_soa *u, const double_soa *phases, double mass, int nsys,
                               const double *shifts, vec3_soa *solutions, const vec3_soa *sources, double res,
                               int max_iter, double delta_frac, int *iters, double *true_res, int *n_reliable);
/* all shifts of approx for nrhs (1..4) right-hand sides: an FP32 multi-shift
 * CG for all right-hand sides together, then every (rhs, shift) system refined
 * by the batched mixed solver to an FP64 true residual <= res.  solutions:
 * nrhs*approx_order vec3_soa, index rhs*order + shift; iters_cgm[nrhs],
 * iters_refine[nrhs*order], true_res[nrhs*order] may be NULL. */
int ostaple_multishift_batch(const su3_soa *u, const double_soa *phases, double mass, const RationalApprox *approx,
                             int nrhs, const vec3_soa *sources, vec3_soa *solutions, double res, int max_iter,
                             double delta_frac, int *iters_cgm, int *iters_refine, double *true_res);

/* ---- learned preconditioner (no reference counterpart) -------------------
 * A linear gauge-covariant network of 4 layers (even -> odd -> even -> odd ->
 * even), 8 channels per colour: each layer transports its input channels
 * along the 8 staggered hops (links and staggered signs) and mixes
 * hops x channels with real weights W[layer][64][8] on the BF16 tensor cores
 * (FP32 accumulation).  Weights are FP32 masters, 4*64*8 floats, row-major
 * [layer][hop*8 + in_channel][out_channel].  Phases must be 0 or pi. */
int ostaple_net_init(unsigned seed, double scale);                 /* uniform in [-scale, scale] */
/* Weight files (host only, no GPU needed): magic "OSTNETWT", version 1,
 * shape 4x64x8, FP32 weights, FNV-1a 64-bit checksum of header and weights.
 * Load returns -17 (cannot open), -18 (truncated, wrong magic, version or
 * shape) or -19 (checksum mismatch) and leaves w untouched on error. */
int ostaple_net_weights_save(const char *path, const float *w);
int ostaple_net_weights_load(const char *path, float *w);
/* Failure-path self-test of the tensor-core kernels' bounded mbarrier wait:
 * with signal = 0 nothing arrives, the wait gives up after its poll limit,
 * the error word is set and -13 is returned (error state set, the context
 * stays usable); with signal = 1 it completes and 0 is returned. */
int ostaple_selftest_bounded_wait(int signal);
int ostaple_net_set_weights(const float *w);
int ostaple_net_get_weights(float *w);
/* out = N(in), in/out FP64 vec3_soa on even sites (computed in BF16/FP32) */
int ostaple_net_apply(const su3_soa *u, const double_soa *phases, const vec3_soa *in, vec3_soa *out);
/* With A = M^+M + shift on even sites (mass, shift as in
 * ostaple_invert_learned): loss = |A (N(source) - target)|^2 / |source|^2,
 * the residual that the preconditioned source leaves when target solves
 * A target = source, and dloss/dW into dw[4*64*8] */
int ostaple_net_gradient(const su3_soa *u, const double_soa *phases, double mass, double shift,
                         const vec3_soa *source, const vec3_soa *target, float *dw, double *loss);
/* full-batch Adam on npairs (source, solution) pairs of A, one step per
 * epoch; loss_history[epochs] receives the mean of the pairs' losses */
int ostaple_net_train(const su3_soa *u, const double_soa *phases, double mass, double shift, int npairs,
                      const vec3_soa *sources, const vec3_soa *solutions, int epochs, double lr,
                      double *loss_history);
/* flexible CG on (M^+M + shift) x = b preconditioned by the network, FP32
 * iteration with FP64 reliable updates, until the FP64 true residual is
 * <= res; if it does not converge within max_iter, or its residual sets no
 * new minimum for 500 iterations, the plain mixed-precision CG finishes the
 * solve and *used_fallback is set to 1 */
int ostaple_invert_learned(const su3_soa *u, const double_soa *phases, double mass, double shift,
                           vec3_soa *solution, const vec3_soa *in, double res, int max_iter, int *iters,
                           double *true_res, int *used_fallback);

#ifdef __cplusplus
}
#endif

#endif /* OSTAPLE_GB300_H_ */
