/* ref_harness.c -- flat C entry points around the reference's OWN compiled
 * double-precision hot-path sources, for use as a test oracle only.
 *
 * This file is linked with the UNMODIFIED reference sources (compiled from
 * where they lie, see oracle/Makefile.ref) into oracle/_ref/libref_<dims>.so,
 * one library per lattice size because the reference fixes the lattice at
 * compile time (src/OpenAcc/geometry.h:28, src/Mpi/geometry_multidev.h:78-85).
 * It supplies the globals the reference's host program would normally define
 * and wraps the structured calls into pointer-only signatures that ctypes can
 * drive from numpy buffers.  Nothing in the product links or loads this.
 *
 * Buffers follow the reference SoA layouts exactly:
 *   vec3_soa  = 3 x sizeh complex double         (struct_c_def.h:16-20)
 *   su3_soa   = 3 rows x vec3_soa                (struct_c_def.h:37-44)
 *   links     = su3_soa[8], index 2*mu+parity    (geometry_multidev.h:284-296)
 *   phases    = double_soa[8]                    (backfield.c:20-187)
 *   tamat_soa = c01,c02,c12 complex + ic00,ic11  (struct_c_def.h:47-53)
 *   thmat_soa = c01,c02,c12 complex + rc00,rc11  (struct_c_def.h:54-60)
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../Include/common_defines.h"
#include "../Mpi/multidev.h"
#include "./action.h"
#include "./geometry.h"
#include "./struct_c_def.h"
#include "./fermion_matrix.h"
#include "./fermionic_utilities.h"
#include "./inverter_full.h"
#include "./inverter_multishift_full.h"
#include "./inverter_package.h"
#include "./find_min_max.h"
#include "../RationalApprox/rationalapprox.h"
#include "./stouting.h"
#include "./fermion_force.h"
#include "./fermion_force_utilities.h"
#include "./backfield.h"
#include "./backfield_parameters.h"
#include "./su3_utilities.h"
#include "./plaquettes.h"
#include "./md_parameters.h"
#include "../Include/debug.h"
#include "../Include/inverter_tricks.h"
#include "../Include/fermion_parameters.h"
#include "../DbgTools/dbgtools.h"
#include "./su3_measurements.h"
#include "./ipdot_gauge.h"
#include "./rectangles.h"
#include "./md_parameters.h"
#include "./md_integrator.h"
#include "./alloc_settings.h"
#include "./io.h"
#include "../Include/setting_file_parser.h"
#include "./sp_struct_c_def.h"
#include "./sp_alloc_vars.h"

/* ---- globals a reference host program defines (main.c / alloc_vars.c) ---- */
int verbosity_lv = 0;
action_param act_params;
dev_info devinfo;
int multishift_invert_iterations;
su3_soa *auxbis_conf_acc, *glocal_staples;
tamat_soa *gipdot, *aux_ta, *ipdot_f_old;
thmat_soa *aux_th;
su3_soa_f *conf_acc_f;
vec3_soa_f *ferm_shiftmulti_acc_f, *aux1_f;
debug_settings_t debug_settings;
md_param md_parameters;
int md_dbg_print_count, md_diag_count_fermion, ipdot_f_reset, nMdInversionPerformed;

tamat_soa *ipdot_g_old;
char input_file_str[MAXLINES * MAXLINELENGTH];
ferm_param *fermions_parameters;
int ipdot_g_reset, md_diag_count_gauge;
/* the benchmark drivers' timing container (test_and_benchmarks.h:31-44) */
typedef struct { double t[16]; int count; } harness_md_times;
harness_md_times gauge_mdtimes;

/* stubs for diagnostics and for parts the wrapped paths never reach at
 * verbosity 0 (the topological force is off: act_params.topo_action = 0) */
void dbg_print_su3_soa(su3_soa *const conf, const char *n, int i) {}
void dbgprint_gl3_soa(su3_soa *const conf, const char *n, int i) {}
void print_tamat_soa(tamat_soa *const t, const char *n) {}
void print_thmat_soa(thmat_soa *const t, const char *n) {}
void print_gl3_soa_wrapper(const su3_soa *t, const char *n) {}
void print_tamat_soa_wrapper(const tamat_soa *t, const char *n) {}
void print_thmat_soa_wrapper(const thmat_soa *t, const char *n) {}
void calc_ipdot_topo(const su3_soa *const u, su3_soa *const s, su3_soa *a, su3_soa *const b,
                     tamat_soa *const ip) {}
void convert_double_to_float_su3_soa(const su3_soa *d, su3_soa_f *f) {}

/* The double-precision branch of the reference's inverter_multishift_wrapper
 * (inverter_wrappers.c:41-114 with singlePInvAccelMultiInv = 0): one call of
 * the reference's multishift_invert with the package's work vectors.
 * inverter_wrappers.c itself is not compiled here because it needs the
 * generated single-precision sources. */
int inverter_multishift_wrapper(inverter_package ip, ferm_param *pars, RationalApprox *approx,
                                vec3_soa *out, const vec3_soa *in, double res, int max_cg, int ci)
{
  int cg = 0;
  multishift_invert(ip.u, pars, approx, out, in, res, ip.loc_r, ip.loc_h, ip.loc_s, ip.loc_p,
                    ip.ferm_shift_temp, max_cg, &cg);
  return cg;
}

static void *xalloc(size_t n)
{
  void *p = NULL;
  if (posix_memalign(&p, 128, n)) { fprintf(stderr, "ref_harness: OOM\n"); exit(2); }
  memset(p, 0, n);
  return p;
}

/* ---- geometry ---- */
int ref_sizeh(void) { return sizeh; }
void ref_dims(int *d) { d[0] = nd0; d[1] = nd1; d[2] = nd2; d[3] = nd3; }

void ref_setup(int verbosity)
{
  verbosity_lv = verbosity;
  devinfo.myrank = 0; devinfo.nranks = 1;
  geom_par.gnx = nd0; geom_par.gny = nd1; geom_par.gnz = nd2; geom_par.gnt = nd3;
  geom_par.xmap = 0; geom_par.ymap = 1; geom_par.zmap = 2; geom_par.tmap = 3;
  set_geom_glv(&geom_par);
  compute_nnp_and_nnm_openacc();
  inverter_tricks.restartingEvery = 10000;
  inverter_tricks.useMixedPrecision = 0;
  inverter_tricks.mixedPrecisionDelta = 0.1;
  inverter_tricks.singlePInvAccelMultiInv = 0;
  act_params.stout_steps = 2;
  act_params.stout_rho = 0.15;
  gl_stout_rho = 0.15;
}

void ref_set_restart(int every) { inverter_tricks.restartingEvery = every; }

/* staggered phases + APBC (+ optional imaginary chemical potential), no B/E. */
void ref_calc_phases(double *phases, double im_chem_pot, double charge)
{
  bf_param bf;
  memset(&bf, 0, sizeof(bf));
  calc_u1_phases((double_soa *)phases, bf, im_chem_pot, charge);
}

/* ---- Dirac operator ---- */
void ref_Deo(const double *u, double *out, const double *in, const double *ph)
{ acc_Deo((const su3_soa *)u, (vec3_soa *)out, (const vec3_soa *)in, (const double_soa *)ph); }

void ref_Doe(const double *u, double *out, const double *in, const double *ph)
{ acc_Doe((const su3_soa *)u, (vec3_soa *)out, (const vec3_soa *)in, (const double_soa *)ph); }

static void make_fp(ferm_param *fp, double *ph, double mass)
{
  memset(fp, 0, sizeof(*fp));
  fp->ferm_mass = mass;
  fp->phases = (double_soa *)ph;
}

void ref_mdagm_shifted(const double *u, double *out, const double *in, double *temp,
                       double *ph, double mass, double shift)
{
  ferm_param fp; make_fp(&fp, ph, mass);
  fermion_matrix_multiplication_shifted((const su3_soa *)u, (vec3_soa *)out, (const vec3_soa *)in,
                                        (vec3_soa *)temp, &fp, shift);
}

/* ---- BLAS / reductions ---- */
double ref_l2norm2(const double *v) { return l2norm2_global((const vec3_soa *)v); }
double ref_real_scal_prod(const double *a, const double *b)
{ return real_scal_prod_global((const vec3_soa *)a, (const vec3_soa *)b); }
void ref_scal_prod(const double *a, const double *b, double *re_im)
{
  d_complex z = scal_prod_global((const vec3_soa *)a, (const vec3_soa *)b);
  re_im[0] = creal(z); re_im[1] = cimag(z);
}

/* ---- single-shift CG (inverter_full.c:19-132) ---- */
int ref_cg(const double *u, double *ph, double mass, double *solution, const double *in,
           double res, int max_cg, double shift, int *cg_out)
{
  size_t vb = sizeof(vec3_soa);
  vec3_soa *r = xalloc(vb), *h = xalloc(vb), *s = xalloc(vb), *p = xalloc(vb);
  ferm_param fp; make_fp(&fp, ph, mass);
  int st = ker_invert_openacc((const su3_soa *)u, &fp, (vec3_soa *)solution, (const vec3_soa *)in,
                              res, r, h, s, p, max_cg, shift, cg_out);
  free(r); free(h); free(s); free(p);
  return st;
}

/* ---- eigenvalue bounds (find_min_max.c:21-117) ---- */
void ref_find_min_max(const double *u, double *ph, double mass, double *p1, double *r, double *minmax)
{
  size_t vb = sizeof(vec3_soa);
  vec3_soa *h = xalloc(vb), *p2 = xalloc(vb);
  ferm_param fp; make_fp(&fp, ph, mass);
  find_min_max_eigenvalue_soloopenacc((su3_soa *)u, &fp, (vec3_soa *)r, h, (vec3_soa *)p1, p2, minmax);
  free(h); free(p2);
}

double ref_find_min(const double *u, double *ph, double mass, double *p, double *r, double max)
{
  size_t vb = sizeof(vec3_soa);
  vec3_soa *h = xalloc(vb);
  ferm_param fp; make_fp(&fp, ph, mass);
  double mn = ker_find_min_eigenvalue_openacc((su3_soa *)u, &fp, (vec3_soa *)r, h, (vec3_soa *)p, max);
  free(h);
  return mn;
}

/* ---- rational approximations (rationalapprox.c:83-236) ---- */
int ref_ra_read(const char *path, RationalApprox *ra) { return rationalapprox_read_custom_nomefile(ra, (char *)path); }
void ref_ra_save(const char *path, RationalApprox *ra) { rationalapprox_save(path, ra); }
void ref_ra_rescale(RationalApprox *in, RationalApprox *out, double *minmax) { rescale_rational_approximation(in, out, minmax); }
void ref_ra_renormalize(RationalApprox *in, RationalApprox *out) { renormalize_rational_approximation(in, out); }
double ref_ra_evaluate(RationalApprox *in, double x) { return rational_approx_evaluate(in, x); }
void ref_ra_filename(double error, int num, int den, double lmin, char *out64)
{
  char *n = rational_approx_filename(error, num, den, lmin);
  strncpy(out64, n, 63); out64[63] = 0; free(n);
}

/* ---- multi-shift CG (inverter_multishift_full.c:23-252) ---- */
int ref_cgm(const double *u, double *ph, double mass, int order, double a0, const double *a,
            const double *b, double *out, const double *in, double res, int max_cg, int *cg_out)
{
  size_t vb = sizeof(vec3_soa);
  vec3_soa *r = xalloc(vb), *h = xalloc(vb), *s = xalloc(vb), *p = xalloc(vb);
  vec3_soa *sf = xalloc(vb * (size_t)order);
  ferm_param fp; make_fp(&fp, ph, mass);
  RationalApprox ra; memset(&ra, 0, sizeof(ra));
  ra.approx_order = order; ra.RA_a0 = a0;
  for (int i = 0; i < order; i++) { ra.RA_a[i] = a[i]; ra.RA_b[i] = b[i]; }
  int st = multishift_invert((const su3_soa *)u, &fp, &ra, (vec3_soa *)out, (const vec3_soa *)in,
                             res, r, h, s, p, sf, max_cg, cg_out);
  free(r); free(h); free(s); free(p); free(sf);
  return st;
}

void ref_recombine(const double *xs, const double *in, double *out, int order, double a0,
                   const double *a)
{
  RationalApprox ra; memset(&ra, 0, sizeof(ra));
  ra.approx_order = order; ra.RA_a0 = a0;
  for (int i = 0; i < order; i++) ra.RA_a[i] = a[i];
  recombine_shifted_vec3_to_vec3((const vec3_soa *)xs, (const vec3_soa *)in, (vec3_soa *)out, &ra);
}

/* ---- stout smearing (stouting.c:36-165) ---- */
void ref_stout_isotropic(const double *u, double *uprime, double rho)
{
  gl_stout_rho = rho;
  su3_soa *stap = xalloc(8 * sizeof(su3_soa));
  su3_soa *aux = xalloc(8 * sizeof(su3_soa));
  tamat_soa *ta = xalloc(8 * sizeof(tamat_soa));
  stout_isotropic((const su3_soa *)u, (su3_soa *)uprime, stap, aux, ta, 0);
  free(stap); free(aux); free(ta);
}

/* the staples times C_ZERO that stout uses (plaquettes.c:196-259) */
void ref_staples(const double *u, double *stap)
{
  set_su3_soa_to_zero((su3_soa *)stap);
  calc_loc_staples_nnptrick_all_onlyferms((const su3_soa *)u, (su3_soa *)stap);
}

/* Q_A = rho/C_ZERO * TA(U*C) (su3_utilities.c:210-239) */
void ref_rho_ta(const double *u, const double *stap, double *qa, double rho)
{
  gl_stout_rho = rho;
  RHO_times_conf_times_staples_ta_part((const su3_soa *)u, (const su3_soa *)stap, (tamat_soa *)qa, 0);
}

/* ---- fermion force pieces (fermion_force_utilities.c:30-201) ---- */
void ref_force_outer_products(const double *u, double *aux_u, const double *xs, double *ph,
                              double mass, int order, const double *a)
{
  size_t vb = sizeof(vec3_soa);
  vec3_soa *s = xalloc(vb), *h = xalloc(vb);
  ferm_param fp; make_fp(&fp, ph, mass);
  fp.approx_md.approx_order = order;
  for (int i = 0; i < order; i++) fp.approx_md.RA_a[i] = a[i];
  ker_openacc_compute_fermion_force((const su3_soa *)u, (su3_soa *)aux_u, (const vec3_soa *)xs,
                                    s, h, &fp);
  free(s); free(h);
}

void ref_backfield_times_force(double *ph, const double *auxmat, double *pseudo_ipdot)
{
  ferm_param fp; make_fp(&fp, ph, 0.0);
  multiply_backfield_times_force(&fp, (const su3_soa *)auxmat, (su3_soa *)pseudo_ipdot);
}

/* Sigma' -> Sigma through one stout level (fermion_force.c:52-162) */
void ref_sigma_prime_to_sigma(double *sigma, const double *u, double rho)
{
  gl_stout_rho = rho;
  thmat_soa *lam = xalloc(8 * sizeof(thmat_soa));
  tamat_soa *qa = xalloc(8 * sizeof(tamat_soa));
  su3_soa *tmp = xalloc(8 * sizeof(su3_soa));
  compute_sigma_from_sigma_prime_backinto_sigma_prime((su3_soa *)sigma, lam, qa, (const su3_soa *)u,
                                                      tmp, 0);
  free(lam); free(qa); free(tmp);
}

void ref_conf_times_force_ta(const double *u, const double *auxmat, double *ipdot)
{
  multiply_conf_times_force_and_take_ta_nophase((const su3_soa *)u, (const su3_soa *)auxmat,
                                                (tamat_soa *)ipdot);
}

void ref_set_tamat_zero(double *t) { set_tamat_soa_to_zero((tamat_soa *)t); }

/* ---- stout chain pieces, one by one (stouting.c:136-165, 516-546, 1175-1302) ---- */
void ref_exp_times_conf(const double *u, const double *qa, double *uout)
{
  su3_soa *aux = xalloc(8 * sizeof(su3_soa));
  exp_minus_QA_times_conf((const su3_soa *)u, (const tamat_soa *)qa, (su3_soa *)uout, aux);
  free(aux);
}

void ref_lambda(double *lam, const double *sp, const double *u, const double *qa)
{
  su3_soa *tmp = xalloc(8 * sizeof(su3_soa));
  compute_lambda((thmat_soa *)lam, (const su3_soa *)sp, (const su3_soa *)u, (const tamat_soa *)qa, tmp);
  free(tmp);
}

void ref_sigma(const double *lam, const double *u, double *s, const double *qa, double rho)
{
  gl_stout_rho = rho;
  su3_soa *tmp = xalloc(8 * sizeof(su3_soa));
  compute_sigma((const thmat_soa *)lam, (const su3_soa *)u, (su3_soa *)s, (const tamat_soa *)qa, tmp, 0);
  free(tmp);
}

/* the parking globals stout_wrapper works in (alloc_vars.c) */
static void stout_globals(int alloc)
{
  if (alloc) {
    auxbis_conf_acc = xalloc(8 * sizeof(su3_soa));
    glocal_staples = xalloc(8 * sizeof(su3_soa));
    gipdot = xalloc(8 * sizeof(tamat_soa));
  } else {
    free(auxbis_conf_acc); free(glocal_staples); free(gipdot);
    auxbis_conf_acc = glocal_staples = NULL; gipdot = NULL;
  }
}

/* act_params.stout_steps levels of stout smearing (stouting.c:27-72) */
void ref_stout_wrapper(const double *u, double *levels, int steps, double rho)
{
  act_params.stout_steps = steps;
  gl_stout_rho = rho;
  stout_globals(1);
  stout_wrapper((const su3_soa *)u, (su3_soa *)levels, 0);
  stout_globals(0);
}

/* The whole rational fermion force of one flavour through the stout levels,
 * by the reference's own fermion_force_soloopenacc (fermion_force.c:166-320):
 * nps pseudofermions phi[nps], the approximation (order, a, b) as approx_md,
 * multi-shift solves to res.  ipdot receives the force (tamat_soa[8]). */
void ref_fermion_force(const double *u, double *levels, double *ipdot, double *ph, double mass, int nps,
                       int order, const double *a, const double *b, const double *phi, double res,
                       int max_cg, int steps, double rho)
{
  size_t vb = sizeof(vec3_soa);
  act_params.stout_steps = steps;
  gl_stout_rho = rho;
  aux_th = xalloc(8 * sizeof(thmat_soa));
  aux_ta = xalloc(8 * sizeof(tamat_soa));
  stout_globals(1);
  su3_soa *gl3 = xalloc(8 * sizeof(su3_soa)), *taux = xalloc(8 * sizeof(su3_soa));
  vec3_soa *shiftmulti = xalloc(vb * (size_t)order), *shifttemp = xalloc(vb * (size_t)order);
  vec3_soa *r = xalloc(vb), *h = xalloc(vb), *s = xalloc(vb), *p = xalloc(vb);
  ferm_param fp; make_fp(&fp, ph, mass);
  fp.number_of_ps = nps;
  fp.index_of_the_first_ps = 0;
  fp.approx_md.approx_order = order;
  for (int i = 0; i < order; i++) { fp.approx_md.RA_a[i] = a[i]; fp.approx_md.RA_b[i] = b[i]; }
  inverter_package ip;
  memset(&ip, 0, sizeof(ip));
  ip.u = (const su3_soa *)u;
  ip.ferm_shift_temp = shifttemp; ip.nshifts = order;
  ip.loc_r = r; ip.loc_h = h; ip.loc_s = s; ip.loc_p = p;
  fermion_force_soloopenacc((su3_soa *)u, (su3_soa *)levels, gl3, (tamat_soa *)ipdot, &fp, 1,
                            (const vec3_soa *)phi, res, taux, shiftmulti, ip, max_cg);
  free(gl3); free(taux); free(shiftmulti); free(shifttemp);
  free(r); free(h); free(s); free(p);
  free(aux_th); free(aux_ta);
  aux_th = NULL; aux_ta = NULL;
  stout_globals(0);
}

/* ---- pure-gauge tree-level Symanzik HMC pieces (ipdot_gauge.c,
 * plaquettes.c, rectangles.c, su3_utilities.c, su3_measurements.c,
 * md_integrator.c, md_parameters.c) ---- */

/* the gauge staples dS/dU: C_ZERO x plaquette staples + C_ONE x the three
 * rectangle types (ipdot_gauge.c:192-212) */
void ref_gauge_staples(const double *u, double *stap)
{
  set_su3_soa_to_zero((su3_soa *)stap);
  calc_loc_staples_nnptrick_all((const su3_soa *)u, (su3_soa *)stap);
  calc_loc_improved_staples_typeA_nnptrick_all((const su3_soa *)u, (su3_soa *)stap);
  calc_loc_improved_staples_typeB_nnptrick_all((const su3_soa *)u, (su3_soa *)stap);
  calc_loc_improved_staples_typeC_nnptrick_all((const su3_soa *)u, (su3_soa *)stap);
}

/* tipdot = TA(U staples) (ipdot_gauge.c:361-426) */
void ref_ipdot_gauge(const double *u, double *stap, double *ipdot)
{
  calc_ipdot_gauge_soloopenacc((const su3_soa *)u, (su3_soa *)stap, (tamat_soa *)ipdot);
}

double ref_plaquette_sum(const double *u)
{
  su3_soa *lp = xalloc(2 * sizeof(su3_soa));
  dcomplex_soa *tr = xalloc(2 * sizeof(dcomplex_soa));
  double r = calc_plaquette_soloopenacc((su3_soa *)u, lp, tr);
  free(lp); free(tr);
  return r;
}

double ref_rectangle_sum(const double *u)
{
  su3_soa *lp = xalloc(2 * sizeof(su3_soa));
  dcomplex_soa *tr = xalloc(2 * sizeof(dcomplex_soa));
  double r = calc_rettangolo_soloopenacc((const su3_soa *)u, lp, tr);
  free(lp); free(tr);
  return r;
}

/* sum over the 8 link directions of 1/2 tr P^2 (su3_measurements.c:138-168) */
double ref_momenta_action(const double *mom)
{
  double_soa *tr = xalloc(sizeof(double_soa));
  double r = 0;
  for (int mu = 0; mu < 8; mu++) r += calc_momenta_action((const thmat_soa *)mom, tr, mu);
  free(tr);
  return r;
}

/* mom += factor x ipdot (su3_utilities.c:241-270) */
void ref_mom_sum_mult(double *mom, const double *ipdot, double factor)
{
  double f[1] = {factor};
  mom_sum_mult((thmat_soa *)mom, (const tamat_soa *)ipdot, f, 0);
}

/* U = exp(i delta P) U, rows 0-1 reunitarised (su3_utilities.c:272-305) */
void ref_mom_exp_times_conf(double *u, const double *mom, double delta)
{
  double f[1] = {delta};
  mom_exp_times_conf_soloopenacc((su3_soa *)u, (const thmat_soa *)mom, f, 0);
}

/* the integrator steps of initialize_md_global_variables (md_parameters.c:11-50) */
void ref_md_deltas(double beta, int no_md, int gauge_scale, double t, double *d7)
{
  act_params.beta = beta;
  md_parameters.no_md = no_md;
  md_parameters.gauge_scale = gauge_scale;
  md_parameters.t = t;
  initialize_md_global_variables(md_parameters);
  for (int i = 0; i < 7; i++) d7[i] = deltas_Omelyan[i];
}

/* ncalls x multistep_2MN_gauge (md_integrator.c:347-376): a pure-gauge
 * trajectory is 2 no_md of them (the fermion kicks of
 * multistep_2MN_SOLOOPENACC vanish without fermions) */
void ref_2mn_gauge(double *u, double *mom, double beta, int no_md, int gauge_scale, double t, int ncalls)
{
  double d7[7];
  ref_md_deltas(beta, no_md, gauge_scale, t, d7);
  su3_soa *stap = xalloc(8 * sizeof(su3_soa));
  tamat_soa *ip = xalloc(8 * sizeof(tamat_soa));
  for (int k = 0; k < ncalls; k++)
    multistep_2MN_gauge((su3_soa *)u, stap, ip, (thmat_soa *)mom);
  free(stap); free(ip);
}

/* ---- molecular dynamics with fermions: the reference's
 * multistep_2MN_SOLOOPENACC (md_integrator.c:502-742) for one flavour of
 * nps pseudofermions chi[nps] with approx_md = (a, b), mass, stout (steps,
 * rho), gauge action beta, integrator (no_md, gauge_scale, t).  u and mom
 * are updated in place. ---- */
void ref_rhmc_md(double *u, double *mom, double *ph, double mass, int nps, int order, const double *a,
                 const double *b, const double *chi, double res, int max_cg, double beta, int no_md,
                 int gauge_scale, double t, int steps, double rho)
{
  size_t vb = sizeof(vec3_soa);
  act_params.stout_steps = steps;
  act_params.topo_action = 0;
  gl_stout_rho = rho;
  double d7[7];
  ref_md_deltas(beta, no_md, gauge_scale, t, d7);
  alloc_info.maxNeededShifts = order;
  alloc_info.NDiffFlavs = 1;
  aux_th = xalloc(8 * sizeof(thmat_soa));
  aux_ta = xalloc(8 * sizeof(tamat_soa));
  stout_globals(1);
  su3_soa *levels = xalloc(8 * (size_t)(steps > 0 ? steps : 1) * sizeof(su3_soa));
  su3_soa *auxbis = xalloc(8 * sizeof(su3_soa)), *aux = xalloc(8 * sizeof(su3_soa));
  tamat_soa *ipdot = xalloc(8 * sizeof(tamat_soa));
  vec3_soa *shiftmulti = xalloc(vb * (size_t)order), *shifttemp = xalloc(vb * (size_t)order);
  vec3_soa *r = xalloc(vb), *h = xalloc(vb), *s = xalloc(vb), *p = xalloc(vb);
  dcomplex_soa *sums = xalloc(2 * sizeof(dcomplex_soa));
  ferm_param fp; make_fp(&fp, ph, mass);
  fp.number_of_ps = nps;
  fp.index_of_the_first_ps = 0;
  fp.approx_md.approx_order = order;
  for (int i = 0; i < order; i++) { fp.approx_md.RA_a[i] = a[i]; fp.approx_md.RA_b[i] = b[i]; }
  inverter_package ip;
  memset(&ip, 0, sizeof(ip));
  ip.u = (const su3_soa *)u;
  ip.ferm_shift_temp = shifttemp; ip.nshifts = order;
  ip.loc_r = r; ip.loc_h = h; ip.loc_s = s; ip.loc_p = p;
  multistep_2MN_SOLOOPENACC(ipdot, (su3_soa *)u, levels, auxbis, aux, &fp, 1, (vec3_soa *)chi, shiftmulti, ip,
                            (thmat_soa *)mom, sums, res, max_cg);
  free(levels); free(auxbis); free(aux); free(ipdot); free(shiftmulti); free(shifttemp);
  free(r); free(h); free(s); free(p); free(sums);
  free(aux_th); free(aux_ta);
  aux_th = NULL; aux_ta = NULL;
  stout_globals(0);
}

/* ---- configuration files (io.c:35-700), host arrays su3_soa[8] ---- */
int ref_write_ascii(const double *u, const char *path, int traj, const double *phases)
{
  return print_su3_soa_ASCII((global_su3_soa *)u, path, traj, (double_soa *)phases);
}
int ref_read_ascii(double *u, const char *path) { int t; int rc = read_su3_soa_ASCII((global_su3_soa *)u, path, &t); return rc ? -rc : t; }
int ref_write_ildg(const double *u, const char *path, int traj, const char *input_text)
{
  strncpy(input_file_str, input_text, sizeof(input_file_str) - 1);
  return print_su3_soa_ildg_binary((global_su3_soa *)u, path, traj);
}
int ref_read_ildg(double *u, const char *path) { int t; int rc = read_su3_soa_ildg_binary((global_su3_soa *)u, path, &t); return rc ? -rc : t; }
void ref_set_beta(double beta) { act_params.beta = beta; }
