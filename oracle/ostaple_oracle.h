/* ostaple_oracle.h -- CPU restatement of the reference's staggered-fermion
 * hot path (GPU-LQCD/OpenStaPLE), used ONLY as the parity checker of the
 * tests and as the CPU baseline of bench.py.  The product never links it.
 *
 * Parity pin: every function here is checked against the reference's own C
 * sources compiled from source (oracle/Makefile.ref -> oracle/_ref) and
 * against the golden vectors committed under tests/golden/, which were
 * produced by that compiled reference.
 *
 * Layouts are the reference's SoA layouts with a run-time lattice:
 *   vec3   : 3 x sizeh double complex
 *   su3    : 9 x sizeh double complex (rows r0,r1,r2 of columns c0,c1,c2)
 *   links  : 8 x su3, index 2*mu + parity
 *   phases : 8 x sizeh double (angles)
 *   tamat  : 3 x sizeh complex (c01,c02,c12) + 2 x sizeh double (ic00,ic11)
 *   thmat  : 3 x sizeh complex (c01,c02,c12) + 2 x sizeh double (rc00,rc11)
 */
#ifndef OSTAPLE_ORACLE_H_
#define OSTAPLE_ORACLE_H_

#include <complex.h>

typedef double complex ocplx;

int orc_init(int n0, int n1, int n2, int n3);   /* returns sizeh */
int orc_sizeh(void);
void orc_set_threads(int n);

void orc_calc_phases(double *phases, double im_chem_pot);
void orc_Deo(const ocplx *u, ocplx *out, const ocplx *in, const double *ph);
void orc_Doe(const ocplx *u, ocplx *out, const ocplx *in, const double *ph);
void orc_mdagm(const ocplx *u, ocplx *out, const ocplx *in, ocplx *tmp, const double *ph, double m2);

double orc_norm2(const ocplx *a);
double orc_rdot(const ocplx *a, const ocplx *b);

int orc_cg(const ocplx *u, const double *ph, double mass, ocplx *x, const ocplx *b, double res, int max_cg,
           double shift, int restart_every, int *cg_out);
int orc_cgm(const ocplx *u, const double *ph, double mass, int order, const double *ra_b, ocplx *xs,
            const ocplx *b, double res, int max_cg, int *cg_out);
void orc_recombine(const ocplx *xs, const ocplx *b, ocplx *out, int order, double a0, const double *a);
double orc_find_max(const ocplx *u, const double *ph, double mass, ocplx *p, ocplx *r, int *loops);
double orc_find_min(const ocplx *u, const double *ph, double mass, ocplx *p, ocplx *r, double max, int *loops);

/* stout smearing and force chain (ostaple_oracle_gauge.c) */
void orc_gauge_init(int n0, int n1, int n2, int n3);
void orc_staples(const ocplx *u, ocplx *stap);
void orc_rho_ta(const ocplx *u, const ocplx *stap, double *qa, double rho);
void orc_exp_times_conf(const ocplx *u, double *qa, ocplx *uout);
void orc_stout(const ocplx *u, ocplx *uout, double rho);
void orc_lambda(double *lam, const ocplx *sp, const ocplx *u, double *qa);
void orc_sigma(double *lam, const ocplx *u, ocplx *s, double *qa, double rho);
void orc_sigma_prime_to_sigma(ocplx *sigma, const ocplx *u, double rho);
void orc_force_outer(const ocplx *u, ocplx *aux, const ocplx *xs, const double *ph, int order, const double *a);
void orc_backfield_times_force(const double *ph, const ocplx *aux, ocplx *pip);
void orc_conf_times_force_ta(const ocplx *u, const ocplx *sigma, double *ipdot);

/* pure-gauge tree-level Symanzik HMC (ostaple_oracle_gauge.c) */
void orc_gauge_staples(const ocplx *u, ocplx *stap);
void orc_ipdot_gauge(const ocplx *u, double *ipdot);
double orc_plaquette_sum(const ocplx *u);
double orc_rectangle_sum(const ocplx *u);
double orc_momenta_action(double *mom);
void orc_mom_sum_mult(double *mom, double *ipdot, double fact);
void orc_mom_exp_times_conf(ocplx *u, double *mom, double delta);
void orc_md_deltas(double beta, int no_md, int gauge_scale, double t, double *d);
void orc_2mn_gauge(ocplx *u, double *mom, double beta, int no_md, int gauge_scale, double t, int ncalls);

#endif
