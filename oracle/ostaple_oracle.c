/* ostaple_oracle.c -- CPU restatement of the reference's fermion hot path.
 * TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg use it, as the checker.  See ostaple_oracle.h.
 *
 * Each function names the reference lines whose algorithm it restates.
 * Loops over sites are OpenMP-parallel (the reference's OpenACC loops are
 * independent loops); reductions use OpenMP's reduction clause.
 */
#include "ostaple_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int N[4];
static long SH;      /* sizeh */
static long VL[4];   /* lexicographic strides */

int orc_init(int n0, int n1, int n2, int n3)
{
  N[0] = n0; N[1] = n1; N[2] = n2; N[3] = n3;
  VL[0] = 1; VL[1] = n0; VL[2] = (long)n0 * n1; VL[3] = (long)n0 * n1 * n2;
  SH = (long)n0 * n1 * n2 * n3 / 2;
  orc_gauge_init(n0, n1, n2, n3);
  return (int)SH;
}

int orc_sizeh(void) { return (int)SH; }

void orc_set_threads(int n)
{
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

/* half-lattice index of a site: lex/2 (geometry_multidev.h:219-229) */
static inline long snum(const int d[4]) { return (d[0] + d[1] * VL[1] + d[2] * VL[2] + d[3] * VL[3]) / 2; }

/* coordinates of half-lattice index h on parity par: d0 = 2*hd0 + parity bit
 * (fermion_matrix.c:67,120) */
static inline void coords(long h, int par, int d[4])
{
  long nh0 = N[0] / 2;
  long hd0 = h % nh0, r = h / nh0;
  d[1] = (int)(r % N[1]); r /= N[1];
  d[2] = (int)(r % N[2]);
  d[3] = (int)(r / N[2]);
  d[0] = (int)(2 * hd0 + ((d[1] + d[2] + d[3] + par) & 1));
}

/* ---- staggered phases: backfield.c:20-187 with zero external fields ----
 * angle/(2pi) = 0.5*[eta_mu = -1] + (t-links) mu_I/(2 N_t) + 0.5*[t = N_t-1],
 * folded to [-1/2, 1/2] and multiplied by 2pi.  eta_x = 1, eta_y = (-1)^x,
 * eta_z = (-1)^(x+y), eta_t = (-1)^(x+y+z) (backfield.h:27-41). */
void orc_calc_phases(double *ph, double im_chem_pot)
{
  const double twopi = 2 * 3.14159265358979323846;
  int d[4];
  for (d[3] = 0; d[3] < N[3]; d[3]++)
    for (d[2] = 0; d[2] < N[2]; d[2]++)
      for (d[1] = 0; d[1] < N[1]; d[1]++)
        for (d[0] = 0; d[0] < N[0]; d[0]++) {
          long h = snum(d);
          int par = (d[0] + d[1] + d[2] + d[3]) % 2;
          int eta_neg[4];
          eta_neg[0] = 0;
          eta_neg[1] = d[0] & 1;
          eta_neg[2] = (d[0] + d[1]) & 1;
          eta_neg[3] = (d[0] + d[1] + d[2]) & 1;
          for (int mu = 0; mu < 4; mu++) {
            double a = eta_neg[mu] ? 0.5 : 0.0;
            if (mu == 3) {
              a += 0.5 * (im_chem_pot / N[3]);
              if (d[3] == N[3] - 1) a += 0.5;
            }
            while (a > 0.5) a -= 1.0;
            while (a < -0.5) a += 1.0;
            ph[(2 * mu + par) * SH + h] = a * twopi;
          }
        }
}

/* ---- link helpers ---- */
static inline const ocplx *lnk(const ocplx *u, int dir, int row, int col)
{
  return u + ((long)dir * 9 + row * 3 + col) * SH;
}

/* U v with the third row rebuilt as conj(r0 x r1) (matvecmul.h:88-131) */
static inline void umul(const ocplx *u, int dir, long i, const ocplx v[3], ocplx o[3])
{
  ocplx a00 = lnk(u, dir, 0, 0)[i], a01 = lnk(u, dir, 0, 1)[i], a02 = lnk(u, dir, 0, 2)[i];
  ocplx a10 = lnk(u, dir, 1, 0)[i], a11 = lnk(u, dir, 1, 1)[i], a12 = lnk(u, dir, 1, 2)[i];
  ocplx a20 = conj(a01 * a12 - a02 * a11);
  ocplx a21 = conj(a02 * a10 - a00 * a12);
  ocplx a22 = conj(a00 * a11 - a01 * a10);
  o[0] = a00 * v[0] + a01 * v[1] + a02 * v[2];
  o[1] = a10 * v[0] + a11 * v[1] + a12 * v[2];
  o[2] = a20 * v[0] + a21 * v[1] + a22 * v[2];
}

/* U^+ v with the same rebuild (matvecmul.h:134-172) */
static inline void udagmul(const ocplx *u, int dir, long i, const ocplx v[3], ocplx o[3])
{
  ocplx a00 = lnk(u, dir, 0, 0)[i], a01 = lnk(u, dir, 0, 1)[i], a02 = lnk(u, dir, 0, 2)[i];
  ocplx a10 = lnk(u, dir, 1, 0)[i], a11 = lnk(u, dir, 1, 1)[i], a12 = lnk(u, dir, 1, 2)[i];
  ocplx c20 = a01 * a12 - a02 * a11;  /* = conj(row-3 element) */
  ocplx c21 = a02 * a10 - a00 * a12;
  ocplx c22 = a00 * a11 - a01 * a10;
  o[0] = conj(a00) * v[0] + conj(a10) * v[1] + c20 * v[2];
  o[1] = conj(a01) * v[0] + conj(a11) * v[1] + c21 * v[2];
  o[2] = conj(a02) * v[0] + conj(a12) * v[1] + c22 * v[2];
}

/* D_eo (P=0) / D_oe (P=1): fermion_matrix.c:47-157.
 * out(x) = 1/2 { sum_mu e^{i th} U_{2mu+P}(x) in(x+mu) - e^{-i th} U_{2mu+1-P}(x-mu)^+ in(x-mu) }
 * with backward terms accumulated first, as in the reference. */
static void dslash(int P, const ocplx *u, ocplx *out, const ocplx *in, const double *ph)
{
  long h;
#pragma omp parallel for schedule(static)
  for (h = 0; h < SH; h++) {
    int d[4], e[4];
    coords(h, P, d);
    ocplx acc[3] = {0, 0, 0};
    for (int mu = 0; mu < 4; mu++) {
      memcpy(e, d, sizeof(e));
      e[mu] = (d[mu] + N[mu] - 1) % N[mu];
      long j = snum(e);
      int dir = 2 * mu + (1 - P);
      double a = ph[(long)dir * SH + j];
      ocplx phase = cos(a) + I * sin(a);
      ocplx v[3] = {in[j] * conj(phase), in[SH + j] * conj(phase), in[2 * SH + j] * conj(phase)}, o[3];
      udagmul(u, dir, j, v, o);
      acc[0] -= o[0]; acc[1] -= o[1]; acc[2] -= o[2];
    }
    for (int mu = 0; mu < 4; mu++) {
      memcpy(e, d, sizeof(e));
      e[mu] = (d[mu] + 1) % N[mu];
      long j = snum(e);
      int dir = 2 * mu + P;
      double a = ph[(long)dir * SH + h];
      ocplx phase = cos(a) + I * sin(a);
      ocplx v[3] = {in[j] * phase, in[SH + j] * phase, in[2 * SH + j] * phase}, o[3];
      umul(u, dir, h, v, o);
      acc[0] += o[0]; acc[1] += o[1]; acc[2] += o[2];
    }
    out[h] = acc[0] * 0.5;
    out[SH + h] = acc[1] * 0.5;
    out[2 * SH + h] = acc[2] * 0.5;
  }
}

void orc_Deo(const ocplx *u, ocplx *out, const ocplx *in, const double *ph) { dslash(0, u, out, in, ph); }
void orc_Doe(const ocplx *u, ocplx *out, const ocplx *in, const double *ph) { dslash(1, u, out, in, ph); }

/* out = m2 in - D_eo D_oe in  (fermion_matrix.c:723-746, fermionic_utilities.c:261-272) */
void orc_mdagm(const ocplx *u, ocplx *out, const ocplx *in, ocplx *tmp, const double *ph, double m2)
{
  dslash(1, u, tmp, in, ph);
  dslash(0, u, out, tmp, ph);
  long i, n = 3 * SH;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n; i++) out[i] = in[i] * m2 - out[i];
}

/* ---- reductions (fermionic_utilities.c:126-175) ---- */
double orc_norm2(const ocplx *a)
{
  double s = 0;
  long i, n = 3 * SH;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (i = 0; i < n; i++) s += creal(a[i]) * creal(a[i]) + cimag(a[i]) * cimag(a[i]);
  return s;
}

double orc_rdot(const ocplx *a, const ocplx *b)
{
  double s = 0;
  long i, n = 3 * SH;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (i = 0; i < n; i++) s += creal(a[i]) * creal(b[i]) + cimag(a[i]) * cimag(b[i]);
  return s;
}

static void axpy(const ocplx *x, double a, const ocplx *y, ocplx *out)
{
  long i, n = 3 * SH;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n; i++) out[i] = x[i] * a + y[i];
}

static void *xmalloc(size_t n)
{
  void *p = calloc(1, n);
  if (!p) { fprintf(stderr, "oracle: out of memory\n"); exit(2); }
  return p;
}

/* ---- CG on (M^+M + shift): inverter_full.c:19-132 ----
 * restarted every restart_every iterations from the true residual; the inner
 * loop stops at sqrt(|r|^2/|b|^2) <= 0.95 res, the outer one at <= res or
 * max_cg; success iff the final true residual is <= res. */
int orc_cg(const ocplx *u, const double *ph, double mass, ocplx *x, const ocplx *b, double res, int max_cg,
           double shift, int restart_every, int *cg_out)
{
  size_t vb = sizeof(ocplx) * 3 * SH;
  ocplx *r = xmalloc(vb), *h = xmalloc(vb), *s = xmalloc(vb), *p = xmalloc(vb);
  double m2 = mass * mass + shift;
  double bn = orc_norm2(b), delta, lambda = 0;
  long i, n = 3 * SH;
  int cg = 0;
  do {
    orc_mdagm(u, s, x, h, ph, m2);
    for (i = 0; i < n; i++) { r[i] = b[i] - s[i]; p[i] = r[i]; }
    delta = orc_norm2(r);
    int inner = 0;
    do {
      cg++; inner++;
      orc_mdagm(u, s, p, h, ph, m2);
      double alpha = orc_rdot(p, s);
      double omega = delta / alpha;
      axpy(p, omega, x, x);
      axpy(s, -omega, r, r);
      lambda = orc_norm2(r);
      double g = lambda / delta;
      delta = lambda;
      axpy(p, g, r, p);
    } while (sqrt(lambda / bn) > res * 0.95 && inner < restart_every);
  } while (sqrt(lambda / bn) > res && cg < max_cg);
  orc_mdagm(u, s, x, h, ph, m2);
  for (i = 0; i < n; i++) h[i] = b[i] - s[i];
  double tr = orc_norm2(h) / bn;
  *cg_out = cg;
  free(r); free(h); free(s); free(p);
  return sqrt(tr) <= res ? 1 : 0;
}

/* ---- eigenvalue bounds of M^+M: find_min_max.c:21-117 ----
 * Power iteration: p <- p / |p|, r = p, p = (M^+M + shift) r, until the
 * relative change of |p| is <= 1e-5.  The largest eigenvalue uses shift 0
 * (find_min_max.c:21-58).  The smallest one (find_min_max.c:62-92) passes
 * shift = (max - m^2) - m^2 to the shifted matrix and returns max - |p|,
 * exactly as the reference does.  p holds the start vector on entry and the
 * last product on exit; r the last normalised vector. */
static double power_iteration(const ocplx *u, const double *ph, double m2_plus_shift, ocplx *p, ocplx *r,
                              int *loops_out)
{
  size_t vb = sizeof(ocplx) * 3 * SH;
  ocplx *h = xmalloc(vb);
  long i, n = 3 * SH;
  double norm = sqrt(orc_norm2(p)), rel;
  int loops = 0;
  do {
    double inorm = 1.0 / norm;
    for (i = 0; i < n; i++) { p[i] = p[i] * inorm; r[i] = p[i]; }
    double old = norm;
    orc_mdagm(u, p, r, h, ph, m2_plus_shift);
    norm = sqrt(orc_norm2(p));
    rel = fabs(old - norm) / norm;
    loops++;
  } while (rel > 1.0e-5);
  free(h);
  if (loops_out) *loops_out = loops;
  return norm;
}

double orc_find_max(const ocplx *u, const double *ph, double mass, ocplx *p, ocplx *r, int *loops)
{
  return power_iteration(u, ph, mass * mass, p, r, loops);
}

double orc_find_min(const ocplx *u, const double *ph, double mass, ocplx *p, ocplx *r, double max, int *loops)
{
  double m2 = mass * mass, delta = max - m2;
  return max - power_iteration(u, ph, m2 + (delta - m2), p, r, loops);
}

/* ---- CG-M for (M^+M + b_k) x_k = b: inverter_multishift_full.c:23-252 ----
 * zeta/omega/gamma recurrences of the shifted systems; shift k is frozen
 * once sqrt(delta zeta_k^2 / |b|^2) < 0.95 res; success iff every final
 * relative residual^2 is <= 1 (the reference's check). */
int orc_cgm(const ocplx *u, const double *ph, double mass, int order, const double *ra_b, ocplx *xs,
            const ocplx *b, double res, int max_cg, int *cg_out)
{
  size_t vb = sizeof(ocplx) * 3 * SH;
  long i, n = 3 * SH;
  ocplx *r = xmalloc(vb), *h = xmalloc(vb), *s = xmalloc(vb), *p = xmalloc(vb);
  ocplx *ps = xmalloc(vb * (size_t)order);
  double z_prev[32], z_cur[32], z_next[32], om_k[32], ga_k[32];
  int live[32];
  double m2 = mass * mass;
  memcpy(r, b, vb);
  memcpy(p, b, vb);
  double delta = orc_norm2(r), bn = orc_norm2(b);
  for (int k = 0; k < order; k++) {
    live[k] = 1;
    memset(xs + k * n, 0, vb);
    memcpy(ps + k * n, b, vb);
    z_prev[k] = 1.0; z_cur[k] = 1.0; ga_k[k] = 0.0;
  }
  double omega = 1.0, gamma = 0.0;
  int cg = 0, top = order;
  do {
    cg++;
    orc_mdagm(u, s, p, h, ph, m2);
    double alpha = orc_rdot(p, s);
    double omega_prev = omega;
    omega = -delta / alpha;
    for (int k = 0; k < top; k++) {
      if (!live[k]) continue;
      z_next[k] = z_prev[k] * z_cur[k] * omega_prev /
                  (omega * gamma * (z_prev[k] - z_cur[k]) + z_prev[k] * omega_prev * (1.0 - ra_b[k] * omega));
      om_k[k] = omega * z_next[k] / z_cur[k];
    }
    for (int k = 0; k < top; k++) {
      if (!live[k]) continue;
      ocplx *xk = xs + k * n, *pk = ps + k * n;
#pragma omp parallel for schedule(static)
      for (i = 0; i < n; i++) xk[i] -= om_k[k] * pk[i];
    }
    axpy(s, omega, r, r);
    double lambda = orc_norm2(r);
    gamma = lambda / delta;
    axpy(p, gamma, r, p);
    for (int k = 0; k < order; k++)
      if (live[k]) ga_k[k] = gamma * z_next[k] * om_k[k] / (z_cur[k] * omega);
    for (int k = 0; k < top; k++) {
      if (!live[k]) continue;
      ocplx *pk = ps + k * n;
#pragma omp parallel for schedule(static)
      for (i = 0; i < n; i++) pk[i] = ga_k[k] * pk[i] + z_next[k] * r[i];
    }
    top = 0;
    for (int k = 0; k < order; k++) {
      if (!live[k]) continue;
      if (sqrt(delta * z_cur[k] * z_cur[k] / bn) < res * 0.95) live[k] = 0;
      else top = k + 1;
      z_prev[k] = z_cur[k];
      z_cur[k] = z_next[k];
    }
    delta = lambda;
  } while (top > 0 && cg < max_cg);
  int ok = 1;
  for (int k = 0; k < order; k++) {
    orc_mdagm(u, s, xs + k * n, h, ph, m2 + ra_b[k]);
    for (i = 0; i < n; i++) h[i] = b[i] - s[i];
    if (orc_norm2(h) / bn > 1) ok = 0;
  }
  *cg_out = cg;
  free(r); free(h); free(s); free(p); free(ps);
  return ok;
}

/* out = a0 b + sum_k a_k x_k  (inverter_multishift_full.c:254-282) */
void orc_recombine(const ocplx *xs, const ocplx *b, ocplx *out, int order, double a0, const double *a)
{
  long i, n = 3 * SH;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n; i++) {
    ocplx v = b[i] * a0;
    for (int k = 0; k < order; k++) v += a[k] * xs[k * n + i];
    out[i] = v;
  }
}
