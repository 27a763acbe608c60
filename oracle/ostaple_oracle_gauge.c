/* ostaple_oracle_gauge.c -- CPU restatement of the reference's stout smearing
 * and rational fermion force chain.  TEST INFRASTRUCTURE (checker only).
 *
 * Matrices are handled as plain 3x3 complex arrays; the SU(3) links of the
 * reference store two rows and rebuild the third as conj(r0 x r1).
 *   su3   : 9 x sizeh complex per link direction   (struct_c_def.h:37-44)
 *   tamat : anti-Hermitian traceless, c01,c02,c12 complex + ic00,ic11 real
 *           [[i a, c01, c02], [-c01*, i b, c12], [-c02*, -c12*, -i(a+b)]]
 *   thmat : Hermitian traceless, c01,c02,c12 complex + rc00,rc11 real
 *           [[a, c01, c02], [c01*, b, c12], [c02*, c12*, -(a+b)]]
 * The exponential and its derivative follow Morningstar & Peardon,
 * Phys. Rev. D 69 (2004) 054501, hep-lat/0311018 (the method the reference
 * cites, cayley_hamilton.h:5-8).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ostaple_oracle.h"

#define C_ZERO (5.0 * 0.33333333333333333333333)  /* tree-level Symanzik c0 (common_defines.h) */

typedef struct { ocplx m[3][3]; } M3;

static int NN[4];
static long SHH, VLL[4];

void orc_gauge_init(int n0, int n1, int n2, int n3)
{
  NN[0] = n0; NN[1] = n1; NN[2] = n2; NN[3] = n3;
  VLL[0] = 1; VLL[1] = n0; VLL[2] = (long)n0 * n1; VLL[3] = (long)n0 * n1 * n2;
  SHH = (long)n0 * n1 * n2 * n3 / 2;
}

static inline long sn(const int d[4]) { return (d[0] + d[1] * VLL[1] + d[2] * VLL[2] + d[3] * VLL[3]) / 2; }

static inline long shift(const int d[4], int mu, int step)
{
  int e[4] = {d[0], d[1], d[2], d[3]};
  e[mu] = (e[mu] + step + NN[mu]) % NN[mu];
  return sn(e);
}

/* ---- matrix helpers ---- */
static M3 mmul(M3 a, M3 b)
{
  M3 c;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
  return c;
}
static M3 mdag(M3 a)
{
  M3 c;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c.m[i][j] = conj(a.m[j][i]);
  return c;
}
static M3 madd(M3 a, M3 b)
{
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) a.m[i][j] += b.m[i][j];
  return a;
}
static M3 mscale(M3 a, ocplx s)
{
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) a.m[i][j] *= s;
  return a;
}
static M3 mzero(void) { M3 z; memset(&z, 0, sizeof(z)); return z; }
static M3 mid(ocplx s) { M3 z = mzero(); z.m[0][0] = z.m[1][1] = z.m[2][2] = s; return z; }
static ocplx mtr(M3 a) { return a.m[0][0] + a.m[1][1] + a.m[2][2]; }

/* link (dir, idx) with the third row rebuilt from the first two */
static M3 ld_link(const ocplx *u, int dir, long i)
{
  M3 a;
  for (int r = 0; r < 2; r++)
    for (int c = 0; c < 3; c++) a.m[r][c] = u[((long)dir * 9 + r * 3 + c) * SHH + i];
  a.m[2][0] = conj(a.m[0][1] * a.m[1][2] - a.m[0][2] * a.m[1][1]);
  a.m[2][1] = conj(a.m[0][2] * a.m[1][0] - a.m[0][0] * a.m[1][2]);
  a.m[2][2] = conj(a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0]);
  return a;
}
/* all three stored rows (general 3x3 such as Sigma or staples) */
static M3 ld_full(const ocplx *u, int dir, long i)
{
  M3 a;
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) a.m[r][c] = u[((long)dir * 9 + r * 3 + c) * SHH + i];
  return a;
}
static void st_full(ocplx *u, int dir, long i, M3 a, int rows)
{
  for (int r = 0; r < rows; r++)
    for (int c = 0; c < 3; c++) u[((long)dir * 9 + r * 3 + c) * SHH + i] = a.m[r][c];
}

/* tamat / thmat blocks: 3 complex arrays then 2 real arrays, per direction */
static ocplx *blk_c(double *t, int dir, int k) { return (ocplx *)(t + (long)dir * 8 * SHH) + (long)k * SHH; }
static double *blk_r(double *t, int dir, int k) { return t + (long)dir * 8 * SHH + 6 * SHH + (long)k * SHH; }

static M3 ld_tamat(double *t, int dir, long i)
{
  ocplx c01 = blk_c(t, dir, 0)[i], c02 = blk_c(t, dir, 1)[i], c12 = blk_c(t, dir, 2)[i];
  double a = blk_r(t, dir, 0)[i], b = blk_r(t, dir, 1)[i];
  M3 m;
  m.m[0][0] = I * a; m.m[0][1] = c01; m.m[0][2] = c02;
  m.m[1][0] = -conj(c01); m.m[1][1] = I * b; m.m[1][2] = c12;
  m.m[2][0] = -conj(c02); m.m[2][1] = -conj(c12); m.m[2][2] = -I * (a + b);
  return m;
}
static M3 ld_thmat(double *t, int dir, long i)
{
  ocplx c01 = blk_c(t, dir, 0)[i], c02 = blk_c(t, dir, 1)[i], c12 = blk_c(t, dir, 2)[i];
  double a = blk_r(t, dir, 0)[i], b = blk_r(t, dir, 1)[i];
  M3 m;
  m.m[0][0] = a; m.m[0][1] = c01; m.m[0][2] = c02;
  m.m[1][0] = conj(c01); m.m[1][1] = b; m.m[1][2] = c12;
  m.m[2][0] = conj(c02); m.m[2][1] = conj(c12); m.m[2][2] = -(a + b);
  return m;
}
static void st_thmat(double *t, int dir, long i, M3 m)
{
  blk_c(t, dir, 0)[i] = m.m[0][1]; blk_c(t, dir, 1)[i] = m.m[0][2]; blk_c(t, dir, 2)[i] = m.m[1][2];
  blk_r(t, dir, 0)[i] = creal(m.m[0][0]); blk_r(t, dir, 1)[i] = creal(m.m[1][1]);
}

/* traceless anti-Hermitian part, stored as tamat, times s:
 * c_ij = s (M_ij - conj(M_ji))/2, ic_kk = s (Im M_kk - Im tr M / 3)
 * (su3_utilities.h:1097-1152) */
static void st_ta(double *t, int dir, long i, M3 m, double s)
{
  double tr = (cimag(m.m[0][0]) + cimag(m.m[1][1]) + cimag(m.m[2][2])) * 0.33333333333333333333333;
  blk_c(t, dir, 0)[i] = s * (0.5 * (m.m[0][1] - conj(m.m[1][0])));
  blk_c(t, dir, 1)[i] = s * (0.5 * (m.m[0][2] - conj(m.m[2][0])));
  blk_c(t, dir, 2)[i] = s * (0.5 * (m.m[1][2] - conj(m.m[2][1])));
  blk_r(t, dir, 0)[i] = s * (cimag(m.m[0][0]) - tr);
  blk_r(t, dir, 1)[i] = s * (cimag(m.m[1][1]) - tr);
}

/* ---- staples: C_mu(x) = C_ZERO sum_nu [ U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+
 *                                       + U_nu(x+mu-nu)^+ U_mu(x-nu)^+ U_nu(x-nu) ]
 * (plaquettes.c:196-259) */
static M3 staple(const ocplx *u, const int d[4], int mu)
{
  int p = (d[0] + d[1] + d[2] + d[3]) & 1;
  long x = sn(d), xpm = shift(d, mu, 1);
  M3 acc = mzero();
  for (int nu = 0; nu < 4; nu++) {
    if (nu == mu) continue;
    long xpn = shift(d, nu, 1), xmn = shift(d, nu, -1);
    int e[4] = {d[0], d[1], d[2], d[3]};
    e[mu] = (e[mu] + 1) % NN[mu];
    long xpmmn = shift(e, nu, -1);
    M3 r = mmul(mmul(ld_link(u, 2 * nu + !p, xpm), mdag(ld_link(u, 2 * mu + !p, xpn))), mdag(ld_link(u, 2 * nu + p, x)));
    M3 l = mmul(mmul(mdag(ld_link(u, 2 * nu + p, xpmmn)), mdag(ld_link(u, 2 * mu + !p, xmn))), ld_link(u, 2 * nu + !p, xmn));
    acc = madd(acc, madd(r, l));
  }
  return mscale(acc, C_ZERO);
}

void orc_staples(const ocplx *u, ocplx *stap)
{
  int d[4];
  for (d[3] = 0; d[3] < NN[3]; d[3]++)
    for (d[2] = 0; d[2] < NN[2]; d[2]++)
      for (d[1] = 0; d[1] < NN[1]; d[1]++)
        for (d[0] = 0; d[0] < NN[0]; d[0]++) {
          int p = (d[0] + d[1] + d[2] + d[3]) & 1;
          for (int mu = 0; mu < 4; mu++) st_full(stap, 2 * mu + p, sn(d), staple(u, d, mu), 3);
        }
}

/* Q_A = rho / C_ZERO * TA(U C) for every link (su3_utilities.c:210-239) */
void orc_rho_ta(const ocplx *u, const ocplx *stap, double *qa, double rho)
{
  for (int dir = 0; dir < 8; dir++)
    for (long i = 0; i < SHH; i++) st_ta(qa, dir, i, mmul(ld_link(u, dir, i), ld_full(stap, dir, i)), rho / C_ZERO);
}

/* ---- Cayley-Hamilton exponential exp(iQ) = f0 + f1 Q + f2 Q^2 for
 * Hermitian traceless Q, with b_1j = d f_j / d c1 and b_2j = d f_j / d c0
 * (c0 = det Q, c1 = tr Q^2 / 2).  Large c1: closed forms of
 * Morningstar-Peardon eqs. (23)-(34), (57)-(65); small c1 (< 4e-3): the
 * power series of exp(iQ) reduced by Q^3 = c1 Q + c0, summed to full
 * precision with the c0/c1 derivatives carried along. */
/* Small-c1 branch: exp(iQ) = sum_n (iQ)^n / n!, each Q^n reduced with
 * Q^3 = c1 Q + c0 to al_n + be_n Q + ga_n Q^2, where al, be, ga are
 * polynomials in (c0, c1).  The sum is truncated at total weight 7 (weight 3
 * for c0, 2 for c1: c1 ~ |Q|^2, c0 ~ |Q|^3), the truncation the reference's
 * small-c1 expansion uses (cayley_hamilton.h:67-72); b_1j, b_2j are the exact
 * c1 and c0 derivatives of the truncated f_j. */
#define SW_MAXW 7
#define SW_NMON 8
static const int sw_i[SW_NMON] = {0, 0, 0, 0, 1, 1, 1, 2};   /* c0 power */
static const int sw_j[SW_NMON] = {0, 1, 2, 3, 0, 1, 2, 0};   /* c1 power */
static int sw_index(int i, int j)
{
  for (int k = 0; k < SW_NMON; k++)
    if (sw_i[k] == i && sw_j[k] == j) return k;
  return -1;
}
typedef struct { ocplx f[3][SW_NMON]; } SwTable;   /* f_j = sum_k f[j][k] c0^i_k c1^j_k */
static SwTable sw_table(void)
{
  double al[SW_NMON] = {1}, be[SW_NMON] = {0}, ga[SW_NMON] = {0};
  SwTable t;
  memset(&t, 0, sizeof(t));
  ocplx in = 1.0;
  for (int n = 0; n <= SW_MAXW + 2; n++) {
    for (int k = 0; k < SW_NMON; k++) { t.f[0][k] += in * al[k]; t.f[1][k] += in * be[k]; t.f[2][k] += in * ga[k]; }
    double nal[SW_NMON] = {0}, nbe[SW_NMON] = {0}, nga[SW_NMON] = {0};
    for (int k = 0; k < SW_NMON; k++) {
      int a = sw_index(sw_i[k] + 1, sw_j[k]), b = sw_index(sw_i[k], sw_j[k] + 1);
      if (a >= 0) nal[a] += ga[k];            /* ga c0 */
      nbe[k] += al[k];
      if (b >= 0) nbe[b] += ga[k];            /* ga c1 */
      nga[k] += be[k];
    }
    memcpy(al, nal, sizeof(al)); memcpy(be, nbe, sizeof(be)); memcpy(ga, nga, sizeof(ga));
    in *= I / (double)(n + 1);
  }
  return t;
}

static void ch_coeffs(double c0, double c1, ocplx f[3], ocplx b1[3], ocplx b2[3], int need_b)
{
  if (c1 < 4.0e-3) {
    static SwTable t;
    static int have = 0;
    if (!have) { t = sw_table(); have = 1; }
    for (int j = 0; j < 3; j++) {
      f[j] = 0; b1[j] = 0; b2[j] = 0;
      for (int k = 0; k < SW_NMON; k++) {
        int i0 = sw_i[k], j1 = sw_j[k];
        f[j] += t.f[j][k] * pow(c0, i0) * pow(c1, j1);
        if (j1 > 0 && 3 * i0 + 2 * j1 - 2 <= SW_MAXW - 2)
          b1[j] += t.f[j][k] * (double)j1 * pow(c0, i0) * pow(c1, j1 - 1);
        if (i0 > 0 && 3 * i0 + 2 * j1 - 3 <= SW_MAXW - 3)
          b2[j] += t.f[j][k] * (double)i0 * pow(c0, i0 - 1) * pow(c1, j1);
      }
    }
    return;
  }
  int neg = c0 < 0;
  if (neg) c0 = -c0;
  double c0max = 2 * pow(c1 / 3, 1.5);
  double eps = (c0max - c0) / c0max, th;
  if (eps < 0) th = 0;
  else if (eps < 1e-3) /* arccos(1 - eps) series */
    th = sqrt(2 * eps) * (1 + (1.0 / 12 + (3.0 / 160 + (5.0 / 896 + (35.0 / 18432 + 63.0 / 90112 * eps) * eps) * eps) * eps) * eps);
  else th = acos(c0 / c0max);
  double u = sqrt(c1 / 3) * cos(th / 3), w = sqrt(c1) * sin(th / 3);
  double u2 = u * u, w2 = w * w;
  double xi0, xi1;
  if (fabs(w) < 0.05) {
    xi0 = 1 - w2 / 6 * (1 - w2 / 20 * (1 - w2 / 42));
    xi1 = -(1 - w2 * (1 - w2 * (1 - w2 / 54) / 28) / 10) / 3;
  } else {
    xi0 = sin(w) / w;
    xi1 = cos(w) / w2 - sin(w) / (w2 * w);
  }
  ocplx e2 = cexp(2 * I * u), em = cexp(-I * u);
  double cw = cos(w);
  ocplx h0 = (u2 - w2) * e2 + em * (8 * u2 * cw + 2 * I * u * (3 * u2 + w2) * xi0);
  ocplx h1 = 2 * u * e2 - em * (2 * u * cw - I * (3 * u2 - w2) * xi0);
  ocplx h2 = e2 - em * (cw + 3 * I * u * xi0);
  double den = 1.0 / (9 * u2 - w2);
  f[0] = h0 * den; f[1] = h1 * den; f[2] = h2 * den;
  if (need_b) {
    ocplx r1[3], r2[3];
    r1[0] = 2 * (u + I * (u2 - w2)) * e2 + 2 * em * (4 * u * (2 - I * u) * cw + I * xi0 * (9 * u2 + w2 - I * u * (3 * u2 + w2)));
    r1[1] = 2 * (1 + 2 * I * u) * e2 + em * (-2 * (1 - I * u) * cw + I * (6 * u + I * (w2 - 3 * u2)) * xi0);
    r1[2] = 2 * I * e2 + I * em * (cw - 3 * (1 - I * u) * xi0);
    r2[0] = -2 * e2 + 2 * I * u * em * (cw + (1 + 4 * I * u) * xi0 + 3 * u2 * xi1);
    r2[1] = -I * em * (cw + (1 + 2 * I * u) * xi0 - 3 * u2 * xi1);
    r2[2] = em * (xi0 - 3 * I * u * xi1);
    for (int j = 0; j < 3; j++) {
      b1[j] = 0.5 * den * den * (2 * u * r1[j] + (3 * u2 - w2) * r2[j] - 2 * (15 * u2 + w2) * f[j]);
      b2[j] = 0.5 * den * den * (r1[j] - 3 * u * r2[j] - 24 * u * f[j]);
    }
  }
  if (neg) { /* f_j(-c0) = (-1)^j f_j(c0)*, b_ij(-c0) = (-1)^(i+j+1) b_ij(c0)* */
    f[0] = conj(f[0]); f[1] = -conj(f[1]); f[2] = conj(f[2]);
    if (need_b) {
      b1[0] = conj(b1[0]); b1[1] = -conj(b1[1]); b1[2] = conj(b1[2]);
      b2[0] = -conj(b2[0]); b2[1] = conj(b2[1]); b2[2] = -conj(b2[2]);
    }
  }
}

/* Q = i Q_A and its invariants */
static M3 q_of(double *qa, int dir, long i, double *c0, double *c1)
{
  M3 q = mscale(ld_tamat(qa, dir, i), I);
  M3 q2 = mmul(q, q);
  *c1 = 0.5 * creal(mtr(q2));
  *c0 = creal(mtr(mmul(q2, q))) / 3.0;   /* det Q = tr Q^3 / 3 for traceless Q */
  return q;
}

static M3 poly(ocplx a0, ocplx a1, ocplx a2, M3 q, M3 q2)
{
  return madd(madd(mid(a0), mscale(q, a1)), mscale(q2, a2));
}

/* U' = exp(-Q_A) U, first two rows written (stouting.c:107-165) */
void orc_exp_times_conf(const ocplx *u, double *qa, ocplx *uout)
{
  for (int dir = 0; dir < 8; dir++)
    for (long i = 0; i < SHH; i++) {
      double c0, c1;
      M3 q = q_of(qa, dir, i, &c0, &c1);
      ocplx f[3], b1[3], b2[3];
      ch_coeffs(c0, c1, f, b1, b2, 0);
      M3 e = poly(f[0], f[1], f[2], q, mmul(q, q));
      st_full(uout, dir, i, mmul(e, ld_link(u, dir, i)), 2);
    }
}

/* one isotropic stout step (stouting.c:74-104) */
void orc_stout(const ocplx *u, ocplx *uout, double rho)
{
  ocplx *stap = calloc(72 * SHH, sizeof(ocplx));
  double *qa = calloc(64 * SHH, sizeof(double));
  orc_staples(u, stap);
  orc_rho_ta(u, stap, qa, rho);
  orc_exp_times_conf(u, qa, uout);
  free(stap);
  free(qa);
}

/* Lambda from Sigma', U, Q_A (stouting.c:171-546; Morningstar-Peardon eqs. 70-74):
 * Gamma = tr(S' B1 U) Q + tr(S' B2 U) Q^2 + f1 U S' + f2 (Q U S' + U S' Q),
 * Lambda = (Gamma + Gamma^+)/2 - tr(Gamma + Gamma^+)/6 */
void orc_lambda(double *lam, const ocplx *sp, const ocplx *u, double *qa)
{
  for (int dir = 0; dir < 8; dir++)
    for (long i = 0; i < SHH; i++) {
      double c0, c1;
      M3 q = q_of(qa, dir, i, &c0, &c1), q2 = mmul(q, q);
      ocplx f[3], b1[3], b2[3];
      ch_coeffs(c0, c1, f, b1, b2, 1);
      M3 U = ld_link(u, dir, i), S = ld_full(sp, dir, i);
      M3 B1 = poly(b1[0], b1[1], b1[2], q, q2), B2 = poly(b2[0], b2[1], b2[2], q, q2);
      ocplx t1 = mtr(mmul(S, mmul(B1, U))), t2 = mtr(mmul(S, mmul(B2, U)));
      M3 US = mmul(U, S);
      M3 G = madd(madd(mscale(q, t1), mscale(q2, t2)),
                  madd(mscale(US, f[1]), mscale(madd(mmul(q, US), mmul(US, q)), f[2])));
      M3 H = madd(G, mdag(G));
      ocplx tr = mtr(H);
      M3 L = madd(mscale(H, 0.5), mid(-tr / 6.0));
      st_thmat(lam, dir, i, L);
    }
}

/* Sigma = Sigma' exp(iQ) + i rho {staple terms with Lambda}
 * (stouting.c:550-1302; Morningstar-Peardon eq. 75) */
void orc_sigma(double *lam, const ocplx *u, ocplx *s, double *qa, double rho)
{
  ocplx *out = calloc(72 * SHH, sizeof(ocplx));
  int d[4];
  const ocplx ir = I * rho;
  for (d[3] = 0; d[3] < NN[3]; d[3]++)
    for (d[2] = 0; d[2] < NN[2]; d[2]++)
      for (d[1] = 0; d[1] < NN[1]; d[1]++)
        for (d[0] = 0; d[0] < NN[0]; d[0]++) {
          int p = (d[0] + d[1] + d[2] + d[3]) & 1;
          long x = sn(d);
          for (int mu = 0; mu < 4; mu++) {
            int dm = 2 * mu + p;
            double c0, c1;
            M3 q = q_of(qa, dm, x, &c0, &c1);
            ocplx f[3], b1[3], b2[3];
            ch_coeffs(c0, c1, f, b1, b2, 0);
            M3 E = poly(f[0], f[1], f[2], q, mmul(q, q));
            /* the reference keeps exp(iQ) as an SU(3) matrix: rebuild its third row */
            E.m[2][0] = conj(E.m[0][1] * E.m[1][2] - E.m[0][2] * E.m[1][1]);
            E.m[2][1] = conj(E.m[0][2] * E.m[1][0] - E.m[0][0] * E.m[1][2]);
            E.m[2][2] = conj(E.m[0][0] * E.m[1][1] - E.m[0][1] * E.m[1][0]);
            M3 acc = mmul(ld_full(s, dm, x), E);
            M3 Lmu = ld_thmat(lam, dm, x);
            long xpm = shift(d, mu, 1);
            for (int nu = 0; nu < 4; nu++) {
              if (nu == mu) continue;
              long xpn = shift(d, nu, 1), xmn = shift(d, nu, -1);
              int e[4] = {d[0], d[1], d[2], d[3]};
              e[mu] = (e[mu] + 1) % NN[mu];
              long xpmmn = shift(e, nu, -1);
              /* right: A = U_nu(x+mu), B = U_mu(x+nu)^+, C = U_nu(x)^+ */
              M3 A = ld_link(u, 2 * nu + !p, xpm), B = mdag(ld_link(u, 2 * mu + !p, xpn)), C = mdag(ld_link(u, 2 * nu + p, x));
              M3 Lnu_x = ld_thmat(lam, 2 * nu + p, x);
              M3 Lnu_xpm = ld_thmat(lam, 2 * nu + !p, xpm);
              M3 Lmu_xpn = ld_thmat(lam, 2 * mu + !p, xpn);
              M3 D = Lmu; for (int a = 0; a < 3; a++) for (int b = 0; b < 3; b++) D.m[a][b] -= Lnu_x.m[a][b];
              acc = madd(acc, mscale(mmul(mmul(A, B), mmul(C, D)), ir));
              acc = madd(acc, mscale(mmul(Lnu_xpm, mmul(A, mmul(B, C))), ir));
              acc = madd(acc, mscale(mmul(mmul(A, B), mmul(Lmu_xpn, C)), -ir));
              /* left: A = U_nu(x+mu-nu)^+, B = U_mu(x-nu)^+, C = U_nu(x-nu) */
              A = mdag(ld_link(u, 2 * nu + p, xpmmn));
              B = mdag(ld_link(u, 2 * mu + !p, xmn));
              C = ld_link(u, 2 * nu + !p, xmn);
              M3 Lnu_xmn = ld_thmat(lam, 2 * nu + !p, xmn), Lmu_xmn = ld_thmat(lam, 2 * mu + !p, xmn);
              M3 Lnu_xpmmn = ld_thmat(lam, 2 * nu + p, xpmmn);
              M3 G = Lnu_xmn; for (int a = 0; a < 3; a++) for (int b = 0; b < 3; b++) G.m[a][b] -= Lmu_xmn.m[a][b];
              acc = madd(acc, mscale(mmul(mmul(A, B), mmul(G, C)), ir));
              acc = madd(acc, mscale(mmul(mmul(A, B), mmul(C, Lmu)), ir));
              acc = madd(acc, mscale(mmul(A, mmul(Lnu_xpmmn, mmul(B, C))), -ir));
            }
            st_full(out, dm, x, acc, 3);
          }
        }
  memcpy(s, out, 72 * SHH * sizeof(ocplx));
  free(out);
}

/* Sigma' -> Sigma through one stout level (fermion_force.c:52-162) */
void orc_sigma_prime_to_sigma(ocplx *sigma, const ocplx *u, double rho)
{
  ocplx *stap = calloc(72 * SHH, sizeof(ocplx));
  double *qa = calloc(64 * SHH, sizeof(double));
  double *lam = calloc(64 * SHH, sizeof(double));
  orc_staples(u, stap);
  orc_rho_ta(u, stap, qa, rho);
  orc_lambda(lam, sigma, u, qa);
  orc_sigma(lam, u, sigma, qa, rho);
  free(stap); free(qa); free(lam);
}

/* aux[2mu](x_e) += a_k Y_k(x_e+mu) (x) X_k(x_e)^+ ;
 * aux[2mu+1](x_o) += -a_k X_k(x_o+mu) (x) Y_k(x_o)^+, Y_k = D_oe X_k
 * (fermion_force_utilities.c:30-93, 183-201) */
void orc_force_outer(const ocplx *u, ocplx *aux, const ocplx *xs, const double *ph, int order, const double *a)
{
  long n = 3 * SHH;
  ocplx *y = calloc(n, sizeof(ocplx));
  for (int k = 0; k < order; k++) {
    const ocplx *x = xs + k * n;
    orc_Doe(u, y, x, ph);
    int d[4];
    for (d[3] = 0; d[3] < NN[3]; d[3]++)
      for (d[2] = 0; d[2] < NN[2]; d[2]++)
        for (d[1] = 0; d[1] < NN[1]; d[1]++)
          for (d[0] = 0; d[0] < NN[0]; d[0]++) {
            int p = (d[0] + d[1] + d[2] + d[3]) & 1;
            long i = sn(d);
            for (int mu = 0; mu < 4; mu++) {
              long j = shift(d, mu, 1);
              const ocplx *l = p ? x : y, *r = p ? y : x;   /* left at x+mu, right at x */
              double f = p ? -a[k] : a[k];
              for (int rr = 0; rr < 3; rr++)
                for (int cc = 0; cc < 3; cc++)
                  aux[((long)(2 * mu + p) * 9 + rr * 3 + cc) * SHH + i] += l[rr * SHH + j] * (f * conj(r[cc * SHH + i]));
            }
          }
  }
  free(y);
}

/* pseudo_ipdot[dir] += e^{i theta} aux[dir] (fermion_force_utilities.c:123-153) */
void orc_backfield_times_force(const double *ph, const ocplx *aux, ocplx *pip)
{
  for (int dir = 0; dir < 8; dir++)
    for (long i = 0; i < SHH; i++) {
      double t = ph[(long)dir * SHH + i];
      ocplx e = cos(t) + I * sin(t);
      for (int k = 0; k < 9; k++) pip[((long)dir * 9 + k) * SHH + i] += aux[((long)dir * 9 + k) * SHH + i] * e;
    }
}

/* ipdot -= TA(U Sigma), TA without the rho/C_ZERO factor
 * (fermion_force_utilities.c:95-121, fermion_force_utilities.h:106-150) */
void orc_conf_times_force_ta(const ocplx *u, const ocplx *sigma, double *ipdot)
{
  double *tmp = calloc(64 * SHH, sizeof(double));
  for (int dir = 0; dir < 8; dir++)
    for (long i = 0; i < SHH; i++) {
      st_ta(tmp, dir, i, mmul(ld_link(u, dir, i), ld_full(sigma, dir, i)), 1.0);
      for (int k = 0; k < 3; k++) blk_c(ipdot, dir, k)[i] -= blk_c(tmp, dir, k)[i];
      for (int k = 0; k < 2; k++) blk_r(ipdot, dir, k)[i] -= blk_r(tmp, dir, k)[i];
    }
  free(tmp);
}

/* f_j, b_1j, b_2j as 18 doubles (re, im interleaved), for tests */
void orc_ch_coeffs(double c0, double c1, double *out)
{
  ocplx f[3], b1[3], b2[3];
  ch_coeffs(c0, c1, f, b1, b2, 1);
  for (int j = 0; j < 3; j++) {
    out[2 * j] = creal(f[j]); out[2 * j + 1] = cimag(f[j]);
    out[6 + 2 * j] = creal(b1[j]); out[7 + 2 * j] = cimag(b1[j]);
    out[12 + 2 * j] = creal(b2[j]); out[13 + 2 * j] = cimag(b2[j]);
  }
}

/* ==== pure-gauge tree-level Symanzik HMC (restated from ipdot_gauge.c,
 * plaquettes.c, rectangles.c, su3_utilities.c, su3_measurements.c,
 * md_integrator.c, md_parameters.c) ==== */

#define C_ONE (-0.25 * 0.33333333333333333333333)   /* tree-level Symanzik c1 (common_defines.h:75) */

/* link U_mu(x + a e_s + b e_t), its parity taken from the shifted site */
static M3 lk(const ocplx *u, const int d[4], int mu, int s, int a, int t, int b)
{
  int e[4] = {d[0], d[1], d[2], d[3]};
  e[s] = ((e[s] + a) % NN[s] + NN[s]) % NN[s];
  e[t] = ((e[t] + b) % NN[t] + NN[t]) % NN[t];
  int p = (e[0] + e[1] + e[2] + e[3]) & 1;
  return ld_link(u, 2 * mu + p, sn(e));
}

static M3 m5(M3 a, M3 b, M3 c, M3 d, M3 e) { return mmul(mmul(mmul(mmul(a, b), c), d), e); }

/* dS/dU of the tree-level Symanzik action for the link (x, mu), the
 * closing paths from x+mu back to x: C_ZERO x the 6 plaquette staples
 * (plaquettes.c:83-195) + C_ONE x the 18 rectangle staples of types A, B, C
 * (rectangles.c:643-917):
 *   A_R = U_n(x+m) U_n(x+m+n) U_m(x+2n)^+ U_n(x+n)^+ U_n(x)^+
 *   A_L = U_n(x+m-n)^+ U_n(x+m-2n)^+ U_m(x-2n)^+ U_n(x-2n) U_n(x-n)
 *   B_R = U_m(x+m) U_n(x+2m) U_m(x+m+n)^+ U_m(x+n)^+ U_n(x)^+
 *   B_L = U_m(x+m) U_n(x+2m-n)^+ U_m(x+m-n)^+ U_m(x-n)^+ U_n(x-n)
 *   C_R = U_n(x+m) U_m(x+n)^+ U_m(x-m+n)^+ U_n(x-m)^+ U_m(x-m)
 *   C_L = U_n(x+m-n)^+ U_m(x-n)^+ U_m(x-m-n)^+ U_n(x-m-n) U_m(x-m) */
static M3 gauge_staple(const ocplx *u, const int d[4], int m)
{
  M3 pl = mzero(), re = mzero();
  for (int n = 0; n < 4; n++) {
    if (n == m) continue;
    M3 r = mmul(mmul(lk(u, d, n, m, 1, n, 0), mdag(lk(u, d, m, n, 1, m, 0))), mdag(lk(u, d, n, m, 0, n, 0)));
    M3 l = mmul(mmul(mdag(lk(u, d, n, m, 1, n, -1)), mdag(lk(u, d, m, n, -1, m, 0))), lk(u, d, n, n, -1, m, 0));
    pl = madd(pl, madd(r, l));
    M3 ar = m5(lk(u, d, n, m, 1, n, 0), lk(u, d, n, m, 1, n, 1), mdag(lk(u, d, m, n, 2, m, 0)),
               mdag(lk(u, d, n, n, 1, m, 0)), mdag(lk(u, d, n, n, 0, m, 0)));
    M3 al = m5(mdag(lk(u, d, n, m, 1, n, -1)), mdag(lk(u, d, n, m, 1, n, -2)), mdag(lk(u, d, m, n, -2, m, 0)),
               lk(u, d, n, n, -2, m, 0), lk(u, d, n, n, -1, m, 0));
    M3 br = m5(lk(u, d, m, m, 1, n, 0), lk(u, d, n, m, 2, n, 0), mdag(lk(u, d, m, m, 1, n, 1)),
               mdag(lk(u, d, m, n, 1, m, 0)), mdag(lk(u, d, n, n, 0, m, 0)));
    M3 bl = m5(lk(u, d, m, m, 1, n, 0), mdag(lk(u, d, n, m, 2, n, -1)), mdag(lk(u, d, m, m, 1, n, -1)),
               mdag(lk(u, d, m, n, -1, m, 0)), lk(u, d, n, n, -1, m, 0));
    M3 cr = m5(lk(u, d, n, m, 1, n, 0), mdag(lk(u, d, m, n, 1, m, 0)), mdag(lk(u, d, m, m, -1, n, 1)),
               mdag(lk(u, d, n, m, -1, n, 0)), lk(u, d, m, m, -1, n, 0));
    M3 cl = m5(mdag(lk(u, d, n, m, 1, n, -1)), mdag(lk(u, d, m, n, -1, m, 0)), mdag(lk(u, d, m, m, -1, n, -1)),
               lk(u, d, n, m, -1, n, -1), lk(u, d, m, m, -1, n, 0));
    re = madd(re, madd(madd(madd(ar, al), madd(br, bl)), madd(cr, cl)));
  }
  return madd(mscale(pl, C_ZERO), mscale(re, C_ONE));
}

void orc_gauge_staples(const ocplx *u, ocplx *stap)
{
  int d[4];
  for (d[3] = 0; d[3] < NN[3]; d[3]++)
    for (d[2] = 0; d[2] < NN[2]; d[2]++)
      for (d[1] = 0; d[1] < NN[1]; d[1]++)
        for (d[0] = 0; d[0] < NN[0]; d[0]++) {
          int p = (d[0] + d[1] + d[2] + d[3]) & 1;
          for (int mu = 0; mu < 4; mu++) st_full(stap, 2 * mu + p, sn(d), gauge_staple(u, d, mu), 3);
        }
}

/* tipdot = TA(U dS/dU) for every link (ipdot_gauge.c:192-212 +
 * su3_utilities.c:146-175, su3_utilities.h:979-1035) */
void orc_ipdot_gauge(const ocplx *u, double *ipdot)
{
  int d[4];
  for (d[3] = 0; d[3] < NN[3]; d[3]++)
    for (d[2] = 0; d[2] < NN[2]; d[2]++)
      for (d[1] = 0; d[1] < NN[1]; d[1]++)
        for (d[0] = 0; d[0] < NN[0]; d[0]++) {
          int p = (d[0] + d[1] + d[2] + d[3]) & 1;
          long x = sn(d);
          for (int mu = 0; mu < 4; mu++) {
            int dir = 2 * mu + p;
            st_ta(ipdot, dir, x, mmul(ld_link(u, dir, x), gauge_staple(u, d, mu)), 1.0);
          }
        }
}

/* sum over sites and planes mu < nu of Re tr of the plaquette
 * U_mu(x) U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+ (su3_measurements.c:191-213,
 * plaquettes.c:14-80) */
double orc_plaquette_sum(const ocplx *u)
{
  double s = 0;
  int d[4];
  for (d[3] = 0; d[3] < NN[3]; d[3]++)
    for (d[2] = 0; d[2] < NN[2]; d[2]++)
      for (d[1] = 0; d[1] < NN[1]; d[1]++)
        for (d[0] = 0; d[0] < NN[0]; d[0]++)
          for (int m = 0; m < 3; m++)
            for (int n = m + 1; n < 4; n++) {
              M3 pq = mmul(mmul(lk(u, d, m, m, 0, n, 0), lk(u, d, n, m, 1, n, 0)),
                           mmul(mdag(lk(u, d, m, n, 1, m, 0)), mdag(lk(u, d, n, m, 0, n, 0))));
              s += creal(mtr(pq));
            }
  return s;
}

/* sum over sites and planes mu < nu of Re tr of the 2x1 and 1x2 rectangles
 * (rectangles.c:16-164, 1890-1909):
 *   U_m(x) U_m(x+m) U_n(x+2m) U_m(x+m+n)^+ U_m(x+n)^+ U_n(x)^+
 *   U_m(x) U_n(x+m) U_n(x+m+n) U_m(x+2n)^+ U_n(x+n)^+ U_n(x)^+ */
double orc_rectangle_sum(const ocplx *u)
{
  double s = 0;
  int d[4];
  for (d[3] = 0; d[3] < NN[3]; d[3]++)
    for (d[2] = 0; d[2] < NN[2]; d[2]++)
      for (d[1] = 0; d[1] < NN[1]; d[1]++)
        for (d[0] = 0; d[0] < NN[0]; d[0]++)
          for (int m = 0; m < 3; m++)
            for (int n = m + 1; n < 4; n++) {
              M3 a = mmul(m5(lk(u, d, m, m, 0, n, 0), lk(u, d, m, m, 1, n, 0), lk(u, d, n, m, 2, n, 0),
                             mdag(lk(u, d, m, m, 1, n, 1)), mdag(lk(u, d, m, n, 1, m, 0))),
                          mdag(lk(u, d, n, m, 0, n, 0)));
              M3 b = mmul(m5(lk(u, d, m, m, 0, n, 0), lk(u, d, n, m, 1, n, 0), lk(u, d, n, m, 1, n, 1),
                             mdag(lk(u, d, m, n, 2, m, 0)), mdag(lk(u, d, n, n, 1, m, 0))),
                          mdag(lk(u, d, n, m, 0, n, 0)));
              s += creal(mtr(a)) + creal(mtr(b));
            }
  return s;
}

/* sum over all links of 1/2 tr P^2 = a^2 + b^2 + ab + |c01|^2 + |c02|^2 + |c12|^2
 * (su3_measurements.c:138-168, su3_utilities.h:1295-1307) */
double orc_momenta_action(double *mom)
{
  double s = 0;
  for (int dir = 0; dir < 8; dir++)
    for (long i = 0; i < SHH; i++) {
      double a = blk_r(mom, dir, 0)[i], b = blk_r(mom, dir, 1)[i];
      ocplx c = blk_c(mom, dir, 0)[i], e = blk_c(mom, dir, 1)[i], f = blk_c(mom, dir, 2)[i];
      s += a * a + b * b + a * b + creal(c) * creal(c) + cimag(c) * cimag(c) + creal(e) * creal(e) +
           cimag(e) * cimag(e) + creal(f) * creal(f) + cimag(f) * cimag(f);
    }
  return s;
}

/* mom -= i fact ipdot on the complex entries, mom_kk += fact ipdot_kk on the
 * real diagonals (su3_utilities.c:241-270, su3_utilities.h:1383-1395) */
void orc_mom_sum_mult(double *mom, double *ipdot, double fact)
{
  for (int dir = 0; dir < 8; dir++)
    for (long i = 0; i < SHH; i++) {
      for (int k = 0; k < 3; k++) blk_c(mom, dir, k)[i] -= I * fact * blk_c(ipdot, dir, k)[i];
      for (int k = 0; k < 2; k++) blk_r(mom, dir, k)[i] += fact * blk_r(ipdot, dir, k)[i];
    }
}

/* U = exp(i delta P) U with rows 0-1 reunitarised by Gram-Schmidt
 * (su3_utilities.c:272-305, su3_utilities.h:1433-1537): exp(-Q_A) of the
 * anti-Hermitian Q_A = -i delta P */
void orc_mom_exp_times_conf(ocplx *u, double *mom, double delta)
{
  double *qa = calloc(64 * SHH, sizeof(double));
  for (int dir = 0; dir < 8; dir++)
    for (long i = 0; i < SHH; i++) {
      for (int k = 0; k < 3; k++) blk_c(qa, dir, k)[i] = -blk_c(mom, dir, k)[i] * delta * I;
      for (int k = 0; k < 2; k++) blk_r(qa, dir, k)[i] = -blk_r(mom, dir, k)[i] * delta;
    }
  for (int dir = 0; dir < 8; dir++)
    for (long i = 0; i < SHH; i++) {
      double c0, c1;
      M3 q = q_of(qa, dir, i, &c0, &c1);
      ocplx f[3], b1[3], b2[3];
      ch_coeffs(c0, c1, f, b1, b2, 0);
      M3 r = mmul(poly(f[0], f[1], f[2], q, mmul(q, q)), ld_link(u, dir, i));
      double n0 = 0;
      for (int c = 0; c < 3; c++) n0 += creal(r.m[0][c]) * creal(r.m[0][c]) + cimag(r.m[0][c]) * cimag(r.m[0][c]);
      n0 = 1.0 / sqrt(n0);
      for (int c = 0; c < 3; c++) r.m[0][c] *= n0;
      ocplx sp = conj(r.m[0][0]) * r.m[1][0] + conj(r.m[0][1]) * r.m[1][1] + conj(r.m[0][2]) * r.m[1][2];
      for (int c = 0; c < 3; c++) r.m[1][c] -= sp * r.m[0][c];
      double n1 = 0;
      for (int c = 0; c < 3; c++) n1 += creal(r.m[1][c]) * creal(r.m[1][c]) + cimag(r.m[1][c]) * cimag(r.m[1][c]);
      n1 = 1.0 / sqrt(n1);
      for (int c = 0; c < 3; c++) r.m[1][c] *= n1;
      st_full(u, dir, i, r, 2);
    }
  free(qa);
}

/* the integrator coefficients of initialize_md_global_variables
 * (md_parameters.c:11-50; Omelyan lambda = 0.1931833275037836) */
void orc_md_deltas(double beta, int no_md, int gauge_scale, double t, double *d)
{
  const double lambda = 0.1931833275037836;
  const double b3 = beta * 0.33333333333333333333333;
  d[0] = -t / no_md * lambda;
  d[1] = -t / no_md * (1.0 - 2.0 * lambda);
  d[2] = -t / no_md * 2.0 * lambda;
  d[3] = -t / (2 * no_md * gauge_scale) * lambda * b3;
  d[4] = 0.5 * t / (2 * no_md * gauge_scale);
  d[5] = -t / (2 * no_md * gauge_scale) * (1.0 - 2.0 * lambda) * b3;
  d[6] = -t / (2 * no_md * gauge_scale) * 2.0 * lambda * b3;
}

/* ncalls x multistep_2MN_gauge (md_integrator.c:256-376):
 *   K(d3) X [K(d5) X K(d6) X]^(gauge_scale-1) K(d5) X K(d3)
 * with K(f): mom += f TA(U dS/dU) and X: U = exp(i d4 P) U */
void orc_2mn_gauge(ocplx *u, double *mom, double beta, int no_md, int gauge_scale, double t, int ncalls)
{
  double d[7];
  orc_md_deltas(beta, no_md, gauge_scale, t, d);
  double *ip = calloc(64 * SHH, sizeof(double));
  for (int c = 0; c < ncalls; c++) {
    orc_ipdot_gauge(u, ip); orc_mom_sum_mult(mom, ip, d[3]); orc_mom_exp_times_conf(u, mom, d[4]);
    for (int k = 1; k < gauge_scale; k++) {
      orc_ipdot_gauge(u, ip); orc_mom_sum_mult(mom, ip, d[5]); orc_mom_exp_times_conf(u, mom, d[4]);
      orc_ipdot_gauge(u, ip); orc_mom_sum_mult(mom, ip, d[6]); orc_mom_exp_times_conf(u, mom, d[4]);
    }
    orc_ipdot_gauge(u, ip); orc_mom_sum_mult(mom, ip, d[5]); orc_mom_exp_times_conf(u, mom, d[4]);
    orc_ipdot_gauge(u, ip); orc_mom_sum_mult(mom, ip, d[3]);
  }
  free(ip);
}
