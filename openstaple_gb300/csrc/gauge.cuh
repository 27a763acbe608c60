// gauge.cuh -- 3x3 complex matrix arithmetic and the Cayley-Hamilton
// exponential exp(iQ) = f0 + f1 Q + f2 Q^2 with its derivative coefficients,
// for the stout smearing and the stout force chain (FP64).
//
// Formats (reference layouts, per link direction, sizeh entries each):
//   su3   : 9 complex arrays r0c0..r2c2 (only r0, r1 stored for links)
//   tamat : c01, c02, c12 complex, ic00, ic11 real  (anti-Hermitian traceless)
//   thmat : c01, c02, c12 complex, rc00, rc11 real  (Hermitian traceless)
#pragma once
#include "common.cuh"

namespace ost {

struct M3 { double2 m[3][3]; };

OST_D double2 zc() { return make_double2(0.0, 0.0); }
OST_D double2 cm(double2 a, double2 b) { return cmul(a, b); }
OST_D double2 cjm(double2 a) { return make_double2(a.x, -a.y); }
OST_D double2 csc(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
OST_D double2 cadd2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
OST_D double2 csub2(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
OST_D double2 cmuli(double2 a) { return make_double2(-a.y, a.x); }    // i a

OST_D M3 mzero() { M3 z; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) z.m[i][j] = zc(); return z; }

OST_D M3 mmul(const M3& a, const M3& b) {
  M3 c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double2 s = cm(a.m[i][0], b.m[0][j]);
      cmac(s, a.m[i][1], b.m[1][j]);
      cmac(s, a.m[i][2], b.m[2][j]);
      c.m[i][j] = s;
    }
  return c;
}
// a^+ b
OST_D M3 mdagmul(const M3& a, const M3& b) {
  M3 c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double2 s = conjmul(a.m[0][i], b.m[0][j]);
      cmacc(s, a.m[1][i], b.m[1][j]);
      cmacc(s, a.m[2][i], b.m[2][j]);
      c.m[i][j] = s;
    }
  return c;
}
// a b^+
OST_D M3 mmuldag(const M3& a, const M3& b) {
  M3 c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double2 s = conjmul(b.m[j][0], a.m[i][0]);
      cmacc(s, b.m[j][1], a.m[i][1]);
      cmacc(s, b.m[j][2], a.m[i][2]);
      c.m[i][j] = s;
    }
  return c;
}
OST_D M3 mdag(const M3& a) {
  M3 c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) c.m[i][j] = cjm(a.m[j][i]);
  return c;
}
OST_D void madd_to(M3& a, const M3& b) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) a.m[i][j] = cadd2(a.m[i][j], b.m[i][j]);
}
OST_D void madd_scaled(M3& a, const M3& b, double2 s) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) cmac(a.m[i][j], b.m[i][j], s);
}
OST_D M3 mscale(const M3& a, double2 s) {
  M3 c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) c.m[i][j] = cm(a.m[i][j], s);
  return c;
}
OST_D double2 mtrace(const M3& a) { return cadd2(cadd2(a.m[0][0], a.m[1][1]), a.m[2][2]); }
// tr(a b)
OST_D double2 mtrace_mul(const M3& a, const M3& b) {
  double2 s = zc();
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) cmac(s, a.m[i][k], b.m[k][i]);
  return s;
}
OST_D void rebuild_row2(M3& a) {
  a.m[2][0] = conj_cross(a.m[0][1], a.m[1][2], a.m[0][2], a.m[1][1]);
  a.m[2][1] = conj_cross(a.m[0][2], a.m[1][0], a.m[0][0], a.m[1][2]);
  a.m[2][2] = conj_cross(a.m[0][0], a.m[1][1], a.m[0][1], a.m[1][0]);
}

// ---- field access ----
struct SU3Field {
  double2* p;
  long sh;
  OST_D double2* at(int dir, int r, int c) const { return p + (long(dir) * 9 + r * 3 + c) * sh; }
};

OST_D M3 ld_link(const SU3Field& f, int dir, long i) {
  M3 a;
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) a.m[r][c] = __ldg(f.at(dir, r, c) + i);
  rebuild_row2(a);
  return a;
}
OST_D M3 ld_full(const SU3Field& f, int dir, long i) {
  M3 a;
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) a.m[r][c] = f.at(dir, r, c)[i];
  return a;
}
OST_D void st_rows(const SU3Field& f, int dir, long i, const M3& a, int rows) {
  for (int r = 0; r < rows; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) f.at(dir, r, c)[i] = a.m[r][c];
}

struct AlgField {    // tamat_soa[8] or thmat_soa[8]: per dir 3 complex + 2 real arrays
  double* p;
  long sh;
  OST_D double2* c(int dir, int k) const { return reinterpret_cast<double2*>(p + long(dir) * 8 * sh) + long(k) * sh; }
  OST_D double* r(int dir, int k) const { return p + long(dir) * 8 * sh + 6 * sh + long(k) * sh; }
};

// Q = i Q_A for an anti-Hermitian traceless Q_A stored as tamat
OST_D M3 ld_q_from_tamat(const AlgField& t, int dir, long i) {
  double2 c01 = t.c(dir, 0)[i], c02 = t.c(dir, 1)[i], c12 = t.c(dir, 2)[i];
  double a = t.r(dir, 0)[i], b = t.r(dir, 1)[i];
  M3 q;
  q.m[0][0] = make_double2(-a, 0.0);
  q.m[1][1] = make_double2(-b, 0.0);
  q.m[2][2] = make_double2(a + b, 0.0);
  q.m[0][1] = cmuli(c01);
  q.m[0][2] = cmuli(c02);
  q.m[1][2] = cmuli(c12);
  q.m[1][0] = cjm(q.m[0][1]);
  q.m[2][0] = cjm(q.m[0][2]);
  q.m[2][1] = cjm(q.m[1][2]);
  return q;
}
OST_D M3 ld_thmat(const AlgField& t, int dir, long i) {
  double2 c01 = t.c(dir, 0)[i], c02 = t.c(dir, 1)[i], c12 = t.c(dir, 2)[i];
  double a = t.r(dir, 0)[i], b = t.r(dir, 1)[i];
  M3 m;
  m.m[0][0] = make_double2(a, 0.0);
  m.m[1][1] = make_double2(b, 0.0);
  m.m[2][2] = make_double2(-(a + b), 0.0);
  m.m[0][1] = c01; m.m[0][2] = c02; m.m[1][2] = c12;
  m.m[1][0] = cjm(c01); m.m[2][0] = cjm(c02); m.m[2][1] = cjm(c12);
  return m;
}
OST_D void st_thmat(const AlgField& t, int dir, long i, const M3& m) {
  t.c(dir, 0)[i] = m.m[0][1];
  t.c(dir, 1)[i] = m.m[0][2];
  t.c(dir, 2)[i] = m.m[1][2];
  t.r(dir, 0)[i] = m.m[0][0].x;
  t.r(dir, 1)[i] = m.m[1][1].x;
}
// s * TA(m): c_ij = s (m_ij - conj(m_ji))/2, ic_kk = s (Im m_kk - Im tr m / 3)
// (su3_utilities.h:1097-1152)
struct TA { double2 c01, c02, c12; double a, b; };
OST_D TA ta_of(const M3& m, double s) {
  TA t;
  const double third = 0.33333333333333333333333;
  double tr = (m.m[0][0].y + m.m[1][1].y + m.m[2][2].y) * third;
  t.c01 = csc(csc(csub2(m.m[0][1], cjm(m.m[1][0])), 0.5), s);
  t.c02 = csc(csc(csub2(m.m[0][2], cjm(m.m[2][0])), 0.5), s);
  t.c12 = csc(csc(csub2(m.m[1][2], cjm(m.m[2][1])), 0.5), s);
  t.a = s * (m.m[0][0].y - tr);
  t.b = s * (m.m[1][1].y - tr);
  return t;
}

// ---- Cayley-Hamilton coefficients ----
// Small c1 (< 4e-3): polynomial in (c0, c1) truncated at total weight 7
// (weight 3 for c0, 2 for c1), table built on the host (gauge.cu).
struct CHTable { double2 f[3][8]; int i0[8]; int j1[8]; };
// Every translation unit that includes this header has its own copy of the
// table in constant memory and uploads fill_ch_table()'s values before use
// (gauge.cu: ensure_ch_table, hmc.cu: its own).
static __constant__ CHTable c_ch_table;
void fill_ch_table(CHTable* table);   // host, gauge.cu

struct CHCoeffs { double2 f[3], b1[3], b2[3]; };

OST_D double ipow(double x, int n) { double r = 1.0; for (int k = 0; k < n; ++k) r *= x; return r; }

// exp(iQ) = f0 + f1 Q + f2 Q^2 and (if NEED_B) b_1j = df_j/dc1, b_2j = df_j/dc0
// (Morningstar & Peardon, hep-lat/0311018, eqs. 23-34 and 57-65).
template <bool NEED_B>
OST_D CHCoeffs ch_coeffs(double c0, double c1) {
  CHCoeffs r;
  if (c1 < 4.0e-3) {
#pragma unroll
    for (int j = 0; j < 3; ++j) { r.f[j] = zc(); r.b1[j] = zc(); r.b2[j] = zc(); }
    for (int k = 0; k < 8; ++k) {
      const int a = c_ch_table.i0[k], b = c_ch_table.j1[k];
      const double mon = ipow(c0, a) * ipow(c1, b);
      const double d1 = b > 0 ? double(b) * ipow(c0, a) * ipow(c1, b - 1) : 0.0;
      const double d0 = a > 0 ? double(a) * ipow(c0, a - 1) * ipow(c1, b) : 0.0;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double2 t = c_ch_table.f[j][k];
        r.f[j] = cadd2(r.f[j], csc(t, mon));
        if (NEED_B) { r.b1[j] = cadd2(r.b1[j], csc(t, d1)); r.b2[j] = cadd2(r.b2[j], csc(t, d0)); }
      }
    }
    return r;
  }
  const bool neg = c0 < 0;
  if (neg) c0 = -c0;
  const double c0max = 2.0 * pow(c1 / 3.0, 1.5);
  const double eps = (c0max - c0) / c0max;
  double th;
  if (eps < 0) th = 0.0;
  else if (eps < 1e-3)   // arccos(1 - eps) series
    th = sqrt(2 * eps) * (1 + (1.0 / 12 + (3.0 / 160 + (5.0 / 896 + (35.0 / 18432 + 63.0 / 90112 * eps) * eps) * eps) * eps) * eps);
  else th = acos(c0 / c0max);
  const double u = sqrt(c1 / 3.0) * cos(th / 3.0), w = sqrt(c1) * sin(th / 3.0);
  const double u2 = u * u, w2 = w * w;
  double xi0, xi1;
  if (fabs(w) < 0.05) {
    xi0 = 1 - w2 / 6 * (1 - w2 / 20 * (1 - w2 / 42));
    xi1 = -(1 - w2 * (1 - w2 * (1 - w2 / 54) / 28) / 10) / 3;
  } else {
    double sw = sin(w);
    xi0 = sw / w;
    xi1 = cos(w) / w2 - sw / (w2 * w);
  }
  double s2u, c2u, su, cu;
  sincos(2 * u, &s2u, &c2u);
  sincos(u, &su, &cu);
  const double2 e2 = make_double2(c2u, s2u);   // e^{2iu}
  const double2 em = make_double2(cu, -su);    // e^{-iu}
  const double cw = cos(w);
  // h0 = (u^2-w^2) e2 + em (8u^2 cos w + 2iu(3u^2+w^2) xi0)
  double2 h0 = cadd2(csc(e2, u2 - w2), cm(em, make_double2(8 * u2 * cw, 2 * u * (3 * u2 + w2) * xi0)));
  // h1 = 2u e2 - em (2u cos w - i(3u^2-w^2) xi0)
  double2 h1 = csub2(csc(e2, 2 * u), cm(em, make_double2(2 * u * cw, -(3 * u2 - w2) * xi0)));
  // h2 = e2 - em (cos w + 3iu xi0)
  double2 h2 = csub2(e2, cm(em, make_double2(cw, 3 * u * xi0)));
  const double den = 1.0 / (9 * u2 - w2);
  r.f[0] = csc(h0, den); r.f[1] = csc(h1, den); r.f[2] = csc(h2, den);
  if (NEED_B) {
    double2 r1[3], r2[3];
    // r0^(1) = 2(u + i(u^2-w^2)) e2 + 2 em (4u(2 - iu) cos w + i xi0 (9u^2 + w^2 - iu(3u^2 + w^2)))
    r1[0] = cadd2(cm(make_double2(2 * u, 2 * (u2 - w2)), e2),
                  csc(cm(em, cadd2(make_double2(8 * u * cw, -4 * u2 * cw),
                                   make_double2(xi0 * u * (3 * u2 + w2), xi0 * (9 * u2 + w2)))), 2.0));
    // r1^(1) = 2(1 + 2iu) e2 + em (-2(1 - iu) cos w + i(6u + i(w^2 - 3u^2)) xi0)
    r1[1] = cadd2(cm(make_double2(2.0, 4 * u), e2),
                  cm(em, make_double2(-2 * cw - (w2 - 3 * u2) * xi0, 2 * u * cw + 6 * u * xi0)));
    // r2^(1) = 2i e2 + i em (cos w - 3(1 - iu) xi0)
    r1[2] = cadd2(cmuli(csc(e2, 2.0)), cmuli(cm(em, make_double2(cw - 3 * xi0, 3 * u * xi0))));
    // r0^(2) = -2 e2 + 2iu em (cos w + (1 + 4iu) xi0 + 3u^2 xi1)
    r2[0] = cadd2(csc(e2, -2.0), cm(make_double2(0.0, 2 * u), cm(em, make_double2(cw + xi0 + 3 * u2 * xi1, 4 * u * xi0))));
    // r1^(2) = -i em (cos w + (1 + 2iu) xi0 - 3u^2 xi1)
    r2[1] = cm(make_double2(0.0, -1.0), cm(em, make_double2(cw + xi0 - 3 * u2 * xi1, 2 * u * xi0)));
    // r2^(2) = em (xi0 - 3iu xi1)
    r2[2] = cm(em, make_double2(xi0, -3 * u * xi1));
    const double hd = 0.5 * den * den;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      r.b1[j] = csc(cadd2(cadd2(csc(r1[j], 2 * u), csc(r2[j], 3 * u2 - w2)), csc(r.f[j], -2 * (15 * u2 + w2))), hd);
      r.b2[j] = csc(cadd2(cadd2(r1[j], csc(r2[j], -3 * u)), csc(r.f[j], -24 * u)), hd);
    }
  }
  if (neg) {   // f_j(-c0) = (-1)^j f_j*, b_ij(-c0) = (-1)^(i+j+1) b_ij*
    r.f[0] = cjm(r.f[0]); r.f[1] = csc(cjm(r.f[1]), -1.0); r.f[2] = cjm(r.f[2]);
    if (NEED_B) {
      r.b1[0] = cjm(r.b1[0]); r.b1[1] = csc(cjm(r.b1[1]), -1.0); r.b1[2] = cjm(r.b1[2]);
      r.b2[0] = csc(cjm(r.b2[0]), -1.0); r.b2[1] = cjm(r.b2[1]); r.b2[2] = csc(cjm(r.b2[2]), -1.0);
    }
  }
  return r;
}

// c0 = det Q = tr Q^3 / 3, c1 = tr Q^2 / 2 for traceless Hermitian Q
OST_D void q_invariants(const M3& q, const M3& q2, double* c0, double* c1) {
  *c1 = 0.5 * mtrace(q2).x;
  *c0 = mtrace_mul(q2, q).x / 3.0;
}

OST_D M3 poly3(double2 a0, double2 a1, double2 a2, const M3& q, const M3& q2) {
  M3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double2 s = cm(q.m[i][j], a1);
      cmac(s, q2.m[i][j], a2);
      if (i == j) s = cadd2(s, a0);
      r.m[i][j] = s;
    }
  return r;
}

}  // namespace ost
