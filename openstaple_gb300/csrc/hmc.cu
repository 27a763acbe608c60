// hmc.cu -- sm_103a kernels of the pure-gauge tree-level Symanzik HMC:
// the gauge force TA(U dS/dU) from the plaquette and 2x1 rectangle staples,
// the momentum kick, the link update U = exp(i delta P) U, the plaquette and
// rectangle sums of the action, 1/2 tr P^2, and Gaussian momenta from a
// counter-based generator.  One thread per link (8 directions x sizeh) or per
// site; every kernel is a template over the real type: double behind the
// reference-named FP64 entry points, float for the FP32 molecular dynamics
// of the link generator.
//
// The staple of link (x, mu) is the sum of the paths from x+mu back to x
// (plaquettes.c:83-195, rectangles.c:643-917):
//   C_ZERO x [ U_n(x+m) U_m(x+n)^+ U_n(x)^+ + U_n(x+m-n)^+ U_m(x-n)^+ U_n(x-n) ]
//   C_ONE  x [ A_R + A_L + B_R + B_L + C_R + C_L ]   (2x1 rectangles, three shapes)
// with C_ZERO = 5/3, C_ONE = -1/12.  Products keep two rows and rebuild the
// third as conj(r0 x r1), as the reference's 5-matrix helpers do.
#include <cstdio>
#include "gauge.cuh"
#include "hmc.cuh"
#include "reduce.cuh"
#include "runtime.cuh"

namespace ost {

static constexpr int H_THREADS = 128;
static constexpr double HMC_C_ZERO = 5.0 * 0.33333333333333333333333;
static constexpr double HMC_C_ONE = -0.25 * 0.33333333333333333333333;

// ---- 3x3 complex matrices in the kernel's precision ----
template <typename C> struct Mt { C m[3][3]; };
template <typename C> struct R2 { C m[2][3]; };   // rows 0, 1 of a product

template <typename C> OST_D C czero() { return cmk<C>(0, 0); }

template <typename C> OST_D void rebuild2(Mt<C>& a) {
  a.m[2][0] = conj_cross(a.m[0][1], a.m[1][2], a.m[0][2], a.m[1][1]);
  a.m[2][1] = conj_cross(a.m[0][2], a.m[1][0], a.m[0][0], a.m[1][2]);
  a.m[2][2] = conj_cross(a.m[0][0], a.m[1][1], a.m[0][1], a.m[1][0]);
}

// U_mu(y), rows 0-1 loaded, row 2 rebuilt.  rows = 9 or 6: structure of
// arrays (rows complex arrays per direction); rows = 0: the link generator's
// array of structures, the 6 complex numbers of a link contiguous (48 bytes
// in FP32: three 16-byte loads)
template <typename C> OST_D void ld_rows(const C* u, int rows, long sh, int dir, long i, C m[6]) {
  if (rows == 0) {
    const C* b = u + (long(dir) * sh + i) * 6;
    if constexpr (sizeof(C) == 8) {
      const float4* q = reinterpret_cast<const float4*>(b);
      const float4 a0 = __ldg(q), a1 = __ldg(q + 1), a2 = __ldg(q + 2);
      m[0] = cmk<C>(a0.x, a0.y); m[1] = cmk<C>(a0.z, a0.w); m[2] = cmk<C>(a1.x, a1.y);
      m[3] = cmk<C>(a1.z, a1.w); m[4] = cmk<C>(a2.x, a2.y); m[5] = cmk<C>(a2.z, a2.w);
    } else {
#pragma unroll
      for (int k = 0; k < 6; ++k) m[k] = __ldg(b + k);
    }
    return;
  }
  const C* b = u + long(dir) * rows * sh + i;
#pragma unroll
  for (int k = 0; k < 6; ++k) m[k] = __ldg(b + k * sh);
}
template <typename C> OST_D Mt<C> ld_u(const C* u, int rows, long sh, int dir, long i) {
  Mt<C> a;
  C m[6];
  ld_rows(u, rows, sh, dir, i, m);
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) a.m[r][c] = m[r * 3 + c];
  rebuild2(a);
  return a;
}
template <typename C> OST_D Mt<C> dagger(const Mt<C>& a) {
  Mt<C> d;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) d.m[i][j] = cconj(a.m[j][i]);
  return d;
}
template <typename C> OST_D R2<C> rows01(const Mt<C>& a) {
  R2<C> r;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j];
  return r;
}
// rows 0-1 of a x b
template <typename C> OST_D R2<C> mul2(const R2<C>& a, const Mt<C>& b) {
  R2<C> c;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      C s = cmul(a.m[i][0], b.m[0][j]);
      cmac(s, a.m[i][1], b.m[1][j]);
      cmac(s, a.m[i][2], b.m[2][j]);
      c.m[i][j] = s;
    }
  return c;
}
// acc += w x (rows 0-1 of p, row 2 rebuilt)
template <typename C> OST_D void add_su3(Mt<C>& acc, const R2<C>& p, decltype(C().x) w) {
  C r2[3] = {conj_cross(p.m[0][1], p.m[1][2], p.m[0][2], p.m[1][1]),
             conj_cross(p.m[0][2], p.m[1][0], p.m[0][0], p.m[1][2]),
             conj_cross(p.m[0][0], p.m[1][1], p.m[0][1], p.m[1][0])};
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    acc.m[0][j] = cmk<C>(fma(w, p.m[0][j].x, acc.m[0][j].x), fma(w, p.m[0][j].y, acc.m[0][j].y));
    acc.m[1][j] = cmk<C>(fma(w, p.m[1][j].x, acc.m[1][j].x), fma(w, p.m[1][j].y, acc.m[1][j].y));
    acc.m[2][j] = cmk<C>(fma(w, r2[j].x, acc.m[2][j].x), fma(w, r2[j].y, acc.m[2][j].y));
  }
}
template <typename C> OST_D Mt<C> mzero_t() {
  Mt<C> z;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) z.m[i][j] = czero<C>();
  return z;
}
template <typename C> OST_D C tr_re_sum(const R2<C>& p, const Mt<C>& last) {
  // Re tr(p x last) with p's row 2 rebuilt
  Mt<C> f;
  f.m[0][0] = p.m[0][0]; f.m[0][1] = p.m[0][1]; f.m[0][2] = p.m[0][2];
  f.m[1][0] = p.m[1][0]; f.m[1][1] = p.m[1][1]; f.m[1][2] = p.m[1][2];
  rebuild2(f);
  C s = czero<C>();
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) cmac(s, f.m[i][k], last.m[k][i]);
  return s;
}

// ---- lattice walking ----
struct Pos { int d[4]; };
OST_D Pos pos_of(const Site& s) { Pos p; p.d[0] = s.d0; p.d[1] = s.d1; p.d[2] = s.d2; p.d[3] = s.d3; return p; }
OST_D int wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

template <typename C> struct Walker {
  const Geom& g;
  const C* u;
  int rows;
  Pos x;
  int px;   // parity of x
  // U_mu(x + a e_s + b e_t), |a|, |b| <= 2; every coordinate shifted and
  // wrapped with selects (no indexed local array)
  OST_D Mt<C> at(int mu, int s, int a, int t, int b) const {
    const int e0 = wrap(x.d[0] + (s == 0 ? a : 0) + (t == 0 ? b : 0), g.n0);
    const int e1 = wrap(x.d[1] + (s == 1 ? a : 0) + (t == 1 ? b : 0), g.n1);
    const int e2 = wrap(x.d[2] + (s == 2 ? a : 0) + (t == 2 ? b : 0), g.n2);
    const int e3 = wrap(x.d[3] + (s == 3 ? a : 0) + (t == 3 ? b : 0), g.n3);
    const long lex = e0 + long(e1) * g.vol1 + long(e2) * g.vol2 + long(e3) * g.vol3;
    const int p = px ^ ((a + b) & 1);
    return ld_u(u, rows, long(g.sizeh), 2 * mu + p, lex >> 1);
  }
};

// the staple parts of link (x, M), C_ZERO / C_ONE included.  M is a
// template parameter and the loop over nu is unrolled, so every neighbour
// offset is a compile-time constant.
template <typename C, int M>
OST_D Mt<C> gauge_staple_t(const Walker<C>& w, int parts) {
  typedef decltype(C().x) Rt;
  const Rt c0 = Rt(HMC_C_ZERO), c1 = Rt(HMC_C_ONE);
  constexpr int m = M;
  Mt<C> S = mzero_t<C>();
#pragma unroll 1
  for (int n = 0; n < 4; ++n) {
    if (n == m) continue;
    if (parts & SP_PLAQ) {
      add_su3(S, mul2(mul2(rows01(w.at(n, m, 1, n, 0)), dagger(w.at(m, n, 1, m, 0))), dagger(w.at(n, m, 0, n, 0))), c0);
      add_su3(S, mul2(mul2(rows01(dagger(w.at(n, m, 1, n, -1))), dagger(w.at(m, n, -1, m, 0))), w.at(n, n, -1, m, 0)),
              c0);
    }
    if (parts & SP_RECT_A) {
      add_su3(S, mul2(mul2(mul2(mul2(rows01(w.at(n, m, 1, n, 0)), w.at(n, m, 1, n, 1)), dagger(w.at(m, n, 2, m, 0))),
                           dagger(w.at(n, n, 1, m, 0))), dagger(w.at(n, n, 0, m, 0))), c1);
      add_su3(S, mul2(mul2(mul2(mul2(rows01(dagger(w.at(n, m, 1, n, -1))), dagger(w.at(n, m, 1, n, -2))),
                                dagger(w.at(m, n, -2, m, 0))), w.at(n, n, -2, m, 0)), w.at(n, n, -1, m, 0)), c1);
    }
    if (parts & SP_RECT_B) {
      add_su3(S, mul2(mul2(mul2(mul2(rows01(w.at(m, m, 1, n, 0)), w.at(n, m, 2, n, 0)), dagger(w.at(m, m, 1, n, 1))),
                           dagger(w.at(m, n, 1, m, 0))), dagger(w.at(n, n, 0, m, 0))), c1);
      add_su3(S, mul2(mul2(mul2(mul2(rows01(w.at(m, m, 1, n, 0)), dagger(w.at(n, m, 2, n, -1))),
                                dagger(w.at(m, m, 1, n, -1))), dagger(w.at(m, n, -1, m, 0))), w.at(n, n, -1, m, 0)), c1);
    }
    if (parts & SP_RECT_C) {
      add_su3(S, mul2(mul2(mul2(mul2(rows01(w.at(n, m, 1, n, 0)), dagger(w.at(m, n, 1, m, 0))),
                                dagger(w.at(m, m, -1, n, 1))), dagger(w.at(n, m, -1, n, 0))), w.at(m, m, -1, n, 0)), c1);
      add_su3(S, mul2(mul2(mul2(mul2(rows01(dagger(w.at(n, m, 1, n, -1))), dagger(w.at(m, n, -1, m, 0))),
                                dagger(w.at(m, m, -1, n, -1))), w.at(n, m, -1, n, -1)), w.at(m, m, -1, n, 0)), c1);
    }
  }
  return S;
}

template <typename C>
OST_D Mt<C> gauge_staple(const Walker<C>& w, int m, int parts) {
  switch (m) {
    case 0: return gauge_staple_t<C, 0>(w, parts);
    case 1: return gauge_staple_t<C, 1>(w, parts);
    case 2: return gauge_staple_t<C, 2>(w, parts);
    default: return gauge_staple_t<C, 3>(w, parts);
  }
}

// tamat / thmat access in precision R (per direction: 3 complex arrays, then 2 real)
template <typename R> struct Alg {
  R* p;
  long sh;
  OST_D typename cplx_t<R>::type* c(int dir, int k) const {
    return reinterpret_cast<typename cplx_t<R>::type*>(p + long(dir) * 8 * sh) + long(k) * sh;
  }
  OST_D R* r(int dir, int k) const { return p + long(dir) * 8 * sh + 6 * sh + long(k) * sh; }
};

// TA(U S): c_ij = (m_ij - conj(m_ji))/2, ic_kk = Im m_kk - Im tr m / 3
// (su3_utilities.h:979-1035)
template <typename C> struct TaT { C c01, c02, c12; decltype(C().x) a, b; };
template <typename C> OST_D TaT<C> ta_of_product(const Mt<C>& U, const Mt<C>& S) {
  typedef decltype(C().x) Rt;
  Mt<C> m;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      C s = cmul(U.m[i][0], S.m[0][j]);
      cmac(s, U.m[i][1], S.m[1][j]);
      cmac(s, U.m[i][2], S.m[2][j]);
      m.m[i][j] = s;
    }
  TaT<C> t;
  const Rt half = Rt(0.5);
  t.c01 = cscale(csub(m.m[0][1], cconj(m.m[1][0])), half);
  t.c02 = cscale(csub(m.m[0][2], cconj(m.m[2][0])), half);
  t.c12 = cscale(csub(m.m[1][2], cconj(m.m[2][1])), half);
  const Rt tr = (m.m[0][0].y + m.m[1][1].y + m.m[2][2].y) * Rt(0.33333333333333333333333);
  t.a = m.m[0][0].y - tr;
  t.b = m.m[1][1].y - tr;
  return t;
}

template <typename C>
__global__ void __launch_bounds__(H_THREADS)
k_gauge_force(Geom g, const C* __restrict__ u, int rows, int parts, int mode, C* stap,
              decltype(C().x)* alg, double fact) {
  typedef decltype(C().x) Rt;
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * g.sizeh) return;
  const int dir = int(t / g.sizeh);
  const long x = t - long(dir) * g.sizeh;
  const int mu = dir >> 1, p = dir & 1;
  const Site s = site_of(g, int(x), p);
  Walker<C> w{g, u, rows, pos_of(s), p};
  const Mt<C> S = gauge_staple(w, mu, parts);
  const long sh = g.sizeh;
  if (mode == GF_STAPLES) {   // staples only, added to stap (reference layout, 9 arrays)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        C* q = stap + (long(dir) * 9 + i * 3 + j) * sh + x;
        *q = cadd(*q, S.m[i][j]);
      }
    return;
  }
  const Mt<C> U = ld_u(u, rows, sh, dir, x);
  const TaT<C> a = ta_of_product(U, S);
  Alg<Rt> A{alg, sh};
  if (mode == GF_IPDOT) {
    if (stap) {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) stap[(long(dir) * 9 + i * 3 + j) * sh + x] = S.m[i][j];
    }
    A.c(dir, 0)[x] = a.c01; A.c(dir, 1)[x] = a.c02; A.c(dir, 2)[x] = a.c12;
    A.r(dir, 0)[x] = a.a; A.r(dir, 1)[x] = a.b;
  } else {   // GF_MOM: mom -= i fact ipdot, mom_kk += fact ipdot_kk (su3_utilities.h:1383-1395)
    const Rt f = Rt(fact);
    C v;
    v = A.c(dir, 0)[x]; A.c(dir, 0)[x] = cmk<C>(fma(f, a.c01.y, v.x), fma(-f, a.c01.x, v.y));
    v = A.c(dir, 1)[x]; A.c(dir, 1)[x] = cmk<C>(fma(f, a.c02.y, v.x), fma(-f, a.c02.x, v.y));
    v = A.c(dir, 2)[x]; A.c(dir, 2)[x] = cmk<C>(fma(f, a.c12.y, v.x), fma(-f, a.c12.x, v.y));
    A.r(dir, 0)[x] = fma(f, a.a, A.r(dir, 0)[x]);
    A.r(dir, 1)[x] = fma(f, a.b, A.r(dir, 1)[x]);
  }
}

static int links_grid(long sh) { return int((8L * sh + H_THREADS - 1) / H_THREADS); }

template <typename R>
void launch_gauge_force(HmcLinks<R> u, int parts, int mode, typename cplx_t<R>::type* stap, R* alg, double fact,
                        cudaStream_t st) {
  const Geom& g = rt().g;
  k_gauge_force<typename cplx_t<R>::type><<<links_grid(g.sizeh), H_THREADS, 0, st>>>(g, u.p, u.rows, parts, mode,
                                                                                       stap, alg, fact);
  OST_LAUNCH_CHECK();
}

__global__ void __launch_bounds__(H_THREADS)
k_conf_times_staples_ta(Geom g, const double2* __restrict__ u, int rows, const double2* __restrict__ stap,
                        double* ipdot) {
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * g.sizeh) return;
  const int dir = int(t / g.sizeh);
  const long x = t - long(dir) * g.sizeh;
  const long sh = g.sizeh;
  Mt<double2> S;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) S.m[i][j] = stap[(long(dir) * 9 + i * 3 + j) * sh + x];
  const TaT<double2> a = ta_of_product(ld_u(u, rows, sh, dir, x), S);
  Alg<double> A{ipdot, sh};
  A.c(dir, 0)[x] = a.c01; A.c(dir, 1)[x] = a.c02; A.c(dir, 2)[x] = a.c12;
  A.r(dir, 0)[x] = a.a; A.r(dir, 1)[x] = a.b;
}

void launch_conf_times_staples_ta(HmcLinks<double> u, const double2* stap, double* ipdot, cudaStream_t st) {
  const Geom& g = rt().g;
  k_conf_times_staples_ta<<<links_grid(g.sizeh), H_THREADS, 0, st>>>(g, u.p, u.rows, stap, ipdot);
  OST_LAUNCH_CHECK();
}

template <typename R>
__global__ void k_mom_sum_mult(Alg<R> mom, Alg<R> ip, R f, long sh) {
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * sh) return;
  const int dir = int(t / sh);
  const long x = t - long(dir) * sh;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    auto v = mom.c(dir, k)[x];
    const auto a = ip.c(dir, k)[x];
    v.x = fma(f, a.y, v.x);
    v.y = fma(-f, a.x, v.y);
    mom.c(dir, k)[x] = v;
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) mom.r(dir, k)[x] = fma(f, ip.r(dir, k)[x], mom.r(dir, k)[x]);
}

template <typename R>
void launch_mom_sum_mult(R* mom, const R* ipdot, double fact, cudaStream_t st) {
  const long sh = rt().g.sizeh;
  k_mom_sum_mult<R><<<links_grid(sh), H_THREADS, 0, st>>>(Alg<R>{mom, sh}, Alg<R>{const_cast<R*>(ipdot), sh},
                                                            R(fact), sh);
  OST_LAUNCH_CHECK();
}

// ---- exp(iQ) for Hermitian traceless Q = delta P ----
// FP64: the Cayley-Hamilton coefficients of gauge.cuh.  FP32: the small-c1
// series of the same table in float (the molecular dynamics steps keep
// c1 = tr Q^2 / 2 far below 4e-3); a larger c1 takes the FP64 path.
template <typename C> OST_D Mt<C> exp_iq(const Mt<C>& q);

template <> OST_D Mt<double2> exp_iq<double2>(const Mt<double2>& qd) {
  M3 q;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) q.m[i][j] = qd.m[i][j];
  M3 q2 = ost::mmul(q, q);
  double c0, c1;
  q_invariants(q, q2, &c0, &c1);
  CHCoeffs f = ch_coeffs<false>(c0, c1);
  M3 e = poly3(f.f[0], f.f[1], f.f[2], q, q2);
  Mt<double2> r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.m[i][j] = e.m[i][j];
  return r;
}

template <> OST_D Mt<float2> exp_iq<float2>(const Mt<float2>& q) {
  Mt<float2> q2;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float2 s = cmul(q.m[i][0], q.m[0][j]);
      cmac(s, q.m[i][1], q.m[1][j]);
      cmac(s, q.m[i][2], q.m[2][j]);
      q2.m[i][j] = s;
    }
  const float c1 = 0.5f * (q2.m[0][0].x + q2.m[1][1].x + q2.m[2][2].x);
  if (c1 >= 4.0e-3f) {
    Mt<double2> qd;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) qd.m[i][j] = make_double2(q.m[i][j].x, q.m[i][j].y);
    Mt<double2> ed = exp_iq<double2>(qd);
    Mt<float2> e;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) e.m[i][j] = make_float2(float(ed.m[i][j].x), float(ed.m[i][j].y));
    return e;
  }
  float c0 = 0.f;   // tr(Q^2 Q) / 3
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) c0 = fmaf(q2.m[i][k].x, q.m[k][i].x, fmaf(-q2.m[i][k].y, q.m[k][i].y, c0));
  c0 *= (1.0f / 3.0f);
  float2 f[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  for (int k = 0; k < 8; ++k) {
    float mon = 1.f;
    for (int a = 0; a < c_ch_table.i0[k]; ++a) mon *= c0;
    for (int b = 0; b < c_ch_table.j1[k]; ++b) mon *= c1;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double2 t = c_ch_table.f[j][k];
      f[j].x = fmaf(float(t.x), mon, f[j].x);
      f[j].y = fmaf(float(t.y), mon, f[j].y);
    }
  }
  Mt<float2> e;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float2 s = cmul(q.m[i][j], f[1]);
      cmac(s, q2.m[i][j], f[2]);
      if (i == j) s = cadd(s, f[0]);
      e.m[i][j] = s;
    }
  return e;
}

// U = exp(i delta P) U, rows 0-1 reunitarised by Gram-Schmidt
// (su3_utilities.h:1433-1537)
template <typename C>
__global__ void __launch_bounds__(H_THREADS)
k_mom_exp(long sh, C* u, int rows, const decltype(C().x)* __restrict__ mom, double delta) {
  typedef decltype(C().x) Rt;
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * sh) return;
  const int dir = int(t / sh);
  const long x = t - long(dir) * sh;
  Alg<Rt> P{const_cast<Rt*>(mom), sh};
  const Rt d = Rt(delta);
  const C c01 = P.c(dir, 0)[x], c02 = P.c(dir, 1)[x], c12 = P.c(dir, 2)[x];
  const Rt a = P.r(dir, 0)[x], b = P.r(dir, 1)[x];
  Mt<C> q;
  q.m[0][0] = cmk<C>(a * d, 0); q.m[1][1] = cmk<C>(b * d, 0); q.m[2][2] = cmk<C>(-(a + b) * d, 0);
  q.m[0][1] = cscale(c01, d); q.m[0][2] = cscale(c02, d); q.m[1][2] = cscale(c12, d);
  q.m[1][0] = cconj(q.m[0][1]); q.m[2][0] = cconj(q.m[0][2]); q.m[2][1] = cconj(q.m[1][2]);
  const Mt<C> E = exp_iq<C>(q);
  const Mt<C> U = ld_u(u, rows, sh, dir, x);
  R2<C> r = mul2(rows01(E), U);
  Rt n0 = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) n0 += r.m[0][c].x * r.m[0][c].x + r.m[0][c].y * r.m[0][c].y;
  n0 = Rt(1) / sqrt(n0);
#pragma unroll
  for (int c = 0; c < 3; ++c) r.m[0][c] = cscale(r.m[0][c], n0);
  C sp = czero<C>();
#pragma unroll
  for (int c = 0; c < 3; ++c) cmacc(sp, r.m[0][c], r.m[1][c]);
#pragma unroll
  for (int c = 0; c < 3; ++c) r.m[1][c] = csub(r.m[1][c], cmul(sp, r.m[0][c]));
  Rt n1 = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) n1 += r.m[1][c].x * r.m[1][c].x + r.m[1][c].y * r.m[1][c].y;
  n1 = Rt(1) / sqrt(n1);
#pragma unroll
  for (int c = 0; c < 3; ++c) r.m[1][c] = cscale(r.m[1][c], n1);
  if (rows == 0) {
    C* base = u + (long(dir) * sh + x) * 6;
#pragma unroll
    for (int c = 0; c < 3; ++c) { base[c] = r.m[0][c]; base[3 + c] = r.m[1][c]; }
  } else {
    C* base = u + long(dir) * rows * sh + x;
#pragma unroll
    for (int c = 0; c < 3; ++c) { base[c * sh] = r.m[0][c]; base[(3 + c) * sh] = r.m[1][c]; }
  }
}

static void ensure_ch_table_hmc(cudaStream_t st) {
  static bool done = false;
  if (done) return;
  CHTable h;
  fill_ch_table(&h);
  OST_CUDA(cudaMemcpyToSymbolAsync(c_ch_table, &h, sizeof(h), 0, cudaMemcpyHostToDevice, st));
  OST_CUDA(cudaStreamSynchronize(st));
  done = true;
}

template <typename R>
void launch_mom_exp_times_conf(HmcLinks<R> u, const R* mom, double delta, cudaStream_t st) {
  ensure_ch_table_hmc(st);
  const long sh = rt().g.sizeh;
  k_mom_exp<typename cplx_t<R>::type><<<links_grid(sh), H_THREADS, 0, st>>>(sh, u.p, u.rows, mom, delta);
  OST_LAUNCH_CHECK();
}

// ---- the gauge action: Re tr of plaquettes and 2x1 / 1x2 rectangles ----
// (plaquettes.c:14-80, rectangles.c:16-164), per site, summed in FP64
template <typename C>
__global__ void __launch_bounds__(RED_THREADS)
k_gauge_action(Geom g, const C* __restrict__ u, int rows, int which, ReduceWs ws, double* dst) {
  double v[2] = {0.0, 0.0};
  const long nsite = 2L * g.sizeh;
  for (long t = blockIdx.x * long(blockDim.x) + threadIdx.x; t < nsite; t += long(gridDim.x) * blockDim.x) {
    const int p = t >= g.sizeh;
    const long x = t - (p ? long(g.sizeh) : 0L);
    const Site s = site_of(g, int(x), p);
    Walker<C> w{g, u, rows, pos_of(s), p};
    for (int m = 0; m < 3; ++m)
      for (int n = m + 1; n < 4; ++n) {
        const Mt<C> um = w.at(m, m, 0, n, 0), unx = dagger(w.at(n, m, 0, n, 0));
        if (which & 1) {
          R2<C> pq = mul2(mul2(rows01(um), w.at(n, m, 1, n, 0)), dagger(w.at(m, n, 1, m, 0)));
          v[0] += double(tr_re_sum(pq, unx).x);
        }
        if (which & 2) {
          R2<C> a = mul2(mul2(mul2(mul2(rows01(um), w.at(m, m, 1, n, 0)), w.at(n, m, 2, n, 0)),
                              dagger(w.at(m, m, 1, n, 1))), dagger(w.at(m, n, 1, m, 0)));
          R2<C> b = mul2(mul2(mul2(mul2(rows01(um), w.at(n, m, 1, n, 0)), w.at(n, m, 1, n, 1)),
                              dagger(w.at(m, n, 2, m, 0))), dagger(w.at(n, n, 1, m, 0)));
          v[1] += double(tr_re_sum(a, unx).x) + double(tr_re_sum(b, unx).x);
        }
      }
  }
  double tot[2];
  if (grid_reduce<2>(v, ws, tot)) { dst[0] = tot[0]; dst[1] = tot[1]; }
}

template <typename R>
void launch_gauge_action(HmcLinks<R> u, int which, double* dst, cudaStream_t st) {
  const Geom& g = rt().g;
  const int grid = reduce_grid(2L * g.sizeh * 8);
  k_gauge_action<typename cplx_t<R>::type><<<grid, RED_THREADS, 0, st>>>(g, u.p, u.rows, which, reduce_ws(2, grid),
                                                                          dst);
  OST_LAUNCH_CHECK();
}

// sum of 1/2 tr P^2 = a^2 + b^2 + ab + |c01|^2 + |c02|^2 + |c12|^2
// (su3_utilities.h:1295-1307)
template <typename R>
__global__ void k_momenta_action(Alg<R> P, int d0, int d1, long sh, ReduceWs ws, double* dst) {
  double v[1] = {0.0};
  const long n = long(d1 - d0) * sh;
  for (long t = blockIdx.x * long(blockDim.x) + threadIdx.x; t < n; t += long(gridDim.x) * blockDim.x) {
    const int dir = d0 + int(t / sh);
    const long x = t - long(dir - d0) * sh;
    const double a = P.r(dir, 0)[x], b = P.r(dir, 1)[x];
    double s = a * a + b * b + a * b;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const auto c = P.c(dir, k)[x];
      s += double(c.x) * double(c.x) + double(c.y) * double(c.y);
    }
    v[0] += s;
  }
  double tot[1];
  if (grid_reduce<1>(v, ws, tot)) dst[0] = tot[0];
}

template <typename R>
void launch_momenta_action(const R* mom, int d0, int d1, double* dst, cudaStream_t st) {
  const long sh = rt().g.sizeh;
  const int grid = reduce_grid(long(d1 - d0) * sh);
  k_momenta_action<R><<<grid, RED_THREADS, 0, st>>>(Alg<R>{const_cast<R*>(mom), sh}, d0, d1, sh, reduce_ws(1, grid),
                                                    dst);
  OST_LAUNCH_CHECK();
}

// ---- counter-based Gaussian momenta ----
// splitmix64 (Steele, Lea & Flood 2014) of (seed, stream) and the counter,
// the 53 high bits as a uniform in (0,1), Box-Muller with radius
// sqrt(-log u1) (variance 1/2, the reference's two_double_gauss,
// random_assignement.c:44-55).  The same generator runs on the host in the
// package's field helpers, so a test can regenerate any momentum field.
OST_HD unsigned long long splitmix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
OST_D double uniform01(unsigned long long seed, unsigned long long stream, unsigned long long ctr) {
  const unsigned long long base = splitmix64((seed & 0xFFFFFFFFull) * 0x100000001ull + stream);
  const unsigned long long bits = splitmix64(ctr * 0xD1B54A32D192ED03ull + base);
  return (double(bits >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

template <typename R>
__global__ void k_gen_momenta(Alg<R> P, long sh, unsigned long long seed, unsigned long long stream) {
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * sh) return;
  const int dir = int(t / sh);
  const long x = t - long(dir) * sh;
  double g[8];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const unsigned long long m = (unsigned long long)t * 4ull + j;
    const double u1 = uniform01(seed, 2 * stream, m), u2 = uniform01(seed, 2 * stream + 1, m);
    const double rad = sqrt(-log(u1));
    double sn, cs;
    sincospi(2.0 * u2, &sn, &cs);
    g[2 * j] = rad * cs;
    g[2 * j + 1] = rad * sn;
  }
  const double r3 = 0.57735026918962576451;   // 1/sqrt(3)
  P.r(dir, 0)[x] = R(g[2] + g[7] * r3);
  P.r(dir, 1)[x] = R(-g[2] + g[7] * r3);
  typedef typename cplx_t<R>::type C;
  P.c(dir, 0)[x] = cmk<C>(R(g[0]), R(-g[1]));
  P.c(dir, 1)[x] = cmk<C>(R(g[3]), R(-g[4]));
  P.c(dir, 2)[x] = cmk<C>(R(g[5]), R(-g[6]));
}

template <typename R>
void launch_gen_momenta(R* mom, unsigned long long seed, unsigned long long stream, cudaStream_t st) {
  const long sh = rt().g.sizeh;
  k_gen_momenta<R><<<links_grid(sh), H_THREADS, 0, st>>>(Alg<R>{mom, sh}, sh, seed, stream);
  OST_LAUNCH_CHECK();
}

// Gaussian complex 3-vectors (vec3_soa over sizeh sites): element k of the
// 3*sizeh complex numbers takes the Box-Muller pair k of (seed, stream), as
// the host field helpers' gaussian_vec3 (the reference's
// generate_vec3_soa_gauss, random_assignement.c:58-92: real and imaginary
// parts of variance 1/2)
__global__ void k_gen_vec3(double2* v, long n, unsigned long long seed, unsigned long long stream) {
  const long k = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (k >= n) return;
  const double u1 = uniform01(seed, 2 * stream, (unsigned long long)k);
  const double u2 = uniform01(seed, 2 * stream + 1, (unsigned long long)k);
  const double rad = sqrt(-log(u1));
  double sn, cs;
  sincospi(2.0 * u2, &sn, &cs);
  v[k] = make_double2(rad * cs, rad * sn);
}

void launch_gen_vec3_gauss(double2* v, unsigned long long seed, unsigned long long stream, cudaStream_t st) {
  const long n = 3L * rt().g.sizeh;
  k_gen_vec3<<<int((n + 255) / 256), 256, 0, st>>>(v, n, seed, stream);
  OST_LAUNCH_CHECK();
}

// ---- precision conversions of the link generator ----
__global__ void k_links_64_to_32(const double2* __restrict__ u64, int rows64, float2* u32, long sh) {
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * sh) return;
  const int dir = int(t / sh);
  const long x = t - long(dir) * sh;
  float2* o = u32 + (long(dir) * sh + x) * 6;   // array of structures: a link's 6 numbers contiguous
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const double2 v = u64[(long(dir) * rows64 + k) * sh + x];
    o[k] = make_float2(float(v.x), float(v.y));
  }
}

// rows 0-1 back to FP64, reunitarised by Gram-Schmidt in FP64, row 2 rebuilt
__global__ void k_links_32_to_64(const float2* __restrict__ u32, double2* u64, int rows64, long sh) {
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * sh) return;
  const int dir = int(t / sh);
  const long x = t - long(dir) * sh;
  Mt<double2> a;
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 v = u32[(long(dir) * sh + x) * 6 + r * 3 + c];
      a.m[r][c] = make_double2(v.x, v.y);
    }
  double n0 = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) n0 += a.m[0][c].x * a.m[0][c].x + a.m[0][c].y * a.m[0][c].y;
  n0 = 1.0 / sqrt(n0);
#pragma unroll
  for (int c = 0; c < 3; ++c) a.m[0][c] = cscale(a.m[0][c], n0);
  double2 sp = make_double2(0, 0);
#pragma unroll
  for (int c = 0; c < 3; ++c) cmacc(sp, a.m[0][c], a.m[1][c]);
#pragma unroll
  for (int c = 0; c < 3; ++c) a.m[1][c] = csub(a.m[1][c], cmul(sp, a.m[0][c]));
  double n1 = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) n1 += a.m[1][c].x * a.m[1][c].x + a.m[1][c].y * a.m[1][c].y;
  n1 = 1.0 / sqrt(n1);
#pragma unroll
  for (int c = 0; c < 3; ++c) a.m[1][c] = cscale(a.m[1][c], n1);
  rebuild2(a);
  const int nr = rows64 == 9 ? 3 : 2;
  for (int r = 0; r < nr; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) u64[(long(dir) * rows64 + r * 3 + c) * sh + x] = a.m[r][c];
}

void launch_links_64_to_32(const double2* u64, int rows64, float2* u32, cudaStream_t st) {
  const long sh = rt().g.sizeh;
  k_links_64_to_32<<<links_grid(sh), H_THREADS, 0, st>>>(u64, rows64, u32, sh);
  OST_LAUNCH_CHECK();
}
void launch_links_32_to_64(const float2* u32, double2* u64, int rows64, cudaStream_t st) {
  const long sh = rt().g.sizeh;
  k_links_32_to_64<<<links_grid(sh), H_THREADS, 0, st>>>(u32, u64, rows64, sh);
  OST_LAUNCH_CHECK();
}

__global__ void k_d2f_n(const double* __restrict__ a, float* b, long n) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) b[i] = float(a[i]);
}
__global__ void k_f2d_n(const float* __restrict__ a, double* b, long n) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) b[i] = a[i];
}
void launch_alg_64_to_32(const double* a64, float* a32, cudaStream_t st) {
  k_d2f_n<<<8 * rt().num_sms, 256, 0, st>>>(a64, a32, 64L * rt().g.sizeh);
  OST_LAUNCH_CHECK();
}
void launch_alg_32_to_64(const float* a32, double* a64, cudaStream_t st) {
  k_f2d_n<<<8 * rt().num_sms, 256, 0, st>>>(a32, a64, 64L * rt().g.sizeh);
  OST_LAUNCH_CHECK();
}

template void launch_gauge_force<double>(HmcLinks<double>, int, int, double2*, double*, double, cudaStream_t);
template void launch_gauge_force<float>(HmcLinks<float>, int, int, float2*, float*, double, cudaStream_t);
template void launch_mom_sum_mult<double>(double*, const double*, double, cudaStream_t);
template void launch_mom_sum_mult<float>(float*, const float*, double, cudaStream_t);
template void launch_mom_exp_times_conf<double>(HmcLinks<double>, const double*, double, cudaStream_t);
template void launch_mom_exp_times_conf<float>(HmcLinks<float>, const float*, double, cudaStream_t);
template void launch_gauge_action<double>(HmcLinks<double>, int, double*, cudaStream_t);
template void launch_gauge_action<float>(HmcLinks<float>, int, double*, cudaStream_t);
template void launch_momenta_action<double>(const double*, int, int, double*, cudaStream_t);
template void launch_momenta_action<float>(const float*, int, int, double*, cudaStream_t);
template void launch_gen_momenta<double>(double*, unsigned long long, unsigned long long, cudaStream_t);
template void launch_gen_momenta<float>(float*, unsigned long long, unsigned long long, cudaStream_t);

}  // namespace ost
