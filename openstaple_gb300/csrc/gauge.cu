// gauge.cu -- FP64 kernels of the stout smearing and of the rational fermion
// force chain: staples + Q_A + exp(-Q_A) U in one pass per link, Lambda,
// Sigma' -> Sigma, the outer products summed over all shifts with the
// staggered phase folded in, and the final traceless anti-Hermitian
// projection.  One thread per link (8 directions x sizeh).
#include <cstring>
#include "gauge.cuh"
#include "gauge_kernels.cuh"
#include "runtime.cuh"

namespace ost {

static constexpr int G_THREADS = 128;
static constexpr double C_ZERO = 5.0 * 0.33333333333333333333333;   // tree-level Symanzik c0

// Small-c1 table: exp(iQ) = sum_n (iQ)^n/n! with Q^n reduced by Q^3 = c1 Q + c0
// to polynomials in (c0, c1), truncated at total weight 7 (c0: 3, c1: 2).
void fill_ch_table(CHTable* table) {
  const int mons[8][2] = {{0, 0}, {0, 1}, {0, 2}, {0, 3}, {1, 0}, {1, 1}, {1, 2}, {2, 0}};
  auto index = [&](int i, int j) {
    for (int k = 0; k < 8; ++k)
      if (mons[k][0] == i && mons[k][1] == j) return k;
    return -1;
  };
  double al[8] = {1}, be[8] = {0}, ga[8] = {0};
  double fr[3][8] = {{0}}, fi[3][8] = {{0}};
  double inr = 1.0, ini = 0.0;   // i^n / n!
  for (int n = 0; n <= 9; ++n) {
    for (int k = 0; k < 8; ++k) {
      fr[0][k] += inr * al[k]; fi[0][k] += ini * al[k];
      fr[1][k] += inr * be[k]; fi[1][k] += ini * be[k];
      fr[2][k] += inr * ga[k]; fi[2][k] += ini * ga[k];
    }
    double nal[8] = {0}, nbe[8] = {0}, nga[8] = {0};
    for (int k = 0; k < 8; ++k) {
      int a = index(mons[k][0] + 1, mons[k][1]), b = index(mons[k][0], mons[k][1] + 1);
      if (a >= 0) nal[a] += ga[k];
      nbe[k] += al[k];
      if (b >= 0) nbe[b] += ga[k];
      nga[k] += be[k];
    }
    memcpy(al, nal, sizeof(al));
    memcpy(be, nbe, sizeof(be));
    memcpy(ga, nga, sizeof(ga));
    double t = inr;       // multiply by i/(n+1)
    inr = -ini / double(n + 1);
    ini = t / double(n + 1);
  }
  for (int j = 0; j < 3; ++j)
    for (int k = 0; k < 8; ++k) table->f[j][k] = make_double2(fr[j][k], fi[j][k]);
  for (int k = 0; k < 8; ++k) { table->i0[k] = mons[k][0]; table->j1[k] = mons[k][1]; }
}

void ensure_ch_table(cudaStream_t st) {
  static bool done = false;
  if (done) return;
  CHTable h;
  fill_ch_table(&h);
  OST_CUDA(cudaMemcpyToSymbolAsync(c_ch_table, &h, sizeof(h), 0, cudaMemcpyHostToDevice, st));
  OST_CUDA(cudaStreamSynchronize(st));
  done = true;
}

// snum of x + a e_mu + b e_nu (periodic)
OST_D long nbr(const Geom& g, const Site& s, int mu, int a, int nu, int b) {
  int d[4] = {s.d0, s.d1, s.d2, s.d3};
  const int n[4] = {g.n0, g.n1, g.n2, g.n3};
  d[mu] += a; if (d[mu] < 0) d[mu] += n[mu]; if (d[mu] >= n[mu]) d[mu] -= n[mu];
  if (b != 0) { d[nu] += b; if (d[nu] < 0) d[nu] += n[nu]; if (d[nu] >= n[nu]) d[nu] -= n[nu]; }
  return (d[0] + long(d[1]) * g.vol1 + long(d[2]) * g.vol2 + long(d[3]) * g.vol3) >> 1;
}

// C_ZERO * sum_nu [ U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+ + U_nu(x+mu-nu)^+ U_mu(x-nu)^+ U_nu(x-nu) ]
// (plaquettes.c:196-259)
OST_D M3 staple_sum(const Geom& g, const SU3Field& u, const Site& s, int mu, int p, long x) {
  M3 acc = mzero();
  const long xpm = nbr(g, s, mu, 1, mu, 0);
#pragma unroll 1
  for (int nu = 0; nu < 4; ++nu) {
    if (nu == mu) continue;
    const long xpn = nbr(g, s, nu, 1, nu, 0), xmn = nbr(g, s, nu, -1, nu, 0), xpmmn = nbr(g, s, mu, 1, nu, -1);
    M3 r = mmuldag(mmuldag(ld_link(u, 2 * nu + !p, xpm), ld_link(u, 2 * mu + !p, xpn)), ld_link(u, 2 * nu + p, x));
    madd_to(acc, r);
    M3 l = mmul(mdagmul(ld_link(u, 2 * nu + p, xpmmn), mdag(ld_link(u, 2 * mu + !p, xmn))), ld_link(u, 2 * nu + !p, xmn));
    madd_to(acc, l);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) acc.m[i][j] = csc(acc.m[i][j], C_ZERO);
  return acc;
}

OST_D void st_ta(const AlgField& t, int dir, long i, const TA& a) {
  t.c(dir, 0)[i] = a.c01; t.c(dir, 1)[i] = a.c02; t.c(dir, 2)[i] = a.c12;
  t.r(dir, 0)[i] = a.a; t.r(dir, 1)[i] = a.b;
}

// One stout step for every link: Q_A = rho/C_ZERO TA(U C), U' = exp(-Q_A) U
// (stouting.c:74-165).  Writes U' rows 0,1, Q_A, and the staples if asked.
__global__ void __launch_bounds__(G_THREADS)
k_stout(Geom g, SU3Field u, SU3Field uout, AlgField qa, SU3Field stap, int write_stap, double rho) {
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * g.sizeh) return;
  const int dir = int(t / g.sizeh);
  const long x = t - long(dir) * g.sizeh;
  const int mu = dir >> 1, p = dir & 1;
  const Site s = site_of(g, int(x), p);
  M3 C = staple_sum(g, u, s, mu, p, x);
  if (write_stap) st_rows(stap, dir, x, C, 3);
  const M3 U = ld_link(u, dir, x);
  TA a = ta_of(mmul(U, C), rho / C_ZERO);
  st_ta(qa, dir, x, a);
  M3 q = ld_q_from_tamat(qa, dir, x);
  M3 q2 = mmul(q, q);
  double c0, c1;
  q_invariants(q, q2, &c0, &c1);
  CHCoeffs f = ch_coeffs<false>(c0, c1);
  M3 E = poly3(f.f[0], f.f[1], f.f[2], q, q2);
  st_rows(uout, dir, x, mmul(E, U), 2);
}

// U' = exp(-Q_A) U for given Q_A (stouting.c:136-165)
__global__ void __launch_bounds__(G_THREADS)
k_exp_times_conf(Geom g, SU3Field u, AlgField qa, SU3Field uout) {
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * g.sizeh) return;
  const int dir = int(t / g.sizeh);
  const long x = t - long(dir) * g.sizeh;
  M3 q = ld_q_from_tamat(qa, dir, x);
  M3 q2 = mmul(q, q);
  double c0, c1;
  q_invariants(q, q2, &c0, &c1);
  CHCoeffs f = ch_coeffs<false>(c0, c1);
  M3 E = poly3(f.f[0], f.f[1], f.f[2], q, q2);
  st_rows(uout, dir, x, mmul(E, ld_link(u, dir, x)), 2);
}

// Lambda = (Gamma + Gamma^+)/2 - tr(Gamma + Gamma^+)/6,
// Gamma = tr(S' B1 U) Q + tr(S' B2 U) Q^2 + f1 U S' + f2 (Q U S' + U S' Q)
// (stouting.c:171-546)
__global__ void __launch_bounds__(G_THREADS)
k_lambda(Geom g, AlgField lam, SU3Field sp, SU3Field u, AlgField qa) {
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * g.sizeh) return;
  const int dir = int(t / g.sizeh);
  const long x = t - long(dir) * g.sizeh;
  M3 q = ld_q_from_tamat(qa, dir, x);
  M3 q2 = mmul(q, q);
  double c0, c1;
  q_invariants(q, q2, &c0, &c1);
  CHCoeffs f = ch_coeffs<true>(c0, c1);
  const M3 U = ld_link(u, dir, x);
  const M3 S = ld_full(sp, dir, x);
  M3 US = mmul(U, S);
  // tr(S B U) = tr(B U S)
  double2 t1 = mtrace_mul(poly3(f.b1[0], f.b1[1], f.b1[2], q, q2), US);
  double2 t2 = mtrace_mul(poly3(f.b2[0], f.b2[1], f.b2[2], q, q2), US);
  M3 G = mscale(q, t1);
  madd_scaled(G, q2, t2);
  madd_scaled(G, US, f.f[1]);
  M3 qus = mmul(q, US);
  madd_to(qus, mmul(US, q));
  madd_scaled(G, qus, f.f[2]);
  M3 H = G;
  madd_to(H, mdag(G));
  const double tr6 = mtrace(H).x / 6.0;
  M3 L;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) L.m[i][j] = csc(H.m[i][j], 0.5);
  L.m[0][0].x -= tr6; L.m[1][1].x -= tr6;
  st_thmat(lam, dir, x, L);
}

// Sigma = Sigma' exp(iQ) + i rho {three right and three left staple terms
// with Lambda} (stouting.c:550-1302; Morningstar & Peardon eq. 75).  Each
// thread reads Lambda and U of neighbours and writes only its own link, so
// Sigma may overwrite Sigma' in place.
__global__ void __launch_bounds__(G_THREADS)
k_sigma(Geom g, AlgField lam, SU3Field u, SU3Field s_io, AlgField qa, double rho) {
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * g.sizeh) return;
  const int dir = int(t / g.sizeh);
  const long x = t - long(dir) * g.sizeh;
  const int mu = dir >> 1, p = dir & 1;
  const Site s = site_of(g, int(x), p);
  M3 q = ld_q_from_tamat(qa, dir, x);
  M3 q2 = mmul(q, q);
  double c0, c1;
  q_invariants(q, q2, &c0, &c1);
  CHCoeffs f = ch_coeffs<false>(c0, c1);
  M3 E = poly3(f.f[0], f.f[1], f.f[2], q, q2);
  rebuild_row2(E);   // the reference keeps exp(iQ) as an SU(3) matrix of two rows
  M3 acc = mmul(ld_full(s_io, dir, x), E);
  const M3 Lmu = ld_thmat(lam, dir, x);
  const double2 ir = make_double2(0.0, rho), mir = make_double2(0.0, -rho);
  const long xpm = nbr(g, s, mu, 1, mu, 0);
#pragma unroll 1
  for (int nu = 0; nu < 4; ++nu) {
    if (nu == mu) continue;
    const long xpn = nbr(g, s, nu, 1, nu, 0), xmn = nbr(g, s, nu, -1, nu, 0), xpmmn = nbr(g, s, mu, 1, nu, -1);
    {  // right: A = U_nu(x+mu), B = U_mu(x+nu)^+, C = U_nu(x)^+
      const M3 A = ld_link(u, 2 * nu + !p, xpm);
      const M3 AB = mmuldag(A, ld_link(u, 2 * mu + !p, xpn));
      const M3 ABC = mmuldag(AB, ld_link(u, 2 * nu + p, x));
      M3 D = Lmu;
      const M3 Lnu = ld_thmat(lam, 2 * nu + p, x);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) D.m[i][j] = csub2(D.m[i][j], Lnu.m[i][j]);
      madd_scaled(acc, mmul(ABC, D), ir);                                          // i rho ABC (L_mu(x) - L_nu(x))
      madd_scaled(acc, mmul(ld_thmat(lam, 2 * nu + !p, xpm), ABC), ir);           // i rho L_nu(x+mu) ABC
      madd_scaled(acc, mmuldag(mmul(AB, ld_thmat(lam, 2 * mu + !p, xpn)), ld_link(u, 2 * nu + p, x)), mir);
    }
    {  // left: A = U_nu(x+mu-nu)^+, B = U_mu(x-nu)^+, C = U_nu(x-nu)
      const M3 Ad = ld_link(u, 2 * nu + p, xpmmn);
      const M3 Bd = ld_link(u, 2 * mu + !p, xmn);
      const M3 C = ld_link(u, 2 * nu + !p, xmn);
      const M3 AB = mmuldag(mdag(Ad), Bd);                                          // A^+ B^+ with A,B as loaded
      M3 G = ld_thmat(lam, 2 * nu + !p, xmn);
      const M3 Em = ld_thmat(lam, 2 * mu + !p, xmn);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) G.m[i][j] = csub2(G.m[i][j], Em.m[i][j]);
      madd_scaled(acc, mmul(mmul(AB, G), C), ir);                                  // i rho A B (L_nu - L_mu)(x-nu) C
      madd_scaled(acc, mmul(mmul(AB, C), Lmu), ir);                                // i rho A B C L_mu(x)
      madd_scaled(acc, mmul(mdagmul(Ad, ld_thmat(lam, 2 * nu + p, xpmmn)), mdagmul(Bd, C)), mir);  // -i rho A L_nu(x+mu-nu) B C
    }
  }
  st_rows(s_io, dir, x, acc, 3);
}

// pip[dir](x) += e^{i theta} sum_k c_k l_k(x+mu) (x) r_k(x)^+, with
// (l, r, c) = (Y_k, X_k, a_k) on even and (X_k, Y_k, -a_k) on odd links,
// Y_k = D_oe X_k: the outer products of ker_openacc_compute_fermion_force
// (fermion_force_utilities.c:30-93, 183-201) for all shifts in one pass,
// with multiply_backfield_times_force (:123-153) folded in.
__global__ void __launch_bounds__(G_THREADS)
k_force_outer(Geom g, const double2* __restrict__ xs, const double2* __restrict__ ys, long vstride, int nshift,
              const double* __restrict__ coef, const double* __restrict__ ph, SU3Field pip, int accumulate_phase) {
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * g.sizeh) return;
  const int dir = int(t / g.sizeh);
  const long x = t - long(dir) * g.sizeh;
  const int mu = dir >> 1, p = dir & 1;
  const Site s = site_of(g, int(x), p);
  const long j = nbr(g, s, mu, 1, mu, 0);
  const long sh = g.sizeh;
  M3 acc = mzero();
  for (int k = 0; k < nshift; ++k) {
    const double2* X = xs + k * vstride;
    const double2* Y = ys + k * vstride;
    const double2* L = p ? X : Y;
    const double2* R = p ? Y : X;
    const double c = p ? -coef[k] : coef[k];
    double2 l[3], r[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) { l[a] = L[a * sh + j]; r[a] = csc(cjm(R[a * sh + x]), c); }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) cmac(acc.m[a][b], l[a], r[b]);
  }
  double2 e = make_double2(1.0, 0.0);
  if (accumulate_phase) {
    double sn, cs;
    sincos(ph[long(dir) * sh + x], &sn, &cs);
    e = make_double2(cs, sn);
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      double2* q = pip.at(dir, a, b) + x;
      *q = cadd2(*q, cm(acc.m[a][b], e));
    }
}

// pip[dir] += e^{i theta} aux[dir] (fermion_force_utilities.c:123-153)
__global__ void k_backfield(Geom g, const double* __restrict__ ph, SU3Field aux, SU3Field pip) {
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * g.sizeh) return;
  const int dir = int(t / g.sizeh);
  const long x = t - long(dir) * g.sizeh;
  double sn, cs;
  sincos(ph[long(dir) * g.sizeh + x], &sn, &cs);
  const double2 e = make_double2(cs, sn);
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      double2* q = pip.at(dir, a, b) + x;
      *q = cadd2(*q, cm(aux.at(dir, a, b)[x], e));
    }
}

// ipdot -= TA(U Sigma) (fermion_force_utilities.c:95-121)
__global__ void k_conf_force_ta(Geom g, SU3Field u, SU3Field sig, AlgField ip) {
  const long t = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (t >= 8L * g.sizeh) return;
  const int dir = int(t / g.sizeh);
  const long x = t - long(dir) * g.sizeh;
  TA a = ta_of(mmul(ld_link(u, dir, x), ld_full(sig, dir, x)), 1.0);
  ip.c(dir, 0)[x] = csub2(ip.c(dir, 0)[x], a.c01);
  ip.c(dir, 1)[x] = csub2(ip.c(dir, 1)[x], a.c02);
  ip.c(dir, 2)[x] = csub2(ip.c(dir, 2)[x], a.c12);
  ip.r(dir, 0)[x] -= a.a;
  ip.r(dir, 1)[x] -= a.b;
}

// ---- launchers ----
static int links_grid() { return blocks_for(8L * rt().g.sizeh, G_THREADS); }

void launch_stout(const double2* u, double2* uout, double* qa, double2* stap, double rho, cudaStream_t st) {
  ensure_ch_table(st);
  const Geom& g = rt().g;
  k_stout<<<links_grid(), G_THREADS, 0, st>>>(g, SU3Field{const_cast<double2*>(u), g.sizeh},
                                              SU3Field{uout, g.sizeh}, AlgField{qa, g.sizeh},
                                              SU3Field{stap, g.sizeh}, stap != nullptr, rho);
  OST_LAUNCH_CHECK();
}

void launch_exp_times_conf(const double2* u, const double* qa, double2* uout, cudaStream_t st) {
  ensure_ch_table(st);
  const Geom& g = rt().g;
  k_exp_times_conf<<<links_grid(), G_THREADS, 0, st>>>(g, SU3Field{const_cast<double2*>(u), g.sizeh},
                                                       AlgField{const_cast<double*>(qa), g.sizeh},
                                                       SU3Field{uout, g.sizeh});
  OST_LAUNCH_CHECK();
}

void launch_lambda(double* lam, const double2* sp, const double2* u, const double* qa, cudaStream_t st) {
  ensure_ch_table(st);
  const Geom& g = rt().g;
  k_lambda<<<links_grid(), G_THREADS, 0, st>>>(g, AlgField{lam, g.sizeh}, SU3Field{const_cast<double2*>(sp), g.sizeh},
                                               SU3Field{const_cast<double2*>(u), g.sizeh},
                                               AlgField{const_cast<double*>(qa), g.sizeh});
  OST_LAUNCH_CHECK();
}

void launch_sigma(const double* lam, const double2* u, double2* s, const double* qa, double rho, cudaStream_t st) {
  ensure_ch_table(st);
  const Geom& g = rt().g;
  k_sigma<<<links_grid(), G_THREADS, 0, st>>>(g, AlgField{const_cast<double*>(lam), g.sizeh},
                                              SU3Field{const_cast<double2*>(u), g.sizeh}, SU3Field{s, g.sizeh},
                                              AlgField{const_cast<double*>(qa), g.sizeh}, rho);
  OST_LAUNCH_CHECK();
}

void launch_force_outer(const double2* xs, const double2* ys, long vstride, int nshift, const double* coef_dev,
                        const double* ph, double2* pip, int with_phase, cudaStream_t st) {
  const Geom& g = rt().g;
  k_force_outer<<<links_grid(), G_THREADS, 0, st>>>(g, xs, ys, vstride, nshift, coef_dev, ph,
                                                    SU3Field{pip, g.sizeh}, with_phase);
  OST_LAUNCH_CHECK();
}

void launch_backfield(const double* ph, const double2* aux, double2* pip, cudaStream_t st) {
  const Geom& g = rt().g;
  k_backfield<<<links_grid(), G_THREADS, 0, st>>>(g, ph, SU3Field{const_cast<double2*>(aux), g.sizeh},
                                                  SU3Field{pip, g.sizeh});
  OST_LAUNCH_CHECK();
}

void launch_conf_force_ta(const double2* u, const double2* sig, double* ip, cudaStream_t st) {
  const Geom& g = rt().g;
  k_conf_force_ta<<<links_grid(), G_THREADS, 0, st>>>(g, SU3Field{const_cast<double2*>(u), g.sizeh},
                                                      SU3Field{const_cast<double2*>(sig), g.sizeh},
                                                      AlgField{ip, g.sizeh});
  OST_LAUNCH_CHECK();
}

}  // namespace ost
