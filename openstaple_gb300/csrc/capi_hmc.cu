// capi_hmc.cu -- C entry points of the pure-gauge tree-level Symanzik HMC:
// the reference-named FP64 pieces (ipdot_gauge.h, plaquettes.h,
// rectangles.h, su3_utilities.h, su3_measurements.h, md_integrator.h,
// md_parameters.h, random_assignement.h) and ostaple_pure_gauge_hmc, the
// link generator that runs whole trajectories on the device.
#include <cmath>
#include <cstdio>
#include <cstring>
#include "hmc.cuh"
#include "runtime.cuh"
#include "../../include/ostaple_gb300.h"

using namespace ost;

extern "C" {
// Integrator globals a reference host program defines itself
// (md_parameters.c:8-9, 57); weak defaults here.
__attribute__((weak)) double deltas_Omelyan[7] = {0, 0, 0, 0, 0, 0, 0};
__attribute__((weak)) md_param md_parameters = {18, 4, 1.0, 1e-10, 0.0, 0, 1e-8, 10000, 0, 0};
}

namespace {

typedef double2 Z;
inline cudaStream_t S() { return rt().stream; }
inline long sh() { return rt().g.sizeh; }
inline size_t alg_bytes() { return 64 * size_t(sh()) * sizeof(double); }

HmcLinks<double> links64(const su3_soa* u, const char* who) {
  return HmcLinks<double>{static_cast<Z*>(resolve(u, who)), 9};
}

double* dsc(int k) {
  double* p = static_cast<double*>(workspace(WS_SCALARS, 64 * sizeof(double)));
  return p ? p + 16 + k : nullptr;   // slots 16.. (the solvers use the first ones)
}
void read_scalars(double* h, const double* d, int n) {
  OST_CUDA(cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, S()));
  OST_CUDA(cudaStreamSynchronize(S()));
}

constexpr double C_ZERO = 5.0 * 0.33333333333333333333333;
constexpr double C_ONE = -0.25 * 0.33333333333333333333333;

// host copy of the device generator (hmc.cu): splitmix64 of (seed, stream)
// and counter, 53 bits to (0, 1)
unsigned long long hsplitmix(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double huniform(unsigned long long seed, unsigned long long stream, unsigned long long ctr) {
  const unsigned long long base = hsplitmix((seed & 0xFFFFFFFFull) * 0x100000001ull + stream);
  const unsigned long long bits = hsplitmix(ctr * 0xD1B54A32D192ED03ull + base);
  return (double(bits >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

// the MD integrator steps of initialize_md_global_variables (md_parameters.c:11-50)
void md_deltas(double beta, int no_md, int gauge_scale, double t, double d[7]) {
  const double lambda = 0.1931833275037836;   // Omelyan et al.
  const double b3 = beta * 0.33333333333333333333333;
  d[0] = -t / no_md * lambda;
  d[1] = -t / no_md * (1.0 - 2.0 * lambda);
  d[2] = -t / no_md * 2.0 * lambda;
  d[3] = -t / (2 * no_md * gauge_scale) * lambda * b3;
  d[4] = 0.5 * t / (2 * no_md * gauge_scale);
  d[5] = -t / (2 * no_md * gauge_scale) * (1.0 - 2.0 * lambda) * b3;
  d[6] = -t / (2 * no_md * gauge_scale) * 2.0 * lambda * b3;
}

// one multistep_2MN_gauge with the kick fused into the force kernel
// (md_integrator.c:347-376):  K(d3) X [K(d5) X K(d6) X]^(gs-1) K(d5) X K(d3)
template <typename R>
void gauge_2mn_fused(HmcLinks<R> u, R* mom, const double d[7], int gauge_scale) {
  auto K = [&](double f) { launch_gauge_force<R>(u, SP_ALL, GF_MOM, nullptr, mom, f, S()); };
  auto X = [&]() { launch_mom_exp_times_conf<R>(u, mom, d[4], S()); };
  K(d[3]); X();
  for (int k = 1; k < gauge_scale; ++k) { K(d[5]); X(); K(d[6]); X(); }
  K(d[5]); X(); K(d[3]);
}

}  // namespace

extern "C" {

// ---- reference-named FP64 pieces ----
void calc_loc_staples_nnptrick_all(const su3_soa* u, su3_soa* loc_stap) {
  if (!require_init("calc_loc_staples_nnptrick_all")) return;
  HmcLinks<double> l = links64(u, "u");
  Z* st = static_cast<Z*>(resolve(loc_stap, "loc_stap"));
  if (l.p && st) launch_gauge_force<double>(l, SP_PLAQ, GF_STAPLES, st, nullptr, 0.0, S());
}
void calc_loc_improved_staples_typeA_nnptrick_all(const su3_soa* u, su3_soa* loc_stap) {
  if (!require_init("calc_loc_improved_staples_typeA_nnptrick_all")) return;
  HmcLinks<double> l = links64(u, "u");
  Z* st = static_cast<Z*>(resolve(loc_stap, "loc_stap"));
  if (l.p && st) launch_gauge_force<double>(l, SP_RECT_A, GF_STAPLES, st, nullptr, 0.0, S());
}
void calc_loc_improved_staples_typeB_nnptrick_all(const su3_soa* u, su3_soa* loc_stap) {
  if (!require_init("calc_loc_improved_staples_typeB_nnptrick_all")) return;
  HmcLinks<double> l = links64(u, "u");
  Z* st = static_cast<Z*>(resolve(loc_stap, "loc_stap"));
  if (l.p && st) launch_gauge_force<double>(l, SP_RECT_B, GF_STAPLES, st, nullptr, 0.0, S());
}
void calc_loc_improved_staples_typeC_nnptrick_all(const su3_soa* u, su3_soa* loc_stap) {
  if (!require_init("calc_loc_improved_staples_typeC_nnptrick_all")) return;
  HmcLinks<double> l = links64(u, "u");
  Z* st = static_cast<Z*>(resolve(loc_stap, "loc_stap"));
  if (l.p && st) launch_gauge_force<double>(l, SP_RECT_C, GF_STAPLES, st, nullptr, 0.0, S());
}

void conf_times_staples_ta_part(const su3_soa* u, const su3_soa* loc_stap, tamat_soa* tipdot) {
  if (!require_init("conf_times_staples_ta_part")) return;
  HmcLinks<double> l = links64(u, "u");
  const Z* st = static_cast<const Z*>(resolve(loc_stap, "loc_stap"));
  double* ip = static_cast<double*>(resolve(tipdot, "tipdot"));
  if (l.p && st && ip) launch_conf_times_staples_ta(l, st, ip, S());
}

void calc_ipdot_gauge_soloopenacc(const su3_soa* tconf_acc, su3_soa* local_staples, tamat_soa* tipdot) {
  if (!require_init("calc_ipdot_gauge_soloopenacc")) return;
  HmcLinks<double> l = links64(tconf_acc, "tconf_acc");
  Z* st = local_staples ? static_cast<Z*>(resolve(local_staples, "local_staples")) : nullptr;
  double* ip = static_cast<double*>(resolve(tipdot, "tipdot"));
  if (l.p && ip) launch_gauge_force<double>(l, SP_ALL, GF_IPDOT, st, ip, 0.0, S());
}

double calc_plaquette_soloopenacc(su3_soa* tconf_acc, su3_soa* local_plaqs, dcomplex_soa* tr_local_plaqs) {
  (void)local_plaqs;
  (void)tr_local_plaqs;
  if (!require_init("calc_plaquette_soloopenacc")) return NAN;
  HmcLinks<double> l = links64(tconf_acc, "tconf_acc");
  double* d = dsc(0);
  if (!l.p || !d) return NAN;
  launch_gauge_action<double>(l, 1, d, S());
  double h[2];
  read_scalars(h, d, 2);
  return h[0];
}

double calc_rettangolo_soloopenacc(const su3_soa* tconf_acc, su3_soa* local_plaqs, dcomplex_soa* tr_local_plaqs) {
  (void)local_plaqs;
  (void)tr_local_plaqs;
  if (!require_init("calc_rettangolo_soloopenacc")) return NAN;
  HmcLinks<double> l = links64(tconf_acc, "tconf_acc");
  double* d = dsc(0);
  if (!l.p || !d) return NAN;
  launch_gauge_action<double>(l, 2, d, S());
  double h[2];
  read_scalars(h, d, 2);
  return h[1];
}

double calc_momenta_action(const thmat_soa* mom, double_soa* tr_local, const int mu) {
  (void)tr_local;
  if (!require_init("calc_momenta_action")) return NAN;
  const double* m = static_cast<const double*>(resolve(mom, "mom"));
  double* d = dsc(2);
  if (!m || !d || mu < 0 || mu > 7) {
    if (mu < 0 || mu > 7) set_error(-11, "calc_momenta_action: direction %d outside [0,7]", mu);
    return NAN;
  }
  launch_momenta_action<double>(m, mu, mu + 1, d, S());
  double h;
  read_scalars(&h, d, 1);
  return h;
}

void mom_sum_mult(thmat_soa* mom, const tamat_soa* ipdot, const double* factor, int id_factor) {
  if (!require_init("mom_sum_mult")) return;
  double* m = static_cast<double*>(resolve(mom, "mom"));
  const double* ip = static_cast<const double*>(resolve(ipdot, "ipdot"));
  if (m && ip) launch_mom_sum_mult<double>(m, ip, factor[id_factor], S());
}

void mom_exp_times_conf_soloopenacc(su3_soa* tconf_acc, const thmat_soa* tmomenta, const double* tdelta,
                                    int id_delta) {
  if (!require_init("mom_exp_times_conf_soloopenacc")) return;
  HmcLinks<double> l = links64(tconf_acc, "tconf_acc");
  const double* m = static_cast<const double*>(resolve(tmomenta, "tmomenta"));
  if (l.p && m) launch_mom_exp_times_conf<double>(l, m, tdelta[id_delta], S());
}

void initialize_md_global_variables(md_param md_params) {
  md_deltas(act_params.beta, md_params.no_md, md_params.gauge_scale, md_params.t, deltas_Omelyan);
}

// md_integrator.c:347-376, with the reference's staples and tipdot left in
// the caller's buffers after the last kick
void multistep_2MN_gauge(su3_soa* tconf_acc, su3_soa* local_staples, tamat_soa* tipdot, thmat_soa* tmomenta) {
  if (!require_init("multistep_2MN_gauge")) return;
  const int gs = md_parameters.gauge_scale;
  auto kick = [&](int k) {
    calc_ipdot_gauge_soloopenacc(tconf_acc, local_staples, tipdot);
    mom_sum_mult(tmomenta, tipdot, deltas_Omelyan, k);
  };
  auto drift = [&]() { mom_exp_times_conf_soloopenacc(tconf_acc, tmomenta, deltas_Omelyan, 4); };
  kick(3); drift();
  for (int k = 1; k < gs; ++k) { kick(5); drift(); kick(6); drift(); }
  kick(5); drift(); kick(3);
}

// random_assignement.c:145-185: eight normal deviates of variance 1/2 per
// link composed into a traceless Hermitian matrix, written to the HOST array
// (the reference fills host memory and then updates the device mirror).
// The deviates come from the library's counter-based generator, stream
// 0x7fffffff of ostaple_set_momenta_seed's seed and a call counter.
static unsigned long long g_mom_seed = 1, g_mom_calls = 0;
void ostaple_set_momenta_seed(unsigned long long seed) { g_mom_seed = seed; g_mom_calls = 0; }

void generate_Momenta_gauss(thmat_soa* mom8) {
  if (!require_init("generate_Momenta_gauss")) return;
  const long n = sh();
  double* m = reinterpret_cast<double*>(mom8);
  const unsigned long long stream = 0x7fffffffull + g_mom_calls++;
  for (int dir = 0; dir < 8; ++dir)
    for (long x = 0; x < n; ++x) {
      double g[8];
      for (int j = 0; j < 4; ++j) {
        const unsigned long long c = (unsigned long long)(long(dir) * n + x) * 4ull + j;
        const double u1 = huniform(g_mom_seed, 2 * stream, c), u2 = huniform(g_mom_seed, 2 * stream + 1, c);
        const double rad = std::sqrt(-std::log(u1));
        g[2 * j] = rad * std::cos(2.0 * M_PI * u2);
        g[2 * j + 1] = rad * std::sin(2.0 * M_PI * u2);
      }
      double* base = m + long(dir) * 8 * n;
      const double r3 = 0.57735026918962576451;
      base[2 * x] = g[0]; base[2 * x + 1] = -g[1];                 // c01
      base[2 * n + 2 * x] = g[3]; base[2 * n + 2 * x + 1] = -g[4]; // c02
      base[4 * n + 2 * x] = g[5]; base[4 * n + 2 * x + 1] = -g[6]; // c12
      base[6 * n + x] = g[2] + g[7] * r3;                          // rc00
      base[7 * n + x] = -g[2] + g[7] * r3;                         // rc11
    }
}

// ---- the link generator ----
int ostaple_gauge_momenta(thmat_soa* mom, unsigned long long seed, unsigned long long stream) {
  if (!require_init("ostaple_gauge_momenta")) return -2;
  double* m = static_cast<double*>(resolve(mom, "mom"));
  if (!m) return -3;
  launch_gen_momenta<double>(m, seed, stream, S());
  return error_code();
}

int ostaple_gaussian_vec3(vec3_soa* v, unsigned long long seed, unsigned long long stream) {
  if (!require_init("ostaple_gaussian_vec3")) return -2;
  double2* d = static_cast<double2*>(resolve(v, "v"));
  if (!d) return -3;
  launch_gen_vec3_gauss(d, seed, stream, S());
  return error_code();
}

int ostaple_gauge_action(const su3_soa* u, double beta, double* plaq_sum, double* rect_sum, double* action) {
  if (!require_init("ostaple_gauge_action")) return -2;
  HmcLinks<double> l = links64(u, "u");
  double* d = dsc(4);
  if (!l.p || !d) return -3;
  launch_gauge_action<double>(l, 3, d, S());
  double h[2];
  read_scalars(h, d, 2);
  if (plaq_sum) *plaq_sum = h[0];
  if (rect_sum) *rect_sum = h[1];
  // the action the Metropolis test compares, -beta/3 (C_ZERO P + C_ONE R)
  // (update_versatile.c:226-230, 540-545)
  if (action) *action = -beta * 0.33333333333333333333333 * (C_ZERO * h[0] + C_ONE * h[1]);
  return error_code();
}

int ostaple_pure_gauge_hmc(su3_soa* u, double beta, int ntraj, int no_md, int gauge_scale, double traj_len,
                           unsigned long long seed, int first_traj, int precision, int metropolis, int* accepted,
                           double* plaquette, double* delta_s) {
  if (!require_init("ostaple_pure_gauge_hmc")) return -2;
  if (ntraj < 0 || no_md < 1 || gauge_scale < 1 || (precision != 0 && precision != 1)) {
    set_error(-11, "ostaple_pure_gauge_hmc: ntraj %d, no_md %d, gauge_scale %d, precision %d", ntraj, no_md,
              gauge_scale, precision);
    return -11;
  }
  cudaStream_t st = S();
  const long n = sh();
  HmcLinks<double> U = links64(u, "u");
  if (!U.p) return -3;
  double* mom = static_cast<double*>(workspace(WS_HMC_MOM, alg_bytes()));
  Z* bkp = static_cast<Z*>(workspace(WS_HMC_BKP, 72 * size_t(n) * sizeof(Z)));
  float2* u32 = nullptr;
  float* mom32 = nullptr;
  if (precision == 1) {
    u32 = static_cast<float2*>(workspace(WS_HMC_F32, 48 * size_t(n) * sizeof(float2) + 64 * size_t(n) * sizeof(float)));
    mom32 = u32 ? reinterpret_cast<float*>(u32 + 48 * size_t(n)) : nullptr;
  }
  double* d = dsc(8);
  if (!mom || !bkp || !d || (precision == 1 && !u32)) return -5;
  double dl[7];
  md_deltas(beta, no_md, gauge_scale, traj_len, dl);
  int acc = 0;
  for (int k = 0; k < ntraj; ++k) {
    const unsigned long long traj = (unsigned long long)first_traj + k;
    if (metropolis) OST_CUDA(cudaMemcpyAsync(bkp, U.p, 72 * size_t(n) * sizeof(Z), cudaMemcpyDeviceToDevice, st));
    launch_gen_momenta<double>(mom, seed, traj, st);
    if (precision == 1) {   // the MD starts from the FP32-rounded momenta
      launch_alg_64_to_32(mom, mom32, st);
      launch_alg_32_to_64(mom32, mom, st);
    }
    launch_gauge_action<double>(U, 3, d, st);
    launch_momenta_action<double>(mom, 0, 8, d + 2, st);
    // MD: 2 no_md gauge multisteps (the fermion kicks of
    // multistep_2MN_SOLOOPENACC vanish without fermions)
    if (precision == 0) {
      for (int c = 0; c < 2 * no_md; ++c) gauge_2mn_fused<double>(U, mom, dl, gauge_scale);
    } else {
      launch_links_64_to_32(U.p, 9, u32, st);
      HmcLinks<float> U32{u32, 0};   // array-of-structures FP32 copy
      for (int c = 0; c < 2 * no_md; ++c) gauge_2mn_fused<float>(U32, mom32, dl, gauge_scale);
      launch_links_32_to_64(u32, U.p, 9, st);
      launch_alg_32_to_64(mom32, mom, st);
    }
    launch_gauge_action<double>(U, 3, d + 3, st);
    launch_momenta_action<double>(mom, 0, 8, d + 5, st);
    double h[6];
    read_scalars(h, d, 6);
    if (error_code()) return error_code();
    const double b3 = beta * 0.33333333333333333333333;
    const double s_in = b3 * (C_ZERO * h[0] + C_ONE * h[1]), s_fin = b3 * (C_ZERO * h[3] + C_ONE * h[4]);
    // delta_S = -(-S_in + K_in) + (-S_fin + K_fin)  (update_versatile.c:572)
    const double ds = -(-s_in + h[2]) + (-s_fin + h[5]);
    int ok = 1;
    if (metropolis && ds >= 0) ok = huniform(seed, 0xA5A5A5A500000000ull + traj, 0) < std::exp(-ds);
    if (!ok) OST_CUDA(cudaMemcpyAsync(U.p, bkp, 72 * size_t(n) * sizeof(Z), cudaMemcpyDeviceToDevice, st));
    acc += ok;
    if (delta_s) delta_s[k] = ds;
    if (plaquette) plaquette[k] = (ok ? h[3] : h[0]) / (18.0 * double(2 * n));   // <Re tr P> / 3 per plaquette
  }
  OST_CUDA(cudaStreamSynchronize(st));
  if (accepted) *accepted = acc;
  return error_code();
}

}  // extern "C"
