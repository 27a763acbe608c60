// capi.cu -- the reference-named C entry points of the Dirac operator, the
// fermion BLAS and the FP64 solvers.  Each function keeps the reference's
// argument meaning and return convention; pointers are translated through
// the residency registry (OpenACC `present`).
#include <cmath>
#include <cstdio>
#include <vector>
#include "dslash.cuh"
#include "kernels.cuh"
#include "runtime.cuh"
#include "solver_kernels.cuh"
#include "../../include/ostaple_gb300.h"

using namespace ost;

// Weak defaults for globals a reference host program defines itself.
extern "C" {
__attribute__((weak)) inv_tricks inverter_tricks = {0, 0, 0.1, 10000};
__attribute__((weak)) int verbosity_lv = 0;
}

namespace {

typedef double2 Z;

inline long vlen() { return 3L * rt().g.sizeh; }           // complex numbers in a vec3_soa
inline long su3len() { return 9L * rt().g.sizeh; }         // complex numbers in a su3_soa
inline cudaStream_t S() { return rt().stream; }

void dslash64(int parity, const su3_soa* u, vec3_soa* out, const vec3_soa* in, const double_soa* bf,
              int epi, const vec3_soa* in0, double mass2, const char* who) {
  if (!require_init(who)) return;
  DslashArgs<double> a;
  a.parity = parity;
  a.phase_mode = PH_ANGLE;
  a.epilogue = epi;
  a.u = dev(reinterpret_cast<const Z*>(u), "u");
  a.out = dev(reinterpret_cast<Z*>(out), "out");
  a.in = dev(reinterpret_cast<const Z*>(in), "in");
  a.phases = resolve(bf, "backfield");
  a.in0 = epi == EPI_MDAGM ? dev(reinterpret_cast<const Z*>(in0), "in") : nullptr;
  a.mass2 = mass2;
  a.stream = S();
  if (!a.u || !a.out || !a.in || !a.phases || (epi == EPI_MDAGM && !a.in0)) return;
  launch_dslash<double>(a);
}

// device-side M^+M with the temp field: tmp = D_oe in ; out = m2 in - D_eo tmp
void mdagm_dev(const Z* u, Z* out, const Z* in, Z* tmp, const void* ph, double m2) {
  DslashArgs<double> a;
  a.phase_mode = PH_ANGLE;
  a.u = u;
  a.phases = ph;
  a.stream = S();
  a.mass2 = 0;
  a.in0 = nullptr;
  a.parity = 1; a.epilogue = EPI_PLAIN; a.out = tmp; a.in = in;
  launch_dslash<double>(a);
  a.parity = 0; a.epilogue = EPI_MDAGM; a.out = out; a.in = tmp; a.in0 = in; a.mass2 = m2;
  launch_dslash<double>(a);
}

// one-double device scalar slots read back by the host solvers
double* dscal(int k) {
  double* p = static_cast<double*>(workspace(WS_SCALARS, 64 * sizeof(double)));
  return p ? p + k : nullptr;
}
double readback(const double* d) {
  double h = 0;
  OST_CUDA(cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, S()));
  OST_CUDA(cudaStreamSynchronize(S()));
  return h;
}

}  // namespace

extern "C" {

void acc_Deo(const su3_soa* u, vec3_soa* out, const vec3_soa* in, const double_soa* bf) {
  dslash64(0, u, out, in, bf, EPI_PLAIN, nullptr, 0.0, "acc_Deo");
}
void acc_Doe(const su3_soa* u, vec3_soa* out, const vec3_soa* in, const double_soa* bf) {
  dslash64(1, u, out, in, bf, EPI_PLAIN, nullptr, 0.0, "acc_Doe");
}
void acc_Deo_unsafe(const su3_soa* u, vec3_soa* out, const vec3_soa* in, const double_soa* bf) {
  dslash64(0, u, out, in, bf, EPI_PLAIN, nullptr, 0.0, "acc_Deo_unsafe");
}
void acc_Doe_unsafe(const su3_soa* u, vec3_soa* out, const vec3_soa* in, const double_soa* bf) {
  dslash64(1, u, out, in, bf, EPI_PLAIN, nullptr, 0.0, "acc_Doe_unsafe");
}

void fermion_matrix_multiplication_shifted(const su3_soa* u, vec3_soa* out, const vec3_soa* in,
                                           vec3_soa* temp1, ferm_param* pars, double shift) {
  // temp1 = D_oe in ; out = (m^2 + shift) in - D_eo temp1   (fermion_matrix.c:736-746)
  dslash64(1, u, temp1, in, pars->phases, EPI_PLAIN, nullptr, 0.0, "fermion_matrix_multiplication");
  dslash64(0, u, out, temp1, pars->phases, EPI_MDAGM, in, pars->ferm_mass * pars->ferm_mass + shift,
           "fermion_matrix_multiplication");
}

void fermion_matrix_multiplication(const su3_soa* u, vec3_soa* out, const vec3_soa* in, vec3_soa* temp1,
                                   ferm_param* pars) {
  fermion_matrix_multiplication_shifted(u, out, in, temp1, pars, 0.0);
}

// ---- reductions (synchronous: they return host scalars) ----
void scal_prod_global_ri(const vec3_soa* a, const vec3_soa* b, double* re_im) {
  if (!require_init("scal_prod_global")) return;
  const Z* da = dev(reinterpret_cast<const Z*>(a), "in_vect1");
  const Z* db = dev(reinterpret_cast<const Z*>(b), "in_vect2");
  if (!da || !db) return;
  blas_cdot<double>(da, db, vlen(), dscal(0), S());
  double h[2];
  OST_CUDA(cudaMemcpyAsync(h, dscal(0), 2 * sizeof(double), cudaMemcpyDeviceToHost, S()));
  OST_CUDA(cudaStreamSynchronize(S()));
  re_im[0] = h[0];
  re_im[1] = h[1];
}

ostaple_dcomplex scal_prod_global(const vec3_soa* a, const vec3_soa* b) {
  double ri[2] = {NAN, NAN};
  scal_prod_global_ri(a, b, ri);
  ostaple_dcomplex z;
  z.re = ri[0];
  z.im = ri[1];
  return z;
}

double real_scal_prod_global(const vec3_soa* a, const vec3_soa* b) {
  if (!require_init("real_scal_prod_global")) return NAN;
  const Z* da = dev(reinterpret_cast<const Z*>(a), "in_vect1");
  const Z* db = dev(reinterpret_cast<const Z*>(b), "in_vect2");
  if (!da || !db) return NAN;
  blas_rdot<double>(da, db, vlen(), dscal(0), S());
  return readback(dscal(0));
}

double l2norm2_global(const vec3_soa* a) {
  if (!require_init("l2norm2_global")) return NAN;
  const Z* da = dev(reinterpret_cast<const Z*>(a), "in_vect1");
  if (!da) return NAN;
  blas_norm2<double>(da, vlen(), dscal(0), S());
  return readback(dscal(0));
}

// ---- streaming BLAS ----
#define DV(p, name) dev(reinterpret_cast<const Z*>(p), name)
#define DVW(p, name) dev(reinterpret_cast<Z*>(p), name)

void combine_in1xfactor_plus_in2(const vec3_soa* in1, const double factor, const vec3_soa* in2, vec3_soa* out) {
  if (!require_init("combine_in1xfactor_plus_in2")) return;
  const Z *a = DV(in1, "in1"), *b = DV(in2, "in2");
  Z* o = DVW(out, "out");
  if (a && b && o) blas_axpy<double>(a, factor, b, o, vlen(), S());
}
void multiply_fermion_x_doublefactor(vec3_soa* in1, const double factor) {
  if (!require_init("multiply_fermion_x_doublefactor")) return;
  Z* a = DVW(in1, "in1");
  if (a) blas_scale<double>(a, factor, vlen(), S());
}
void combine_add_factor_x_in2_to_in1(vec3_soa* in1, const vec3_soa* in2, double factor) {
  if (!require_init("combine_add_factor_x_in2_to_in1")) return;
  Z* a = DVW(in1, "in1");
  const Z* b = DV(in2, "in2");
  if (a && b) blas_axpy<double>(b, factor, a, a, vlen(), S());
}
void combine_in1xferm_mass2_minus_in2_minus_in3(const vec3_soa* in1, double m, const vec3_soa* in2,
                                                const vec3_soa* in3, vec3_soa* out) {
  if (!require_init("combine_in1xferm_mass2_minus_in2_minus_in3")) return;
  const Z *a = DV(in1, "in1"), *b = DV(in2, "in2"), *c = DV(in3, "in3");
  Z* o = DVW(out, "out");
  if (a && b && c && o) blas_axmymz<double>(a, m, b, c, o, vlen(), S());
}
void combine_inside_loop(vec3_soa* vout, vec3_soa* vr, const vec3_soa* vs, const vec3_soa* vp, const double w) {
  if (!require_init("combine_inside_loop")) return;
  Z *o = DVW(vout, "out"), *r = DVW(vr, "r");
  const Z *s = DV(vs, "s"), *p = DV(vp, "p");
  if (o && r && s && p) blas_inside_loop<double>(o, r, s, p, w, vlen(), S());
}
void combine_in1xferm_mass_minus_in2(const vec3_soa* in1, double m2, vec3_soa* in2) {
  if (!require_init("combine_in1xferm_mass_minus_in2")) return;
  const Z* a = DV(in1, "in1");
  Z* b = DVW(in2, "in2");
  if (a && b) blas_axmy<double>(a, m2, b, b, vlen(), S());
}
void combine_in1_minus_in2(const vec3_soa* in1, const vec3_soa* in2, vec3_soa* out) {
  if (!require_init("combine_in1_minus_in2")) return;
  const Z *a = DV(in1, "in1"), *b = DV(in2, "in2");
  Z* o = DVW(out, "out");
  if (a && b && o) blas_axmy<double>(a, 1.0, b, o, vlen(), S());
}
void assign_in_to_out(const vec3_soa* in1, vec3_soa* out) {
  if (!require_init("assign_in_to_out")) return;
  const Z* a = DV(in1, "in");
  Z* o = DVW(out, "out");
  if (a && o) blas_copy<double>(a, o, vlen(), S());
}
void set_vec3_soa_to_zero(vec3_soa* f) {
  if (!require_init("set_vec3_soa_to_zero")) return;
  Z* a = DVW(f, "fermion");
  if (a) blas_zero<double>(a, vlen(), S());
}
void multiple_combine_in1_minus_in2x_factor_back_into_in1(vec3_soa* out, const vec3_soa* in, const int maxiter,
                                                          const int* flag, const double* omegas) {
  if (!require_init("multiple_combine_in1_minus_in2x_factor_back_into_in1")) return;
  Z* o = DVW(out, "out");
  const Z* a = DV(in, "in");
  if (!o || !a) return;
  for (int k = 0; k < maxiter; ++k)
    if (flag[k] == 1) blas_axpy<double>(a + k * vlen(), -omegas[k], o + k * vlen(), o + k * vlen(), vlen(), S());
}
void multiple1_combine_in1_x_fact1_plus_in2_x_fact2_back_into_in1(vec3_soa* in1, int maxiter, const int* flag,
                                                                  const double* gammas, const vec3_soa* in2,
                                                                  const double* zeta_iii) {
  if (!require_init("multiple1_combine_in1_x_fact1_plus_in2_x_fact2_back_into_in1")) return;
  Z* a = DVW(in1, "in1");
  const Z* b = DV(in2, "in2");
  if (!a || !b) return;
  for (int k = 0; k < maxiter; ++k) {
    if (flag[k] != 1) continue;
    // in1_k = gammas_k in1_k + zeta_k in2
    blas_scale<double>(a + k * vlen(), gammas[k], vlen(), S());
    blas_axpy<double>(b, zeta_iii[k], a + k * vlen(), a + k * vlen(), vlen(), S());
  }
}
void combine_in1_x_fact1_minus_in2_back_into_in2(const vec3_soa* in1, double f, vec3_soa* in2) {
  if (!require_init("combine_in1_x_fact1_minus_in2_back_into_in2")) return;
  const Z* a = DV(in1, "in1");
  Z* b = DVW(in2, "in2");
  if (a && b) blas_axmy<double>(a, f, b, b, vlen(), S());
}
void combine_in1_minus_in2_allxfact(const vec3_soa* in1, const vec3_soa* in2, double f, vec3_soa* out) {
  if (!require_init("combine_in1_minus_in2_allxfact")) return;
  const Z *a = DV(in1, "in1"), *b = DV(in2, "in2");
  Z* o = DVW(out, "out");
  if (a && b && o) blas_scaled_diff<double>(a, b, f, o, vlen(), S());
}

// ---- single-shift CG (inverter_full.c:19-132) ----
int ker_invert_openacc(const su3_soa* u, ferm_param* pars, vec3_soa* solution, const vec3_soa* in, double res,
                       vec3_soa* loc_r, vec3_soa* loc_h, vec3_soa* loc_s, vec3_soa* loc_p, const int max_cg,
                       double shift, int* cg_return) {
  if (!require_init("ker_invert_openacc")) return INVERTER_FAILURE;
  const Z* du = DV(u, "u");
  Z* x = DVW(solution, "solution");
  const Z* b = DV(in, "in");
  Z *r = DVW(loc_r, "loc_r"), *h = DVW(loc_h, "loc_h"), *s = DVW(loc_s, "loc_s"), *p = DVW(loc_p, "loc_p");
  const void* ph = resolve(pars->phases, "phases");
  if (!du || !x || !b || !r || !h || !s || !p || !ph) return INVERTER_FAILURE;
  const long n = vlen();
  const double m2 = pars->ferm_mass * pars->ferm_mass + shift;
  const double SAFETY = 0.95;
  const int restart = inverter_tricks.restartingEvery > 0 ? inverter_tricks.restartingEvery : 10000;

  blas_norm2<double>(b, n, dscal(0), S());
  const double source_norm = readback(dscal(0));
  int cg = 0;
  double delta, alpha, lambda = 0, omega, gammag;
  do {
    mdagm_dev(du, s, x, h, ph, m2);
    blas_axmy<double>(b, 1.0, s, r, n, S());      // r = in - s
    blas_copy<double>(r, p, n, S());
    blas_norm2<double>(r, n, dscal(0), S());
    delta = readback(dscal(0));
    int cg_restarted = 0;
    do {
      cg++;
      cg_restarted++;
      mdagm_dev(du, s, p, h, ph, m2);
      blas_rdot<double>(p, s, n, dscal(1), S());
      alpha = readback(dscal(1));
      omega = delta / alpha;
      blas_axpy<double>(p, omega, x, x, n, S());    // x += omega p
      fused_axpy_norm<double>(r, s, -omega, n, dscal(2), S());  // r -= omega s ; lambda
      lambda = readback(dscal(2));
      gammag = lambda / delta;
      delta = lambda;
      blas_axpy<double>(p, gammag, r, p, n, S());   // p = r + gammag p
      if (error_code()) return INVERTER_FAILURE;
    } while (std::sqrt(lambda / source_norm) > res * SAFETY && cg_restarted < restart);
  } while (std::sqrt(lambda / source_norm) > res && cg < max_cg);

  mdagm_dev(du, s, x, h, ph, m2);
  blas_axmy<double>(b, 1.0, s, h, n, S());
  blas_norm2<double>(h, n, dscal(3), S());
  const double current_res = readback(dscal(3)) / source_norm;
  if (verbosity_lv > 1)
    printf("Terminated invert after   %d    iterations[res/stop_res=  %e , stop_res=%e ]\n", cg,
           std::sqrt(current_res) / res, res);
  if (cg == max_cg) printf("WARNING: maximum number of iterations reached in invert\n");
  *cg_return = cg;
  if (error_code()) return INVERTER_FAILURE;
  return std::sqrt(current_res) <= res ? INVERTER_SUCCESS : INVERTER_FAILURE;
}

// ---- multi-shift CG (inverter_multishift_full.c:23-252) ----
int multishift_invert(const su3_soa* u, ferm_param* pars, RationalApprox* approx, vec3_soa* out,
                      const vec3_soa* in, double residuo, vec3_soa* loc_r, vec3_soa* loc_h, vec3_soa* loc_s,
                      vec3_soa* loc_p, vec3_soa* shiftferm, const int max_cg, int* cg_return) {
  if (!require_init("multishift_invert")) return INVERTER_FAILURE;
  const int order = approx->approx_order;
  if (order < 1 || order > OST_MAX_SHIFTS) {
    set_error(-11, "multishift_invert: approx_order %d outside [1,%d]", order, OST_MAX_SHIFTS);
    return INVERTER_FAILURE;
  }
  const Z* du = DV(u, "u");
  Z* xs = DVW(out, "out");
  const Z* b = DV(in, "in");
  Z *r = DVW(loc_r, "loc_r"), *h = DVW(loc_h, "loc_h"), *s = DVW(loc_s, "loc_s"), *p = DVW(loc_p, "loc_p");
  Z* ps = DVW(shiftferm, "shiftferm");
  const void* ph = resolve(pars->phases, "phases");
  if (!du || !xs || !b || !r || !h || !s || !p || !ps || !ph) return INVERTER_FAILURE;
  const long n = vlen();
  const double m2 = pars->ferm_mass * pars->ferm_mass;
  const double SAFETY = 0.95;

  double zeta_i[OST_MAX_SHIFTS], zeta_ii[OST_MAX_SHIFTS], zeta_iii[OST_MAX_SHIFTS];
  double omegas[OST_MAX_SHIFTS], gammas[OST_MAX_SHIFTS];
  int flag[OST_MAX_SHIFTS];
  for (int k = 0; k < order; ++k) {
    flag[k] = 1;
    blas_zero<double>(xs + k * n, n, S());
  }
  blas_copy<double>(b, r, n, S());
  blas_copy<double>(r, p, n, S());
  blas_norm2<double>(r, n, dscal(0), S());
  double delta = readback(dscal(0));
  blas_norm2<double>(b, n, dscal(1), S());
  const double source_norm = readback(dscal(1));
  double omega = 1.0, omega_save, alpha, lambda, gammag = 0.0;
  for (int k = 0; k < order; ++k) {
    blas_copy<double>(b, ps + k * n, n, S());
    zeta_i[k] = 1.0;
    zeta_ii[k] = 1.0;
    gammas[k] = 0.0;
  }
  int cg = 0;
  int maxiter = order;
  do {
    cg++;
    mdagm_dev(du, s, p, h, ph, m2);
    blas_rdot<double>(p, s, n, dscal(2), S());
    alpha = readback(dscal(2));
    omega_save = omega;
    omega = -delta / alpha;
    for (int k = 0; k < maxiter; ++k) {
      if (flag[k] == 1) {
        zeta_iii[k] = (zeta_i[k] * zeta_ii[k] * omega_save) /
                      (omega * gammag * (zeta_i[k] - zeta_ii[k]) +
                       zeta_i[k] * omega_save * (1.0 - (approx->RA_b[k]) * omega));
        omegas[k] = omega * zeta_iii[k] / zeta_ii[k];
      }
    }
    fused_axpy_norm<double>(r, s, omega, n, dscal(3), S());   // r += omega s ; lambda
    lambda = readback(dscal(3));
    gammag = lambda / delta;
    for (int k = 0; k < order; ++k)
      if (flag[k] == 1) gammas[k] = gammag * zeta_iii[k] * omegas[k] / (zeta_ii[k] * omega);
    CgmCoeffs cf;
    cf.nshift = maxiter;
    for (int k = 0; k < maxiter; ++k) {
      cf.active[k] = flag[k] == 1;
      cf.omega[k] = omegas[k];
      cf.gamma[k] = gammas[k];
      cf.zeta[k] = zeta_iii[k];
    }
    // p = r + gammag p ; x_k -= omegas_k ps_k ; ps_k = gammas_k ps_k + zeta_k r
    fused_cgm_update<double>(p, r, gammag, xs, ps, n, cf, n, S());
    maxiter = 0;
    for (int k = 0; k < order; ++k) {
      if (flag[k] == 1) {
        double fact = std::sqrt(delta * zeta_ii[k] * zeta_ii[k] / source_norm);
        if (fact < residuo * SAFETY) flag[k] = 0;
        else maxiter = k + 1;
        zeta_i[k] = zeta_ii[k];
        zeta_ii[k] = zeta_iii[k];
      }
    }
    delta = lambda;
    if (error_code()) return INVERTER_FAILURE;
  } while (maxiter > 0 && cg < max_cg);
  if (cg == max_cg) printf("WARNING: maximum number of iterations reached in invert\n");

  int check = 1;
  for (int k = 0; k < order; ++k) {
    mdagm_dev(du, s, xs + k * n, h, ph, m2 + approx->RA_b[k]);
    blas_axmy<double>(b, 1.0, s, h, n, S());
    blas_norm2<double>(h, n, dscal(4), S());
    double rr = readback(dscal(4)) / source_norm;
    check *= (rr <= 1) ? 1 : 0;
  }
  *cg_return = cg;
  if (error_code()) return INVERTER_FAILURE;
  return check ? INVERTER_SUCCESS : INVERTER_FAILURE;
}

void recombine_shifted_vec3_to_vec3(const vec3_soa* in_shifted, const vec3_soa* in, vec3_soa* out,
                                    const RationalApprox* approx) {
  if (!require_init("recombine_shifted_vec3_to_vec3")) return;
  const Z* xs = DV(in_shifted, "in_shifted");
  const Z* b = DV(in, "in");
  Z* o = DVW(out, "out");
  if (!xs || !b || !o) return;
  RecombCoeffs rc;
  rc.order = approx->approx_order;
  rc.a0 = approx->RA_a0;
  for (int k = 0; k < rc.order && k < OST_MAX_SHIFTS; ++k) rc.a[k] = approx->RA_a[k];
  recombine<double>(xs, vlen(), b, o, rc, vlen(), S());
}

// ---- eigenvalue bounds of M^+M (the rational approximation's range) ----
//
// Power iteration, find_min_max.c:21-92: p <- p/|p|, r = p,
// p = (m^2 + shift) r - D_eo D_oe r, until the relative change of |p| is at
// most 1e-5.  p holds the (Gaussian) start vector on entry and the last
// product on exit, r the last normalised vector; |p| is read back once per
// iteration for the stopping test, as in the reference.
static double power_iteration(const char* who, const su3_soa* u, ferm_param* pars, double shift, vec3_soa* loc_r,
                              vec3_soa* loc_h, vec3_soa* loc_p) {
  if (!require_init(who)) return NAN;
  const Z* du = DV(u, "u");
  Z* p = DVW(loc_p, "loc_p");
  Z* r = DVW(loc_r, "loc_r");
  Z* h = DVW(loc_h, "loc_h");
  const void* ph = resolve(pars->phases, "phases");
  if (!du || !p || !r || !h || !ph) return NAN;
  const double m2 = pars->ferm_mass * pars->ferm_mass + shift;
  double* d = dscal(0);
  blas_norm2<double>(p, vlen(), d, S());
  double norm = std::sqrt(readback(d)), rel;
  int loops = 0;
  do {
    blas_scale<double>(p, 1.0 / norm, vlen(), S());
    blas_copy<double>(p, r, vlen(), S());
    const double old = norm;
    mdagm_dev(du, p, r, h, ph, m2);
    blas_norm2<double>(p, vlen(), d, S());
    norm = std::sqrt(readback(d));
    rel = std::fabs(old - norm) / norm;
    ++loops;
    if (loops % 100 == 0 && verbosity_lv > 2)
      printf("        iterations of max computat  = %d, norm = %lf, old_norm = %lf\n", loops, norm, rel);
    if (loops >= 1000000) {
      set_error(-15, "%s: power iteration did not settle in %d iterations", who, loops);
      break;
    }
  } while (rel > 1.0e-5 && error_code() == 0);
  return norm;
}

double ker_find_max_eigenvalue_openacc(const su3_soa* u, ferm_param* pars, vec3_soa* loc_r, vec3_soa* loc_h,
                                       vec3_soa* loc_p) {
  return power_iteration("ker_find_max_eigenvalue_openacc", u, pars, 0.0, loc_r, loc_h, loc_p);
}

// The reference passes shift = (max - m^2) - m^2 to the shifted matrix and
// returns max - |p| (find_min_max.c:62-92); kept as it is.  Its caller does
// not use it: the minimum is set to m^2.
double ker_find_min_eigenvalue_openacc(const su3_soa* u, ferm_param* pars, vec3_soa* loc_r, vec3_soa* loc_h,
                                       vec3_soa* loc_p, double max) {
  const double m2 = pars->ferm_mass * pars->ferm_mass;
  const double delta = max - m2;
  return max - power_iteration("ker_find_min_eigenvalue_openacc", u, pars, delta - m2, loc_r, loc_h, loc_p);
}

void find_min_max_eigenvalue_soloopenacc(const su3_soa* u, ferm_param* pars, vec3_soa* loc_r, vec3_soa* loc_h,
                                         vec3_soa* loc_p1, vec3_soa* loc_p2, double* minmax) {
  (void)loc_p2;
  minmax[0] = pars->ferm_mass * pars->ferm_mass;
  minmax[1] = ker_find_max_eigenvalue_openacc(u, pars, loc_r, loc_h, loc_p1);
  if (verbosity_lv > 3)
    printf("    Computed the min and max eigs : [ min= %.18lf; max= %.18lf ]  \n", minmax[0], minmax[1]);
}

}  // extern "C"
