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
#include "solvers_fp.cuh"
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

using fp::dscal;
using fp::readback;

inline void mdagm_dev(const Z* u, Z* out, const Z* in, Z* tmp, const void* ph, double m2) {
  fp::mdagm<double>(u, out, in, tmp, ph, m2);
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
  if (maxiter < 0 || maxiter > OST_MAX_SHIFTS) {
    set_error(-11, "multiple_combine_in1_minus_in2x_factor_back_into_in1: maxiter %d outside [0,%d]", maxiter,
              OST_MAX_SHIFTS);
    return;
  }
  Z* o = DVW(out, "out");
  const Z* a = DV(in, "in");
  if (!o || !a || maxiter == 0) return;
  CgmCoeffs cf{};
  cf.nshift = maxiter;
  for (int k = 0; k < maxiter; ++k) {
    cf.active[k] = flag[k] == 1;
    cf.omega[k] = omegas[k];
  }
  multi_xupdate<double>(o, a, vlen(), cf, vlen(), S());   // out_k -= omegas_k in_k, one pass
}
void multiple1_combine_in1_x_fact1_plus_in2_x_fact2_back_into_in1(vec3_soa* in1, int maxiter, const int* flag,
                                                                  const double* gammas, const vec3_soa* in2,
                                                                  const double* zeta_iii) {
  if (!require_init("multiple1_combine_in1_x_fact1_plus_in2_x_fact2_back_into_in1")) return;
  if (maxiter < 0 || maxiter > OST_MAX_SHIFTS) {
    set_error(-11, "multiple1_combine_in1_x_fact1_plus_in2_x_fact2_back_into_in1: maxiter %d outside [0,%d]",
              maxiter, OST_MAX_SHIFTS);
    return;
  }
  Z* a = DVW(in1, "in1");
  const Z* b = DV(in2, "in2");
  if (!a || !b || maxiter == 0) return;
  CgmCoeffs cf{};
  cf.nshift = maxiter;
  for (int k = 0; k < maxiter; ++k) {
    cf.active[k] = flag[k] == 1;
    cf.gamma[k] = gammas[k];
    cf.zeta[k] = zeta_iii[k];
  }
  multi_pupdate<double>(a, b, vlen(), cf, vlen(), S());   // in1_k = gammas_k in1_k + zeta_k in2, one pass
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
  return fp::cg<double>(du, ph, pars->ferm_mass, x, b, res, r, h, s, p, max_cg, shift,
                         inverter_tricks.restartingEvery, cg_return);
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
  return fp::cgm<double>(du, ph, pars->ferm_mass, approx->RA_b, order, xs, b, residuo, r, h, s, p, ps, max_cg,
                          cg_return);
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

double ker_find_max_eigenvalue_openacc(su3_soa* u, ferm_param* pars, vec3_soa* loc_r, vec3_soa* loc_h,
                                       vec3_soa* loc_p) {
  return power_iteration("ker_find_max_eigenvalue_openacc", u, pars, 0.0, loc_r, loc_h, loc_p);
}

// The reference passes shift = (max - m^2) - m^2 to the shifted matrix and
// returns max - |p| (find_min_max.c:62-92); kept as it is.  Its caller does
// not use it: the minimum is set to m^2.
double ker_find_min_eigenvalue_openacc(su3_soa* u, ferm_param* pars, vec3_soa* loc_r, vec3_soa* loc_h,
                                       vec3_soa* loc_p, double max) {
  const double m2 = pars->ferm_mass * pars->ferm_mass;
  const double delta = max - m2;
  return max - power_iteration("ker_find_min_eigenvalue_openacc", u, pars, delta - m2, loc_r, loc_h, loc_p);
}

void find_min_max_eigenvalue_soloopenacc(su3_soa* u, ferm_param* pars, vec3_soa* loc_r, vec3_soa* loc_h,
                                         vec3_soa* loc_p1, vec3_soa* loc_p2, double* minmax) {
  (void)loc_p2;
  minmax[0] = pars->ferm_mass * pars->ferm_mass;
  minmax[1] = ker_find_max_eigenvalue_openacc(u, pars, loc_r, loc_h, loc_p1);
  if (verbosity_lv > 3)
    printf("    Computed the min and max eigs : [ min= %.18lf; max= %.18lf ]  \n", minmax[0], minmax[1]);
}

}  // extern "C"
