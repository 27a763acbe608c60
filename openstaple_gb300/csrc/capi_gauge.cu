// capi_gauge.cu -- C entry points of stout smearing and the rational fermion
// force (stouting.h:13-44, fermion_force.h:15-36,
// fermion_force_utilities.h:204-240), plus the multi-shift dispatch wrapper
// (inverter_wrappers.c:41-114).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include "batched.cuh"
#include "dslash.cuh"
#include "gauge_kernels.cuh"
#include "kernels.cuh"
#include "runtime.cuh"
#include "../../include/ostaple_gb300.h"

using namespace ost;

extern "C" {
// Globals a reference host program defines itself (action.h:22-23,
// action.c); weak defaults here: 2 stout steps of rho = 0.15.
__attribute__((weak)) double gl_stout_rho = 0.15;
__attribute__((weak)) double gl_topo_rho = 0.15;
__attribute__((weak)) action_param act_params = {0.0, 2, 0.15, 0, 0.0, 0.0, {0}, 0, 0.15};
}

namespace {

typedef double2 Z;
inline cudaStream_t S() { return rt().stream; }
inline long sh() { return rt().g.sizeh; }
inline size_t su3_bytes() { return 8 * 9 * size_t(sh()) * sizeof(Z); }      // su3_soa[8]
inline size_t alg_bytes() { return 8 * 8 * size_t(sh()) * sizeof(double); }  // tamat_soa[8] / thmat_soa[8]
inline long vlen() { return 3L * sh(); }

double rho_of(int istopo) { return istopo ? gl_topo_rho : gl_stout_rho; }

template <typename T> T* D(T* p, const char* n) { return static_cast<T*>(resolve(p, n)); }
template <typename T> const T* D(const T* p, const char* n) { return static_cast<const T*>(resolve(p, n)); }

void zero_bytes(void* p, size_t n) { OST_CUDA(cudaMemsetAsync(p, 0, n, S())); }


// The pseudofermions of one flavour in groups of up to 4: all shifts of a
// group solved together by the two-phase multi-shift solver (FP32 CG-M to the
// reference's single-precision target, then FP64 refinement: batched mixed
// when mixed != 0, else ker_invert_openacc per system), then D_oe of every
// solution and the outer products of the whole group accumulated into aux in
// one pass (fermion_force.c:222-249 loops over the pseudofermions one by one).
// The last pseudofermion's solutions are left in shiftmulti and its last
// shift's X and D_oe X in ip.loc_s / ip.loc_h, as after the reference's loop.
void force_pseudofermion_groups(inverter_package ip, ferm_param* fp, const Z* first_src, su3_soa* aux_u,
                                vec3_soa* shiftmulti, double res, int max_cg, int mixed) {
  const int order = fp->approx_md.approx_order;
  const int nps = fp->number_of_ps;
  if (order < 1 || order > MAX_APPROX_ORDER) {
    set_error(-11, "fermion force: approx_md order %d out of range", order);
    return;
  }
  const long n = vlen();
  const Z* u = D(reinterpret_cast<const Z*>(ip.u), "ip.u");
  const double* ph = static_cast<const double*>(resolve(fp->phases, "phases"));
  const Z* b = D(first_src, "ferm_in_acc");
  Z* aux = D(reinterpret_cast<Z*>(aux_u), "aux_u");
  Z* last = D(reinterpret_cast<Z*>(shiftmulti), "tferm_shiftmulti_acc");
  const int group = std::min(nps, 4);
  Z* xs = static_cast<Z*>(workspace(WS_FORCE1, size_t(group) * order * n * sizeof(Z)));
  Z* ys = static_cast<Z*>(workspace(WS_MULTI2, std::max<size_t>(size_t(group) * order * n * sizeof(Z),
                                                                2 * size_t(BATCH_MAX) * n * sizeof(Z))));
  double* coef = static_cast<double*>(workspace(WS_FORCE3, 128 * sizeof(double)));
  if (!u || !ph || !b || !aux || !last || !xs || !ys || !coef) return;
  double res_sp = double(8e-7f * sqrtf(float(sh())));
  if (res_sp < res) res_sp = res;
  double c[128];
  for (int p0 = 0; p0 < nps; p0 += 4) {
    const int m = std::min(4, nps - p0);
    int it_cgm[4];
    int st = multishift_two_phase(u, ph, fp->ferm_mass, fp->approx_md.RA_b, order, m, b + long(p0) * n, xs, res_sp,
                                  res, max_cg, 0.0, mixed, it_cgm, nullptr, nullptr);
    convergence_messages(CONVERGENCE_NONCRITICAL, st);
    if (!mixed) {
      for (int r = 0; r < m; ++r)
        for (int k = 0; k < order; ++k) {
          vec3_soa* xk = reinterpret_cast<vec3_soa*>(xs + (long(r) * order + k) * n);
          const vec3_soa* src = reinterpret_cast<const vec3_soa*>(b + long(p0 + r) * n);
          inverter_wrapper(ip, fp, xk, src, res, max_cg, fp->approx_md.RA_b[k], CONVERGENCE_NONCRITICAL);
        }
    }
    // ys = D_oe xs (the ys buffer is reused by the refinement stage, so after it)
    for (int k = 0; k < m * order; ++k) {
      DslashArgs<double> a;
      a.parity = 1; a.phase_mode = PH_ANGLE; a.epilogue = EPI_PLAIN; a.u = u; a.out = ys + k * n;
      a.in = xs + k * n; a.phases = ph; a.in0 = nullptr; a.mass2 = 0; a.stream = S(); a.compact_links = 0;
      launch_dslash<double>(a);
    }
    for (int r = 0; r < m; ++r)
      for (int k = 0; k < order; ++k) c[r * order + k] = fp->approx_md.RA_a[k];
    OST_CUDA(cudaMemcpyAsync(coef, c, size_t(m) * order * sizeof(double), cudaMemcpyHostToDevice, S()));
    launch_force_outer(xs, ys, n, m * order, coef, nullptr, aux, 0, S());
    if (p0 + m == nps) {
      const Z* xl = xs + long(m - 1) * order * n;
      blas_copy<double>(xl, last, long(order) * n, S());
      Z* s = ip.loc_s ? D(reinterpret_cast<Z*>(ip.loc_s), "loc_s") : nullptr;
      Z* h = ip.loc_h ? D(reinterpret_cast<Z*>(ip.loc_h), "loc_h") : nullptr;
      if (s) blas_copy<double>(xl + (order - 1) * n, s, n, S());
      if (h) blas_copy<double>(ys + (long(m - 1) * order + order - 1) * n, h, n, S());
    }
    // the host coefficient buffer is reused by the next group
    OST_CUDA(cudaStreamSynchronize(S()));
  }
}

}  // namespace

extern "C" {

void set_su3_soa_to_zero(su3_soa* m) {
  if (!require_init("set_su3_soa_to_zero")) return;
  void* d = resolve(m, "matrix");
  if (d) zero_bytes(d, su3_bytes());
}

void set_tamat_soa_to_zero(tamat_soa* m) {
  if (!require_init("set_tamat_soa_to_zero")) return;
  void* d = resolve(m, "matrix");
  if (d) zero_bytes(d, alg_bytes());
}

void stout_isotropic(const su3_soa* u, su3_soa* uprime, su3_soa* local_staples, su3_soa* auxiliary,
                     tamat_soa* tipdot, const int istopo) {
  if (!require_init("stout_isotropic")) return;
  (void)auxiliary;  // parking variable of the reference; not needed here
  const Z* du = D(reinterpret_cast<const Z*>(u), "u");
  Z* dout = D(reinterpret_cast<Z*>(uprime), "uprime");
  double* qa = D(reinterpret_cast<double*>(tipdot), "tipdot");
  Z* st = local_staples ? D(reinterpret_cast<Z*>(local_staples), "local_staples") : nullptr;
  if (!du || !dout || !qa) return;
  launch_stout(du, dout, qa, st, rho_of(istopo), S());
}

void stout_wrapper(const su3_soa* tconf_acc, su3_soa* tstout_conf_acc_arr, const int istopo) {
  if (!require_init("stout_wrapper")) return;
  const int steps = (istopo & act_params.topo_action) ? act_params.topo_stout_steps : act_params.stout_steps;
  const Z* u = D(reinterpret_cast<const Z*>(tconf_acc), "tconf_acc");
  Z* out = D(reinterpret_cast<Z*>(tstout_conf_acc_arr), "tstout_conf_acc_arr");
  double* qa = static_cast<double*>(workspace(WS_FORCE0, alg_bytes()));
  if (!u || !out || !qa) return;
  const long lvl = 8L * 9 * sh();
  for (int k = 0; k < steps; ++k) launch_stout(k == 0 ? u : out + (k - 1) * lvl, out + k * lvl, qa, nullptr,
                                               rho_of(istopo), S());
}

void exp_minus_QA_times_conf(const su3_soa* tu, const tamat_soa* QA, su3_soa* tu_out, su3_soa* exp_aux) {
  if (!require_init("exp_minus_QA_times_conf")) return;
  (void)exp_aux;
  const Z* u = D(reinterpret_cast<const Z*>(tu), "tu");
  const double* qa = D(reinterpret_cast<const double*>(QA), "QA");
  Z* out = D(reinterpret_cast<Z*>(tu_out), "tu_out");
  if (u && qa && out) launch_exp_times_conf(u, qa, out, S());
}

void compute_lambda(thmat_soa* L, const su3_soa* SP, const su3_soa* U, const tamat_soa* QA, su3_soa* TMP) {
  if (!require_init("compute_lambda")) return;
  (void)TMP;
  double* l = D(reinterpret_cast<double*>(L), "L");
  const Z* sp = D(reinterpret_cast<const Z*>(SP), "SP");
  const Z* u = D(reinterpret_cast<const Z*>(U), "U");
  const double* qa = D(reinterpret_cast<const double*>(QA), "QA");
  if (l && sp && u && qa) launch_lambda(l, sp, u, qa, S());
}

void compute_sigma(const thmat_soa* L, const su3_soa* U, su3_soa* Sg, const tamat_soa* QA, su3_soa* TMP,
                   const int istopo) {
  if (!require_init("compute_sigma")) return;
  (void)TMP;
  const double* l = D(reinterpret_cast<const double*>(L), "L");
  const Z* u = D(reinterpret_cast<const Z*>(U), "U");
  Z* s = D(reinterpret_cast<Z*>(Sg), "S");
  const double* qa = D(reinterpret_cast<const double*>(QA), "QA");
  if (l && u && s && qa) launch_sigma(l, u, s, qa, rho_of(istopo), S());
}

void compute_sigma_from_sigma_prime_backinto_sigma_prime(su3_soa* Sigma, thmat_soa* Lambda, tamat_soa* QA,
                                                         const su3_soa* U, su3_soa* TMP, const int istopo) {
  if (!require_init("compute_sigma_from_sigma_prime_backinto_sigma_prime")) return;
  Z* s = D(reinterpret_cast<Z*>(Sigma), "Sigma");
  double* l = D(reinterpret_cast<double*>(Lambda), "Lambda");
  double* qa = D(reinterpret_cast<double*>(QA), "QA");
  const Z* u = D(reinterpret_cast<const Z*>(U), "U");
  Z* tmp = D(reinterpret_cast<Z*>(TMP), "TMP");
  if (!s || !l || !qa || !u || !tmp) return;
  const double rho = rho_of(istopo);
  // TMP receives the staples and QA = rho/C0 TA(U C), as in the reference;
  // the link output of the stout kernel goes to the workspace.
  Z* scratch = static_cast<Z*>(workspace(WS_FORCE1, su3_bytes()));
  if (!scratch) return;
  launch_stout(u, scratch, qa, tmp, rho, S());
  launch_lambda(l, s, u, qa, S());
  launch_sigma(l, u, s, qa, rho, S());
}

void direct_product_of_fermions_into_auxmat(const vec3_soa* loc_s, const vec3_soa* loc_h, su3_soa* aux_u,
                                            const RationalApprox* approx, int iter) {
  if (!require_init("direct_product_of_fermions_into_auxmat")) return;
  const Z* x = D(reinterpret_cast<const Z*>(loc_s), "loc_s");
  const Z* y = D(reinterpret_cast<const Z*>(loc_h), "loc_h");
  Z* aux = D(reinterpret_cast<Z*>(aux_u), "aux_u");
  double* coef = static_cast<double*>(workspace(WS_FORCE3, 128 * sizeof(double)));
  if (!x || !y || !aux || !coef) return;
  OST_CUDA(cudaMemcpyAsync(coef, &approx->RA_a[iter], sizeof(double), cudaMemcpyHostToDevice, S()));
  launch_force_outer(x, y, vlen(), 1, coef, nullptr, aux, 0, S());
}

void ker_openacc_compute_fermion_force(const su3_soa* u, su3_soa* aux_u, const vec3_soa* in_shiftmulti,
                                       vec3_soa* loc_s, vec3_soa* loc_h, ferm_param* tpars) {
  if (!require_init("ker_openacc_compute_fermion_force")) return;
  const int order = tpars->approx_md.approx_order;
  const Z* du = D(reinterpret_cast<const Z*>(u), "u");
  Z* aux = D(reinterpret_cast<Z*>(aux_u), "aux_u");
  const Z* xs = D(reinterpret_cast<const Z*>(in_shiftmulti), "in_shiftmulti");
  const void* ph = resolve(tpars->phases, "phases");
  Z* ys = static_cast<Z*>(workspace(WS_MULTI2, size_t(order > 0 ? order : 1) * vlen() * sizeof(Z)));
  double* coef = static_cast<double*>(workspace(WS_FORCE3, 128 * sizeof(double)));
  if (!du || !aux || !xs || !ph || !ys || !coef || order < 1 || order > MAX_APPROX_ORDER) {
    if (order < 1 || order > MAX_APPROX_ORDER) set_error(-11, "approx_md order %d out of range", order);
    return;
  }
  // Y_k = D_oe X_k for every shift, then all outer products in one pass
  for (int k = 0; k < order; ++k) {
    DslashArgs<double> a;
    a.parity = 1; a.phase_mode = PH_ANGLE; a.epilogue = EPI_PLAIN; a.u = du; a.out = ys + k * vlen();
    a.in = xs + k * vlen(); a.phases = ph; a.in0 = nullptr; a.mass2 = 0; a.stream = S(); a.compact_links = 0;
    launch_dslash<double>(a);
  }
  OST_CUDA(cudaMemcpyAsync(coef, tpars->approx_md.RA_a, order * sizeof(double), cudaMemcpyHostToDevice, S()));
  launch_force_outer(xs, ys, vlen(), order, coef, nullptr, aux, 0, S());
  // leave the last shift's X and D_oe X in the parking vectors, as the reference does
  Z* s = loc_s ? D(reinterpret_cast<Z*>(loc_s), "loc_s") : nullptr;
  Z* h = loc_h ? D(reinterpret_cast<Z*>(loc_h), "loc_h") : nullptr;
  if (s) blas_copy<double>(xs + (order - 1) * vlen(), s, vlen(), S());
  if (h) blas_copy<double>(ys + (order - 1) * vlen(), h, vlen(), S());
}

void multiply_backfield_times_force(ferm_param* tpars, const su3_soa* auxmat, su3_soa* pseudo_ipdot) {
  if (!require_init("multiply_backfield_times_force")) return;
  const double* ph = static_cast<const double*>(resolve(tpars->phases, "phases"));
  const Z* aux = D(reinterpret_cast<const Z*>(auxmat), "auxmat");
  Z* pip = D(reinterpret_cast<Z*>(pseudo_ipdot), "pseudo_ipdot");
  if (ph && aux && pip) launch_backfield(ph, aux, pip, S());
}

void multiply_conf_times_force_and_take_ta_nophase(const su3_soa* u, const su3_soa* auxmat, tamat_soa* ipdot) {
  if (!require_init("multiply_conf_times_force_and_take_ta_nophase")) return;
  const Z* du = D(reinterpret_cast<const Z*>(u), "u");
  const Z* aux = D(reinterpret_cast<const Z*>(auxmat), "auxmat");
  double* ip = D(reinterpret_cast<double*>(ipdot), "ipdot");
  if (du && aux && ip) launch_conf_force_ta(du, aux, ip, S());
}

// Multi-shift solve dispatch (inverter_wrappers.c:41-114).
//
// Default: the FP64 multishift_invert to res.  With
// inverter_tricks.singlePInvAccelMultiInv, as in the reference, a
// single-precision CG-M runs first to max(8e-7 sqrt(sizeh), res) (:57-60) and
// every shift is then refined to res in FP64: with useMixedPrecision all
// shifts together by the batched mixed solver (each to an FP64 true residual
// <= res), otherwise one after the other by ker_invert_openacc from the
// single-precision guess (inverter_wrapper, :82-96).  The single-precision
// phase is the library's FP32 CG-M on its own FP32 copy of ip.u (ip.u_f is
// not read).  Returns the total iteration count: the CG-M iterations plus
// those of every refinement (the reference adds the CG-M count once per
// shift instead, :97; no caller reads it).
int inverter_multishift_wrapper(inverter_package ip, ferm_param* pars, RationalApprox* approx, vec3_soa* out,
                                const vec3_soa* in, double res, int max_cg, int convergence_importance) {
  int cg = 0;
  if (!inverter_tricks.singlePInvAccelMultiInv) {
    const int st = multishift_invert(ip.u, pars, approx, out, in, res, ip.loc_r, ip.loc_h, ip.loc_s, ip.loc_p,
                                     ip.ferm_shift_temp, max_cg, &cg);
    convergence_messages(convergence_importance, st);
    return cg;
  }
  if (!require_init("inverter_multishift_wrapper")) return 0;
  const int order = approx->approx_order;
  const Z* u = D(reinterpret_cast<const Z*>(ip.u), "ip.u");
  const double* ph = static_cast<const double*>(resolve(pars->phases, "phases"));
  const Z* b = D(reinterpret_cast<const Z*>(in), "in");
  Z* xs = D(reinterpret_cast<Z*>(out), "out");
  if (!u || !ph || !b || !xs) {
    convergence_messages(convergence_importance, INVERTER_FAILURE);
    return 0;
  }
  double res_sp = double(8e-7f * sqrtf(float(sh())));
  if (res_sp < res) res_sp = res;
  int it_cgm = 0, total = 0;
  if (inverter_tricks.useMixedPrecision) {
    int it_ref[MAX_APPROX_ORDER] = {0};
    const int st = multishift_two_phase(u, ph, pars->ferm_mass, approx->RA_b, order, 1, b, xs, res_sp, res, max_cg,
                                        0.0, 1, &it_cgm, it_ref, nullptr);
    total = it_cgm;
    for (int k = 0; k < order; ++k) total += it_ref[k];
    convergence_messages(convergence_importance, st);
    return total;
  }
  const int st = multishift_two_phase(u, ph, pars->ferm_mass, approx->RA_b, order, 1, b, xs, res_sp, res, max_cg,
                                      0.0, 0, &it_cgm, nullptr, nullptr);
  convergence_messages(convergence_importance, st);
  total = it_cgm;
  for (int k = 0; k < order; ++k) {
    vec3_soa* xk = reinterpret_cast<vec3_soa*>(reinterpret_cast<Z*>(out) + k * vlen());
    total += inverter_wrapper(ip, pars, xk, in, res, max_cg, approx->RA_b[k], convergence_importance);
  }
  return total;
}

// The fermion force of all flavours through the stout levels
// (fermion_force.c:166-320): stout, multi-shift solves with approx_md,
// outer products with phases, Sigma' -> Sigma per level, and
// ipdot = -TA(U Sigma).
void fermion_force_soloopenacc(su3_soa* tconf_acc, su3_soa* tstout_conf_acc_arr, su3_soa* gl3_aux,
                               tamat_soa* tipdot_acc, ferm_param* tfermion_parameters, int tNDiffFlavs,
                               const vec3_soa* ferm_in_acc, double res, su3_soa* taux_conf_acc,
                               vec3_soa* tferm_shiftmulti_acc, inverter_package ipt, const int max_cg) {
  if (!require_init("fermion_force_soloopenacc")) return;
  const int steps = act_params.stout_steps;
  const long lvl = 8L * 9 * sh();
  stout_wrapper(tconf_acc, tstout_conf_acc_arr, 0);
  const su3_soa* conf_to_use =
      steps > 0 ? reinterpret_cast<su3_soa*>(reinterpret_cast<Z*>(tstout_conf_acc_arr) + (steps - 1) * lvl) : tconf_acc;
  set_su3_soa_to_zero(gl3_aux);
  set_tamat_soa_to_zero(tipdot_acc);
  ipt.u = conf_to_use;
  for (int f = 0; f < tNDiffFlavs; ++f) {
    ferm_param* fp = &tfermion_parameters[f];
    set_su3_soa_to_zero(taux_conf_acc);
    const Z* first_src = reinterpret_cast<const Z*>(ferm_in_acc) + long(fp->index_of_the_first_ps) * vlen();
    if (inverter_tricks.singlePInvAccelMultiInv && fp->number_of_ps > 1 && !inverter_tricks.useMixedPrecision) {
      // accelerated mode with FP64 refinement: the pseudofermions share one
      // FP32 CG-M launch sequence per group of 4, each shift then refined
      // by ker_invert_openacc, and all outer products of a group in one pass
      force_pseudofermion_groups(ipt, fp, first_src, taux_conf_acc, tferm_shiftmulti_acc, res, max_cg, 0);
    } else if (inverter_tricks.singlePInvAccelMultiInv && fp->number_of_ps > 1) {
      // accelerated mode with mixed refinement: FP32 CG-M and refinement of
      // every (pseudofermion, shift) system batched
      force_pseudofermion_groups(ipt, fp, first_src, taux_conf_acc, tferm_shiftmulti_acc, res, max_cg, 1);
    } else {
      for (int ps = 0; ps < fp->number_of_ps; ++ps) {
        const vec3_soa* src = reinterpret_cast<const vec3_soa*>(first_src + long(ps) * vlen());
        inverter_multishift_wrapper(ipt, fp, &fp->approx_md, tferm_shiftmulti_acc, src, res, max_cg,
                                    CONVERGENCE_NONCRITICAL);
        ker_openacc_compute_fermion_force(ipt.u, taux_conf_acc, tferm_shiftmulti_acc, ipt.loc_s, ipt.loc_h, fp);
      }
    }
    multiply_backfield_times_force(fp, taux_conf_acc, gl3_aux);
  }
  double* lam = static_cast<double*>(workspace(WS_FORCE0, alg_bytes()));
  double* qa = static_cast<double*>(workspace(WS_FORCE2, alg_bytes()));
  if (!lam || !qa) return;
  thmat_soa* L = reinterpret_cast<thmat_soa*>(lam);
  tamat_soa* Q = reinterpret_cast<tamat_soa*>(qa);
  for (int level = steps; level > 1; --level) {
    const su3_soa* c = reinterpret_cast<su3_soa*>(reinterpret_cast<Z*>(tstout_conf_acc_arr) + (level - 2) * lvl);
    compute_sigma_from_sigma_prime_backinto_sigma_prime(gl3_aux, L, Q, c, taux_conf_acc, 0);
  }
  if (steps > 0) compute_sigma_from_sigma_prime_backinto_sigma_prime(gl3_aux, L, Q, tconf_acc, taux_conf_acc, 0);
  multiply_conf_times_force_and_take_ta_nophase(tconf_acc, gl3_aux, tipdot_acc);
}

}  // extern "C"
