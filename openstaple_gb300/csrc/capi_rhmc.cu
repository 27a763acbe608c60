// capi_rhmc.cu -- the RHMC trajectory on top of the hot path: the
// molecular dynamics with fermions of the reference (multistep_2MN_SOLOOPENACC,
// md_integrator.c:502-742) and ostaple_rhmc_trajectory, one whole update of
// the reference's UPDATE_SOLOACC_UNOSTEP_VERSATILE (update_versatile.c:44-665)
// with explicit arguments: momenta and pseudofermion heatbath, eigenvalue
// bounds and rescaled rational approximations, chi = r_fi(M^+M) phi, the
// molecular dynamics, the last inversion with r_li and the Metropolis test.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#include "hmc.cuh"
#include "runtime.cuh"
#include "../../include/ostaple_gb300.h"

using namespace ost;

namespace {

typedef double2 Z;
inline cudaStream_t S() { return rt().stream; }
inline long sh() { return rt().g.sizeh; }
inline long vlen() { return 3L * sh(); }

double* dsc(int k) {
  double* p = static_cast<double*>(workspace(WS_SCALARS, 64 * sizeof(double)));
  return p ? p + 40 + k : nullptr;   // slots 40.. (the link generator uses 16-29)
}

// host copy of the counter-based generator (hmc.cu)
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

}  // namespace

extern "C" {

// md_integrator.c:502-742: with the fermion force F and the gauge multistep G,
//   F(d0) [G F(d1) G F(d2)]^(no_md - 1) G F(d1) G F(d0)
// (the steps d in deltas_Omelyan, md_parameters.no_md steps).  The gauge
// multisteps park the staples in taux_conf_acc and the force in tipdot_acc;
// the fermion force uses tauxbis_conf_acc and taux_conf_acc as parking, as in
// the reference.  local_sums is not used.
void multistep_2MN_SOLOOPENACC(tamat_soa* tipdot_acc, su3_soa* tconf_acc, su3_soa* tstout_conf_acc_arr,
                               su3_soa* tauxbis_conf_acc, su3_soa* taux_conf_acc, ferm_param* tfermions_parameters,
                               int tNDiffFlavs, vec3_soa* ferm_in_acc, vec3_soa* tferm_shiftmulti_acc,
                               inverter_package ip, thmat_soa* tmomenta, dcomplex_soa* local_sums, double res,
                               const int max_cg) {
  (void)local_sums;
  if (!require_init("multistep_2MN_SOLOOPENACC")) return;
  auto F = [&](int k) {
    fermion_force_soloopenacc(tconf_acc, tstout_conf_acc_arr, tauxbis_conf_acc, tipdot_acc, tfermions_parameters,
                              tNDiffFlavs, ferm_in_acc, res, taux_conf_acc, tferm_shiftmulti_acc, ip, max_cg);
    mom_sum_mult(tmomenta, tipdot_acc, deltas_Omelyan, k);
  };
  auto G = [&]() { multistep_2MN_gauge(tconf_acc, taux_conf_acc, tipdot_acc, tmomenta); };
  F(0);
  for (int md = 1; md < md_parameters.no_md; ++md) {
    G(); F(1);
    G(); F(2);
  }
  G(); F(1);
  G(); F(0);
}

// One RHMC update (update_versatile.c:44-665) of the links u with
// nflavs flavours fpars[f] (mass, phases, number_of_ps,
// index_of_the_first_ps, and the mother approximations approx_fi_mother,
// approx_md_mother, approx_li_mother on [lambda_min, 1], as read from
// .REMEZ files) and the gauge action of beta (act_params.stout_steps stout
// levels of gl_stout_rho for the fermions).  The integrator is the
// reference's 2MN with no_md steps of gauge_scale gauge substeps
// (md_parameters and deltas_Omelyan are set from the arguments); the
// solvers follow inverter_tricks exactly as in the reference.  Random
// numbers: the counter-based generator of (seed, trajectory traj).  With
// metropolis != 0 the update is accepted with probability min(1, exp(-dS))
// and rejected updates restore u.  action[6] (may be NULL) receives the
// gauge, momentum and fermion actions before and after.
int ostaple_rhmc_trajectory(su3_soa* u, ferm_param* fpars, int nflavs, double beta, int no_md, int gauge_scale,
                            double traj_len, double res_metro, double res_md, int max_cg, unsigned long long seed,
                            int traj, int metropolis, int* accepted, double* delta_s, double* action) {
  if (!require_init("ostaple_rhmc_trajectory")) return -2;
  if (nflavs < 0 || no_md < 1 || gauge_scale < 1) {
    set_error(-11, "ostaple_rhmc_trajectory: nflavs %d, no_md %d, gauge_scale %d", nflavs, no_md, gauge_scale);
    return -11;
  }
  cudaStream_t st = S();
  const long n = sh(), nv = vlen();
  int nps_tot = 0, max_order = 1;
  for (int f = 0; f < nflavs; ++f) {
    nps_tot = std::max(nps_tot, fpars[f].index_of_the_first_ps + fpars[f].number_of_ps);
    max_order = std::max({max_order, fpars[f].approx_fi_mother.approx_order, fpars[f].approx_md_mother.approx_order,
                          fpars[f].approx_li_mother.approx_order});
  }
  if (max_order > MAX_APPROX_ORDER) {
    set_error(-11, "ostaple_rhmc_trajectory: approximation order %d above %d", max_order, MAX_APPROX_ORDER);
    return -11;
  }
  Z* U = static_cast<Z*>(resolve(u, "u"));
  if (!U) return -3;
  const int steps = act_params.stout_steps > 0 ? act_params.stout_steps : 0;
  // one device buffer for the trajectory's fields
  const size_t su3 = 72 * size_t(n), alg = 64 * size_t(n);
  const size_t nz = su3 * (size_t(std::max(steps, 1)) + 3) + size_t(nv) * (2 * size_t(nps_tot) + 2 * max_order + 6);
  const size_t nd = 2 * alg;
  char* base = static_cast<char*>(workspace(WS_RHMC, nz * sizeof(Z) + nd * sizeof(double)));
  if (!base) return -5;
  Z* z = reinterpret_cast<Z*>(base);
  Z* levels = z;            z += su3 * std::max(steps, 1);
  Z* bkp = z;               z += su3;
  Z* auxbis = z;            z += su3;
  Z* aux = z;               z += su3;
  Z* phi = z;               z += nv * nps_tot;
  Z* chi = z;               z += nv * nps_tot;
  Z* shiftmulti = z;        z += nv * max_order;
  Z* shifttemp = z;         z += nv * max_order;
  Z* r = z; z += nv; Z* h = z; z += nv; Z* s = z; z += nv; Z* p = z; z += nv;
  Z* kp = z; z += nv; Z* ks = z; z += nv;
  double* mom = reinterpret_cast<double*>(z);
  double* ipdot = mom + alg;
  double* d = dsc(0);
  if (!d) return -5;

  md_parameters.no_md = no_md;
  md_parameters.gauge_scale = gauge_scale;
  md_parameters.t = traj_len;
  act_params.beta = beta;
  initialize_md_global_variables(md_parameters);

  su3_soa* U_ = reinterpret_cast<su3_soa*>(U);
  su3_soa* lev = reinterpret_cast<su3_soa*>(levels);
  const su3_soa* conf_f = steps > 0 ? reinterpret_cast<su3_soa*>(levels + su3 * (steps - 1)) : U_;
  auto vec = [](Z* q, long k) { return reinterpret_cast<vec3_soa*>(q + k); };
  inverter_package ip{};
  ip.u = conf_f;
  ip.ferm_shift_temp = vec(shifttemp, 0);
  ip.nshifts = max_order;
  ip.loc_r = vec(r, 0); ip.loc_h = vec(h, 0); ip.loc_s = vec(s, 0); ip.loc_p = vec(p, 0);
  const unsigned long long tr = (unsigned long long)traj;
  unsigned long long stream = tr * 4096ull;   // a block of generator streams per trajectory

  if (metropolis) OST_CUDA(cudaMemcpyAsync(bkp, U, su3 * sizeof(Z), cudaMemcpyDeviceToDevice, st));
  launch_gen_momenta<double>(mom, seed, stream++, st);
  for (int k = 0; k < nps_tot; ++k) launch_gen_vec3_gauss(phi + k * nv, seed, stream++, st);
  if (steps > 0 && nflavs > 0) stout_wrapper(U_, lev, 0);

  // eigenvalue bounds on the smeared links and the rescaled approximations
  // (update_versatile.c:164-196)
  std::vector<double> minmax(2 * std::max(nflavs, 1));
  auto bounds = [&]() {
    for (int f = 0; f < nflavs; ++f) {
      launch_gen_vec3_gauss(kp, seed, stream++, st);
      launch_gen_vec3_gauss(ks, seed, stream++, st);
      find_min_max_eigenvalue_soloopenacc(const_cast<su3_soa*>(conf_f), &fpars[f], vec(r, 0), vec(h, 0), vec(kp, 0),
                                          vec(ks, 0), &minmax[2 * f]);
    }
  };
  bounds();
  for (int f = 0; f < nflavs; ++f)
    rescale_rational_approximation(&fpars[f].approx_fi_mother, &fpars[f].approx_fi, &minmax[2 * f]);

  auto gauge_and_mom = [&](double* out) {
    double pl = 0, re = 0;
    ostaple_gauge_action(U_, beta, &pl, &re, nullptr);
    launch_momenta_action<double>(mom, 0, 8, d, st);
    double km;
    OST_CUDA(cudaMemcpyAsync(&km, d, sizeof(double), cudaMemcpyDeviceToHost, st));
    OST_CUDA(cudaStreamSynchronize(st));
    const double b3 = beta * 0.33333333333333333333333;
    out[0] = b3 * (5.0 * 0.33333333333333333333333 * pl - 0.25 * 0.33333333333333333333333 * re);   // action_in/fin
    out[1] = km;
  };
  double gm_in[2] = {0, 0}, gm_fin[2] = {0, 0}, f_in = 0, f_fin = 0;
  if (metropolis) {
    gauge_and_mom(gm_in);
    for (int k = 0; k < nps_tot; ++k) f_in += real_scal_prod_global(vec(phi, k * nv), vec(phi, k * nv));
  }
  // heatbath: chi = r_fi(M^+M) phi (update_versatile.c:255-275)
  for (int f = 0; f < nflavs; ++f)
    for (int ps = 0; ps < fpars[f].number_of_ps; ++ps) {
      const long k = fpars[f].index_of_the_first_ps + ps;
      inverter_multishift_wrapper(ip, &fpars[f], &fpars[f].approx_fi, vec(shiftmulti, 0), vec(phi, k * nv), res_metro,
                                  max_cg, CONVERGENCE_CRITICAL);
      recombine_shifted_vec3_to_vec3(vec(shiftmulti, 0), vec(phi, k * nv), vec(chi, k * nv), &fpars[f].approx_fi);
    }
  for (int f = 0; f < nflavs; ++f)
    rescale_rational_approximation(&fpars[f].approx_md_mother, &fpars[f].approx_md, &minmax[2 * f]);

  // molecular dynamics (update_versatile.c:347-359)
  inverter_package ipm = ip;
  multistep_2MN_SOLOOPENACC(reinterpret_cast<tamat_soa*>(ipdot), U_, lev, reinterpret_cast<su3_soa*>(auxbis),
                            reinterpret_cast<su3_soa*>(aux), fpars, nflavs, vec(chi, 0), vec(shiftmulti, 0), ipm,
                            reinterpret_cast<thmat_soa*>(mom), nullptr, res_md, max_cg);

  int ok = 1;
  double ds = 0;
  if (metropolis) {
    if (steps > 0 && nflavs > 0) stout_wrapper(U_, lev, 0);
    bounds();
    for (int f = 0; f < nflavs; ++f)
      rescale_rational_approximation(&fpars[f].approx_li_mother, &fpars[f].approx_li, &minmax[2 * f]);
    // last inversion: phi' = r_li(M^+M) chi (update_versatile.c:480-491)
    for (int f = 0; f < nflavs; ++f)
      for (int ps = 0; ps < fpars[f].number_of_ps; ++ps) {
        const long k = fpars[f].index_of_the_first_ps + ps;
        inverter_multishift_wrapper(ip, &fpars[f], &fpars[f].approx_li, vec(shiftmulti, 0), vec(chi, k * nv),
                                    res_metro, max_cg, CONVERGENCE_CRITICAL);
        recombine_shifted_vec3_to_vec3(vec(shiftmulti, 0), vec(chi, k * nv), vec(phi, k * nv), &fpars[f].approx_li);
        f_fin += real_scal_prod_global(vec(chi, k * nv), vec(phi, k * nv));
      }
    gauge_and_mom(gm_fin);
    // delta_S = -(-S_in + K_in + F_in) + (-S_fin + K_fin + F_fin)  (update_versatile.c:566-572)
    ds = -(-gm_in[0] + gm_in[1] + f_in) + (-gm_fin[0] + gm_fin[1] + f_fin);
    if (ds >= 0) ok = huniform(seed, 0x5A5A5A5A00000000ull + tr, 0) < std::exp(-ds);
    if (!ok) OST_CUDA(cudaMemcpyAsync(U, bkp, su3 * sizeof(Z), cudaMemcpyDeviceToDevice, st));
  }
  OST_CUDA(cudaStreamSynchronize(st));
  if (accepted) *accepted = ok;
  if (delta_s) *delta_s = ds;
  if (action) {
    const double v[6] = {-gm_in[0], gm_in[1], f_in, -gm_fin[0], gm_fin[1], f_fin};
    memcpy(action, v, sizeof(v));
  }
  return error_code();
}

}  // extern "C"
