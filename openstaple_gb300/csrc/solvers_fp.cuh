// solvers_fp.cuh -- the reference's CG (inverter_full.c:19-132) and CG-M
// (inverter_multishift_full.c:23-252) on the library's Dirac operator and
// BLAS, templated on the vector precision: T = double behind
// ker_invert_openacc / multishift_invert, T = float behind their FP32 twins
// ker_invert_openacc_f / multishift_invert_f (the reference's generated
// sp_inverter_full.c / sp_inverter_multishift_full.c, which keep FP32 links
// and vectors and double scalars).  Scalars and global reductions are FP64
// in both.  Stopping rules, restarts and success criteria follow the
// reference, which fixes the iteration counts and status codes callers see.
#pragma once
#include <cmath>
#include <cstdio>
#include "dslash.cuh"
#include "kernels.cuh"
#include "runtime.cuh"
#include "solver_kernels.cuh"
#include "../../include/ostaple_gb300.h"

extern "C" int verbosity_lv;

namespace ost {
namespace fp {

template <typename T> using Cx = typename cplx_t<T>::type;

inline cudaStream_t S() { return rt().stream; }
inline long vlen() { return 3L * rt().g.sizeh; }   // complex numbers in a vec3_soa

// one-double device scalar slots read back by the host-driven solvers
inline double* dscal(int k) {
  double* p = static_cast<double*>(workspace(WS_SCALARS, 64 * sizeof(double)));
  return p ? p + k : nullptr;
}
inline double readback(const double* d) {
  double h = 0;
  OST_CUDA(cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, S()));
  OST_CUDA(cudaStreamSynchronize(S()));
  return h;
}

// one hop application on the reference layouts (9 complex arrays per link
// direction, angle phases of type T): out = 0.5 hop(in) or out = m2 in0 - 0.5 hop(in)
template <typename T>
void dslash(int parity, const Cx<T>* u, Cx<T>* out, const Cx<T>* in, const void* ph, int epi, const Cx<T>* in0,
            double m2) {
  DslashArgs<T> a;
  a.parity = parity;
  a.phase_mode = PH_ANGLE;
  a.epilogue = epi;
  a.u = u;
  a.out = out;
  a.in = in;
  a.phases = ph;
  a.in0 = in0;
  a.mass2 = T(m2);
  a.stream = S();
  launch_dslash<T>(a);
}

// tmp = D_oe in ; out = m2 in - D_eo tmp   (fermion_matrix.c:736-746)
template <typename T>
void mdagm(const Cx<T>* u, Cx<T>* out, const Cx<T>* in, Cx<T>* tmp, const void* ph, double m2) {
  dslash<T>(1, u, tmp, in, ph, EPI_PLAIN, nullptr, 0.0);
  dslash<T>(0, u, out, tmp, ph, EPI_MDAGM, in, m2);
}

// CG on (M^+M + shift) x = b, restarted every `restart` iterations
// (inverter_full.c:19-132).  Returns INVERTER_SUCCESS when the final true
// residual sqrt(|b - A x|^2 / |b|^2) is <= res.
template <typename T>
int cg(const Cx<T>* u, const void* ph, double mass, Cx<T>* x, const Cx<T>* b, double res, Cx<T>* r, Cx<T>* h,
       Cx<T>* s, Cx<T>* p, int max_cg, double shift, int restart, int* cg_return) {
  const long n = vlen();
  const double m2 = mass * mass + shift;
  const double SAFETY = 0.95;
  if (restart <= 0) restart = 10000;
  blas_norm2<T>(b, n, dscal(0), S());
  const double source_norm = readback(dscal(0));
  int iters = 0;
  double delta, alpha, lambda = 0, omega, gammag;
  do {
    mdagm<T>(u, s, x, h, ph, m2);
    blas_axmy<T>(b, 1.0, s, r, n, S());      // r = b - s
    blas_copy<T>(r, p, n, S());
    blas_norm2<T>(r, n, dscal(0), S());
    delta = readback(dscal(0));
    int restarted = 0;
    do {
      iters++;
      restarted++;
      mdagm<T>(u, s, p, h, ph, m2);
      blas_rdot<T>(p, s, n, dscal(1), S());
      alpha = readback(dscal(1));
      omega = delta / alpha;
      blas_axpy<T>(p, omega, x, x, n, S());                     // x += omega p
      fused_axpy_norm<T>(r, s, -omega, n, dscal(2), S());       // r -= omega s ; lambda
      lambda = readback(dscal(2));
      gammag = lambda / delta;
      delta = lambda;
      blas_axpy<T>(p, gammag, r, p, n, S());                    // p = r + gammag p
      if (error_code()) return INVERTER_FAILURE;
    } while (std::sqrt(lambda / source_norm) > res * SAFETY && restarted < restart);
  } while (std::sqrt(lambda / source_norm) > res && iters < max_cg);

  mdagm<T>(u, s, x, h, ph, m2);
  blas_axmy<T>(b, 1.0, s, h, n, S());
  blas_norm2<T>(h, n, dscal(3), S());
  const double current_res = readback(dscal(3)) / source_norm;
  if (verbosity_lv > 1)
    printf("Terminated invert after   %d    iterations[res/stop_res=  %e , stop_res=%e ]\n", iters,
           std::sqrt(current_res) / res, res);
  if (iters == max_cg) printf("WARNING: maximum number of iterations reached in invert\n");
  *cg_return = iters;
  if (error_code()) return INVERTER_FAILURE;
  return std::sqrt(current_res) <= res ? INVERTER_SUCCESS : INVERTER_FAILURE;
}

// CG-M for (M^+M + shift_k) x_k = b, k < order (inverter_multishift_full.c:
// 23-252): zeta/omega/gamma recurrences on the host, all shifted updates in
// one fused pass per iteration, shift k frozen when
// sqrt(delta zeta_k^2 / |b|^2) < residuo * 0.95; success when every final
// relative residual is <= 1 (the reference's check, :211-229).
template <typename T>
int cgm(const Cx<T>* u, const void* ph, double mass, const double* shifts, int order, Cx<T>* xs, const Cx<T>* b,
        double residuo, Cx<T>* r, Cx<T>* h, Cx<T>* s, Cx<T>* p, Cx<T>* ps, int max_cg, int* cg_return) {
  const long n = vlen();
  const double m2 = mass * mass;
  const double SAFETY = 0.95;
  double zeta_i[OST_MAX_SHIFTS], zeta_ii[OST_MAX_SHIFTS], zeta_iii[OST_MAX_SHIFTS];
  double omegas[OST_MAX_SHIFTS], gammas[OST_MAX_SHIFTS];
  int flag[OST_MAX_SHIFTS];
  for (int k = 0; k < order; ++k) {
    flag[k] = 1;
    blas_zero<T>(xs + k * n, n, S());
  }
  blas_copy<T>(b, r, n, S());
  blas_copy<T>(r, p, n, S());
  blas_norm2<T>(r, n, dscal(0), S());
  double delta = readback(dscal(0));
  blas_norm2<T>(b, n, dscal(1), S());
  const double source_norm = readback(dscal(1));
  double omega = 1.0, omega_save, alpha, lambda, gammag = 0.0;
  for (int k = 0; k < order; ++k) {
    blas_copy<T>(b, ps + k * n, n, S());
    zeta_i[k] = 1.0;
    zeta_ii[k] = 1.0;
    gammas[k] = 0.0;
  }
  int iters = 0;
  int maxiter = order;
  do {
    iters++;
    mdagm<T>(u, s, p, h, ph, m2);
    blas_rdot<T>(p, s, n, dscal(2), S());
    alpha = readback(dscal(2));
    omega_save = omega;
    omega = -delta / alpha;
    for (int k = 0; k < maxiter; ++k) {
      if (flag[k] == 1) {
        zeta_iii[k] = (zeta_i[k] * zeta_ii[k] * omega_save) /
                      (omega * gammag * (zeta_i[k] - zeta_ii[k]) +
                       zeta_i[k] * omega_save * (1.0 - shifts[k] * omega));
        omegas[k] = omega * zeta_iii[k] / zeta_ii[k];
      }
    }
    fused_axpy_norm<T>(r, s, omega, n, dscal(3), S());   // r += omega s ; lambda
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
    fused_cgm_update<T>(p, r, gammag, xs, ps, n, cf, n, S());
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
  } while (maxiter > 0 && iters < max_cg);
  if (iters == max_cg) printf("WARNING: maximum number of iterations reached in invert\n");

  int check = 1;
  for (int k = 0; k < order; ++k) {
    mdagm<T>(u, s, xs + k * n, h, ph, m2 + shifts[k]);
    blas_axmy<T>(b, 1.0, s, h, n, S());
    blas_norm2<T>(h, n, dscal(4), S());
    double rr = readback(dscal(4)) / source_norm;
    check *= (rr <= 1) ? 1 : 0;
  }
  *cg_return = iters;
  if (error_code()) return INVERTER_FAILURE;
  return check ? INVERTER_SUCCESS : INVERTER_FAILURE;
}

}  // namespace fp
}  // namespace ost
