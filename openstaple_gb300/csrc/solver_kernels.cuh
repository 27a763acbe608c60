// solver_kernels.cuh -- fused CG / CG-M vector kernels.
#pragma once
#include "common.cuh"

namespace ost {

static constexpr int OST_MAX_SHIFTS = 25;   // MAX_APPROX_ORDER (rationalapprox.h:8)

struct CgmCoeffs {
  int nshift;
  int active[OST_MAX_SHIFTS];
  double omega[OST_MAX_SHIFTS];
  double gamma[OST_MAX_SHIFTS];
  double zeta[OST_MAX_SHIFTS];
};

struct RecombCoeffs {
  int order;
  double a0;
  double a[OST_MAX_SHIFTS];
};

template <typename T>
void fused_axpy_norm(typename cplx_t<T>::type* r, const typename cplx_t<T>::type* s, double w, long n,
                     double* dst, cudaStream_t st);
template <typename T>
void fused_cgm_update(typename cplx_t<T>::type* p, const typename cplx_t<T>::type* r, double g,
                      typename cplx_t<T>::type* x, typename cplx_t<T>::type* ps, long stride,
                      const CgmCoeffs& cf, long n, cudaStream_t st);
// x_k -= omega_k ps_k  /  ps_k = gamma_k ps_k + zeta_k r, over the active shifts
template <typename T>
void multi_xupdate(typename cplx_t<T>::type* x, const typename cplx_t<T>::type* ps, long stride, const CgmCoeffs& cf,
                   long n, cudaStream_t st);
template <typename T>
void multi_pupdate(typename cplx_t<T>::type* ps, const typename cplx_t<T>::type* r, long stride, const CgmCoeffs& cf,
                   long n, cudaStream_t st);
template <typename T>
void recombine(const typename cplx_t<T>::type* xs, long stride, const typename cplx_t<T>::type* in,
               typename cplx_t<T>::type* out, const RecombCoeffs& rc, long n, cudaStream_t st);

}  // namespace ost
