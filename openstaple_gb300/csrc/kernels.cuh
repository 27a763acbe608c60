// kernels.cuh -- launch interfaces shared between the kernel translation
// units and the C ABI layer.
#pragma once
#include <cuda_runtime.h>
#include "common.cuh"

namespace ost {

enum Epilogue { EPI_PLAIN = 0, EPI_MDAGM = 1 };

template <typename T>
struct DslashArgs {
  typedef typename cplx_t<T>::type C;
  int parity;                 // parity of the OUTPUT sites: 0 -> D_eo, 1 -> D_oe
  int phase_mode;             // PhaseMode
  int epilogue;               // Epilogue
  const C* u;                 // 8 su3_soa
  C* out;
  const C* in;
  const void* phases;         // angle soa[8] or sign bytes [8][sizeh]
  const C* in0;               // EPI_MDAGM: the vector multiplied by mass2
  T mass2;
  cudaStream_t stream;
  int compact_links = 0;      // 1: 6 complex arrays per direction (two rows only)
};

template <typename T> void launch_dslash(const DslashArgs<T>& a);

// ---- BLAS over vec3 fields (n = 3*sizeh complex numbers) ----
// Reductions are deterministic: fixed block partials summed in a fixed order
// by the last block to finish.  Results land in device memory at `dst`.
template <typename T> void blas_norm2(const typename cplx_t<T>::type* a, long n, double* dst, cudaStream_t st);
template <typename T> void blas_rdot(const typename cplx_t<T>::type* a, const typename cplx_t<T>::type* b, long n,
                                     double* dst, cudaStream_t st);
template <typename T> void blas_cdot(const typename cplx_t<T>::type* a, const typename cplx_t<T>::type* b, long n,
                                     double* dst /*[2]*/, cudaStream_t st);
// out = a*x + y
template <typename T> void blas_axpy(const typename cplx_t<T>::type* x, double a, const typename cplx_t<T>::type* y,
                                     typename cplx_t<T>::type* out, long n, cudaStream_t st);
// out = a*x - y
template <typename T> void blas_axmy(const typename cplx_t<T>::type* x, double a, const typename cplx_t<T>::type* y,
                                     typename cplx_t<T>::type* out, long n, cudaStream_t st);
// out = a*(x - y)
template <typename T> void blas_scaled_diff(const typename cplx_t<T>::type* x, const typename cplx_t<T>::type* y,
                                            double a, typename cplx_t<T>::type* out, long n, cudaStream_t st);
// out = a*x - y - z
template <typename T> void blas_axmymz(const typename cplx_t<T>::type* x, double a, const typename cplx_t<T>::type* y,
                                       const typename cplx_t<T>::type* z, typename cplx_t<T>::type* out, long n,
                                       cudaStream_t st);
// x *= a
template <typename T> void blas_scale(typename cplx_t<T>::type* x, double a, long n, cudaStream_t st);
// out += w*p ; r -= w*s
template <typename T> void blas_inside_loop(typename cplx_t<T>::type* out, typename cplx_t<T>::type* r,
                                            const typename cplx_t<T>::type* s, const typename cplx_t<T>::type* p,
                                            double w, long n, cudaStream_t st);
template <typename T> void blas_copy(const typename cplx_t<T>::type* x, typename cplx_t<T>::type* y, long n,
                                     cudaStream_t st);
template <typename T> void blas_zero(typename cplx_t<T>::type* x, long n, cudaStream_t st);

// float <-> double conversions of complex arrays
void conv_d2f(const double2* d, float2* f, long n, cudaStream_t st);
void conv_f2d(const float2* f, double2* d, long n, cudaStream_t st);
// d += (double) f
void acc_f2d(const float2* f, double2* d, long n, cudaStream_t st);

}  // namespace ost
