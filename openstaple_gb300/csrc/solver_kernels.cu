// solver_kernels.cu -- fused vector kernels of the CG and CG-M iterations.
#include "kernels.cuh"
#include "reduce.cuh"
#include "solver_kernels.cuh"

namespace ost {

#define OST_GRID_LOOP(i, n) \
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < (n); i += long(gridDim.x) * blockDim.x)

// r += w*s ; dst = |r|^2
template <typename C, typename S>
__global__ void k_axpy_norm(C* r, const C* __restrict__ s, S w, long n, ReduceWs ws, double* dst) {
  double v[1] = {0.0};
  OST_GRID_LOOP(i, n) {
    C a = r[i], b = s[i];
    a = cmk<C>(fma(b.x, w, a.x), fma(b.y, w, a.y));
    r[i] = a;
    v[0] += double(a.x) * double(a.x) + double(a.y) * double(a.y);
  }
  double t[1];
  if (grid_reduce<1>(v, ws, t)) dst[0] = t[0];
}

template <typename T>
void fused_axpy_norm(typename cplx_t<T>::type* r, const typename cplx_t<T>::type* s, double w, long n,
                     double* dst, cudaStream_t st) {
  int g = reduce_grid(n);
  k_axpy_norm<<<g, RED_THREADS, 0, st>>>(r, s, T(w), n, reduce_ws(1, g), dst);
  OST_LAUNCH_CHECK();
}

// p = g*p + r ; for active shifts k:  x_k -= om_k * ps_k ; ps_k = ga_k * ps_k + ze_k * r
template <typename C, typename S>
__global__ void k_cgm_update(C* p, const C* __restrict__ r, S g, C* x, C* ps, long stride, CgmCoeffs cf,
                             long n) {
  OST_GRID_LOOP(i, n) {
    C rr = r[i];
    C pp = p[i];
    p[i] = cmk<C>(fma(pp.x, g, rr.x), fma(pp.y, g, rr.y));
    for (int k = 0; k < cf.nshift; ++k) {
      if (!cf.active[k]) continue;
      C* xk = x + k * stride;
      C* pk = ps + k * stride;
      C xv = xk[i], pv = pk[i];
      S om = S(cf.omega[k]), ga = S(cf.gamma[k]), ze = S(cf.zeta[k]);
      xk[i] = cmk<C>(fma(-om, pv.x, xv.x), fma(-om, pv.y, xv.y));
      pk[i] = cmk<C>(fma(ga, pv.x, ze * rr.x), fma(ga, pv.y, ze * rr.y));
    }
  }
}

template <typename T>
void fused_cgm_update(typename cplx_t<T>::type* p, const typename cplx_t<T>::type* r, double g,
                      typename cplx_t<T>::type* x, typename cplx_t<T>::type* ps, long stride,
                      const CgmCoeffs& cf, long n, cudaStream_t st) {
  long b = (n + 255) / 256;
  long cap = 8L * rt().num_sms;
  int grid = int(b < cap ? b : cap);
  k_cgm_update<<<grid, 256, 0, st>>>(p, r, T(g), x, ps, stride, cf, n);
  OST_LAUNCH_CHECK();
}

// x_k -= om_k * ps_k for every active shift k, all shifts in one pass
// (multiple_combine_in1_minus_in2x_factor_back_into_in1,
// fermionic_utilities.c:315-339)
template <typename C, typename S>
__global__ void k_multi_xupdate(C* x, const C* __restrict__ ps, long stride, CgmCoeffs cf, long n) {
  OST_GRID_LOOP(i, n) {
    for (int k = 0; k < cf.nshift; ++k) {
      if (!cf.active[k]) continue;
      C xv = x[k * stride + i], pv = ps[k * stride + i];
      const S om = S(cf.omega[k]);
      x[k * stride + i] = cmk<C>(fma(-om, pv.x, xv.x), fma(-om, pv.y, xv.y));
    }
  }
}

// ps_k = ga_k * ps_k + ze_k * r for every active shift k
// (multiple1_combine_in1_x_fact1_plus_in2_x_fact2_back_into_in1,
// fermionic_utilities.c:341-377)
template <typename C, typename S>
__global__ void k_multi_pupdate(C* ps, const C* __restrict__ r, long stride, CgmCoeffs cf, long n) {
  OST_GRID_LOOP(i, n) {
    const C rr = r[i];
    for (int k = 0; k < cf.nshift; ++k) {
      if (!cf.active[k]) continue;
      C pv = ps[k * stride + i];
      const S ga = S(cf.gamma[k]), ze = S(cf.zeta[k]);
      ps[k * stride + i] = cmk<C>(fma(ga, pv.x, ze * rr.x), fma(ga, pv.y, ze * rr.y));
    }
  }
}

template <typename T>
void multi_xupdate(typename cplx_t<T>::type* x, const typename cplx_t<T>::type* ps, long stride, const CgmCoeffs& cf,
                   long n, cudaStream_t st) {
  long b = (n + 255) / 256;
  long cap = 8L * rt().num_sms;
  k_multi_xupdate<typename cplx_t<T>::type, T><<<int(b < cap ? b : cap), 256, 0, st>>>(x, ps, stride, cf, n);
  OST_LAUNCH_CHECK();
}

template <typename T>
void multi_pupdate(typename cplx_t<T>::type* ps, const typename cplx_t<T>::type* r, long stride, const CgmCoeffs& cf,
                   long n, cudaStream_t st) {
  long b = (n + 255) / 256;
  long cap = 8L * rt().num_sms;
  k_multi_pupdate<typename cplx_t<T>::type, T><<<int(b < cap ? b : cap), 256, 0, st>>>(ps, r, stride, cf, n);
  OST_LAUNCH_CHECK();
}

// out = a0*in + sum_k a_k x_k
template <typename C>
__global__ void k_recombine(const C* __restrict__ xs, long stride, const C* __restrict__ in, C* out, RecombCoeffs rc,
                            long n) {
  OST_GRID_LOOP(i, n) {
    C v = in[i];
    double re = double(v.x) * rc.a0, im = double(v.y) * rc.a0;
    for (int k = 0; k < rc.order; ++k) {
      C xv = xs[k * stride + i];
      re += rc.a[k] * double(xv.x);
      im += rc.a[k] * double(xv.y);
    }
    out[i] = cmk<C>(re, im);
  }
}

template <typename T>
void recombine(const typename cplx_t<T>::type* xs, long stride, const typename cplx_t<T>::type* in,
               typename cplx_t<T>::type* out, const RecombCoeffs& rc, long n, cudaStream_t st) {
  long b = (n + 255) / 256;
  long cap = 8L * rt().num_sms;
  int grid = int(b < cap ? b : cap);
  k_recombine<<<grid, 256, 0, st>>>(xs, stride, in, out, rc, n);
  OST_LAUNCH_CHECK();
}

template void fused_axpy_norm<double>(double2*, const double2*, double, long, double*, cudaStream_t);
template void fused_axpy_norm<float>(float2*, const float2*, double, long, double*, cudaStream_t);
template void fused_cgm_update<double>(double2*, const double2*, double, double2*, double2*, long,
                                       const CgmCoeffs&, long, cudaStream_t);
template void fused_cgm_update<float>(float2*, const float2*, double, float2*, float2*, long, const CgmCoeffs&,
                                      long, cudaStream_t);
template void multi_xupdate<double>(double2*, const double2*, long, const CgmCoeffs&, long, cudaStream_t);
template void multi_xupdate<float>(float2*, const float2*, long, const CgmCoeffs&, long, cudaStream_t);
template void multi_pupdate<double>(double2*, const double2*, long, const CgmCoeffs&, long, cudaStream_t);
template void multi_pupdate<float>(float2*, const float2*, long, const CgmCoeffs&, long, cudaStream_t);
template void recombine<double>(const double2*, long, const double2*, double2*, const RecombCoeffs&, long,
                                cudaStream_t);
template void recombine<float>(const float2*, long, const float2*, float2*, const RecombCoeffs&, long,
                               cudaStream_t);

}  // namespace ost
