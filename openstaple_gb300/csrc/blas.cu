// blas.cu -- vector kernels over vec3_soa fields (3*sizeh contiguous complex
// numbers): the reference's fermion BLAS and global reductions
// (fermionic_utilities.c:126-455).  All streaming kernels use grid-stride
// loops sized to a multiple of the SM count; reductions are deterministic.
#include "kernels.cuh"
#include "reduce.cuh"

namespace ost {

static constexpr int BLAS_THREADS = 256;

static int stream_grid(long n) {
  long b = (n + BLAS_THREADS - 1) / BLAS_THREADS;
  long cap = 8L * (rt().num_sms > 0 ? rt().num_sms : 132);
  return int(b < cap ? (b < 1 ? 1 : b) : cap);
}

ReduceWs reduce_ws(int nv, int max_blocks) {
  // layout: RED_COUNTERS ticket counters | nv*max_blocks partials | nv*max_groups group totals
  ReduceWs w;
  if (max_blocks > RED_GROUP * (RED_COUNTERS - 1)) {
    set_error(-16, "reduction over %d blocks exceeds the workspace's %d", max_blocks, RED_GROUP * (RED_COUNTERS - 1));
    max_blocks = RED_GROUP * (RED_COUNTERS - 1);
  }
  const int max_groups = (max_blocks + RED_GROUP - 1) / RED_GROUP;
  const size_t head = sizeof(unsigned int) * RED_COUNTERS;
  size_t bytes = head + sizeof(double) * size_t(nv) * (size_t(max_blocks) + size_t(max_groups));
  // the ticket counters must read zero before the first reduction into a
  // freshly allocated buffer; afterwards every reduction leaves them at zero
  static unsigned long long zeroed_in = 0;
  char* base = static_cast<char*>(workspace(WS_REDUCE, bytes));
  if (base && zeroed_in != runtime_epoch()) {
    cudaMemsetAsync(base, 0, head, rt().stream);
    zeroed_in = runtime_epoch();
  }
  w.counter = reinterpret_cast<unsigned int*>(base);
  w.partials = reinterpret_cast<double*>(base + head);
  w.gpartials = w.partials + size_t(nv) * max_blocks;
  w.max_blocks = max_blocks;
  w.max_groups = max_groups;
  return w;
}

void reduce_ws_reserve(size_t partials) {
  // nv*max_blocks <= partials implies nv*(max_blocks + max_groups) <= partials*(1 + 1/64) + 8*nv
  const size_t bytes = sizeof(unsigned int) * RED_COUNTERS + sizeof(double) * (partials + partials / RED_GROUP + 64);
  workspace(WS_REDUCE, bytes);
}

// ---- reductions ----
template <typename C>
__global__ void k_norm2(const C* __restrict__ a, long n, ReduceWs ws, double* dst) {
  double v[1] = {0.0};
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    C x = a[i];
    v[0] += double(x.x) * double(x.x) + double(x.y) * double(x.y);
  }
  double t[1];
  if (grid_reduce<1>(v, ws, t)) dst[0] = t[0];
}

template <typename C>
__global__ void k_rdot(const C* __restrict__ a, const C* __restrict__ b, long n, ReduceWs ws, double* dst) {
  double v[1] = {0.0};
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    C x = a[i], y = b[i];
    v[0] += double(x.x) * double(y.x) + double(x.y) * double(y.y);
  }
  double t[1];
  if (grid_reduce<1>(v, ws, t)) dst[0] = t[0];
}

template <typename C>
__global__ void k_cdot(const C* __restrict__ a, const C* __restrict__ b, long n, ReduceWs ws, double* dst) {
  double v[2] = {0.0, 0.0};
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    C x = a[i], y = b[i];
    v[0] += double(x.x) * double(y.x) + double(x.y) * double(y.y);
    v[1] += double(x.x) * double(y.y) - double(x.y) * double(y.x);
  }
  double t[2];
  if (grid_reduce<2>(v, ws, t)) { dst[0] = t[0]; dst[1] = t[1]; }
}

template <typename T>
void blas_norm2(const typename cplx_t<T>::type* a, long n, double* dst, cudaStream_t st) {
  int g = reduce_grid(n);
  k_norm2<<<g, RED_THREADS, 0, st>>>(a, n, reduce_ws(1, g), dst);
  OST_LAUNCH_CHECK();
}
template <typename T>
void blas_rdot(const typename cplx_t<T>::type* a, const typename cplx_t<T>::type* b, long n, double* dst,
               cudaStream_t st) {
  int g = reduce_grid(n);
  k_rdot<<<g, RED_THREADS, 0, st>>>(a, b, n, reduce_ws(1, g), dst);
  OST_LAUNCH_CHECK();
}
template <typename T>
void blas_cdot(const typename cplx_t<T>::type* a, const typename cplx_t<T>::type* b, long n, double* dst,
               cudaStream_t st) {
  int g = reduce_grid(n);
  k_cdot<<<g, RED_THREADS, 0, st>>>(a, b, n, reduce_ws(2, g), dst);
  OST_LAUNCH_CHECK();
}

// ---- streaming updates ----
#define OST_GRID_LOOP(i, n) \
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < (n); i += long(gridDim.x) * blockDim.x)

template <typename C, typename S>
__global__ void k_axpy(const C* __restrict__ x, S a, const C* __restrict__ y, C* out, long n) {
  OST_GRID_LOOP(i, n) { C p = x[i], q = y[i]; out[i] = cmk<C>(fma(p.x, a, q.x), fma(p.y, a, q.y)); }
}
template <typename C, typename S>
__global__ void k_axmy(const C* __restrict__ x, S a, const C* __restrict__ y, C* out, long n) {
  OST_GRID_LOOP(i, n) { C p = x[i], q = y[i]; out[i] = cmk<C>(fma(p.x, a, -q.x), fma(p.y, a, -q.y)); }
}
template <typename C, typename S>
__global__ void k_scaled_diff(const C* __restrict__ x, const C* __restrict__ y, S a, C* out, long n) {
  OST_GRID_LOOP(i, n) { C p = x[i], q = y[i]; out[i] = cmk<C>(a * (p.x - q.x), a * (p.y - q.y)); }
}
template <typename C, typename S>
__global__ void k_axmymz(const C* __restrict__ x, S a, const C* __restrict__ y, const C* __restrict__ z, C* out,
                         long n) {
  OST_GRID_LOOP(i, n) {
    C p = x[i], q = y[i], r = z[i];
    out[i] = cmk<C>(p.x * a - q.x - r.x, p.y * a - q.y - r.y);
  }
}
template <typename C, typename S>
__global__ void k_scale(C* x, S a, long n) {
  OST_GRID_LOOP(i, n) { C p = x[i]; x[i] = cmk<C>(a * p.x, a * p.y); }
}
template <typename C, typename S>
__global__ void k_inside_loop(C* out, C* r, const C* __restrict__ s, const C* __restrict__ p, S w, long n) {
  OST_GRID_LOOP(i, n) {
    C o = out[i], pp = p[i], rr = r[i], ss = s[i];
    out[i] = cmk<C>(fma(pp.x, w, o.x), fma(pp.y, w, o.y));
    r[i] = cmk<C>(fma(-ss.x, w, rr.x), fma(-ss.y, w, rr.y));
  }
}
template <typename C>
__global__ void k_copy(const C* __restrict__ x, C* y, long n) { OST_GRID_LOOP(i, n) y[i] = x[i]; }
template <typename C>
__global__ void k_zero(C* x, long n) { OST_GRID_LOOP(i, n) x[i] = cmk<C>(0, 0); }

__global__ void k_d2f(const double2* __restrict__ d, float2* f, long n) {
  OST_GRID_LOOP(i, n) { double2 v = d[i]; f[i] = make_float2(float(v.x), float(v.y)); }
}
__global__ void k_f2d(const float2* __restrict__ f, double2* d, long n) {
  OST_GRID_LOOP(i, n) { float2 v = f[i]; d[i] = make_double2(double(v.x), double(v.y)); }
}
__global__ void k_acc_f2d(const float2* __restrict__ f, double2* d, long n) {
  OST_GRID_LOOP(i, n) {
    float2 v = f[i]; double2 w = d[i];
    d[i] = make_double2(w.x + double(v.x), w.y + double(v.y));
  }
}

#define OST_STREAM(kernel, n, ...)                                                 \
  do {                                                                             \
    kernel<<<stream_grid(n), BLAS_THREADS, 0, st>>>(__VA_ARGS__);                  \
    OST_LAUNCH_CHECK();                                                            \
  } while (0)

template <typename T>
void blas_axpy(const typename cplx_t<T>::type* x, double a, const typename cplx_t<T>::type* y,
               typename cplx_t<T>::type* out, long n, cudaStream_t st) {
  OST_STREAM(k_axpy, n, x, T(a), y, out, n);
}
template <typename T>
void blas_axmy(const typename cplx_t<T>::type* x, double a, const typename cplx_t<T>::type* y,
               typename cplx_t<T>::type* out, long n, cudaStream_t st) {
  OST_STREAM(k_axmy, n, x, T(a), y, out, n);
}
template <typename T>
void blas_scaled_diff(const typename cplx_t<T>::type* x, const typename cplx_t<T>::type* y, double a,
                      typename cplx_t<T>::type* out, long n, cudaStream_t st) {
  OST_STREAM(k_scaled_diff, n, x, y, T(a), out, n);
}
template <typename T>
void blas_axmymz(const typename cplx_t<T>::type* x, double a, const typename cplx_t<T>::type* y,
                 const typename cplx_t<T>::type* z, typename cplx_t<T>::type* out, long n, cudaStream_t st) {
  OST_STREAM(k_axmymz, n, x, T(a), y, z, out, n);
}
template <typename T>
void blas_scale(typename cplx_t<T>::type* x, double a, long n, cudaStream_t st) {
  OST_STREAM(k_scale, n, x, T(a), n);
}
template <typename T>
void blas_inside_loop(typename cplx_t<T>::type* out, typename cplx_t<T>::type* r, const typename cplx_t<T>::type* s,
                      const typename cplx_t<T>::type* p, double w, long n, cudaStream_t st) {
  OST_STREAM(k_inside_loop, n, out, r, s, p, T(w), n);
}
template <typename T>
void blas_copy(const typename cplx_t<T>::type* x, typename cplx_t<T>::type* y, long n, cudaStream_t st) {
  OST_STREAM(k_copy, n, x, y, n);
}
template <typename T>
void blas_zero(typename cplx_t<T>::type* x, long n, cudaStream_t st) {
  OST_STREAM(k_zero, n, x, n);
}

void conv_d2f(const double2* d, float2* f, long n, cudaStream_t st) { OST_STREAM(k_d2f, n, d, f, n); }
void conv_f2d(const float2* f, double2* d, long n, cudaStream_t st) { OST_STREAM(k_f2d, n, f, d, n); }
void acc_f2d(const float2* f, double2* d, long n, cudaStream_t st) { OST_STREAM(k_acc_f2d, n, f, d, n); }

#define OST_INST(T)                                                                                              \
  template void blas_norm2<T>(const cplx_t<T>::type*, long, double*, cudaStream_t);                              \
  template void blas_rdot<T>(const cplx_t<T>::type*, const cplx_t<T>::type*, long, double*, cudaStream_t);       \
  template void blas_cdot<T>(const cplx_t<T>::type*, const cplx_t<T>::type*, long, double*, cudaStream_t);       \
  template void blas_axpy<T>(const cplx_t<T>::type*, double, const cplx_t<T>::type*, cplx_t<T>::type*, long,     \
                             cudaStream_t);                                                                      \
  template void blas_axmy<T>(const cplx_t<T>::type*, double, const cplx_t<T>::type*, cplx_t<T>::type*, long,     \
                             cudaStream_t);                                                                      \
  template void blas_scaled_diff<T>(const cplx_t<T>::type*, const cplx_t<T>::type*, double, cplx_t<T>::type*,    \
                                    long, cudaStream_t);                                                         \
  template void blas_axmymz<T>(const cplx_t<T>::type*, double, const cplx_t<T>::type*, const cplx_t<T>::type*,   \
                               cplx_t<T>::type*, long, cudaStream_t);                                            \
  template void blas_scale<T>(cplx_t<T>::type*, double, long, cudaStream_t);                                     \
  template void blas_inside_loop<T>(cplx_t<T>::type*, cplx_t<T>::type*, const cplx_t<T>::type*,                  \
                                    const cplx_t<T>::type*, double, long, cudaStream_t);                         \
  template void blas_copy<T>(const cplx_t<T>::type*, cplx_t<T>::type*, long, cudaStream_t);                      \
  template void blas_zero<T>(cplx_t<T>::type*, long, cudaStream_t);
OST_INST(double)
OST_INST(float)

}  // namespace ost
