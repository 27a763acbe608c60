// probe.cu -- the benchmark library (libostaple_gb300_bench.so, not part of
// the drop-in): the device's FP64 and FP32 FMA throughput, the roofline
// ceiling of the compute-bound FP64 kernels (the measured peaks of the
// machine cover HBM bandwidth and BF16 tensor throughput only), and the
// per-launch timing of the hot kernels that the benchmark's roofline uses.
#include <cstdio>
#include "../runtime.cuh"
#include "../../../include/ostaple_gb300.h"
#include "../../../include/ostaple_gb300_bench.h"

namespace ost {
int time_hot_kernel(int which, const su3_soa* u, const double_soa* phases, int reps, double* ms);
}

namespace {

template <typename T>
__global__ void k_fma_chain(T* out, int iters, T a, T b) {
  // 8 independent dependency chains per thread hide the FMA latency.
  T x0 = T(threadIdx.x) * T(1e-7), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == T(-12345.678)) out[0] = s;  // keeps the chains alive
}

template <typename T>
double run(int iters) {
  ost::Runtime& r = ost::rt();
  T* out = nullptr;
  cudaMalloc(&out, sizeof(T));
  const int threads = 256;
  const int blocks = r.num_sms * 8;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chain<T><<<blocks, threads, 0, r.stream>>>(out, 16, T(0.999999), T(1e-6));  // warm-up
  cudaEventRecord(e0, r.stream);
  k_fma_chain<T><<<blocks, threads, 0, r.stream>>>(out, iters, T(0.999999), T(1e-6));
  cudaEventRecord(e1, r.stream);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  double flops = 2.0 * 64.0 * double(iters) * threads * blocks;
  return flops / (ms * 1e-3) / 1e12;
}

}  // namespace

extern "C" int ostaple_probe_fma_tflops(int fp64, double* tflops) {
  if (!ost::require_init("ostaple_probe_fma_tflops")) return -2;
  *tflops = fp64 ? run<double>(256) : run<float>(8192);
  return ost::error_code();
}

extern "C" int ostaple_time_kernel(int which, const su3_soa* u, const double_soa* phases, int reps, double* ms) {
  return ost::time_hot_kernel(which, u, phases, reps, ms);
}
