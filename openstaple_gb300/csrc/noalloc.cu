// noalloc.cu -- an allocation-free variant of real_scal_prod_global.
//
// Some callers cannot allocate device memory at the moment they need a
// global reduction: code that must not pay the implicit device
// synchronisation of cudaMalloc/cudaFree inside a latency-critical loop, and
// processes that run under a fixed device-memory budget (an MPS client with a
// memory limit, or a host program that has already divided HBM among its own
// pools and forbids further raw allocations).  For them this entry point
// keeps its scratch -- the per-block partial sums, the ticket counter and the
// result slot -- in one file-scope device array of fixed size that every GPU
// loading the library holds until the process exits.  Lattices with
// 3*sizeh > 8,388,608 complex numbers are rejected with error -14.
#include <cstdio>
#include "reduce.cuh"
#include "runtime.cuh"
#include "../../include/ostaple_gb300.h"

namespace ost {

// Layout in doubles: [0, 64) ticket counters (the final one and one per
// group of blocks, 65 used), [64] the result, [80, 80 + 4096) block
// partials, then 64 group totals: 33,920 bytes per device.
static constexpr int NOALLOC_MAX_BLOCKS = 4096;
static constexpr int NOALLOC_MAX_GROUPS = NOALLOC_MAX_BLOCKS / RED_GROUP;
static constexpr int NOALLOC_RESULT = 64;
static constexpr int NOALLOC_HEADER = 80;
static_assert((NOALLOC_MAX_GROUPS + 1) * sizeof(unsigned int) <= NOALLOC_RESULT * sizeof(double),
              "ticket counters overlap the result slot");
static constexpr int NOALLOC_THREADS = 256;
static constexpr int NOALLOC_PER_THREAD = 8;                                     // complex numbers per thread
static constexpr long NOALLOC_PER_BLOCK = long(NOALLOC_THREADS) * NOALLOC_PER_THREAD;
static constexpr long NOALLOC_MAX_N = NOALLOC_MAX_BLOCKS * NOALLOC_PER_BLOCK;     // 8,388,608 complex numbers

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_HEADER + NOALLOC_MAX_BLOCKS + NOALLOC_MAX_GROUPS];

// Each block reduces a fixed chunk of NOALLOC_PER_BLOCK complex numbers, so
// the number of partials is n / chunk and the scratch bounds n.
__global__ void k_rdot_noalloc(const double2* __restrict__ a, const double2* __restrict__ b, long n,
                               double* scratch) {
  double v[1] = {0.0};
  const long base = long(blockIdx.x) * NOALLOC_PER_BLOCK;
#pragma unroll
  for (int k = 0; k < NOALLOC_PER_THREAD; ++k) {
    const long i = base + long(k) * NOALLOC_THREADS + threadIdx.x;
    if (i < n) {
      double2 x = a[i], y = b[i];
      v[0] += x.x * y.x + x.y * y.y;
    }
  }
  ReduceWs ws;
  ws.counter = reinterpret_cast<unsigned int*>(scratch);
  ws.partials = scratch + NOALLOC_HEADER;
  ws.gpartials = ws.partials + NOALLOC_MAX_BLOCKS;
  ws.max_blocks = NOALLOC_MAX_BLOCKS;
  ws.max_groups = NOALLOC_MAX_GROUPS;
  double tot[1];
  if (grid_reduce<1>(v, ws, tot)) scratch[NOALLOC_RESULT] = tot[0];
}

}  // namespace ost

using namespace ost;

extern "C" double ostaple_real_scal_prod_global_noalloc(const vec3_soa* in_vect1, const vec3_soa* in_vect2) {
  if (!require_init("ostaple_real_scal_prod_global_noalloc")) return NAN;
  const long n = 3L * rt().g.sizeh;
  if (n > NOALLOC_MAX_N) {
    set_error(-14,
              "ostaple_real_scal_prod_global_noalloc: %ld complex numbers exceed the fixed scratch (at most %ld, "
              "i.e. sizeh <= %ld); use real_scal_prod_global",
              n, NOALLOC_MAX_N, NOALLOC_MAX_N / 3);
    return NAN;
  }
  // device address of the static scratch, looked up once per device with that
  // device current (the first call on a device does this set-up)
  static double* s_addr[64] = {nullptr};
  int devid = -1;
  if (cudaGetDevice(&devid) != cudaSuccess) {
    cudaGetLastError();
    set_error(-14, "ostaple_real_scal_prod_global_noalloc: no current CUDA device");
    return NAN;
  }
  if (devid < 0 || devid >= 64) {
    set_error(-14, "ostaple_real_scal_prod_global_noalloc: device id %d out of range", devid);
    return NAN;
  }
  if (!s_addr[devid]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error(int(e), "ostaple_real_scal_prod_global_noalloc: cudaGetSymbolAddress failed: %s",
                cudaGetErrorString(e));
      return NAN;
    }
    s_addr[devid] = static_cast<double*>(p);
  }
  double* scratch = s_addr[devid];
  const double2* a = dev(reinterpret_cast<const double2*>(in_vect1), "in_vect1");
  const double2* b = dev(reinterpret_cast<const double2*>(in_vect2), "in_vect2");
  if (!a || !b) return NAN;  // pointer neither registered nor device memory (error recorded)
  cudaStream_t st = rt().stream;
  // This call's own CUDA status decides the result: the library's error word
  // keeps the first failure of any earlier call, so it cannot tell whether
  // this reduction succeeded.
  // The array keeps the previous call's contents: the ticket counters must
  // start at zero.
  cudaError_t e = cudaMemsetAsync(scratch, 0, NOALLOC_RESULT * sizeof(double), st);
  if (e == cudaSuccess) {
    const int grid = int((n + NOALLOC_PER_BLOCK - 1) / NOALLOC_PER_BLOCK);
    k_rdot_noalloc<<<grid, NOALLOC_THREADS, 0, st>>>(a, b, n, scratch);
    ++g_kernel_launches;
    e = cudaGetLastError();
  }
  double h = NAN;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&h, scratch + NOALLOC_RESULT, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(int(e), "ostaple_real_scal_prod_global_noalloc: %s", cudaGetErrorString(e));
    return NAN;
  }
  return h;
}
