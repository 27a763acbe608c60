// reduce.cuh -- deterministic single-pass grid reductions.
//
// Every block reduces its values with warp shuffles and shared memory, writes
// one partial per block, and the last block to finish (ticket counter with a
// device-scope fence) sums the partials in block order.  The grid size only
// depends on the problem size and the SM count, so results are bitwise
// reproducible run to run; no floating-point atomics are used.
#pragma once
#include "runtime.cuh"

namespace ost {

static constexpr int RED_THREADS = 256;

struct ReduceWs {
  unsigned int* counter;   // zero between reductions
  double* partials;        // [NV * max_blocks]
  int max_blocks;
};

// Workspace for reductions of up to NV values over at most max_blocks blocks.
ReduceWs reduce_ws(int nv, int max_blocks);

// Grid for streaming reductions: enough blocks to keep every SM's load
// queues full (up to 16 blocks of 256 threads per SM), each thread handling a
// few elements.
inline int reduce_grid(long n_items) {
  long b = (n_items + 2 * RED_THREADS - 1) / (2 * RED_THREADS);
  long cap = 16L * (rt().num_sms > 0 ? rt().num_sms : 132);
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return int(b);
}

template <int NV>
OST_D void block_reduce(double v[NV], double* smem /* [NV * 32] */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) smem[k * 32 + warp] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = (lane < nwarps) ? smem[k * 32 + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      v[k] = t;
    }
  }
}

// Called by every thread of every block after computing its local values.
// Returns true in thread 0 of the last block, with the totals in `tot`.
template <int NV>
OST_D bool grid_reduce(double v[NV], ReduceWs ws, double tot[NV]) {
  __shared__ double smem[NV * 32];
  __shared__ bool am_last;
  block_reduce<NV>(v, smem);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) ws.partials[k * ws.max_blocks + blockIdx.x] = v[k];
    __threadfence();
    unsigned int t = atomicAdd(ws.counter, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  // last block: sum partials in fixed order, one value per warp-strided lane
  double s[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) s[k] = 0.0;
  for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
#pragma unroll
    for (int k = 0; k < NV; ++k) s[k] += __ldcg(ws.partials + k * ws.max_blocks + b);
  }
  __syncthreads();
  block_reduce<NV>(s, smem);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) tot[k] = s[k];
    *ws.counter = 0;
    return true;
  }
  return false;
}

// Variant for single-precision solvers: per-thread values and the
// intra-warp tree in FP32 (GB300 runs FP64 at 1/64 of the FP32 rate, so FP64
// per-thread accumulation would cost as much as the memory traffic), the
// cross-warp and cross-block sums in FP64.  Same fixed order, so results
// stay bitwise reproducible.
template <int NV>
OST_D bool grid_reduce_f32w(float vf[NV], ReduceWs ws, double tot[NV]) {
  __shared__ double smem[NV * 32];
  __shared__ bool am_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vf[k] += __shfl_down_sync(0xffffffffu, vf[k], o);
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) smem[k * 32 + warp] = double(vf[k]);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = 0.0;
      for (int w = 0; w < nwarps; ++w) t += smem[k * 32 + w];
      ws.partials[k * ws.max_blocks + blockIdx.x] = t;
    }
    __threadfence();
    unsigned int t = atomicAdd(ws.counter, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  double s[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) s[k] = 0.0;
  for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
#pragma unroll
    for (int k = 0; k < NV; ++k) s[k] += __ldcg(ws.partials + k * ws.max_blocks + b);
  }
  __syncthreads();
  block_reduce<NV>(s, smem);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) tot[k] = s[k];
    *ws.counter = 0;
    return true;
  }
  return false;
}

}  // namespace ost
