// reduce.cuh -- deterministic single-pass grid reductions.
//
// Every block reduces its values with warp shuffles and shared memory and
// writes one partial per block.  The partials are then summed in two levels
// inside the same kernel: the last block to finish in each group of
// RED_GROUP consecutive blocks sums that group's partials (ticket counter
// per group, device-scope fences), and the last group to finish sums the
// group totals.  A single last block summing every partial would read them
// one L2 round trip after another; with 10^4 blocks that tail alone costs
// tens of microseconds.  All sums run in a fixed order that depends only on
// the grid size, so results are bitwise reproducible run to run; no
// floating-point atomics are used.
#pragma once
#include "runtime.cuh"

namespace ost {

static constexpr int RED_THREADS = 256;
static constexpr int RED_GROUP = 64;          // blocks per first-level group
static constexpr int RED_COUNTERS = 16384;    // ticket counters: [0] final, [1 + g] group g

struct ReduceWs {
  unsigned int* counter;   // [RED_COUNTERS], all zero between reductions
  double* partials;        // [NV * max_blocks] block partials
  double* gpartials;       // [NV * max_groups] group totals
  int max_blocks;
  int max_groups;
};

// Workspace for reductions of up to NV values over at most max_blocks blocks
// (max_blocks <= RED_GROUP * (RED_COUNTERS - 1)).
ReduceWs reduce_ws(int nv, int max_blocks);
// Allocates the workspace for reductions with up to `partials` = NV x blocks
// block partials ahead of a graph capture (nothing may allocate inside one).
void reduce_ws_reserve(size_t partials);

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

// Second and third stage shared by every variant: bv[NV] holds this block's
// partials in thread 0.  Returns true in thread 0 of the block that finishes
// last, with the grid totals in tot.  smem must hold NV * 32 doubles and be
// free for reuse (callers synchronise before the call).
template <int NV>
OST_D bool grid_finish(const double bv[NV], ReduceWs ws, double tot[NV], double* smem) {
  __shared__ int stage;   // 1: this block closed its group, 2: it closed the grid
  const int g = blockIdx.x / RED_GROUP;
  const int ng = (gridDim.x + RED_GROUP - 1) / RED_GROUP;
  const int gsize = min(RED_GROUP, int(gridDim.x) - g * RED_GROUP);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) ws.partials[k * ws.max_blocks + blockIdx.x] = bv[k];
    __threadfence();
    const unsigned int t = atomicAdd(ws.counter + 1 + g, 1u);
    stage = (t == unsigned(gsize - 1)) ? 1 : 0;
  }
  __syncthreads();
  if (stage == 0) return false;
  __threadfence();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    double gs[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double* src = ws.partials + k * ws.max_blocks + g * RED_GROUP;
      double a = lane < gsize ? __ldcg(src + lane) : 0.0;
      if (lane + 32 < gsize) a += __ldcg(src + lane + 32);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
      gs[k] = a;
    }
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < NV; ++k) ws.gpartials[k * ws.max_groups + g] = gs[k];
      ws.counter[1 + g] = 0;
      __threadfence();
      const unsigned int t = atomicAdd(ws.counter, 1u);
      stage = (t == unsigned(ng - 1)) ? 2 : 0;
    }
  }
  __syncthreads();
  if (stage != 2) return false;
  __threadfence();
  double s[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) s[k] = 0.0;
  for (int i = threadIdx.x; i < ng; i += blockDim.x) {
#pragma unroll
    for (int k = 0; k < NV; ++k) s[k] += __ldcg(ws.gpartials + k * ws.max_groups + i);
  }
  block_reduce<NV>(s, smem);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) tot[k] = s[k];
    *ws.counter = 0;
    return true;
  }
  return false;
}

// Called by every thread of every block after computing its local values.
// Returns true in thread 0 of the last block, with the totals in `tot`.
template <int NV>
OST_D bool grid_reduce(double v[NV], ReduceWs ws, double tot[NV]) {
  __shared__ double smem[NV * 32];
  block_reduce<NV>(v, smem);
  __syncthreads();
  return grid_finish<NV>(v, ws, tot, smem);
}

// Variant for single-precision solvers: per-thread values and the
// intra-warp tree in FP32 (GB300 runs FP64 at 1/64 of the FP32 rate, so FP64
// per-thread accumulation would cost as much as the memory traffic), the
// cross-warp and cross-block sums in FP64.  Same fixed order, so results
// stay bitwise reproducible.
template <int NV>
OST_D bool grid_reduce_f32w(float vf[NV], ReduceWs ws, double tot[NV]) {
  __shared__ double smem[NV * 32];
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
  double bv[NV];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = 0.0;
      for (int w = 0; w < nwarps; ++w) t += smem[k * 32 + w];
      bv[k] = t;
    }
  }
  __syncthreads();
  return grid_finish<NV>(bv, ws, tot, smem);
}

// Per-system reduction for kernels that give each system of a batch its own
// lane: system k = lane % NSP (NSP a power of two <= 32).  Each thread passes
// one FP32 value (zero if it has none); returns true in thread 0 of the last
// block with tot[k] = the sum over all threads of system k.  The intra-warp
// tree is FP32, the cross-warp and cross-block sums FP64, in a fixed order.
template <int NSP>
OST_D bool grid_reduce_lanes(float vf, ReduceWs ws, double tot[NSP]) {
  __shared__ double smem[NSP * 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int o = 16; o >= NSP; o >>= 1) vf += __shfl_xor_sync(0xffffffffu, vf, o);
  if (lane < NSP) smem[lane * 32 + warp] = double(vf);
  __syncthreads();
  double bv[NSP];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NSP; ++k) {
      double t = 0.0;
      for (int w = 0; w < nwarps; ++w) t += smem[k * 32 + w];
      bv[k] = t;
    }
  }
  __syncthreads();
  return grid_finish<NSP>(bv, ws, tot, smem);
}

// Segmented reduction: the grid's blocks form NSEG consecutive segments of
// seg_blocks blocks (segment = blockIdx.x / seg_blocks, one system each).
// Each thread passes one FP32 value; returns true in thread 0 of the last
// block with tot[k] = the sum over segment k.  FP32 intra-warp, FP64 above.
template <int NSEG>
OST_D bool grid_reduce_seg(float vf, int seg_blocks, ReduceWs ws, double tot[NSEG]) {
  __shared__ double smem[NSEG * 32 > 32 ? NSEG * 32 : 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) vf += __shfl_down_sync(0xffffffffu, vf, o);
  if (lane == 0) smem[warp] = double(vf);
  __syncthreads();
  double bv[NSEG];
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < nwarps; ++w) t += smem[w];
    const int seg = blockIdx.x / seg_blocks;
#pragma unroll
    for (int k = 0; k < NSEG; ++k) bv[k] = (k == seg) ? t : 0.0;
  }
  __syncthreads();
  return grid_finish<NSEG>(bv, ws, tot, smem);
}

}  // namespace ost
