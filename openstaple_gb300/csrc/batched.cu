// batched.cu -- multi-system FP32 solvers: a batch of up to BATCH_MAX
// independent mixed-precision CG systems (own source, own shift, own
// scalars, own reliable updates), and a multi-shift CG for several
// right-hand sides at once.  In both, one thread per site loads each link
// and its sign once and applies it to every system of the batch, so the
// link stream (384 of the 440 bytes per site of a single-system hop) is
// shared by the batch.  All scalars stay on the device; iteration chunks
// are captured as CUDA graphs and polled once per chunk.
#include <cmath>
#include <cstring>
#include "batched.cuh"
#include "dslash.cuh"
#include "kernels.cuh"
#include "reduce.cuh"
#include "runtime.cuh"

namespace ost {

static constexpr int BT = 128;

// hop term of NS systems at output index idx of parity P, skipping systems
// whose bit in `mask` is clear.
template <int NS, int P, int PH>
OST_D void hop_batch(const Geom& g, const LinkView<float2>& u, const float2* in, long vstride, const void* ph,
                     int idx, unsigned mask, float2 aux[NS][3]) {
  typedef unsigned int M;
  const long sh = g.sizeh;
  Site s = site_of(g, idx, P);
  int fwd[4], bwd[4];
  neighbours(g, s, fwd, bwd);
#pragma unroll
  for (int k = 0; k < NS; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) aux[k][c] = make_float2(0.f, 0.f);
#pragma unroll
  for (int half = 0; half < 2; ++half) {
#pragma unroll
    for (int mu = 0; mu < 4; ++mu) {
      const bool back = half == 0;
      const int dir = back ? 2 * mu + (1 - P) : 2 * mu + P;
      const int j = back ? bwd[mu] : fwd[mu];      // neighbour holding the input spinor
      const int li = back ? j : idx;               // index of the link
      float2 m[6];
      load_two_rows(u, dir, li, m);
      M mask_sign;
      float2 phz = make_float2(1.f, 0.f);
      bool generic = false;
      if (PH == PH_SIGN8) {
        unsigned char sb = __ldg(static_cast<const unsigned char*>(ph) + long(dir) * sh + li);
        mask_sign = (sb ? 0x80000000u : 0u) ^ (back ? 0x80000000u : 0u);
      } else {
        float a = __ldg(static_cast<const float*>(ph) + long(dir) * sh + li);
        unsigned bits = __float_as_uint(a);
        if (bits == 0u || bits == PiBits<float>::bits()) {
          mask_sign = (bits == 0u ? 0u : 0x80000000u) ^ (back ? 0x80000000u : 0u);
        } else {
          float sn, cs;
          sincosf(a, &sn, &cs);
          phz = make_float2(cs, back ? -sn : sn);
          mask_sign = back ? 0x80000000u : 0u;
          generic = true;
        }
      }
#pragma unroll
      for (int k = 0; k < NS; ++k) {
        if (!(mask >> k & 1u)) continue;
        float2 v[3];
        load_vec(in + k * vstride, sh, j, v);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (generic) v[c] = cmul(v[c], phz);
          v[c].x = flip_sign(v[c].x, mask_sign);
          v[c].y = flip_sign(v[c].y, mask_sign);
        }
        if (back) mac_Udag(aux[k], m, v);
        else mac_U(aux[k], m, v);
      }
    }
  }
}

OST_D unsigned active_mask(const BatchScal* sc) {
  unsigned m = 0;
  for (int k = 0; k < sc->nsys; ++k)
    if (!(*(volatile const int*)&sc->done[k]) && !(*(volatile const int*)&sc->need_rel[k])) m |= 1u << k;
  return m;
}

// t_k = D_oe p_k
template <int NS, int PH>
__global__ void __launch_bounds__(BT)
k_b_doe(Geom g, LinkView<float2> u, const void* __restrict__ ph, const float2* __restrict__ p, float2* __restrict__ t,
        long vs, const BatchScal* sc) {
  const unsigned mask = active_mask(sc);
  if (!mask) return;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.sizeh) return;
  float2 aux[NS][3];
  hop_batch<NS, 1, PH>(g, u, p, vs, ph, idx, mask, aux);
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    if (!(mask >> k & 1u)) continue;
#pragma unroll
    for (int c = 0; c < 3; ++c)
      t[k * vs + c * long(g.sizeh) + idx] = make_float2(0.5f * aux[k][c].x, 0.5f * aux[k][c].y);
  }
}

// s_k = m2_k p_k - D_eo t_k ; pAp_k ; alpha_k = delta_k / pAp_k
template <int NS, int PH>
__global__ void __launch_bounds__(BT)
k_b_deo_dot(Geom g, LinkView<float2> u, const void* __restrict__ ph, const float2* __restrict__ t,
            const float2* __restrict__ p, float2* __restrict__ s, long vs, BatchScal* sc, ReduceWs ws) {
  const unsigned mask = active_mask(sc);
  if (!mask) return;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  float v[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) v[k] = 0.f;
  if (idx < g.sizeh) {
    float2 aux[NS][3];
    hop_batch<NS, 0, PH>(g, u, t, vs, ph, idx, mask, aux);
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      if (!(mask >> k & 1u)) continue;
      const float m2 = float(sc->m2[k]);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const long q = k * vs + c * long(g.sizeh) + idx;
        float2 pv = p[q];
        float2 r = make_float2(fmaf(pv.x, m2, -0.5f * aux[k][c].x), fmaf(pv.y, m2, -0.5f * aux[k][c].y));
        s[q] = r;
        v[k] = fmaf(pv.x, r.x, fmaf(pv.y, r.y, v[k]));
      }
    }
  }
  double tot[NS];
  if (grid_reduce_f32w<NS>(v, ws, tot)) {
    for (int k = 0; k < NS; ++k)
      if (mask >> k & 1u) { sc->pAp[k] = tot[k]; sc->alpha[k] = sc->delta[k] / tot[k]; }
  }
}

// x_f += alpha p ; unless a reliable update is due: r -= alpha s, lambda = |r|^2
template <int NS>
__global__ void k_b_update(float4* __restrict__ xf, float4* __restrict__ r, const float4* __restrict__ p,
                           const float4* __restrict__ s, long n4, long vs4, BatchScal* sc, ReduceWs ws) {
  const unsigned mask = active_mask(sc);
  if (!mask) return;
  bool rel[NS];
  float a[NS], v[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    const double delta = sc->delta[k];
    const double lm = sc->last_max[k] > delta ? sc->last_max[k] : delta;
    rel[k] = sc->every > 0 ? ((sc->iter[k] + 1) % sc->every == 0) : (delta < sc->frac * lm);
    a[k] = float(sc->alpha[k]);
    v[k] = 0.f;
  }
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n4; i += long(gridDim.x) * blockDim.x) {
    float4 pv[NS], xv[NS], sv[NS], rv[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {       // all loads of this element first
      if (!(mask >> k & 1u)) continue;
      const long q = k * vs4 + i;
      pv[k] = p[q]; xv[k] = xf[q];
      if (!rel[k]) { sv[k] = s[q]; rv[k] = r[q]; }
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      if (!(mask >> k & 1u)) continue;
      const long q = k * vs4 + i;
      xv[k].x = fmaf(a[k], pv[k].x, xv[k].x); xv[k].y = fmaf(a[k], pv[k].y, xv[k].y);
      xv[k].z = fmaf(a[k], pv[k].z, xv[k].z); xv[k].w = fmaf(a[k], pv[k].w, xv[k].w);
      xf[q] = xv[k];
      if (!rel[k]) {
        rv[k].x = fmaf(-a[k], sv[k].x, rv[k].x); rv[k].y = fmaf(-a[k], sv[k].y, rv[k].y);
        rv[k].z = fmaf(-a[k], sv[k].z, rv[k].z); rv[k].w = fmaf(-a[k], sv[k].w, rv[k].w);
        r[q] = rv[k];
        v[k] = fmaf(rv[k].x, rv[k].x, fmaf(rv[k].y, rv[k].y, fmaf(rv[k].z, rv[k].z, fmaf(rv[k].w, rv[k].w, v[k]))));
      }
    }
  }
  double tot[NS];
  if (grid_reduce_f32w<NS>(v, ws, tot)) {
    for (int k = 0; k < NS; ++k) {
      if (!(mask >> k & 1u)) continue;
      const double delta = sc->delta[k];
      sc->iter[k] += 1;
      sc->last_max[k] = sc->last_max[k] > delta ? sc->last_max[k] : delta;
      if (rel[k]) {
        sc->need_rel[k] = 1;
      } else {
        sc->lambda[k] = tot[k];
        sc->beta[k] = tot[k] / delta;
        sc->delta[k] = tot[k];
        if (tot[k] <= sc->target2[k] || sc->iter[k] >= sc->max_iter) sc->done[k] = 1;
      }
    }
  }
}

// p = r + beta p  (mode 0: active systems; mode 1: system `only`)
template <int NS>
__global__ void k_b_pupdate(float4* __restrict__ p, const float4* __restrict__ r, long n4, long vs4,
                            const BatchScal* sc, int only) {
  unsigned mask;
  if (only >= 0) mask = 1u << only;
  else {
    mask = active_mask(sc);
    if (!mask) return;
  }
  float b[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) b[k] = float(sc->beta[k]);
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n4; i += long(gridDim.x) * blockDim.x) {
    float4 pv[NS], rv[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      if (!(mask >> k & 1u)) continue;
      pv[k] = p[k * vs4 + i]; rv[k] = r[k * vs4 + i];
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      if (!(mask >> k & 1u)) continue;
      p[k * vs4 + i] = make_float4(fmaf(b[k], pv[k].x, rv[k].x), fmaf(b[k], pv[k].y, rv[k].y),
                                   fmaf(b[k], pv[k].z, rv[k].z), fmaf(b[k], pv[k].w, rv[k].w));
    }
  }
}

// p_k = r_k + beta_k p_k for one system (after its reliable update)
__global__ void k_b_pupdate_sys(float4* __restrict__ p, const float4* __restrict__ r, long n4, const BatchScal* sc,
                                int k) {
  const float b = float(sc->beta[k]);
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n4; i += long(gridDim.x) * blockDim.x) {
    float4 pv = p[i], rv = r[i];
    p[i] = make_float4(fmaf(b, pv.x, rv.x), fmaf(b, pv.y, rv.y), fmaf(b, pv.z, rv.z), fmaf(b, pv.w, rv.w));
  }
}

// FP64 side of system k: x += x_f, x_f = 0
__global__ void k_b_accumulate(double2* __restrict__ x, float2* __restrict__ xf, long n) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    float2 f = xf[i];
    double2 d = x[i];
    x[i] = make_double2(d.x + double(f.x), d.y + double(f.y));
    xf[i] = make_float2(0.f, 0.f);
  }
}

// r64 = b - Ax, r = (float) r64 for system k; mode 0 initial, mode 1 reliable update
__global__ void k_b_residual(const double2* __restrict__ b, const double2* __restrict__ ax, double2* __restrict__ r64,
                             float2* __restrict__ r, float2* __restrict__ p, long n, BatchScal* sc, int k,
                             ReduceWs ws, int mode) {
  double v[2] = {0.0, 0.0};
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    double2 bb = b[i], a = ax[i];
    double2 d = make_double2(bb.x - a.x, bb.y - a.y);
    r64[i] = d;
    float2 f = make_float2(float(d.x), float(d.y));
    r[i] = f;
    if (mode == 0) p[i] = f;
    v[0] += double(f.x) * f.x + double(f.y) * f.y;
    v[1] += d.x * d.x + d.y * d.y;
  }
  double tot[2];
  if (grid_reduce<2>(v, ws, tot)) {
    sc->true_r2[k] = tot[1];
    sc->lambda[k] = tot[0];
    if (mode == 0) {
      sc->delta[k] = tot[0];
      sc->beta[k] = 0.0;
    } else {
      sc->beta[k] = tot[0] / sc->delta[k];
      sc->delta[k] = tot[0];
      sc->n_rel[k] += 1;
    }
    sc->last_max[k] = 0.0;
    sc->need_rel[k] = 0;
    sc->done[k] = (tot[0] <= sc->target2[k] || sc->iter[k] >= sc->max_iter) ? 1 : 0;
  }
}

// ---- host engine ----
namespace {

struct BGraph {
  cudaGraphExec_t exec = nullptr;
  BatchBuffers key{};
  BatchScal* sc = nullptr;
  int chunk = 0;
  unsigned long long epoch = 0;
};
BGraph g_bgraph;
cudaStream_t g_bcap = nullptr;
BatchScal* g_bhost = nullptr;

void fp64_mdagm(const BatchBuffers& B, double2* out, const double2* in, double m2, cudaStream_t st) {
  DslashArgs<double> a;
  a.phase_mode = PH_ANGLE; a.u = B.u64; a.phases = B.ph64; a.stream = st; a.compact_links = 0;
  a.parity = 1; a.epilogue = EPI_PLAIN; a.out = B.t64b; a.in = in; a.in0 = nullptr; a.mass2 = 0;
  launch_dslash<double>(a);
  a.parity = 0; a.epilogue = EPI_MDAGM; a.out = out; a.in = B.t64b; a.in0 = in; a.mass2 = m2;
  launch_dslash<double>(a);
}

template <int NS>
void enqueue_batch_iteration(const BatchBuffers& B, BatchScal* sc, cudaStream_t st) {
  const Geom& g = rt().g;
  LinkView<float2> u{B.u32, g.sizeh, 6};
  const int nb = blocks_for(g.sizeh, BT);
  const long n = 3L * g.sizeh, n4 = n / 2;
  const int gr = reduce_grid(n4);
  ReduceWs ws = reduce_ws(NS, nb > gr ? nb : gr);
  if (B.ph32_mode == PH_SIGN8) {
    k_b_doe<NS, PH_SIGN8><<<nb, BT, 0, st>>>(g, u, B.ph32, B.p, B.t, n, sc);
    k_b_deo_dot<NS, PH_SIGN8><<<nb, BT, 0, st>>>(g, u, B.ph32, B.t, B.p, B.s, n, sc, ws);
  } else {
    k_b_doe<NS, PH_ANGLE><<<nb, BT, 0, st>>>(g, u, B.ph32, B.p, B.t, n, sc);
    k_b_deo_dot<NS, PH_ANGLE><<<nb, BT, 0, st>>>(g, u, B.ph32, B.t, B.p, B.s, n, sc, ws);
  }
  k_b_update<NS><<<gr, RED_THREADS, 0, st>>>(reinterpret_cast<float4*>(B.xf), reinterpret_cast<float4*>(B.r),
                                              reinterpret_cast<const float4*>(B.p),
                                              reinterpret_cast<const float4*>(B.s), n4, n4, sc, ws);
  k_b_pupdate<NS><<<gr, RED_THREADS, 0, st>>>(reinterpret_cast<float4*>(B.p), reinterpret_cast<const float4*>(B.r),
                                               n4, n4, sc, -1);
}

void enqueue_chunk(const BatchBuffers& B, BatchScal* sc, int chunk, cudaStream_t st) {
  for (int c = 0; c < chunk; ++c) {
    switch (B.nsys) {
      case 1: enqueue_batch_iteration<1>(B, sc, st); break;
      case 2: enqueue_batch_iteration<2>(B, sc, st); break;
      case 3: enqueue_batch_iteration<3>(B, sc, st); break;
      case 4: enqueue_batch_iteration<4>(B, sc, st); break;
      case 5: enqueue_batch_iteration<5>(B, sc, st); break;
      case 6: enqueue_batch_iteration<6>(B, sc, st); break;
      case 7: enqueue_batch_iteration<7>(B, sc, st); break;
      default: enqueue_batch_iteration<8>(B, sc, st); break;
    }
  }
}

void pupdate_one(const BatchBuffers& B, BatchScal* sc, int k, cudaStream_t st) {
  const long n4 = 3L * rt().g.sizeh / 2;
  k_b_pupdate_sys<<<reduce_grid(n4), RED_THREADS, 0, st>>>(reinterpret_cast<float4*>(B.p) + k * n4,
                                                            reinterpret_cast<const float4*>(B.r) + k * n4, n4, sc, k);
  OST_LAUNCH_CHECK();
}

}  // namespace

BatchResult batched_mixed_cg(const BatchBuffers& B, const double* m2, double res, int max_iter, double delta_frac,
                             BatchScal* sc, cudaStream_t st) {
  BatchResult out;
  memset(&out, 0, sizeof(out));
  const Geom& g = rt().g;
  const long n = 3L * g.sizeh;
  const int NSY = B.nsys;
  if (!g_bcap) {
    OST_CUDA(cudaStreamCreateWithFlags(&g_bcap, cudaStreamNonBlocking));
    OST_CUDA(cudaMallocHost(&g_bhost, sizeof(BatchScal)));
  }
  cudaEvent_t ev;
  OST_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  OST_CUDA(cudaEventRecord(ev, st));
  OST_CUDA(cudaStreamWaitEvent(g_bcap, ev, 0));
  cudaStream_t cs = g_bcap;
  {
    const int nb = blocks_for(g.sizeh, BT), gr = reduce_grid(n);
    reduce_ws(BATCH_MAX, nb > gr ? nb : gr);
  }
  BatchScal init;
  memset(&init, 0, sizeof(init));
  init.frac = delta_frac;
  init.max_iter = max_iter;
  init.every = 0;
  init.nsys = NSY;
  for (int k = 0; k < NSY; ++k) init.m2[k] = m2[k];
  OST_CUDA(cudaMemcpyAsync(sc, &init, sizeof(BatchScal), cudaMemcpyHostToDevice, cs));
  for (int k = 0; k < NSY; ++k) blas_norm2<double>(B.b + k * n, n, &sc->bnorm2[k], cs);
  OST_CUDA(cudaMemcpyAsync(g_bhost, sc, sizeof(BatchScal), cudaMemcpyDeviceToHost, cs));
  OST_CUDA(cudaStreamSynchronize(cs));
  double bn[BATCH_MAX], fp32_target[BATCH_MAX];
  for (int k = 0; k < NSY; ++k) {
    bn[k] = g_bhost->bnorm2[k];
    fp32_target[k] = 0.9 * res;
    init.bnorm2[k] = bn[k];
    init.target2[k] = fp32_target[k] * fp32_target[k] * bn[k];
  }
  OST_CUDA(cudaMemcpyAsync(sc, &init, sizeof(BatchScal), cudaMemcpyHostToDevice, cs));
  blas_zero<float>(B.xf, NSY * n, cs);
  for (int k = 0; k < NSY; ++k) {
    fp64_mdagm(B, B.t64, B.x + k * n, m2[k], cs);
    const int gr = reduce_grid(n);
    k_b_residual<<<gr, RED_THREADS, 0, cs>>>(B.b + k * n, B.t64, B.r64, B.r + k * n, B.p + k * n, n, sc, k,
                                             reduce_ws(2, gr), 0);
    OST_LAUNCH_CHECK();
  }
  const int chunk = 8;
  if (!g_bgraph.exec || g_bgraph.sc != sc || g_bgraph.chunk != chunk || g_bgraph.key.nsys != B.nsys ||
      g_bgraph.key.p != B.p || g_bgraph.key.r != B.r || g_bgraph.key.s != B.s || g_bgraph.key.t != B.t ||
      g_bgraph.key.xf != B.xf || g_bgraph.key.u32 != B.u32 || g_bgraph.key.ph32 != B.ph32 ||
      g_bgraph.key.ph32_mode != B.ph32_mode || g_bgraph.epoch != runtime_epoch()) {
    if (g_bgraph.exec) cudaGraphExecDestroy(g_bgraph.exec);
    cudaGraph_t graph;
    OST_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    enqueue_chunk(B, sc, chunk, cs);
    OST_CUDA(cudaStreamEndCapture(cs, &graph));
    OST_CUDA(cudaGraphInstantiate(&g_bgraph.exec, graph, 0));
    cudaGraphDestroy(graph);
    g_bgraph.key = B;
    g_bgraph.sc = sc;
    g_bgraph.chunk = chunk;
    g_bgraph.epoch = runtime_epoch();
  }
  bool finished[BATCH_MAX] = {false};
  for (int guard = 0; guard < 1000000; ++guard) {
    if (error_code()) break;
    OST_CUDA(cudaGraphLaunch(g_bgraph.exec, cs));
    g_kernel_launches += 4ull * chunk;
    OST_CUDA(cudaMemcpyAsync(g_bhost, sc, sizeof(BatchScal), cudaMemcpyDeviceToHost, cs));
    OST_CUDA(cudaStreamSynchronize(cs));
    BatchScal h = *g_bhost;
    bool all = true;
    for (int k = 0; k < NSY; ++k) {
      if (finished[k]) continue;
      if (h.need_rel[k] || h.done[k]) {
        const bool was_done = h.done[k];
        k_b_accumulate<<<8 * rt().num_sms, 256, 0, cs>>>(B.x + k * n, B.xf + k * n, n);
        OST_LAUNCH_CHECK();
        fp64_mdagm(B, B.t64, B.x + k * n, m2[k], cs);
        const int gr = reduce_grid(n);
        k_b_residual<<<gr, RED_THREADS, 0, cs>>>(B.b + k * n, B.t64, B.r64, B.r + k * n, B.p + k * n, n, sc, k,
                                                 reduce_ws(2, gr), 1);
        OST_LAUNCH_CHECK();
        if (was_done) {
          OST_CUDA(cudaMemcpyAsync(g_bhost, sc, sizeof(BatchScal), cudaMemcpyDeviceToHost, cs));
          OST_CUDA(cudaStreamSynchronize(cs));
          const double tr2 = g_bhost->true_r2[k];
          out.iters[k] = g_bhost->iter[k];
          out.n_reliable[k] = g_bhost->n_rel[k] - 1;
          out.true_res[k] = std::sqrt(tr2 / bn[k]);
          out.converged[k] = tr2 <= res * res * bn[k];
          if (out.converged[k] || g_bhost->iter[k] >= max_iter) {
            finished[k] = true;
            // keep the system halted: done stays set
            const int one = 1;
            OST_CUDA(cudaMemcpyAsync(&sc->done[k], &one, sizeof(int), cudaMemcpyHostToDevice, cs));
            continue;
          }
          fp32_target[k] *= 0.5;
          const double t2 = fp32_target[k] * fp32_target[k] * bn[k];
          const int dn = g_bhost->lambda[k] <= t2 ? 1 : 0;
          OST_CUDA(cudaMemcpyAsync(&sc->target2[k], &t2, sizeof(double), cudaMemcpyHostToDevice, cs));
          OST_CUDA(cudaMemcpyAsync(&sc->done[k], &dn, sizeof(int), cudaMemcpyHostToDevice, cs));
        }
        pupdate_one(B, sc, k, cs);
      }
      all = false;
    }
    if (all) break;
  }
  OST_CUDA(cudaEventRecord(ev, cs));
  OST_CUDA(cudaStreamWaitEvent(st, ev, 0));
  OST_CUDA(cudaEventDestroy(ev));
  return out;
}

// ---- batched multi-shift CG (FP32) ----
struct CgmScal {
  double delta[BATCH_MAX], omega[BATCH_MAX], omega_prev[BATCH_MAX], gamma[BATCH_MAX], bnorm2[BATCH_MAX];
  double zi[BATCH_MAX][CGM_MAX_SHIFTS], zii[BATCH_MAX][CGM_MAX_SHIFTS], ziii[BATCH_MAX][CGM_MAX_SHIFTS];
  double omk[BATCH_MAX][CGM_MAX_SHIFTS], gak[BATCH_MAX][CGM_MAX_SHIFTS];
  double shift[CGM_MAX_SHIFTS];
  double m2, stop2;        // stop: sqrt(delta zii^2 / |b|^2) < 0.95 res
  int flag[BATCH_MAX][CGM_MAX_SHIFTS], flag_next[BATCH_MAX][CGM_MAX_SHIFTS];
  int done[BATCH_MAX], iter[BATCH_MAX];
  int nrhs, nshift, max_iter;
};

OST_D unsigned cgm_mask(const CgmScal* sc) {
  unsigned m = 0;
  for (int r = 0; r < sc->nrhs; ++r)
    if (!(*(volatile const int*)&sc->done[r])) m |= 1u << r;
  return m;
}

template <int NR, int PH>
__global__ void __launch_bounds__(BT)
k_cgm_doe(Geom g, LinkView<float2> u, const void* __restrict__ ph, const float2* __restrict__ p, float2* __restrict__ t,
          long vs, const CgmScal* sc) {
  const unsigned mask = cgm_mask(sc);
  if (!mask) return;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.sizeh) return;
  float2 aux[NR][3];
  hop_batch<NR, 1, PH>(g, u, p, vs, ph, idx, mask, aux);
#pragma unroll
  for (int k = 0; k < NR; ++k) {
    if (!(mask >> k & 1u)) continue;
#pragma unroll
    for (int c = 0; c < 3; ++c)
      t[k * vs + c * long(g.sizeh) + idx] = make_float2(0.5f * aux[k][c].x, 0.5f * aux[k][c].y);
  }
}

// s = m2 p - D_eo t ; alpha = <p,s> ; then the shifted recurrences
// (inverter_multishift_full.c:116-137)
template <int NR, int PH>
__global__ void __launch_bounds__(BT)
k_cgm_deo_dot(Geom g, LinkView<float2> u, const void* __restrict__ ph, const float2* __restrict__ t,
              const float2* __restrict__ p, float2* __restrict__ s, long vs, CgmScal* sc, ReduceWs ws) {
  const unsigned mask = cgm_mask(sc);
  if (!mask) return;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  float v[NR];
#pragma unroll
  for (int k = 0; k < NR; ++k) v[k] = 0.f;
  if (idx < g.sizeh) {
    const float m2 = float(sc->m2);
    float2 aux[NR][3];
    hop_batch<NR, 0, PH>(g, u, t, vs, ph, idx, mask, aux);
#pragma unroll
    for (int k = 0; k < NR; ++k) {
      if (!(mask >> k & 1u)) continue;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const long q = k * vs + c * long(g.sizeh) + idx;
        float2 pv = p[q];
        float2 r = make_float2(fmaf(pv.x, m2, -0.5f * aux[k][c].x), fmaf(pv.y, m2, -0.5f * aux[k][c].y));
        s[q] = r;
        v[k] = fmaf(pv.x, r.x, fmaf(pv.y, r.y, v[k]));
      }
    }
  }
  double tot[NR];
  if (grid_reduce_f32w<NR>(v, ws, tot)) {
    for (int r = 0; r < sc->nrhs; ++r) {
      if (!(mask >> r & 1u)) continue;
      for (int k = 0; k < sc->nshift; ++k) sc->flag[r][k] = sc->flag_next[r][k];
      const double alpha = tot[r];
      sc->omega_prev[r] = sc->omega[r];
      const double om = -sc->delta[r] / alpha, omp = sc->omega_prev[r], ga = sc->gamma[r];
      sc->omega[r] = om;
      for (int k = 0; k < sc->nshift; ++k) {
        if (!sc->flag[r][k]) continue;
        const double zi = sc->zi[r][k], zii = sc->zii[r][k];
        const double z3 = (zi * zii * omp) / (om * ga * (zi - zii) + zi * omp * (1.0 - sc->shift[k] * om));
        sc->ziii[r][k] = z3;
        sc->omk[r][k] = om * z3 / zii;
      }
    }
  }
}

// r += omega s ; lambda = |r|^2 ; gamma = lambda/delta ; gamma_k ; freeze
// decisions for the next iteration (inverter_multishift_full.c:139-171)
template <int NR>
__global__ void k_cgm_r(float4* __restrict__ r, const float4* __restrict__ s, long n4, long vs4, CgmScal* sc,
                        ReduceWs ws) {
  const unsigned mask = cgm_mask(sc);
  if (!mask) return;
  float om[NR], v[NR];
#pragma unroll
  for (int k = 0; k < NR; ++k) { om[k] = float(sc->omega[k]); v[k] = 0.f; }
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n4; i += long(gridDim.x) * blockDim.x) {
#pragma unroll
    for (int k = 0; k < NR; ++k) {
      if (!(mask >> k & 1u)) continue;
      const long q = k * vs4 + i;
      float4 rv = r[q], sv = s[q];
      rv.x = fmaf(om[k], sv.x, rv.x); rv.y = fmaf(om[k], sv.y, rv.y);
      rv.z = fmaf(om[k], sv.z, rv.z); rv.w = fmaf(om[k], sv.w, rv.w);
      r[q] = rv;
      v[k] = fmaf(rv.x, rv.x, fmaf(rv.y, rv.y, fmaf(rv.z, rv.z, fmaf(rv.w, rv.w, v[k]))));
    }
  }
  double tot[NR];
  if (grid_reduce_f32w<NR>(v, ws, tot)) {
    for (int r2 = 0; r2 < sc->nrhs; ++r2) {
      if (!(mask >> r2 & 1u)) continue;
      const double lambda = tot[r2], delta = sc->delta[r2], om2 = sc->omega[r2];
      const double gam = lambda / delta;
      sc->gamma[r2] = gam;
      int any = 0;
      for (int k = 0; k < sc->nshift; ++k) {
        if (!sc->flag[r2][k]) { sc->flag_next[r2][k] = 0; continue; }
        sc->gak[r2][k] = gam * sc->ziii[r2][k] * sc->omk[r2][k] / (sc->zii[r2][k] * om2);
        const double zii = sc->zii[r2][k];
        const int keep = !(delta * zii * zii < sc->stop2 * sc->bnorm2[r2]);
        sc->flag_next[r2][k] = keep;
        any |= keep;
        sc->zi[r2][k] = zii;
        sc->zii[r2][k] = sc->ziii[r2][k];
      }
      sc->delta[r2] = lambda;
      sc->iter[r2] += 1;
      if (!any || sc->iter[r2] >= sc->max_iter) sc->done[r2] = 1;
    }
  }
}

// p = r + gamma p ; x_k -= omega_k ps_k ; ps_k = gamma_k ps_k + zeta_k r   (active shifts)
template <int NR>
OST_D void cgm_xp_body(float4* __restrict__ p, const float4* __restrict__ r, float4* __restrict__ xs,
                       float4* __restrict__ ps, long n4, long vs4, const CgmScal* sc, int was_active_mask) {
  // systems that were active when this iteration started: their flag arrays
  // hold this iteration's active shifts
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n4; i += long(gridDim.x) * blockDim.x) {
    for (int rr = 0; rr < sc->nrhs; ++rr) {
      if (!(was_active_mask >> rr & 1u)) continue;
      const long q = rr * vs4 + i;
      const float4 rv = r[q];
      float4 pv = p[q];
      const float ga = float(sc->gamma[rr]);
      p[q] = make_float4(fmaf(ga, pv.x, rv.x), fmaf(ga, pv.y, rv.y), fmaf(ga, pv.z, rv.z), fmaf(ga, pv.w, rv.w));
      for (int k = 0; k < sc->nshift; ++k) {
        if (!sc->flag[rr][k]) continue;
        const long qk = (long(rr) * sc->nshift + k) * vs4 + i;
        float4 xv = xs[qk], pk = ps[qk];
        const float om = float(sc->omk[rr][k]), gk = float(sc->gak[rr][k]), z = float(sc->ziii[rr][k]);
        xv.x = fmaf(-om, pk.x, xv.x); xv.y = fmaf(-om, pk.y, xv.y);
        xv.z = fmaf(-om, pk.z, xv.z); xv.w = fmaf(-om, pk.w, xv.w);
        xs[qk] = xv;
        ps[qk] = make_float4(fmaf(gk, pk.x, z * rv.x), fmaf(gk, pk.y, z * rv.y), fmaf(gk, pk.z, z * rv.z),
                             fmaf(gk, pk.w, z * rv.w));
      }
    }
  }
}

// the active-system mask entering an iteration, kept on the device for k_cgm_xp
__global__ void k_cgm_snapshot(const CgmScal* sc, int* mask_out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *mask_out = int(cgm_mask(sc));
}

template <int NR>
__global__ void k_cgm_xp_dev(float4* __restrict__ p, const float4* __restrict__ r, float4* __restrict__ xs,
                             float4* __restrict__ ps, long n4, long vs4, const CgmScal* sc, const int* mask_in) {
  const int m = *mask_in;
  if (!m) return;
  cgm_xp_body<NR>(p, r, xs, ps, n4, vs4, sc, m);
}

namespace {

template <int NR>
void enqueue_cgm_iteration(const CgmBatchBuffers& B, CgmScal* sc, int* snap, cudaStream_t st) {
  const Geom& g = rt().g;
  LinkView<float2> u{B.u32, g.sizeh, 6};
  const int nb = blocks_for(g.sizeh, BT);
  const long n = 3L * g.sizeh, n4 = n / 2;
  const int gr = reduce_grid(n4);
  ReduceWs ws = reduce_ws(NR, nb > gr ? nb : gr);
  k_cgm_snapshot<<<1, 32, 0, st>>>(sc, snap);
  if (B.ph32_mode == PH_SIGN8) {
    k_cgm_doe<NR, PH_SIGN8><<<nb, BT, 0, st>>>(g, u, B.ph32, B.p, B.t, n, sc);
    k_cgm_deo_dot<NR, PH_SIGN8><<<nb, BT, 0, st>>>(g, u, B.ph32, B.t, B.p, B.s, n, sc, ws);
  } else {
    k_cgm_doe<NR, PH_ANGLE><<<nb, BT, 0, st>>>(g, u, B.ph32, B.p, B.t, n, sc);
    k_cgm_deo_dot<NR, PH_ANGLE><<<nb, BT, 0, st>>>(g, u, B.ph32, B.t, B.p, B.s, n, sc, ws);
  }
  k_cgm_r<NR><<<gr, RED_THREADS, 0, st>>>(reinterpret_cast<float4*>(B.r), reinterpret_cast<const float4*>(B.s), n4,
                                          n4, sc, ws);
  k_cgm_xp_dev<NR><<<gr, RED_THREADS, 0, st>>>(reinterpret_cast<float4*>(B.p), reinterpret_cast<const float4*>(B.r),
                                               reinterpret_cast<float4*>(B.xs), reinterpret_cast<float4*>(B.ps), n4,
                                               n4, sc, snap);
}

}  // namespace

__global__ void k_cgm_copy_f(float2* __restrict__ dst, const float2* __restrict__ src, long n) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) dst[i] = src[i];
}

CgmBatchResult batched_cgm_f32(const CgmBatchBuffers& B, double mass2, const double* shifts, double res,
                               int max_iter, cudaStream_t st) {
  CgmBatchResult out;
  memset(&out, 0, sizeof(out));
  const Geom& g = rt().g;
  const long n = 3L * g.sizeh;
  const int NR = B.nrhs, NK = B.nshift;
  char* ws = static_cast<char*>(workspace(WS_CGM, sizeof(CgmScal) + 1024));
  if (!ws) return out;
  CgmScal* sc = reinterpret_cast<CgmScal*>(ws);
  int* snap = reinterpret_cast<int*>(ws + sizeof(CgmScal) + 64);
  double* norms = reinterpret_cast<double*>(ws + sizeof(CgmScal) + 128);
  {
    const int nb = blocks_for(g.sizeh, BT), gr = reduce_grid(n);
    reduce_ws(BATCH_MAX, nb > gr ? nb : gr);
  }
  CgmScal* h = nullptr;
  OST_CUDA(cudaMallocHost(&h, sizeof(CgmScal)));
  memset(h, 0, sizeof(CgmScal));
  h->nrhs = NR; h->nshift = NK; h->max_iter = max_iter; h->m2 = mass2;
  h->stop2 = (0.95 * res) * (0.95 * res);
  for (int k = 0; k < NK; ++k) h->shift[k] = shifts[k];
  for (int r = 0; r < NR; ++r) {
    h->omega[r] = 1.0; h->gamma[r] = 0.0;
    for (int k = 0; k < NK; ++k) {
      h->zi[r][k] = 1.0; h->zii[r][k] = 1.0; h->gak[r][k] = 0.0;
      h->flag[r][k] = 1; h->flag_next[r][k] = 1;
    }
  }
  // r = p = b ; x = 0 ; ps_k = b ; delta = |b|^2
  for (int r = 0; r < NR; ++r) {
    k_cgm_copy_f<<<8 * rt().num_sms, 256, 0, st>>>(B.r + r * n, B.b + r * n, n);
    k_cgm_copy_f<<<8 * rt().num_sms, 256, 0, st>>>(B.p + r * n, B.b + r * n, n);
    for (int k = 0; k < NK; ++k)
      k_cgm_copy_f<<<8 * rt().num_sms, 256, 0, st>>>(B.ps + (long(r) * NK + k) * n, B.b + r * n, n);
    blas_norm2<float>(B.b + r * n, n, norms + r, st);
  }
  blas_zero<float>(B.xs, long(NR) * NK * n, st);
  double hn[BATCH_MAX];
  OST_CUDA(cudaMemcpyAsync(hn, norms, NR * sizeof(double), cudaMemcpyDeviceToHost, st));
  OST_CUDA(cudaStreamSynchronize(st));
  for (int r = 0; r < NR; ++r) { h->delta[r] = hn[r]; h->bnorm2[r] = hn[r]; }
  OST_CUDA(cudaMemcpyAsync(sc, h, sizeof(CgmScal), cudaMemcpyHostToDevice, st));
  // capture a chunk of iterations once per call (the buffers change per call)
  const int chunk = 8;
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  const unsigned long long counted = g_kernel_launches;
  OST_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  for (int c = 0; c < chunk; ++c) {
    switch (NR) {
      case 1: enqueue_cgm_iteration<1>(B, sc, snap, st); break;
      case 2: enqueue_cgm_iteration<2>(B, sc, snap, st); break;
      case 3: enqueue_cgm_iteration<3>(B, sc, snap, st); break;
      default: enqueue_cgm_iteration<4>(B, sc, snap, st); break;
    }
  }
  OST_CUDA(cudaStreamEndCapture(st, &graph));
  g_kernel_launches = counted;
  OST_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  cudaGraphDestroy(graph);
  int dn[BATCH_MAX];
  for (int guard = 0; guard < 1000000 && !error_code(); ++guard) {
    OST_CUDA(cudaGraphLaunch(exec, st));
    g_kernel_launches += 5ull * chunk;
    OST_CUDA(cudaMemcpyAsync(dn, sc->done, NR * sizeof(int), cudaMemcpyDeviceToHost, st));
    OST_CUDA(cudaStreamSynchronize(st));
    bool all = true;
    for (int r = 0; r < NR; ++r) all = all && dn[r];
    if (all) break;
  }
  OST_CUDA(cudaMemcpyAsync(h, sc, sizeof(CgmScal), cudaMemcpyDeviceToHost, st));
  OST_CUDA(cudaStreamSynchronize(st));
  for (int r = 0; r < NR; ++r) out.iters[r] = h->iter[r];
  cudaGraphExecDestroy(exec);
  cudaFreeHost(h);
  return out;
}

}  // namespace ost
