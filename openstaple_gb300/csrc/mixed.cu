// mixed.cu -- mixed-precision CG on (M^+M + shift): the iteration runs in
// FP32 (links, vectors, Dslash; reductions accumulate in FP64), the solution
// accumulates in FP64, and the residual is periodically recomputed in FP64
// ("reliable updates", the reference's "magic touch", inverter_mixedp.c:41-181,
// after arXiv:0911.3191).
//
// Per iteration four kernels run, all reading their scalars from device
// memory (MixScal), so a chunk of iterations is captured once as a CUDA graph
// and replayed; the host polls the flags once per chunk.  Each kernel returns
// immediately when the recursion has converged (done) or asks for a reliable
// update (need_rel), so replaying a chunk past either point does no work.
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>
#include "autotune.cuh"
#include "dslash.cuh"
#include "kernels.cuh"
#include "mixed.cuh"
#include "reduce.cuh"
#include "runtime.cuh"

namespace ost {

static constexpr int MX_THREADS = 128;

OST_D bool halted(const MixScal* s) { return (*(volatile const int*)&s->done) | (*(volatile const int*)&s->need_rel); }

// ---- preparation kernels ----
// blockIdx.y = link plane (direction x 6 entries of rows 0-1); x runs over
// the half lattice.  With u_lo, also the lo parts of the double-float links
// from the same FP64 loads.
__global__ void k_links_f32(const double2* __restrict__ u64, float2* __restrict__ u32, float2* __restrict__ u_lo,
                            long sh) {
  const int plane = blockIdx.y;
  const int dir = plane / 6, k = plane - 6 * (plane / 6);
  const double2* src = u64 + (long(dir) * 9 + k) * sh;
  float2* hi = u32 + long(plane) * sh;
  float2* lo = u_lo ? u_lo + long(plane) * sh : nullptr;
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < sh; i += long(gridDim.x) * blockDim.x) {
    const double2 v = __ldcs(src + i);
    const float hx = float(v.x), hy = float(v.y);
    hi[i] = make_float2(hx, hy);
    if (lo) lo[i] = make_float2(df_lo_part(v.x, hx), df_lo_part(v.y, hy));
  }
}

void links_to_f32_compact(const double2* u64, float2* u32, long sh, cudaStream_t st, float2* u_lo) {
  const long bx = (sh + 255) / 256;
  k_links_f32<<<dim3(unsigned(bx < 128 ? bx : 128), 48), 256, 0, st>>>(u64, u32, u_lo, sh);
  OST_LAUNCH_CHECK();
}

// one thread per (direction, site): the six FP32 entries of the two rows
// (compact layout [dir][6][sizeh]) -> the link's 16- and 8-byte words
__global__ void k_links_q16(const float2* __restrict__ u32, uint4* __restrict__ a, uint2* __restrict__ b, long sh) {
  const long n = 8L * sh;
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    const int dir = int(i / sh);
    const long idx = i - long(dir) * sh;
    unsigned w[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float2 v = __ldcs(u32 + (long(dir) * 6 + k) * sh + idx);
      w[k] = q16_encode_f32(v.x) | (q16_encode_f32(v.y) << 16);
    }
    a[i] = make_uint4(w[0], w[1], w[2], w[3]);
    b[i] = make_uint2(w[4], w[5]);
  }
}

void links_to_q16(const float2* u32, uint4* a, uint2* b, long sh, cudaStream_t st) {
  k_links_q16<<<8 * rt().num_sms, 256, 0, st>>>(u32, a, b, sh);
  OST_LAUNCH_CHECK();
}

__global__ void k_signs(const double* __restrict__ ph, unsigned char* sg, int* all_exact, long n) {
  const unsigned long long PI = 0x400921FB54442D18ull;
  bool ok = true;
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(ph[i]);
    sg[i] = (b == PI) ? 1 : 0;
    ok = ok && (b == 0 || b == PI);
  }
  if (!__all_sync(0xffffffffu, ok) && (threadIdx.x & 31) == 0) atomicAnd(all_exact, 0);
}

void phases_to_signs(const double* ph64, unsigned char* sg, int* all_exact, long sh, cudaStream_t st) {
  k_signs<<<4 * rt().num_sms, 256, 0, st>>>(ph64, sg, all_exact, 8 * sh);
  OST_LAUNCH_CHECK();
}

__global__ void k_ph32(const double* __restrict__ ph, float* out, long n) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x)
    out[i] = float(ph[i]);
}

void phases_to_f32(const double* ph64, float* ph32, long sh, cudaStream_t st) {
  k_ph32<<<4 * rt().num_sms, 256, 0, st>>>(ph64, ph32, 8 * sh);
  OST_LAUNCH_CHECK();
}

// ---- FP32 iteration kernels ----
// One thread per site; HB hops' loads in flight per thread.

// t = D_oe p (any block size up to 256: the autotuner picks the shape)
template <int PH, typename LV, int HB>
__global__ void __launch_bounds__(256)
k_mx_doe(Geom g, LV u, const void* __restrict__ ph, const float2* __restrict__ p, float2* __restrict__ t,
         const MixScal* sc) {
  if (halted(sc)) return;   // set by k_mx_update, two launches back
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  // launched early (programmatic dependent launch): fetch the links, which
  // no kernel of the solve writes, while the previous kernel finishes
  if (idx < g.sizeh) prefetch_links<1>(g, u, idx);
  pdl_wait();               // p from k_mx_pupdate
  pdl_trigger();
  if (idx >= g.sizeh) return;
  float2 aux[3];
  hop_fb<1, PH, LV, HB>(g, u, p, ph, idx, aux);
#pragma unroll
  for (int c = 0; c < 3; ++c) t[c * long(g.sizeh) + idx] = make_float2(0.5f * aux[c].x, 0.5f * aux[c].y);
}

// s = m2 p - D_eo t ; pAp = Re<p, s> ; alpha = delta / pAp
template <int PH, typename LV, int HB>
__global__ void __launch_bounds__(MX_THREADS)
k_mx_deo_dot(Geom g, LV u, const void* __restrict__ ph, const float2* __restrict__ t, const float2* __restrict__ p,
             float2* __restrict__ s, MixScal* sc, ReduceWs ws) {
  if (halted(sc)) return;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < g.sizeh) prefetch_links<0>(g, u, idx);   // as in k_mx_doe
  pdl_wait();               // t from k_mx_doe
  pdl_trigger();
  float v[1] = {0.0f};
  if (idx < g.sizeh) {
    const float m2 = float(sc->m2);
    float2 aux[3];
    hop_fb<0, PH, LV, HB>(g, u, t, ph, idx, aux);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long k = c * long(g.sizeh) + idx;
      float2 pv = p[k];
      float2 r = make_float2(fmaf(pv.x, m2, -0.5f * aux[c].x), fmaf(pv.y, m2, -0.5f * aux[c].y));
      s[k] = r;
      v[0] = fmaf(pv.x, r.x, fmaf(pv.y, r.y, v[0]));
    }
  }
  double tot[1];
  if (grid_reduce_f32w<1>(v, ws, tot)) {
    sc->pAp = tot[0];
    sc->alpha = sc->delta / tot[0];
  }
}

// x_f += alpha p ; unless a reliable update is due: r -= alpha s, lambda = |r|^2,
// beta = lambda / delta, delta = lambda.
__global__ void k_mx_update(float4* __restrict__ xf, float4* __restrict__ r, const float4* __restrict__ p,
                            const float4* __restrict__ s, long n4, MixScal* sc, ReduceWs ws) {
  if (halted(sc)) return;   // set by this kernel, four launches back
  const long stride = long(gridDim.x) * blockDim.x;
  // launched early: p, x_f and r are not written by k_mx_deo_dot; one lane
  // in eight prefetches the 128-byte lines of its neighbours' elements
  if ((threadIdx.x & 7) == 0)
    for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n4; i += stride) {
      prefetch_l2(p + i);
      prefetch_l2(xf + i);
      prefetch_l2(r + i);
    }
  pdl_wait();               // s and alpha from k_mx_deo_dot
  pdl_trigger();
  const double delta = sc->delta;
  const double lm = sc->last_max > delta ? sc->last_max : delta;
  const bool rel = sc->every > 0 ? ((sc->iter + 1) % sc->every == 0) : (delta < sc->frac * lm);
  const float a = float(sc->alpha);
  float v[1] = {0.0f};
  // two elements per pass, all loads issued before use
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n4; i += 2 * stride) {
    const long j = i + stride;
    const bool two = j < n4;
    float4 pv0 = p[i], xv0 = xf[i], pv1, xv1, sv0, rv0, sv1, rv1;
    if (two) { pv1 = p[j]; xv1 = xf[j]; }
    if (!rel) { sv0 = s[i]; rv0 = r[i]; if (two) { sv1 = s[j]; rv1 = r[j]; } }
    xv0.x = fmaf(a, pv0.x, xv0.x); xv0.y = fmaf(a, pv0.y, xv0.y); xv0.z = fmaf(a, pv0.z, xv0.z); xv0.w = fmaf(a, pv0.w, xv0.w);
    xf[i] = xv0;
    if (two) {
      xv1.x = fmaf(a, pv1.x, xv1.x); xv1.y = fmaf(a, pv1.y, xv1.y); xv1.z = fmaf(a, pv1.z, xv1.z); xv1.w = fmaf(a, pv1.w, xv1.w);
      xf[j] = xv1;
    }
    if (!rel) {
      rv0.x = fmaf(-a, sv0.x, rv0.x); rv0.y = fmaf(-a, sv0.y, rv0.y); rv0.z = fmaf(-a, sv0.z, rv0.z); rv0.w = fmaf(-a, sv0.w, rv0.w);
      r[i] = rv0;
      v[0] = fmaf(rv0.x, rv0.x, fmaf(rv0.y, rv0.y, fmaf(rv0.z, rv0.z, fmaf(rv0.w, rv0.w, v[0]))));
      if (two) {
        rv1.x = fmaf(-a, sv1.x, rv1.x); rv1.y = fmaf(-a, sv1.y, rv1.y); rv1.z = fmaf(-a, sv1.z, rv1.z); rv1.w = fmaf(-a, sv1.w, rv1.w);
        r[j] = rv1;
        v[0] = fmaf(rv1.x, rv1.x, fmaf(rv1.y, rv1.y, fmaf(rv1.z, rv1.z, fmaf(rv1.w, rv1.w, v[0]))));
      }
    }
  }
  double tot[1];
  if (grid_reduce_f32w<1>(v, ws, tot)) {
    sc->iter += 1;
    sc->last_max = lm;
    if (rel) {
      sc->need_rel = 1;
    } else {
      sc->lambda = tot[0];
      sc->beta = tot[0] / delta;
      sc->delta = tot[0];
      if (tot[0] <= sc->target2 || sc->iter >= sc->max_iter) sc->done = 1;
    }
  }
}

// p = r + beta p
__global__ void k_mx_pupdate(float4* __restrict__ p, const float4* __restrict__ r, long n4, const MixScal* sc,
                             int guarded) {
  const long stride = long(gridDim.x) * blockDim.x;
  if (guarded && (threadIdx.x & 7) == 0)   // launched early: p is not written by k_mx_update
    for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n4; i += stride) prefetch_l2(p + i);
  pdl_wait();               // r, beta and the flags from k_mx_update
  if (guarded && halted(sc)) return;
  pdl_trigger();
  const float b = float(sc->beta);
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n4; i += 2 * stride) {
    const long j = i + stride;
    float4 pv = p[i], rv = r[i], pw, rw;
    if (j < n4) { pw = p[j]; rw = r[j]; }
    p[i] = make_float4(fmaf(b, pv.x, rv.x), fmaf(b, pv.y, rv.y), fmaf(b, pv.z, rv.z), fmaf(b, pv.w, rv.w));
    if (j < n4) p[j] = make_float4(fmaf(b, pw.x, rw.x), fmaf(b, pw.y, rw.y), fmaf(b, pw.z, rw.z), fmaf(b, pw.w, rw.w));
  }
}

// ---- FP64 reliable-update kernels ----
// x += x_f ; x_f = 0
__global__ void k_mx_accumulate(double2* __restrict__ x, float2* __restrict__ xf, long n) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    float2 f = xf[i];
    double2 d = x[i];
    x[i] = make_double2(d.x + double(f.x), d.y + double(f.y));
    xf[i] = make_float2(0.f, 0.f);
  }
}

// r64 = b - Ax ; r = (float) r64 ; lambda = |r|^2 ; true_r2 = |r64|^2
// mode 0: initial (p = r, delta = lambda); mode 1: reliable update
// (delta = lambda, last_max = 0, and beta for p = r + beta p below).
//
// The reference's reliable update keeps beta = lambda/delta
// (inverter_mixedp.c:124-150).  That formula assumes the new residual is
// the recursed one; a recomputed residual that differs from it by more than
// the recursion's own progress (a late update, or sloppy links coarser than
// FP32) then makes beta large and the next direction repeats the last one,
// which can stall the solve.  Here beta = -<r, s>/<p, s> with s = A p of the
// last iteration (Hestenes-Stiefel), which keeps the next direction
// A-conjugate to the last one whatever the size of the correction; with
// FP32 links it gives the same iteration counts as the reference's formula.
__global__ void k_mx_residual(const double2* __restrict__ b, const double2* __restrict__ ax, double2* __restrict__ r64,
                              float2* __restrict__ r, float2* __restrict__ p, const float2* __restrict__ s, long n,
                              MixScal* sc, ReduceWs ws, int mode) {
  double v[3] = {0.0, 0.0, 0.0};
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    double2 bb = b[i], a = ax[i];
    double2 d = make_double2(bb.x - a.x, bb.y - a.y);
    r64[i] = d;
    float2 f = make_float2(float(d.x), float(d.y));
    r[i] = f;
    if (mode == 0) {
      p[i] = f;
    } else {
      const float2 sv = s[i];
      v[2] += double(f.x) * sv.x + double(f.y) * sv.y;
    }
    v[0] += double(f.x) * f.x + double(f.y) * f.y;
    v[1] += d.x * d.x + d.y * d.y;
  }
  double tot[3];
  if (grid_reduce<3>(v, ws, tot)) {
    sc->true_r2 = tot[1];
    sc->lambda = tot[0];
    if (mode == 0) {
      sc->delta = tot[0];
      sc->beta = 0.0;
    } else {
      // no iteration yet (or a degenerate one): restart along r
      sc->beta = (sc->iter > 0 && sc->pAp > 0.0) ? -tot[2] / sc->pAp : 0.0;
      sc->delta = tot[0];
      sc->n_rel += 1;
    }
    sc->last_max = 0.0;
    sc->need_rel = 0;
    sc->done = (tot[0] <= sc->target2 || sc->iter >= sc->max_iter) ? 1 : 0;
  }
}

// ---- host engine ----
namespace {

struct GraphCache {
  cudaGraphExec_t exec = nullptr;
  MixedBuffers key{};
  int chunk = 0;
  MixScal* sc = nullptr;
  unsigned long long epoch = 0;
  int hop_shapes = -1;
};
GraphCache g_cache;
cudaStream_t g_cap = nullptr;
MixScal* g_host = nullptr;

bool same_key(const MixedBuffers& a, const MixedBuffers& b) {
  return a.u32 == b.u32 && a.ph32 == b.ph32 && a.ph32_mode == b.ph32_mode && a.u32_compact == b.u32_compact &&
         a.q16 == b.q16 && a.uq.a == b.uq.a && a.uq.b == b.uq.b && a.r == b.r && a.p == b.p && a.s == b.s &&
         a.xf == b.xf && a.t == b.t;
}

void fp64_mdagm(const MixedBuffers& B, double2* out, const double2* in, double2* tmp, double m2, cudaStream_t st) {
  DslashArgs<double> a;
  a.phase_mode = PH_ANGLE;
  a.u = B.u64;
  a.phases = B.ph64;
  a.stream = st;
  a.compact_links = 0;
  a.parity = 1; a.epilogue = EPI_PLAIN; a.out = tmp; a.in = in; a.in0 = nullptr; a.mass2 = 0;
  launch_dslash<double>(a);
  a.parity = 0; a.epilogue = EPI_MDAGM; a.out = out; a.in = tmp; a.in0 = in; a.mass2 = m2;
  launch_dslash<double>(a);
}

// Launch shapes the autotuner tries (the first is the default): block size
// and hops in flight.  The block size of k_mx_deo_dot fixes the summation
// order of <p, Ap>, so only its hops in flight are tuned.
struct HopShape {
  int threads, hb;
};
constexpr int N_DOE_SHAPES = 7, N_DEO_SHAPES = 3;
static const HopShape kDoeShapes[N_DOE_SHAPES] = {{MX_THREADS, 1}, {256, 1}, {64, 1}, {MX_THREADS, 2},
                                                  {MX_THREADS, 4}, {256, 2}, {64, 2}};
static const HopShape kDeoShapes[N_DEO_SHAPES] = {{MX_THREADS, 1}, {MX_THREADS, 2}, {MX_THREADS, 4}};

// Calls f with the view of the sloppy links the FP32 iteration reads.
template <typename F>
void with_sloppy_links(const MixedBuffers& B, F&& f) {
  if (B.q16) f(B.uq);
  else f(LinkView<float2>{B.u32, rt().g.sizeh, B.u32_compact ? 6 : 9});
}

template <int HB>
void launch_mx_doe_t(int threads, const MixedBuffers& B, const MixScal* sc, cudaStream_t st) {
  const Geom& g = rt().g;
  const int nb = blocks_for(g.sizeh, threads);
  with_sloppy_links(B, [&](const auto& u) {
    typedef typename std::decay<decltype(u)>::type LV;
    if (B.ph32_mode == PH_SIGN8)
      launch_pdl(k_mx_doe<PH_SIGN8, LV, HB>, nb, threads, st, g, u, B.ph32, B.p, B.t, sc);
    else launch_pdl(k_mx_doe<PH_ANGLE, LV, HB>, nb, threads, st, g, u, B.ph32, B.p, B.t, sc);
  });
}

void launch_mx_doe(HopShape sh, const MixedBuffers& B, const MixScal* sc, cudaStream_t st) {
  if (sh.hb == 4) launch_mx_doe_t<4>(sh.threads, B, sc, st);
  else if (sh.hb == 2) launch_mx_doe_t<2>(sh.threads, B, sc, st);
  else launch_mx_doe_t<1>(sh.threads, B, sc, st);
}

template <int HB>
void launch_mx_deo_dot_t(const MixedBuffers& B, MixScal* sc, ReduceWs ws, cudaStream_t st) {
  const Geom& g = rt().g;
  const int nb = blocks_for(g.sizeh, MX_THREADS);
  with_sloppy_links(B, [&](const auto& u) {
    typedef typename std::decay<decltype(u)>::type LV;
    if (B.ph32_mode == PH_SIGN8)
      launch_pdl(k_mx_deo_dot<PH_SIGN8, LV, HB>, nb, MX_THREADS, st, g, u, B.ph32, B.t, B.p, B.s, sc, ws);
    else launch_pdl(k_mx_deo_dot<PH_ANGLE, LV, HB>, nb, MX_THREADS, st, g, u, B.ph32, B.t, B.p, B.s, sc, ws);
  });
}

void launch_mx_deo_dot(HopShape sh, const MixedBuffers& B, MixScal* sc, ReduceWs ws, cudaStream_t st) {
  if (sh.hb == 4) launch_mx_deo_dot_t<4>(B, sc, ws, st);
  else if (sh.hb == 2) launch_mx_deo_dot_t<2>(B, sc, ws, st);
  else launch_mx_deo_dot_t<1>(B, sc, ws, st);
}

// blocks of the k_mx_deo_dot launch (the reductions' partial sums)
int mx_deo_blocks() { return blocks_for(rt().g.sizeh, MX_THREADS); }

int doe_variant(const MixedBuffers& B) { return (B.ph32_mode == PH_SIGN8) + 2 * (B.q16 != 0); }

HopShape mx_doe_shape(const MixedBuffers& B) {
  const int pick = autotune_cached(TUNE_MX_DOE, rt().g.sizeh, doe_variant(B));
  return kDoeShapes[pick > 0 && pick < N_DOE_SHAPES ? pick : 0];
}

HopShape mx_deo_shape(const MixedBuffers& B) {
  const int pick = autotune_cached(TUNE_MX_DEO, rt().g.sizeh, doe_variant(B));
  return kDeoShapes[pick > 0 && pick < N_DEO_SHAPES ? pick : 0];
}

// Tunes the launch shapes of both hops once per lattice and link format
// (t and s are scratch; the timing launches see a copy of the scalars with
// the solve running and write their <p, Ap> into that copy).  Returns a key
// of the chosen shapes for the graph cache.
int tune_mx_hops(const MixedBuffers& B, cudaStream_t st) {
  const int variant = doe_variant(B);
  const long sh = rt().g.sizeh;
  if (autotune_enabled() && (autotune_cached(TUNE_MX_DOE, sh, variant) < 0 ||
                             autotune_cached(TUNE_MX_DEO, sh, variant) < 0)) {
    MixScal h;
    memset(&h, 0, sizeof(h));
    h.delta = 1.0;
    MixScal* sc = static_cast<MixScal*>(autotune_scalars(&h, sizeof(h), st));
    if (sc) {
      autotune_pick(TUNE_MX_DOE, sh, variant, N_DOE_SHAPES,
                    [&](int c) { launch_mx_doe(kDoeShapes[c], B, sc, st); }, st);
      ReduceWs ws = reduce_ws(1, mx_deo_blocks());
      autotune_pick(TUNE_MX_DEO, sh, variant, N_DEO_SHAPES,
                    [&](int c) { launch_mx_deo_dot(kDeoShapes[c], B, sc, ws, st); }, st);
    }
  }
  const int a = autotune_cached(TUNE_MX_DOE, sh, variant), b = autotune_cached(TUNE_MX_DEO, sh, variant);
  return (a < 0 ? 0 : a) * 16 + (b < 0 ? 0 : b);
}

void enqueue_iteration(const MixedBuffers& B, MixScal* sc, cudaStream_t st) {
  const Geom& g = rt().g;
  const long n4 = 3L * g.sizeh / 2;
  int gr = reduce_grid(n4);
  int gd = mx_deo_blocks();
  ReduceWs wsd = reduce_ws(1, gd > gr ? gd : gr);
  launch_mx_doe(mx_doe_shape(B), B, sc, st);
  launch_mx_deo_dot(mx_deo_shape(B), B, sc, wsd, st);
  g_kernel_launches += 2;
  launch_pdl(k_mx_update, gr, RED_THREADS, st, reinterpret_cast<float4*>(B.xf), reinterpret_cast<float4*>(B.r),
             reinterpret_cast<const float4*>(B.p), reinterpret_cast<const float4*>(B.s), n4, sc, wsd);
  launch_pdl(k_mx_pupdate, gr, RED_THREADS, st, reinterpret_cast<float4*>(B.p), reinterpret_cast<const float4*>(B.r),
             n4, static_cast<const MixScal*>(sc), 1);
  g_kernel_launches += 2;
}

// ---- the whole solve on the device ----
// One graph launch runs the iteration until the FP32 recursion has converged:
// a while node whose body is a captured chunk of iterations, then an if node
// that performs a due reliable update, then the loop test.  The two tests are
// single-thread kernels that set the nodes' conditions from the device
// scalars; the loop is bounded by a pass count beyond the iteration limit.
__global__ void k_mx_rel_test(cudaGraphConditionalHandle h_rel, const MixScal* sc) {
  cudaGraphSetConditional(h_rel, (sc->need_rel && !sc->done) ? 1u : 0u);
}

__global__ void k_mx_loop_test(cudaGraphConditionalHandle h_loop, const MixScal* sc, int* trips, int max_trips) {
  const int t = *trips + 1;
  *trips = t;
  int go = !sc->done;
  if (go && t >= max_trips) {
    *trips = -t;
    go = 0;
  }
  cudaGraphSetConditional(h_loop, go ? 1u : 0u);
}

// the reliable update of the host loop below, as stream work
void enqueue_reliable_update(const MixedBuffers& B, double m2, MixScal* sc, cudaStream_t cs) {
  const long n = 3L * rt().g.sizeh, n4 = n / 2;
  k_mx_accumulate<<<8 * rt().num_sms, 256, 0, cs>>>(B.x, B.xf, n);
  OST_LAUNCH_CHECK();
  if (B.use_df) df_mdagm(B.df, B.dfw, B.t64, B.x, m2, cs);
  else fp64_mdagm(B, B.t64, B.x, B.t64b, m2, cs);
  const int gr = reduce_grid(n);
  k_mx_residual<<<gr, RED_THREADS, 0, cs>>>(B.b, B.t64, B.r64, B.r, B.p, B.s, n, sc, reduce_ws(3, gr), 1);
  OST_LAUNCH_CHECK();
  k_mx_pupdate<<<reduce_grid(n4), RED_THREADS, 0, cs>>>(reinterpret_cast<float4*>(B.p),
                                                        reinterpret_cast<const float4*>(B.r), n4, sc, 0);
  OST_LAUNCH_CHECK();
}

// the nodes of g that no other node depends on
std::vector<cudaGraphNode_t> leaf_nodes(cudaGraph_t g) {
  size_t n = 0;
  std::vector<cudaGraphNode_t> leaves;
  if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return leaves;
  std::vector<cudaGraphNode_t> nodes(n);
  if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return leaves;
  for (cudaGraphNode_t v : nodes) {
    size_t d = 0;
    if (cudaGraphNodeGetDependentNodes(v, nullptr, nullptr, &d) == cudaSuccess && d == 0) leaves.push_back(v);
  }
  return leaves;
}

struct LoopCache {
  cudaGraphExec_t exec = nullptr;
  MixedBuffers key{};
  int chunk = 0, hop_shapes = -1, max_trips = 0;
  double m2 = 0;
  MixScal* sc = nullptr;
  unsigned long long epoch = 0;
};
LoopCache g_loop;

bool same_loop_key(const LoopCache& c, const MixedBuffers& B, const MixedOptions& o, MixScal* sc, int hop_shapes,
                   int max_trips) {
  return c.exec && same_key(c.key, B) && c.key.x == B.x && c.key.b == B.b && c.key.u64 == B.u64 &&
         c.key.ph64 == B.ph64 && c.key.t64 == B.t64 && c.key.r64 == B.r64 && c.key.t64b == B.t64b &&
         c.key.use_df == B.use_df && c.chunk == o.chunk && c.m2 == o.mass2 && c.sc == sc &&
         c.hop_shapes == hop_shapes && c.max_trips == max_trips && c.epoch == runtime_epoch();
}

// The executable graph of the device loop (cached per buffers and options),
// or nullptr where this device or driver cannot build it.
cudaGraphExec_t device_loop(const MixedBuffers& B, const MixedOptions& o, MixScal* sc, int* trips, int max_trips,
                            int hop_shapes, cudaStream_t cs) {
  if (same_loop_key(g_loop, B, o, sc, hop_shapes, max_trips)) return g_loop.exec;
  if (g_loop.exec) cudaGraphExecDestroy(g_loop.exec);
  g_loop.exec = nullptr;
  const unsigned long long counted = g_kernel_launches;   // building launches nothing
  // graph: while (h_loop) { chunk of iterations; k_mx_rel_test;
  //                         if (h_rel) { reliable update }; k_mx_loop_test }
  // Both condition-setting kernels sit directly in the while body.
  cudaGraph_t graph = nullptr;
  cudaGraphConditionalHandle h_loop{}, h_rel{};
  bool ok = cudaGraphCreate(&graph, 0) == cudaSuccess;
  ok = ok && cudaGraphConditionalHandleCreate(&h_loop, graph, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  ok = ok && cudaGraphConditionalHandleCreate(&h_rel, graph, 0, cudaGraphCondAssignDefault) == cudaSuccess;
  cudaGraphNodeParams wp{};
  cudaGraphNode_t wnode;
  if (ok) {
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = h_loop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    ok = cudaGraphAddNode(&wnode, graph, nullptr, nullptr, 0, &wp) == cudaSuccess;
  }
  cudaGraph_t body = ok ? wp.conditional.phGraph_out[0] : nullptr;
  // the chunk and the reliable-update test, captured into the body
  if (ok) {
    ok = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
         cudaSuccess;
    if (ok) {
      for (int k = 0; k < o.chunk; ++k) enqueue_iteration(B, sc, cs);
      k_mx_rel_test<<<1, 1, 0, cs>>>(h_rel, sc);
      ok = cudaStreamEndCapture(cs, &body) == cudaSuccess;
    }
  }
  std::vector<cudaGraphNode_t> leaves = ok ? leaf_nodes(body) : std::vector<cudaGraphNode_t>{};
  ok = ok && leaves.size() == 1;
  cudaGraphNodeParams ip{};
  cudaGraphNode_t inode, tnode;
  if (ok) {
    ip.type = cudaGraphNodeTypeConditional;
    ip.conditional.handle = h_rel;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    ok = cudaGraphAddNode(&inode, body, leaves.data(), nullptr, 1, &ip) == cudaSuccess;
  }
  if (ok) {   // the reliable update, captured into the if body
    cudaGraph_t ibody = ip.conditional.phGraph_out[0];
    ok = cudaStreamBeginCaptureToGraph(cs, ibody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
         cudaSuccess;
    if (ok) {
      enqueue_reliable_update(B, o.mass2, sc, cs);
      ok = cudaStreamEndCapture(cs, &ibody) == cudaSuccess;
    }
  }
  if (ok) {   // the loop test after the if node
    const MixScal* csc = sc;
    int mt = max_trips;
    void* args[] = {&h_loop, &csc, &trips, &mt};
    cudaKernelNodeParams kp{};
    kp.func = reinterpret_cast<void*>(k_mx_loop_test);
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(1);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    kp.extra = nullptr;
    ok = cudaGraphAddKernelNode(&tnode, body, &inode, 1, &kp) == cudaSuccess;
  }
  cudaGraphExec_t exec = nullptr;
  if (ok) ok = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
  if (graph) cudaGraphDestroy(graph);
  g_kernel_launches = counted;
  if (!ok) {
    if (exec) cudaGraphExecDestroy(exec);
    cudaGetLastError();
    return nullptr;
  }
  g_loop.exec = exec;
  g_loop.key = B;
  g_loop.chunk = o.chunk;
  g_loop.m2 = o.mass2;
  g_loop.sc = sc;
  g_loop.hop_shapes = hop_shapes;
  g_loop.max_trips = max_trips;
  g_loop.epoch = runtime_epoch();
  return exec;
}

__device__ int g_mx_trips;

int* device_loop_trips() {
  static int* p = nullptr;
  if (!p && cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_mx_trips) != cudaSuccess) {
    cudaGetLastError();
    p = nullptr;
  }
  return p;
}

}  // namespace

MixedResult mixed_cg(const MixedBuffers& B, const MixedOptions& o, MixScal* sc, cudaStream_t st) {
  MixedResult res{0, 0, NAN, 0};
  const Geom& g = rt().g;
  const long n = 3L * g.sizeh;
  if (!g_cap) {
    OST_CUDA(cudaStreamCreateWithFlags(&g_cap, cudaStreamNonBlocking));
    OST_CUDA(cudaMallocHost(&g_host, 2 * sizeof(MixScal)));
  }
  // order the private stream after the caller's stream
  cudaEvent_t ev;
  OST_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  OST_CUDA(cudaEventRecord(ev, st));
  OST_CUDA(cudaStreamWaitEvent(g_cap, ev, 0));
  cudaStream_t cs = g_cap;

  // |b|^2 and the initial residual from the FP64 guess
  MixScal init;
  memset(&init, 0, sizeof(init));
  init.m2 = o.mass2;
  init.frac = o.delta_frac;
  init.max_iter = o.max_iter;
  init.every = o.reliable_every;
  OST_CUDA(cudaMemcpyAsync(sc, &init, sizeof(MixScal), cudaMemcpyHostToDevice, cs));
  blas_norm2<double>(B.b, n, &sc->bnorm2, cs);
  blas_norm2<double>(B.x, n, &sc->true_r2, cs);     // |x0|^2, overwritten below
  OST_CUDA(cudaMemcpyAsync(g_host, sc, sizeof(MixScal), cudaMemcpyDeviceToHost, cs));
  OST_CUDA(cudaStreamSynchronize(cs));
  const double bn = g_host->bnorm2;
  const bool zero_guess = g_host->true_r2 == 0.0;
  if (!std::isfinite(bn) || !std::isfinite(g_host->true_r2)) {
    // a non-finite source or guess cannot converge: report failure at once
    // instead of iterating on NaNs up to max_iter
    OST_CUDA(cudaEventRecord(ev, cs));
    OST_CUDA(cudaStreamWaitEvent(st, ev, 0));
    OST_CUDA(cudaEventDestroy(ev));
    return res;
  }
  double fp32_target = o.safety * o.res;
  init.target2 = fp32_target * fp32_target * bn;
  init.bnorm2 = bn;
  OST_CUDA(cudaMemcpyAsync(sc, &init, sizeof(MixScal), cudaMemcpyHostToDevice, cs));
  blas_zero<float>(B.xf, n, cs);
  // r0 = b - A x0; a zero guess (the usual start) needs no operator application
  if (zero_guess) OST_CUDA(cudaMemsetAsync(B.t64, 0, n * sizeof(double2), cs));
  else if (B.use_df) df_mdagm(B.df, B.dfw, B.t64, B.x, o.mass2, cs);   // the closing residual is FP64
  else fp64_mdagm(B, B.t64, B.x, B.t64b, o.mass2, cs);
  {
    int gr = reduce_grid(n);
    k_mx_residual<<<gr, RED_THREADS, 0, cs>>>(B.b, B.t64, B.r64, B.r, B.p, B.s, n, sc, reduce_ws(3, gr), 0);
    OST_LAUNCH_CHECK();
  }

  // workspace used inside the captured chunk is allocated before capture
  {
    const int nb = mx_deo_blocks();
    const int gr = reduce_grid(n);
    reduce_ws(3, nb > gr ? nb : gr);   // the reliable updates' k_mx_residual sums 3 values
  }
  // launch shape of the D_oe (numerics-invariant), chosen before the capture
  const int hop_shapes = tune_mx_hops(B, cs);
  // (re)capture the iteration chunk
  if (!g_cache.exec || !same_key(g_cache.key, B) || g_cache.chunk != o.chunk || g_cache.sc != sc ||
      g_cache.epoch != runtime_epoch() || g_cache.hop_shapes != hop_shapes) {
    if (g_cache.exec) cudaGraphExecDestroy(g_cache.exec);
    g_cache.exec = nullptr;
    cudaGraph_t graph;
    const unsigned long long counted = g_kernel_launches;   // capture launches nothing
    OST_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < o.chunk; ++k) enqueue_iteration(B, sc, cs);
    OST_CUDA(cudaStreamEndCapture(cs, &graph));
    g_kernel_launches = counted;
    OST_CUDA(cudaGraphInstantiate(&g_cache.exec, graph, 0));
    cudaGraphDestroy(graph);
    g_cache.key = B;
    g_cache.chunk = o.chunk;
    g_cache.sc = sc;
    g_cache.epoch = runtime_epoch();
    g_cache.hop_shapes = hop_shapes;
  }

  const long n4 = n / 2;
  const double res2 = o.res * o.res * bn;
  // The recursion has converged: fold the FP32 correction in and measure the
  // FP64 true residual.  Returns true when the solve is finished; otherwise
  // the FP32 target is tightened and the iteration continues from the
  // recomputed residual (the closing residual acts as a reliable update).
  auto close_or_tighten = [&]() -> bool {
    k_mx_accumulate<<<8 * rt().num_sms, 256, 0, cs>>>(B.x, B.xf, n);
    OST_LAUNCH_CHECK();
    fp64_mdagm(B, B.t64, B.x, B.t64b, o.mass2, cs);
    int gr = reduce_grid(n);
    // mode 1 recomputes r, resets last_max and re-evaluates done
    k_mx_residual<<<gr, RED_THREADS, 0, cs>>>(B.b, B.t64, B.r64, B.r, B.p, B.s, n, sc, reduce_ws(3, gr), 1);
    OST_LAUNCH_CHECK();
    OST_CUDA(cudaMemcpyAsync(g_host, sc, sizeof(MixScal), cudaMemcpyDeviceToHost, cs));
    OST_CUDA(cudaStreamSynchronize(cs));
    const MixScal f = *g_host;
    res.iters = f.iter;
    res.n_reliable = f.n_rel - 1;   // the closing residual is not an update
    res.true_res = std::sqrt(f.true_r2 / bn);
    res.converged = f.true_r2 <= res2;
    if (res.converged || !o.guarantee || f.iter >= o.max_iter) return true;
    fp32_target *= 0.5;
    MixScal upd = f;
    upd.target2 = fp32_target * fp32_target * bn;
    upd.done = (f.lambda <= upd.target2) ? 1 : 0;
    OST_CUDA(cudaMemcpyAsync(sc, &upd, sizeof(MixScal), cudaMemcpyHostToDevice, cs));
    k_mx_pupdate<<<reduce_grid(n4), RED_THREADS, 0, cs>>>(reinterpret_cast<float4*>(B.p),
                                                          reinterpret_cast<const float4*>(B.r), n4, sc, 0);
    OST_LAUNCH_CHECK();
    return false;
  };

  // the iteration as one graph launch with its loop on the device
  int* trips = device_loop_enabled() ? device_loop_trips() : nullptr;
  const int max_trips = 2 * (o.max_iter / (o.chunk > 0 ? o.chunk : 1)) + 16;
  cudaGraphExec_t loop = trips ? device_loop(B, o, sc, trips, max_trips, hop_shapes, cs) : nullptr;
  if (loop) {
    int* trips_h = reinterpret_cast<int*>(g_host + 1);
    for (int round = 0; round < 64 && !error_code(); ++round) {
      OST_CUDA(cudaMemsetAsync(trips, 0, sizeof(int), cs));
      OST_CUDA(cudaGraphLaunch(loop, cs));
      OST_CUDA(cudaMemcpyAsync(trips_h, trips, sizeof(int), cudaMemcpyDeviceToHost, cs));
      OST_CUDA(cudaStreamSynchronize(cs));
      const int passes = *trips_h < 0 ? -*trips_h : *trips_h;
      g_kernel_launches += (4ull * o.chunk + 2) * passes;
      if (*trips_h < 0) {
        set_error(-15, "mixed CG: the device loop stopped at its bound of %d passes", max_trips);
        break;
      }
      if (close_or_tighten()) break;
    }
    OST_CUDA(cudaEventRecord(ev, cs));
    OST_CUDA(cudaStreamWaitEvent(st, ev, 0));
    OST_CUDA(cudaEventDestroy(ev));
    return res;
  }

  // Chunks run one ahead of the flag check: the flags copied after chunk k
  // are read while chunk k+1 runs, so the GPU does not wait for the host
  // between chunks.  Once the recursion has halted (converged, or a reliable
  // update is due) every kernel of the chunk launched ahead returns at once;
  // that chunk's flags are discarded.
  static cudaEvent_t flag_ev[2] = {nullptr, nullptr};
  for (int k = 0; k < 2; ++k)
    if (!flag_ev[k]) OST_CUDA(cudaEventCreateWithFlags(&flag_ev[k], cudaEventDisableTiming));
  auto launch_chunk = [&](int slot) {
    OST_CUDA(cudaGraphLaunch(g_cache.exec, cs));
    g_kernel_launches += 4ull * o.chunk;
    OST_CUDA(cudaMemcpyAsync(g_host + slot, sc, sizeof(MixScal), cudaMemcpyDeviceToHost, cs));
    OST_CUDA(cudaEventRecord(flag_ev[slot], cs));
  };
  int cur = 0;
  bool primed = false;
  for (int guard = 0; guard < 1000000; ++guard) {
    if (error_code()) break;
    if (!primed) {
      launch_chunk(cur);
      primed = true;
    }
    launch_chunk(cur ^ 1);
    OST_CUDA(cudaEventSynchronize(flag_ev[cur]));
    const MixScal h = g_host[cur];
    if (!h.need_rel && !h.done) {
      cur ^= 1;   // the chunk ahead becomes the current one
      continue;
    }
    OST_CUDA(cudaEventSynchronize(flag_ev[cur ^ 1]));
    primed = false;
    if (h.need_rel) {
      k_mx_accumulate<<<8 * rt().num_sms, 256, 0, cs>>>(B.x, B.xf, n);
      OST_LAUNCH_CHECK();
      // an intermediate reliable update needs ~1e-14 relative accuracy:
      // double-float suffices; the closing residual below stays in FP64
      if (B.use_df) df_mdagm(B.df, B.dfw, B.t64, B.x, o.mass2, cs);
      else fp64_mdagm(B, B.t64, B.x, B.t64b, o.mass2, cs);
      int gr = reduce_grid(n);
      k_mx_residual<<<gr, RED_THREADS, 0, cs>>>(B.b, B.t64, B.r64, B.r, B.p, B.s, n, sc, reduce_ws(3, gr), 1);
      OST_LAUNCH_CHECK();
      k_mx_pupdate<<<reduce_grid(n4), RED_THREADS, 0, cs>>>(reinterpret_cast<float4*>(B.p),
                                                            reinterpret_cast<const float4*>(B.r), n4, sc, 0);
      OST_LAUNCH_CHECK();
      continue;
    }
    if (h.done) {
      if (close_or_tighten()) break;
      continue;
    }
  }
  OST_CUDA(cudaEventRecord(ev, cs));
  OST_CUDA(cudaStreamWaitEvent(st, ev, 0));
  OST_CUDA(cudaEventDestroy(ev));
  return res;
}

// out = m2 in - D_eo D_oe in through the FP32 iteration kernels (the sloppy
// operator of the solve, with B's link format), FP64 in and out.  Uses B.p,
// B.t and B.s as work and sc as scratch scalars.
void sloppy_mdagm(const MixedBuffers& B, double m2, const double2* in, double2* out, MixScal* sc, cudaStream_t st) {
  const long n = 3L * rt().g.sizeh;
  MixScal init;
  memset(&init, 0, sizeof(init));
  init.m2 = m2;
  init.delta = 1.0;
  OST_CUDA(cudaMemcpyAsync(sc, &init, sizeof(MixScal), cudaMemcpyHostToDevice, st));
  ReduceWs ws = reduce_ws(1, mx_deo_blocks());
  conv_d2f(in, B.p, n, st);
  launch_mx_doe(kDoeShapes[0], B, sc, st);
  launch_mx_deo_dot(kDeoShapes[0], B, sc, ws, st);
  OST_LAUNCH_CHECK();
  conv_f2d(B.s, out, n, st);
  OST_CUDA(cudaStreamSynchronize(st));
}

// Times `reps` launches of one FP32 solver kernel on stream st with CUDA
// events recorded on that stream; returns the mean milliseconds per launch.
// which = 1: D_oe (t = D_oe p); which = 2: fused D_eo + M^+M epilogue + dot.
double time_mixed_kernel(const MixedBuffers& B, MixScal* sc, int which, int reps, cudaStream_t st) {
  const Geom& g = rt().g;
  const int nb = mx_deo_blocks();
  MixScal init;
  memset(&init, 0, sizeof(init));
  init.m2 = 0.01;
  init.delta = 1.0;
  OST_CUDA(cudaMemcpyAsync(sc, &init, sizeof(MixScal), cudaMemcpyHostToDevice, st));
  ReduceWs ws = reduce_ws(1, nb);
  tune_mx_hops(B, st);
  const HopShape doe_shape = mx_doe_shape(B);
  const HopShape deo_shape = mx_deo_shape(B);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float ms = 0;
  for (int pass = 0; pass < 2; ++pass) {       // pass 0 warms up
    cudaEventRecord(e0, st);
    for (int k = 0; k < reps; ++k) {
      if (which == 1) {
        launch_mx_doe(doe_shape, B, sc, st);
      } else {
        launch_mx_deo_dot(deo_shape, B, sc, ws, st);
      }
      OST_LAUNCH_CHECK();
    }
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return double(ms) / reps;
}

}  // namespace ost
