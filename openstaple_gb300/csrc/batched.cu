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
#include <type_traits>
#include "autotune.cuh"
#include "batched.cuh"
#include "dslash.cuh"
#include "kernels.cuh"
#include "reduce.cuh"
#include "runtime.cuh"

namespace ost {

static constexpr int BT = 128;

// Layout of the hop kernels.  A thread applies each link it loads to SPL
// systems (1 for a single system, 2 for up to 4, else 4); the batch is spread over
// LANES = (NS / SPL rounded up to a power of two) consecutive lanes that
// share one site and load the same link words in the same instruction, so a
// link is fetched from memory once per batch.  The link loads, the staggered
// sign and the rebuilt third row are shared by SPL systems per thread, while
// the register footprint stays close to a single-system hop's.
template <int NS, int SPL_ = 0>
struct HopLayout {
  static constexpr int SPL = SPL_ > 0 ? SPL_ : (NS <= 1 ? 1 : NS <= 4 ? 2 : 4);
  static constexpr int NL = (NS + SPL - 1) / SPL;
  static constexpr int LANES = NL <= 1 ? 1 : NL <= 2 ? 2 : NL <= 4 ? 4 : 8;
  static constexpr int SLOTS = LANES * SPL;   // per-site system slots, >= NS
};

template <int NS, int SPL_ = 0>
inline int hop_blocks(long sizeh) {
  return int((sizeh * HopLayout<NS, SPL_>::LANES + BT - 1) / BT);
}

OST_D bool batch_active(const BatchScal* sc, int k) {
  return !(*(volatile const int*)&sc->done[k]) && !(*(volatile const int*)&sc->need_rel[k]);
}

OST_D unsigned active_mask(const BatchScal* sc) {
  unsigned m = 0;
  for (int k = 0; k < sc->nsys; ++k)
    if (batch_active(sc, k)) m |= 1u << k;
  return m;
}

// Hop term at output index idx of parity P for SPL systems whose input
// fields start at in + sys[j] * vs.  All loads of one hop are issued before
// its arithmetic; the link, its sign and its rebuilt third row serve all SPL
// systems.
template <int SPL, int P, int PH, typename LV>
OST_D void hop_multi(const Geom& g, const LV& u, const float2* in, long vs, const int sys[SPL], const void* phases,
                     int idx, float2 aux[SPL][3]) {
  const long sh = g.sizeh;
  Site st = site_of(g, idx, P);
  int fwd[4], bwd[4];
  neighbours(g, st, fwd, bwd);
#pragma unroll
  for (int j = 0; j < SPL; ++j)
#pragma unroll
    for (int c = 0; c < 3; ++c) aux[j][c] = make_float2(0.f, 0.f);
#pragma unroll
  for (int hm = 0; hm < 8; ++hm) {
    const bool back = hm < 4;       // backward hops first, as in the reference
    const int mu = hm & 3;
    const int dir = back ? 2 * mu + (1 - P) : 2 * mu + P;
    const int nb = back ? bwd[mu] : fwd[mu];     // site of the input spinor
    const int li = back ? nb : idx;              // site the link leaves
    float2 m[6], v[SPL][3];
    load_two_rows(u, dir, li, m);
#pragma unroll
    for (int j = 0; j < SPL; ++j) load_vec(in + sys[j] * vs, sh, nb, v[j]);
    unsigned mask = back ? 0x80000000u : 0u;
    float2 phz = make_float2(1.f, 0.f);
    bool generic = false;
    if (PH == PH_SIGN8) {
      const unsigned char sb = __ldg(static_cast<const unsigned char*>(phases) + long(dir) * sh + li);
      mask ^= sb ? 0x80000000u : 0u;
    } else {
      const float a = __ldcs(static_cast<const float*>(phases) + long(dir) * sh + li);
      const unsigned bits = __float_as_uint(a);
      if (bits == PiBits<float>::bits()) {
        mask ^= 0x80000000u;
      } else if (bits != 0u) {
        float sn, cs;
        sincosf(a, &sn, &cs);
        phz = make_float2(cs, back ? -sn : sn);
        generic = true;
      }
    }
    const float2 r20 = conj_cross(m[1], m[5], m[2], m[4]);
    const float2 r21 = conj_cross(m[2], m[3], m[0], m[5]);
    const float2 r22 = conj_cross(m[0], m[4], m[1], m[3]);
#pragma unroll
    for (int j = 0; j < SPL; ++j) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (generic) v[j][c] = cmul(v[j][c], phz);
        v[j][c].x = flip_sign(v[j][c].x, mask);
        v[j][c].y = flip_sign(v[j][c].y, mask);
      }
      if (back) {
        cmacc(aux[j][0], m[0], v[j][0]); cmacc(aux[j][0], m[3], v[j][1]); cmacc(aux[j][0], r20, v[j][2]);
        cmacc(aux[j][1], m[1], v[j][0]); cmacc(aux[j][1], m[4], v[j][1]); cmacc(aux[j][1], r21, v[j][2]);
        cmacc(aux[j][2], m[2], v[j][0]); cmacc(aux[j][2], m[5], v[j][1]); cmacc(aux[j][2], r22, v[j][2]);
      } else {
        cmac(aux[j][0], m[0], v[j][0]); cmac(aux[j][0], m[1], v[j][1]); cmac(aux[j][0], m[2], v[j][2]);
        cmac(aux[j][1], m[3], v[j][0]); cmac(aux[j][1], m[4], v[j][1]); cmac(aux[j][1], m[5], v[j][2]);
        cmac(aux[j][2], r20, v[j][0]); cmac(aux[j][2], r21, v[j][1]); cmac(aux[j][2], r22, v[j][2]);
      }
    }
  }
}

// Launched early (programmatic dependent launch): the first lane of each
// site fetches the links of its eight hops into L2 while the previous kernel
// finishes (no kernel of the solve writes the links).
template <int LANES, int P, typename LV>
OST_D void prefetch_site_links(const Geom& g, const LV& u) {
  const long tid = long(blockIdx.x) * BT + threadIdx.x;
  const long site = tid / LANES;
  if (tid % LANES == 0 && site < g.sizeh) prefetch_links<P>(g, u, int(site));
}

// thread -> (site, first system slot of its lane); slots beyond NS read a
// valid system (slot 0) and discard the result.  Returns idx < sizeh.
template <int NS, int SPL_ = 0>
OST_D bool hop_thread(long sizeh, int& idx, int sys[HopLayout<NS, SPL_>::SPL], bool valid[HopLayout<NS, SPL_>::SPL]) {
  typedef HopLayout<NS, SPL_> H;
  const long tid = long(blockIdx.x) * BT + threadIdx.x;
  idx = int(tid / H::LANES);
  const int lane = int(tid % H::LANES);
#pragma unroll
  for (int j = 0; j < H::SPL; ++j) {
    const int k = lane * H::SPL + j;
    valid[j] = k < NS;
    sys[j] = valid[j] ? k : 0;
  }
  return idx < sizeh;
}

// t_k = D_oe p_k (every system of the batch; converged ones are recomputed
// harmlessly since t is a temporary)
template <int NS, int SPL_, int PH, typename LV>
__global__ void __launch_bounds__(BT)
k_b_doe(Geom g, LV u, const void* __restrict__ ph, const float2* __restrict__ p, float2* __restrict__ t, long vs,
        const BatchScal* sc) {
  typedef HopLayout<NS, SPL_> H;
  if (!active_mask(sc)) return;   // flags of k_b_update, two launches back
  prefetch_site_links<H::LANES, 1>(g, u);
  pdl_wait();                     // p from k_b_pupdate
  pdl_trigger();
  int idx, sys[H::SPL];
  bool valid[H::SPL];
  const bool live = hop_thread<NS, SPL_>(g.sizeh, idx, sys, valid);
  float2 aux[H::SPL][3];
  if (live) hop_multi<H::SPL, 1, PH>(g, u, p, vs, sys, ph, idx, aux);
  if (!live) return;
#pragma unroll
  for (int j = 0; j < H::SPL; ++j) {
    if (!valid[j]) continue;
#pragma unroll
    for (int c = 0; c < 3; ++c)
      t[sys[j] * vs + c * long(g.sizeh) + idx] = make_float2(0.5f * aux[j][c].x, 0.5f * aux[j][c].y);
  }
}

// Per-thread values v[j] of system slot lane*SPL + j -> per-system grid totals.
template <int NS>
OST_D bool hop_reduce(const float v[HopLayout<NS>::SPL], ReduceWs ws, double tot[HopLayout<NS>::SLOTS]) {
  typedef HopLayout<NS> H;
  __shared__ double smem[H::SLOTS * 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  float w[H::SPL];
#pragma unroll
  for (int j = 0; j < H::SPL; ++j) {
    w[j] = v[j];
#pragma unroll
    for (int o = 16; o >= H::LANES; o >>= 1) w[j] += __shfl_xor_sync(0xffffffffu, w[j], o);
  }
  if (lane < H::LANES) {
#pragma unroll
    for (int j = 0; j < H::SPL; ++j) smem[(lane * H::SPL + j) * 32 + warp] = double(w[j]);
  }
  __syncthreads();
  double bv[H::SLOTS];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < H::SLOTS; ++k) {
      double t = 0.0;
      for (int q = 0; q < nwarps; ++q) t += smem[k * 32 + q];
      bv[k] = t;
    }
  }
  __syncthreads();
  return grid_finish<H::SLOTS>(bv, ws, tot, smem);
}

// s_k = m2_k p_k - D_eo t_k ; pAp_k ; alpha_k = delta_k / pAp_k
template <int NS, int PH, typename LV>
__global__ void __launch_bounds__(BT)
k_b_deo_dot(Geom g, LV u, const void* __restrict__ ph, const float2* __restrict__ t, const float2* __restrict__ p,
            float2* __restrict__ s, long vs, BatchScal* sc, ReduceWs ws) {
  typedef HopLayout<NS> H;
  if (!active_mask(sc)) return;
  prefetch_site_links<H::LANES, 0>(g, u);
  pdl_wait();                     // t from k_b_doe
  pdl_trigger();
  int idx, sys[H::SPL];
  bool valid[H::SPL];
  const bool live = hop_thread<NS>(g.sizeh, idx, sys, valid);
  float v[H::SPL];
  float2 aux[H::SPL][3];
  if (live) hop_multi<H::SPL, 0, PH>(g, u, t, vs, sys, ph, idx, aux);
#pragma unroll
  for (int j = 0; j < H::SPL; ++j) {
    v[j] = 0.f;
    if (!live || !valid[j]) continue;
    const float m2 = float(sc->m2[sys[j]]);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long q = sys[j] * vs + c * long(g.sizeh) + idx;
      const float2 pv = p[q];
      const float2 r = make_float2(fmaf(pv.x, m2, -0.5f * aux[j][c].x), fmaf(pv.y, m2, -0.5f * aux[j][c].y));
      s[q] = r;
      v[j] = fmaf(pv.x, r.x, fmaf(pv.y, r.y, v[j]));
    }
  }
  double tot[H::SLOTS];
  if (hop_reduce<NS>(v, ws, tot)) {
    const unsigned mask = active_mask(sc);
    for (int k = 0; k < NS; ++k)
      if (mask >> k & 1u) { sc->pAp[k] = tot[k]; sc->alpha[k] = sc->delta[k] / tot[k]; }
  }
}

// Streaming kernels split the grid into one segment of blocks per system.
inline int seg_blocks(long n4, int nsys) {
  const int total = reduce_grid(n4 * nsys);
  const int b = (total + nsys - 1) / nsys;
  return b < 1 ? 1 : b;
}

// x_f += alpha p ; unless a reliable update is due: r -= alpha s, lambda = |r|^2,
// beta = lambda / delta, convergence test (per system)
template <int NS>
__global__ void k_b_update(float4* __restrict__ xf, float4* __restrict__ r, const float4* __restrict__ p,
                           const float4* __restrict__ s, long n4, long vs4, int bps, BatchScal* sc, ReduceWs ws) {
  pdl_wait();                     // s and alpha from k_b_deo_dot
  pdl_trigger();
  const int k = blockIdx.x / bps;
  const bool act = k < NS && batch_active(sc, k);
  bool rel = false;
  float a = 0.f, v = 0.f;
  if (act) {
    const double delta = sc->delta[k];
    const double lm = sc->last_max[k] > delta ? sc->last_max[k] : delta;
    rel = sc->every > 0 ? ((sc->iter[k] + 1) % sc->every == 0) : (delta < sc->frac * lm);
    a = float(sc->alpha[k]);
    const long base = k * vs4;
    const long stride = long(bps) * blockDim.x;
    for (long i = long(blockIdx.x - k * bps) * blockDim.x + threadIdx.x; i < n4; i += 2 * stride) {
      const long i2 = i + stride;
      const bool two = i2 < n4;
      float4 pv0 = p[base + i], xv0 = xf[base + i], pv1, xv1, sv0, rv0, sv1, rv1;
      if (two) { pv1 = p[base + i2]; xv1 = xf[base + i2]; }
      if (!rel) {
        sv0 = s[base + i]; rv0 = r[base + i];
        if (two) { sv1 = s[base + i2]; rv1 = r[base + i2]; }
      }
      xv0 = make_float4(fmaf(a, pv0.x, xv0.x), fmaf(a, pv0.y, xv0.y), fmaf(a, pv0.z, xv0.z), fmaf(a, pv0.w, xv0.w));
      xf[base + i] = xv0;
      if (two) {
        xv1 = make_float4(fmaf(a, pv1.x, xv1.x), fmaf(a, pv1.y, xv1.y), fmaf(a, pv1.z, xv1.z), fmaf(a, pv1.w, xv1.w));
        xf[base + i2] = xv1;
      }
      if (!rel) {
        rv0 = make_float4(fmaf(-a, sv0.x, rv0.x), fmaf(-a, sv0.y, rv0.y), fmaf(-a, sv0.z, rv0.z),
                          fmaf(-a, sv0.w, rv0.w));
        r[base + i] = rv0;
        v = fmaf(rv0.x, rv0.x, fmaf(rv0.y, rv0.y, fmaf(rv0.z, rv0.z, fmaf(rv0.w, rv0.w, v))));
        if (two) {
          rv1 = make_float4(fmaf(-a, sv1.x, rv1.x), fmaf(-a, sv1.y, rv1.y), fmaf(-a, sv1.z, rv1.z),
                            fmaf(-a, sv1.w, rv1.w));
          r[base + i2] = rv1;
          v = fmaf(rv1.x, rv1.x, fmaf(rv1.y, rv1.y, fmaf(rv1.z, rv1.z, fmaf(rv1.w, rv1.w, v))));
        }
      }
    }
  }
  double tot[NS];
  if (grid_reduce_seg<NS>(v, bps, ws, tot)) {
    const unsigned mask = active_mask(sc);
    for (int j = 0; j < NS; ++j) {
      if (!(mask >> j & 1u)) continue;
      const double delta = sc->delta[j];
      const double lm = sc->last_max[j] > delta ? sc->last_max[j] : delta;
      const bool rj = sc->every > 0 ? ((sc->iter[j] + 1) % sc->every == 0) : (delta < sc->frac * lm);
      sc->iter[j] += 1;
      sc->last_max[j] = lm;
      if (rj) {
        sc->need_rel[j] = 1;
      } else {
        sc->lambda[j] = tot[j];
        sc->beta[j] = tot[j] / delta;
        sc->delta[j] = tot[j];
        if (tot[j] <= sc->target2[j] || sc->iter[j] >= sc->max_iter) sc->done[j] = 1;
      }
    }
  }
}

// p = r + beta p for every active system
template <int NS>
__global__ void k_b_pupdate(float4* __restrict__ p, const float4* __restrict__ r, long n4, long vs4, int bps,
                            const BatchScal* sc) {
  pdl_wait();                     // r, beta and the flags from k_b_update
  pdl_trigger();
  const int k = blockIdx.x / bps;
  if (k >= NS || !batch_active(sc, k)) return;
  const float b = float(sc->beta[k]);
  const long base = k * vs4;
  const long stride = long(bps) * blockDim.x;
  for (long i = long(blockIdx.x - k * bps) * blockDim.x + threadIdx.x; i < n4; i += 2 * stride) {
    const long i2 = i + stride;
    const bool two = i2 < n4;
    float4 pv0 = p[base + i], rv0 = r[base + i], pv1, rv1;
    if (two) { pv1 = p[base + i2]; rv1 = r[base + i2]; }
    p[base + i] = make_float4(fmaf(b, pv0.x, rv0.x), fmaf(b, pv0.y, rv0.y), fmaf(b, pv0.z, rv0.z),
                              fmaf(b, pv0.w, rv0.w));
    if (two)
      p[base + i2] = make_float4(fmaf(b, pv1.x, rv1.x), fmaf(b, pv1.y, rv1.y), fmaf(b, pv1.z, rv1.z),
                                 fmaf(b, pv1.w, rv1.w));
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
// (mode 1: beta = -<r, s>/<p, s> with s = A p of system k's last iteration,
// the Hestenes-Stiefel form the single-system solver uses at its reliable
// updates, k_mx_residual)
__global__ void k_b_residual(const double2* __restrict__ b, const double2* __restrict__ ax, double2* __restrict__ r64,
                             float2* __restrict__ r, float2* __restrict__ p, const float2* __restrict__ s, long n,
                             BatchScal* sc, int k, ReduceWs ws, int mode) {
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
    sc->true_r2[k] = tot[1];
    sc->lambda[k] = tot[0];
    if (mode == 0) {
      sc->delta[k] = tot[0];
      sc->beta[k] = 0.0;
    } else {
      sc->beta[k] = (sc->iter[k] > 0 && sc->pAp[k] > 0.0) ? -tot[2] / sc->pAp[k] : 0.0;
      sc->delta[k] = tot[0];
      sc->n_rel[k] += 1;
    }
    sc->last_max[k] = 0.0;
    sc->need_rel[k] = 0;
    sc->done[k] = (tot[0] <= sc->target2[k] || sc->iter[k] >= sc->max_iter) ? 1 : 0;
  }
}

// Launches of the D_oe hops with a given number of systems per thread
// (0 = the default layout); the autotuner picks among them (no reduction,
// so the results are the same for every choice).
static const int kSplCand[4] = {0, 1, 2, 4};

// Calls f with the view of the sloppy links of the batched iteration.
template <typename F>
void with_batch_links(const BatchBuffers& B, F&& f) {
  if (B.q16) f(B.uq);
  else f(LinkView<float2>{B.u32, rt().g.sizeh, 6});
}

template <int NS, int SPL_>
void launch_b_doe_spl(const BatchBuffers& B, BatchScal* sc, cudaStream_t st) {
  const Geom& g = rt().g;
  const long n = 3L * g.sizeh;
  const int nb = hop_blocks<NS, SPL_>(g.sizeh);
  with_batch_links(B, [&](const auto& u) {
    typedef typename std::decay<decltype(u)>::type LV;
    if (B.ph32_mode == PH_SIGN8)
      launch_pdl(k_b_doe<NS, SPL_, PH_SIGN8, LV>, nb, BT, st, g, u, B.ph32, B.p, B.t, n, static_cast<const BatchScal*>(sc));
    else launch_pdl(k_b_doe<NS, SPL_, PH_ANGLE, LV>, nb, BT, st, g, u, B.ph32, B.p, B.t, n,
                    static_cast<const BatchScal*>(sc));
  });
  OST_LAUNCH_CHECK();
}

// tuning key of k_b_doe: systems, phase mode, link format
template <int NS>
int b_doe_variant(const BatchBuffers& B) {
  return NS * 4 + (B.ph32_mode == PH_SIGN8) * 2 + (B.q16 != 0);
}

template <int NS>
void launch_b_doe(int spl, const BatchBuffers& B, BatchScal* sc, cudaStream_t st) {
  if (spl == 1) launch_b_doe_spl<NS, 1>(B, sc, st);
  else if (spl == 2 && NS >= 2) launch_b_doe_spl<NS, 2>(B, sc, st);
  else if (spl == 4 && NS >= 3) launch_b_doe_spl<NS, 4>(B, sc, st);
  else launch_b_doe_spl<NS, 0>(B, sc, st);
}

// ---- host engine ----
namespace {

struct BGraph {
  cudaGraphExec_t exec = nullptr;
  BatchBuffers key{};
  BatchScal* sc = nullptr;
  int chunk = 0;
  unsigned long long epoch = 0;
  int doe_pick = -1;
};
BGraph g_bgraph;
cudaStream_t g_bcap = nullptr;
BatchScal* g_bhost = nullptr;
BatchScal* g_bflags = nullptr;   // two slots: the flags after the current chunk and after the chunk ahead

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
  const int nb = hop_blocks<NS>(g.sizeh);
  const long n = 3L * g.sizeh, n4 = n / 2;
  const int bps = seg_blocks(n4, NS);
  // one workspace for both reductions: hop (SLOTS x nb partials) and
  // segments (NS x bps partials)
  ReduceWs wh = reduce_ws(HopLayout<NS>::SLOTS, nb > NS * bps ? nb : NS * bps);
  const int pick = autotune_cached(TUNE_B_DOE, g.sizeh, b_doe_variant<NS>(B));
  launch_b_doe<NS>(kSplCand[pick > 0 && pick < 4 ? pick : 0], B, sc, st);
  with_batch_links(B, [&](const auto& u) {
    typedef typename std::decay<decltype(u)>::type LV;
    if (B.ph32_mode == PH_SIGN8)
      launch_pdl(k_b_deo_dot<NS, PH_SIGN8, LV>, nb, BT, st, g, u, B.ph32, B.t, B.p, B.s, n, sc, wh);
    else launch_pdl(k_b_deo_dot<NS, PH_ANGLE, LV>, nb, BT, st, g, u, B.ph32, B.t, B.p, B.s, n, sc, wh);
  });
  launch_pdl(k_b_update<NS>, NS * bps, RED_THREADS, st, reinterpret_cast<float4*>(B.xf),
             reinterpret_cast<float4*>(B.r), reinterpret_cast<const float4*>(B.p),
             reinterpret_cast<const float4*>(B.s), n4, n4, bps, sc, wh);
  launch_pdl(k_b_pupdate<NS>, NS * bps, RED_THREADS, st, reinterpret_cast<float4*>(B.p),
             reinterpret_cast<const float4*>(B.r), n4, n4, bps, static_cast<const BatchScal*>(sc));
}

// partial sums that the batched reductions need at most, for pre-sizing the
// workspace before a graph capture
inline size_t batch_reduce_partials(long sizeh) {
  const long n4 = 3L * sizeh / 2;
  const long hop = long(HopLayout<BATCH_MAX>::SLOTS) * hop_blocks<BATCH_MAX>(sizeh);
  const long seg = long(BATCH_MAX) * BATCH_MAX * seg_blocks(n4, BATCH_MAX);
  const long red = long(BATCH_MAX) * reduce_grid(3L * sizeh);
  long m = hop > seg ? hop : seg;
  return size_t(m > red ? m : red);
}

template <int NS>
int tune_b_doe(const BatchBuffers& B, cudaStream_t st) {
  const int variant = b_doe_variant<NS>(B);
  const int cached = autotune_cached(TUNE_B_DOE, rt().g.sizeh, variant);
  if (cached >= 0 || !autotune_enabled()) return cached > 0 ? cached : 0;
  BatchScal h;
  memset(&h, 0, sizeof(h));
  h.nsys = NS;
  BatchScal* sc = static_cast<BatchScal*>(autotune_scalars(&h, sizeof(h), st));
  if (!sc) return 0;
  return autotune_pick(TUNE_B_DOE, rt().g.sizeh, variant, 4,
                       [&](int c) { launch_b_doe<NS>(kSplCand[c], B, sc, st); }, st);
}

int tune_batch(const BatchBuffers& B, cudaStream_t st) {
  switch (B.nsys) {
    case 1: return tune_b_doe<1>(B, st);
    case 2: return tune_b_doe<2>(B, st);
    case 3: return tune_b_doe<3>(B, st);
    case 4: return tune_b_doe<4>(B, st);
    case 5: return tune_b_doe<5>(B, st);
    case 6: return tune_b_doe<6>(B, st);
    case 7: return tune_b_doe<7>(B, st);
    default: return tune_b_doe<8>(B, st);
  }
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
    OST_CUDA(cudaMallocHost(&g_bflags, 2 * sizeof(BatchScal)));
  }
  cudaEvent_t ev;
  OST_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  OST_CUDA(cudaEventRecord(ev, st));
  OST_CUDA(cudaStreamWaitEvent(g_bcap, ev, 0));
  cudaStream_t cs = g_bcap;
  reduce_ws_reserve(batch_reduce_partials(g.sizeh));   // allocated before any capture
  BatchScal init;
  memset(&init, 0, sizeof(init));
  init.frac = delta_frac;
  init.max_iter = max_iter;
  init.every = 0;
  init.nsys = NSY;
  for (int k = 0; k < NSY; ++k) init.m2[k] = m2[k];
  OST_CUDA(cudaMemcpyAsync(sc, &init, sizeof(BatchScal), cudaMemcpyHostToDevice, cs));
  for (int k = 0; k < NSY; ++k) {
    blas_norm2<double>(B.b + k * n, n, &sc->bnorm2[k], cs);
    blas_norm2<double>(B.x + k * n, n, &sc->true_r2[k], cs);   // |x0|^2, overwritten below
  }
  OST_CUDA(cudaMemcpyAsync(g_bhost, sc, sizeof(BatchScal), cudaMemcpyDeviceToHost, cs));
  OST_CUDA(cudaStreamSynchronize(cs));
  bool zero_guess[BATCH_MAX];
  for (int k = 0; k < NSY; ++k) zero_guess[k] = g_bhost->true_r2[k] == 0.0;
  // a system with a non-finite source or guess cannot converge: it is
  // reported as failed at once and kept out of the iteration
  bool bad[BATCH_MAX];
  for (int k = 0; k < NSY; ++k) bad[k] = !std::isfinite(g_bhost->bnorm2[k]) || !std::isfinite(g_bhost->true_r2[k]);
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
    // r0 = b - A x0; a zero guess needs no operator application, any other
    // guess takes the double-float operator (the closing residual is FP64)
    if (zero_guess[k]) OST_CUDA(cudaMemsetAsync(B.t64, 0, n * sizeof(double2), cs));
    else if (B.use_df) df_mdagm(B.df, B.dfw, B.t64, B.x + k * n, m2[k], cs);
    else fp64_mdagm(B, B.t64, B.x + k * n, m2[k], cs);
    const int gr = reduce_grid(n);
    k_b_residual<<<gr, RED_THREADS, 0, cs>>>(B.b + k * n, B.t64, B.r64, B.r + k * n, B.p + k * n, B.s + k * n, n, sc, k,
                                             reduce_ws(3, gr), 0);
    OST_LAUNCH_CHECK();
  }
  bool finished[BATCH_MAX] = {false};
  for (int k = 0; k < NSY; ++k) {
    if (!bad[k]) continue;
    const int one = 1;
    OST_CUDA(cudaMemcpyAsync(&sc->done[k], &one, sizeof(int), cudaMemcpyHostToDevice, cs));
    out.true_res[k] = NAN;
    finished[k] = true;
  }
  const int chunk = 8;
  // launch shape of the D_oe (numerics-invariant), chosen before the capture
  const int doe_pick = tune_batch(B, cs);
  if (!g_bgraph.exec || g_bgraph.sc != sc || g_bgraph.chunk != chunk || g_bgraph.key.nsys != B.nsys ||
      g_bgraph.doe_pick != doe_pick ||
      g_bgraph.key.p != B.p || g_bgraph.key.r != B.r || g_bgraph.key.s != B.s || g_bgraph.key.t != B.t ||
      g_bgraph.key.xf != B.xf || g_bgraph.key.u32 != B.u32 || g_bgraph.key.ph32 != B.ph32 ||
      g_bgraph.key.q16 != B.q16 || g_bgraph.key.uq.a != B.uq.a ||
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
    g_bgraph.doe_pick = doe_pick;
  }
  // Chunks run one ahead of the flag check (as in the single-system solver):
  // the flags copied after chunk k are read while chunk k+1 runs.  When a
  // system has halted (converged or a reliable update due), the chunk ahead
  // did nothing for it; after that chunk has finished its flags are
  // discarded and the pipeline restarts behind the host's work.
  static cudaEvent_t flag_ev[2] = {nullptr, nullptr};
  for (int k = 0; k < 2; ++k)
    if (!flag_ev[k]) OST_CUDA(cudaEventCreateWithFlags(&flag_ev[k], cudaEventDisableTiming));
  auto launch_chunk = [&](int slot) {
    OST_CUDA(cudaGraphLaunch(g_bgraph.exec, cs));
    g_kernel_launches += 4ull * chunk;
    OST_CUDA(cudaMemcpyAsync(g_bflags + slot, sc, sizeof(BatchScal), cudaMemcpyDeviceToHost, cs));
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
    BatchScal h = g_bflags[cur];
    bool halted_any = false;
    for (int k = 0; k < NSY; ++k)
      if (!finished[k] && (h.need_rel[k] || h.done[k])) halted_any = true;
    if (!halted_any) {
      cur ^= 1;
      continue;
    }
    OST_CUDA(cudaEventSynchronize(flag_ev[cur ^ 1]));
    primed = false;
    bool all = true;
    for (int k = 0; k < NSY; ++k) {
      if (finished[k]) continue;
      if (h.need_rel[k] || h.done[k]) {
        const bool was_done = h.done[k];
        k_b_accumulate<<<8 * rt().num_sms, 256, 0, cs>>>(B.x + k * n, B.xf + k * n, n);
        OST_LAUNCH_CHECK();
        // intermediate reliable updates in double-float, closing residuals in FP64
        if (!was_done && B.use_df) df_mdagm(B.df, B.dfw, B.t64, B.x + k * n, m2[k], cs);
        else fp64_mdagm(B, B.t64, B.x + k * n, m2[k], cs);
        const int gr = reduce_grid(n);
        k_b_residual<<<gr, RED_THREADS, 0, cs>>>(B.b + k * n, B.t64, B.r64, B.r + k * n, B.p + k * n, B.s + k * n, n, sc, k,
                                                 reduce_ws(3, gr), 1);
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

OST_D bool cgm_active(const CgmScal* sc, int r) { return !(*(volatile const int*)&sc->done[r]); }

template <int NR, int SPL_, int PH>
__global__ void __launch_bounds__(BT)
k_cgm_doe(Geom g, LinkView<float2> u, const void* __restrict__ ph, const float2* __restrict__ p, float2* __restrict__ t,
          long vs, const CgmScal* sc) {
  typedef HopLayout<NR, SPL_> H;
  if (!cgm_mask(sc)) return;
  int idx, sys[H::SPL];
  bool valid[H::SPL];
  const bool live = hop_thread<NR, SPL_>(g.sizeh, idx, sys, valid);
  float2 aux[H::SPL][3];
  if (live) hop_multi<H::SPL, 1, PH>(g, u, p, vs, sys, ph, idx, aux);
  if (!live) return;
#pragma unroll
  for (int j = 0; j < H::SPL; ++j) {
    if (!valid[j]) continue;
#pragma unroll
    for (int c = 0; c < 3; ++c)
      t[sys[j] * vs + c * long(g.sizeh) + idx] = make_float2(0.5f * aux[j][c].x, 0.5f * aux[j][c].y);
  }
}

template <int NR, int SPL_>
void launch_cgm_doe_spl(const CgmBatchBuffers& B, const CgmScal* sc, cudaStream_t st) {
  const Geom& g = rt().g;
  LinkView<float2> u{B.u32, g.sizeh, 6};
  const long n = 3L * g.sizeh;
  const int nb = hop_blocks<NR, SPL_>(g.sizeh);
  if (B.ph32_mode == PH_SIGN8) k_cgm_doe<NR, SPL_, PH_SIGN8><<<nb, BT, 0, st>>>(g, u, B.ph32, B.p, B.t, n, sc);
  else k_cgm_doe<NR, SPL_, PH_ANGLE><<<nb, BT, 0, st>>>(g, u, B.ph32, B.p, B.t, n, sc);
  OST_LAUNCH_CHECK();
}

template <int NR>
void launch_cgm_doe(int spl, const CgmBatchBuffers& B, const CgmScal* sc, cudaStream_t st) {
  if (spl == 1) launch_cgm_doe_spl<NR, 1>(B, sc, st);
  else if (spl == 2 && NR >= 2) launch_cgm_doe_spl<NR, 2>(B, sc, st);
  else if (spl == 4 && NR >= 3) launch_cgm_doe_spl<NR, 4>(B, sc, st);
  else launch_cgm_doe_spl<NR, 0>(B, sc, st);
}

template <int NR>
void tune_cgm_doe(const CgmBatchBuffers& B, cudaStream_t st) {
  const int variant = NR * 2 + (B.ph32_mode == PH_SIGN8);
  if (autotune_cached(TUNE_CGM_DOE, rt().g.sizeh, variant) >= 0 || !autotune_enabled()) return;
  CgmScal h;
  memset(&h, 0, sizeof(h));
  h.nrhs = NR;
  const CgmScal* sc = static_cast<const CgmScal*>(autotune_scalars(&h, sizeof(h), st));
  if (!sc) return;
  autotune_pick(TUNE_CGM_DOE, rt().g.sizeh, variant, 4,
                [&](int c) { launch_cgm_doe<NR>(kSplCand[c], B, sc, st); }, st);
}

// s = m2 p - D_eo t ; alpha = <p,s> ; then the shifted recurrences
// (inverter_multishift_full.c:116-137)
template <int NR, int PH>
__global__ void __launch_bounds__(BT)
k_cgm_deo_dot(Geom g, LinkView<float2> u, const void* __restrict__ ph, const float2* __restrict__ t,
              const float2* __restrict__ p, float2* __restrict__ s, long vs, CgmScal* sc, ReduceWs ws) {
  typedef HopLayout<NR> H;
  if (!cgm_mask(sc)) return;
  int idx, sys[H::SPL];
  bool valid[H::SPL];
  const bool live = hop_thread<NR>(g.sizeh, idx, sys, valid);
  float v[H::SPL];
  float2 aux[H::SPL][3];
  if (live) hop_multi<H::SPL, 0, PH>(g, u, t, vs, sys, ph, idx, aux);
  const float m2 = float(sc->m2);
#pragma unroll
  for (int j = 0; j < H::SPL; ++j) {
    v[j] = 0.f;
    if (!live || !valid[j]) continue;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long q = sys[j] * vs + c * long(g.sizeh) + idx;
      const float2 pv = p[q];
      const float2 r = make_float2(fmaf(pv.x, m2, -0.5f * aux[j][c].x), fmaf(pv.y, m2, -0.5f * aux[j][c].y));
      s[q] = r;
      v[j] = fmaf(pv.x, r.x, fmaf(pv.y, r.y, v[j]));
    }
  }
  double tot[H::SLOTS];
  if (hop_reduce<NR>(v, ws, tot)) {
    const unsigned mask = cgm_mask(sc);
    for (int r = 0; r < sc->nrhs; ++r) {
      if (!(mask >> r & 1u)) continue;
      for (int k2 = 0; k2 < sc->nshift; ++k2) sc->flag[r][k2] = sc->flag_next[r][k2];
      const double alpha = tot[r];
      sc->omega_prev[r] = sc->omega[r];
      const double om = -sc->delta[r] / alpha, omp = sc->omega_prev[r], ga = sc->gamma[r];
      sc->omega[r] = om;
      for (int k2 = 0; k2 < sc->nshift; ++k2) {
        if (!sc->flag[r][k2]) continue;
        const double zi = sc->zi[r][k2], zii = sc->zii[r][k2];
        const double z3 = (zi * zii * omp) / (om * ga * (zi - zii) + zi * omp * (1.0 - sc->shift[k2] * om));
        sc->ziii[r][k2] = z3;
        sc->omk[r][k2] = om * z3 / zii;
      }
    }
  }
}

// r += omega s ; lambda = |r|^2 ; gamma = lambda/delta ; gamma_k ; freeze
// decisions for the next iteration (inverter_multishift_full.c:139-171).
// One segment of bps blocks per right-hand side.
template <int NR>
__global__ void k_cgm_r(float4* __restrict__ r, const float4* __restrict__ s, long n4, long vs4, int bps,
                        CgmScal* sc, ReduceWs ws) {
  const int rr = blockIdx.x / bps;
  float v = 0.f;
  if (rr < NR && cgm_active(sc, rr)) {
    const float om = float(sc->omega[rr]);
    const long base = rr * vs4;
    const long stride = long(bps) * blockDim.x;
    for (long i = long(blockIdx.x - rr * bps) * blockDim.x + threadIdx.x; i < n4; i += stride) {
      float4 rv = r[base + i];
      const float4 sv = s[base + i];
      rv = make_float4(fmaf(om, sv.x, rv.x), fmaf(om, sv.y, rv.y), fmaf(om, sv.z, rv.z), fmaf(om, sv.w, rv.w));
      r[base + i] = rv;
      v = fmaf(rv.x, rv.x, fmaf(rv.y, rv.y, fmaf(rv.z, rv.z, fmaf(rv.w, rv.w, v))));
    }
  }
  double tot[NR];
  if (grid_reduce_seg<NR>(v, bps, ws, tot)) {
    const unsigned mask = cgm_mask(sc);
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

// the active-system mask entering an iteration, kept on the device for k_cgm_xp
__global__ void k_cgm_snapshot(const CgmScal* sc, int* mask_out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *mask_out = int(cgm_mask(sc));
}

// p = r + gamma p ; x_k -= omega_k ps_k ; ps_k = gamma_k ps_k + zeta_k r over
// the shifts still active in this iteration.  One segment of bps blocks per
// right-hand side; a block stages its side's coefficients in shared memory.
// Only sides that were active when the iteration started are updated.
__global__ void k_cgm_xp_dev(float4* __restrict__ p, const float4* __restrict__ r, float4* __restrict__ xs,
                             float4* __restrict__ ps, long n4, long vs4, int bps, const CgmScal* sc,
                             const int* mask_in) {
  __shared__ float s_om[CGM_MAX_SHIFTS], s_gk[CGM_MAX_SHIFTS], s_z[CGM_MAX_SHIFTS];
  __shared__ int s_list[CGM_MAX_SHIFTS], s_n;
  const int rr = blockIdx.x / bps;
  if (rr >= sc->nrhs || !(*mask_in >> rr & 1)) return;
  const int nk = sc->nshift;
  if (threadIdx.x == 0) {
    int c = 0;
    for (int k = 0; k < nk; ++k) {
      if (!sc->flag[rr][k]) continue;
      s_list[c] = k;
      s_om[c] = float(sc->omk[rr][k]);
      s_gk[c] = float(sc->gak[rr][k]);
      s_z[c] = float(sc->ziii[rr][k]);
      ++c;
    }
    s_n = c;
  }
  __syncthreads();
  const int na = s_n;
  const float ga = float(sc->gamma[rr]);
  const long base = rr * vs4;
  const long stride = long(bps) * blockDim.x;
  for (long i = long(blockIdx.x - rr * bps) * blockDim.x + threadIdx.x; i < n4; i += stride) {
    const float4 rv = r[base + i];
    const float4 pv = p[base + i];
    p[base + i] = make_float4(fmaf(ga, pv.x, rv.x), fmaf(ga, pv.y, rv.y), fmaf(ga, pv.z, rv.z), fmaf(ga, pv.w, rv.w));
    for (int j = 0; j < na; ++j) {
      const long qk = (long(rr) * nk + s_list[j]) * vs4 + i;
      float4 xv = xs[qk];
      const float4 pk = ps[qk];
      const float om = s_om[j], gk = s_gk[j], z = s_z[j];
      xv = make_float4(fmaf(-om, pk.x, xv.x), fmaf(-om, pk.y, xv.y), fmaf(-om, pk.z, xv.z), fmaf(-om, pk.w, xv.w));
      xs[qk] = xv;
      ps[qk] = make_float4(fmaf(gk, pk.x, z * rv.x), fmaf(gk, pk.y, z * rv.y), fmaf(gk, pk.z, z * rv.z),
                           fmaf(gk, pk.w, z * rv.w));
    }
  }
}

namespace {

template <int NR>
void enqueue_cgm_iteration(const CgmBatchBuffers& B, CgmScal* sc, int* snap, cudaStream_t st) {
  const Geom& g = rt().g;
  LinkView<float2> u{B.u32, g.sizeh, 6};
  const int nb = hop_blocks<NR>(g.sizeh);
  const long n = 3L * g.sizeh, n4 = n / 2;
  const int bps = seg_blocks(n4, NR);
  ReduceWs ws = reduce_ws(HopLayout<NR>::SLOTS, nb > NR * bps ? nb : NR * bps);
  k_cgm_snapshot<<<1, 32, 0, st>>>(sc, snap);
  const int pick = autotune_cached(TUNE_CGM_DOE, g.sizeh, NR * 2 + (B.ph32_mode == PH_SIGN8));
  launch_cgm_doe<NR>(kSplCand[pick > 0 && pick < 4 ? pick : 0], B, sc, st);
  if (B.ph32_mode == PH_SIGN8) k_cgm_deo_dot<NR, PH_SIGN8><<<nb, BT, 0, st>>>(g, u, B.ph32, B.t, B.p, B.s, n, sc, ws);
  else k_cgm_deo_dot<NR, PH_ANGLE><<<nb, BT, 0, st>>>(g, u, B.ph32, B.t, B.p, B.s, n, sc, ws);
  k_cgm_r<NR><<<NR * bps, RED_THREADS, 0, st>>>(reinterpret_cast<float4*>(B.r), reinterpret_cast<const float4*>(B.s),
                                                n4, n4, bps, sc, ws);
  // the x/p update streams nshift+1 fields per side: give it more blocks
  const int bxp = seg_blocks(n4 * (B.nshift + 1), NR);
  k_cgm_xp_dev<<<NR * bxp, RED_THREADS, 0, st>>>(reinterpret_cast<float4*>(B.p), reinterpret_cast<const float4*>(B.r),
                                                 reinterpret_cast<float4*>(B.xs), reinterpret_cast<float4*>(B.ps), n4,
                                                 n4, bxp, sc, snap);
}

}  // namespace

__global__ void k_cgm_copy_f(float2* __restrict__ dst, const float2* __restrict__ src, long n) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) dst[i] = src[i];
}

// The loop test of the device-side CG-M loop: continue while any
// right-hand side is still iterating.  trips counts the passes of the loop
// body; at max_trips (beyond the iteration limit, which sets done by
// itself) the loop stops and trips turns negative.
__global__ void k_cgm_continue(cudaGraphConditionalHandle h, const CgmScal* sc, int* trips, int max_trips) {
  int all = 1;
  for (int r = 0; r < sc->nrhs; ++r) all &= (sc->done[r] != 0);
  const int t = *trips + 1;
  *trips = t;
  if (!all && t >= max_trips) {
    *trips = -t;
    all = 1;
  }
  cudaGraphSetConditional(h, all ? 0u : 1u);
}

// All iterations of the batched CG-M as one graph launch: a while node whose
// body is `chunk` captured iterations followed by k_cgm_continue.  Returns
// false (nothing launched, no error recorded) where the graph cannot be
// built, and the caller runs its host-driven loop instead.
template <typename Enq>
bool cgm_device_loop(const Enq& enqueue_chunk, const CgmScal* sc, int* trips, int max_trips, int* trips_out,
                     cudaStream_t st) {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool ok = cudaGraphCreate(&graph, 0) == cudaSuccess;
  cudaGraphConditionalHandle handle{};
  if (ok) ok = cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  cudaGraphNodeParams cp{};
  cudaGraphNode_t node;
  if (ok) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    ok = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp) == cudaSuccess;
  }
  if (ok) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    ok = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
         cudaSuccess;
    if (ok) {
      const unsigned long long counted = g_kernel_launches;
      enqueue_chunk();
      k_cgm_continue<<<1, 1, 0, st>>>(handle, sc, trips, max_trips);
      g_kernel_launches = counted;
      ok = cudaStreamEndCapture(st, &body) == cudaSuccess;
    }
  }
  if (ok) ok = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
  if (graph) cudaGraphDestroy(graph);
  if (!ok) {
    if (exec) cudaGraphExecDestroy(exec);
    cudaGetLastError();
    return false;
  }
  OST_CUDA(cudaMemsetAsync(trips, 0, sizeof(int), st));
  OST_CUDA(cudaGraphLaunch(exec, st));
  OST_CUDA(cudaMemcpyAsync(trips_out, trips, sizeof(int), cudaMemcpyDeviceToHost, st));
  OST_CUDA(cudaStreamSynchronize(st));
  cudaGraphExecDestroy(exec);
  return true;
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
  reduce_ws_reserve(batch_reduce_partials(g.sizeh));   // allocated before any capture
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
  // launch shape of the D_oe (numerics-invariant; t is scratch), chosen before the capture
  switch (NR) {
    case 1: tune_cgm_doe<1>(B, st); break;
    case 2: tune_cgm_doe<2>(B, st); break;
    case 3: tune_cgm_doe<3>(B, st); break;
    default: tune_cgm_doe<4>(B, st); break;
  }
  // capture a chunk of iterations once per call (the buffers change per call)
  const int chunk = 8;
  auto enqueue_chunk = [&]() {
    for (int c = 0; c < chunk; ++c) {
      switch (NR) {
        case 1: enqueue_cgm_iteration<1>(B, sc, snap, st); break;
        case 2: enqueue_cgm_iteration<2>(B, sc, snap, st); break;
        case 3: enqueue_cgm_iteration<3>(B, sc, snap, st); break;
        default: enqueue_cgm_iteration<4>(B, sc, snap, st); break;
      }
    }
  };
  // the whole iteration on the device: one graph launch with a while node
  int* trips = snap + 8;
  const int max_trips = max_iter / chunk + 2;
  int trips_h = 0;
  out.device_loop = device_loop_enabled() && cgm_device_loop(enqueue_chunk, sc, trips, max_trips, &trips_h, st);
  if (out.device_loop) {
    const int passes = trips_h < 0 ? -trips_h : trips_h;
    g_kernel_launches += (5ull * chunk + 1) * passes;
    if (trips_h < 0) set_error(-15, "batched CG-M: the device loop stopped at its bound of %d passes", max_trips);
  } else {
    // host-driven: replay a captured chunk, poll the flags after each
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    const unsigned long long counted = g_kernel_launches;
    OST_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    enqueue_chunk();
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
    cudaGraphExecDestroy(exec);
  }
  OST_CUDA(cudaMemcpyAsync(h, sc, sizeof(CgmScal), cudaMemcpyDeviceToHost, st));
  OST_CUDA(cudaStreamSynchronize(st));
  for (int r = 0; r < NR; ++r) out.iters[r] = h->iter[r];
  cudaFreeHost(h);
  return out;
}

}  // namespace ost
