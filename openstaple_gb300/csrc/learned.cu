// learned.cu -- forward and backward kernels of the gauge-covariant network
// (see learned.cuh).  Forward: one thread per output site builds the 64
// transported vectors h_{d,c} in FP32, rounds them to BF16 into shared-memory
// tiles laid out for tcgen05 (one tile per real colour component), one
// thread issues the 6 x 4 BF16 MMAs (M = 128 sites, N = 16, K = 64) into
// tensor memory, and every warp reads its 32 rows back.  Weight gradient:
// the same transport, with tiles transposed so that the MMA contracts over
// the 128 sites of a tile and accumulates over all tiles of the CTA.  Input
// gradient: the adjoint hop structure in FP32 SIMT.
//
// Every wait on an MMA completion is bounded; a timeout sets nb.err and the
// kernel still releases its tensor memory.
#include <cstring>
#include "dslash.cuh"
#include "learned.cuh"
#include "reduce.cuh"
#include "runtime.cuh"
#include "tc.cuh"

namespace ost {

static constexpr int NT = 128;                       // threads = sites per tile
static constexpr long WAIT_LIMIT = 1L << 22;         // mbarrier polls before giving up

// ---- transport of the 8 input channels along hop d for output site idx ----
struct HopCtx {
  int j;              // neighbour (input parity) index
  int li;             // link index
  int dir;
  bool back;
};

OST_D HopCtx hop_ctx(const int fwd[4], const int bwd[4], int idx, int d, int p_out) {
  HopCtx h;
  const int mu = d & 3;
  h.back = d >= 4;
  h.dir = h.back ? 2 * mu + (1 - p_out) : 2 * mu + p_out;
  h.j = h.back ? bwd[mu] : fwd[mu];
  h.li = h.back ? bwd[mu] : idx;
  return h;
}

// h[a][c], a = 2*colour + (0 re, 1 im), for channels c0 .. c0+NCH-1 of
// activation act
template <int NCH>
OST_D void transport_ch(const LinkView<float2>& u, const unsigned char* signs, long sh, const HopCtx& hc,
                        const __nv_bfloat162* act, int c0, float h[6][NCH]) {
  float2 m[6];
  load_two_rows(u, hc.dir, hc.li, m);
  const unsigned char sb = __ldg(signs + long(hc.dir) * sh + hc.li);
  float2 vin[NCH][3];
#pragma unroll
  for (int c = 0; c < NCH; ++c)     // every load of the hop first
#pragma unroll
    for (int col = 0; col < 3; ++col) vin[c][col] = __bfloat1622float2(act[(long(c0 + c) * 3 + col) * sh + hc.j]);
  // the staggered sign multiplies the whole matrix (third row rebuilt from the
  // unsigned rows, then all nine entries flipped) instead of every channel
  float2 r3[3] = {conj_cross(m[1], m[5], m[2], m[4]), conj_cross(m[2], m[3], m[0], m[5]),
                  conj_cross(m[0], m[4], m[1], m[3])};
  const unsigned mask = sb ? 0x80000000u : 0u;
#pragma unroll
  for (int e = 0; e < 6; ++e) { m[e].x = flip_sign(m[e].x, mask); m[e].y = flip_sign(m[e].y, mask); }
#pragma unroll
  for (int e = 0; e < 3; ++e) { r3[e].x = flip_sign(r3[e].x, mask); r3[e].y = flip_sign(r3[e].y, mask); }
#pragma unroll
  for (int c = 0; c < NCH; ++c) {
    float2 aux[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    const float2* v = vin[c];
    if (hc.back) {   // U^+ v
      cmacc(aux[0], m[0], v[0]); cmacc(aux[0], m[3], v[1]); cmacc(aux[0], r3[0], v[2]);
      cmacc(aux[1], m[1], v[0]); cmacc(aux[1], m[4], v[1]); cmacc(aux[1], r3[1], v[2]);
      cmacc(aux[2], m[2], v[0]); cmacc(aux[2], m[5], v[1]); cmacc(aux[2], r3[2], v[2]);
    } else {         // U v
      cmac(aux[0], m[0], v[0]); cmac(aux[0], m[1], v[1]); cmac(aux[0], m[2], v[2]);
      cmac(aux[1], m[3], v[0]); cmac(aux[1], m[4], v[1]); cmac(aux[1], m[5], v[2]);
      cmac(aux[2], r3[0], v[0]); cmac(aux[2], r3[1], v[1]); cmac(aux[2], r3[2], v[2]);
    }
#pragma unroll
    for (int col = 0; col < 3; ++col) { h[2 * col][c] = aux[col].x; h[2 * col + 1][c] = aux[col].y; }
  }
}

OST_D void transport8(const LinkView<float2>& u, const unsigned char* signs, long sh, const HopCtx& hc,
                      const __nv_bfloat162* act, float h[6][NET_C]) {
  transport_ch<NET_C>(u, signs, sh, hc, act, 0, h);
}

OST_D uint4 pack8_bf16(const float* v) {
  __nv_bfloat162 a = __floats2bfloat162_rn(v[0], v[1]), b = __floats2bfloat162_rn(v[2], v[3]);
  __nv_bfloat162 c = __floats2bfloat162_rn(v[4], v[5]), d = __floats2bfloat162_rn(v[6], v[7]);
  uint4 r;
  r.x = *reinterpret_cast<uint32_t*>(&a); r.y = *reinterpret_cast<uint32_t*>(&b);
  r.z = *reinterpret_cast<uint32_t*>(&c); r.w = *reinterpret_cast<uint32_t*>(&d);
  return r;
}

OST_D uint2 pack4_bf16(const float* v) {
  __nv_bfloat162 a = __floats2bfloat162_rn(v[0], v[1]), b = __floats2bfloat162_rn(v[2], v[3]);
  uint2 r;
  r.x = *reinterpret_cast<uint32_t*>(&a);
  r.y = *reinterpret_cast<uint32_t*>(&b);
  return r;
}

// ---- forward layer ----
// dynamic shared memory: 6 A tiles [128 x 64] BF16 (16 KB each), B tile [16 x 64] BF16.
// Two threads per site: thread half 0 transports channels 0-3, half 1
// channels 4-7, so a tile of 128 sites runs 8 warps (two CTAs per SM).
static constexpr int FWD_A_BYTES = NT * NET_K * 2;
static constexpr int FWD_SMEM = 6 * FWD_A_BYTES + NET_N * NET_K * 2;
static constexpr int FWD_THREADS = 2 * NT;
static constexpr int FWD_HALF = NET_C / 2;

template <int P_OUT, bool OUT_F32>
__global__ void __launch_bounds__(FWD_THREADS, 2)
k_net_fwd(Geom g, LinkView<float2> u, const unsigned char* __restrict__ signs, const __nv_bfloat162* __restrict__ act_in,
          const __nv_bfloat16* __restrict__ w, __nv_bfloat162* __restrict__ act_out, float2* __restrict__ out_f32,
          int* err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & (NT - 1);          // site of the tile = TMEM lane
  const int half = tid / NT;               // channel half
  const long sh = g.sizeh;
  const int idx = blockIdx.x * NT + row;
  const bool valid = idx < g.sizeh;
  unsigned char* Abase = smem;
  unsigned char* B = smem + 6 * FWD_A_BYTES;
  if (warp == 0) tc::tmem_alloc(&tslot, 128);
  if (tid == 0) tc::mbar_init(&mbar, 1);
  // weights as the B operand: B[n][k] = W[k][n]
  for (int e = tid; e < NET_N * NET_K; e += FWD_THREADS) {
    const int n = e / NET_K, k = e % NET_K;
    *reinterpret_cast<__nv_bfloat16*>(B + tc::kmajor_offset(n, k, NET_K)) = w[e];
  }
  int fwd[4] = {0, 0, 0, 0}, bwd[4] = {0, 0, 0, 0};
  if (valid) {
    Site s = site_of(g, idx, P_OUT);
    neighbours(g, s, fwd, bwd);
  }
#pragma unroll
  for (int d = 0; d < 8; ++d) {
    float h[6][FWD_HALF];
    if (valid) {
      transport_ch<FWD_HALF>(u, signs, sh, hop_ctx(fwd, bwd, idx, d, P_OUT), act_in, half * FWD_HALF, h);
    } else {
#pragma unroll
      for (int a = 0; a < 6; ++a)
#pragma unroll
        for (int c = 0; c < FWD_HALF; ++c) h[a][c] = 0.f;
    }
#pragma unroll
    for (int a = 0; a < 6; ++a)
      *reinterpret_cast<uint2*>(Abase + a * FWD_A_BYTES + tc::kmajor_offset(row, d * NET_C + half * FWD_HALF, NET_K)) =
          pack4_bf16(h[a]);
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = tslot;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, NET_N);
    for (int a = 0; a < 6; ++a)
      for (int ks = 0; ks < NET_K / 16; ++ks) {
        uint64_t ad = tc::make_desc(tc::smem_u32(Abase + a * FWD_A_BYTES) + ks * 256, 128, NET_K * 16);
        uint64_t bd = tc::make_desc(tc::smem_u32(B) + ks * 256, 128, NET_K * 16);
        tc::mma_bf16(taddr + a * NET_N, ad, bd, idesc, ks > 0);
      }
    tc::mma_commit(&mbar);
  }
  const bool ok = tc::mbar_wait_bounded(&mbar, 0, WAIT_LIMIT);
  if (!ok && (tid & 31) == 0) atomicExch(err, 1);
  tc::fence_after_sync();
  // a warp reads the TMEM lanes of its sub-partition (warp % 4): both
  // halves see the same 32 sites and store their own output channels
  float o[6][NET_N];
#pragma unroll
  for (int a = 0; a < 6; ++a) tc::tmem_ld16(taddr + (uint32_t((warp & 3) * 32) << 16) + a * NET_N, o[a]);
  if (valid && ok) {
    if (OUT_F32) {
      if (half == 0) {
#pragma unroll
        for (int col = 0; col < 3; ++col) out_f32[col * sh + idx] = make_float2(o[2 * col][0], o[2 * col + 1][0]);
      }
    } else {
#pragma unroll
      for (int c = 0; c < FWD_HALF; ++c)
#pragma unroll
        for (int col = 0; col < 3; ++col) {
          // compile-time register indices, selected by the half
          const float re = half ? o[2 * col][FWD_HALF + c] : o[2 * col][c];
          const float im = half ? o[2 * col + 1][FWD_HALF + c] : o[2 * col + 1][c];
          act_out[(long(half * FWD_HALF + c) * 3 + col) * sh + idx] = __floats2bfloat162_rn(re, im);
        }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, 128);
}

// ---- weight gradient: dW[k][n] = sum_{sites, a} h_a[site][k] g_a[site][n] ----
// A tile of component pair p: rows 0..63 = h_{2p}^T, rows 64..127 = h_{2p+1}^T,
// K = 128 sites; B tile: rows 0..7 = g_{2p}^T, rows 8..15 = g_{2p+1}^T.  The
// wanted blocks are D[0:64][0:8] and D[64:128][8:16].
static constexpr int DW_A_BYTES = 128 * NT * 2;     // [128 x 128] BF16
static constexpr int DW_B_BYTES = NET_N * NT * 2;   // [16 x 128] BF16
static constexpr int DW_SMEM = 3 * DW_A_BYTES + 3 * DW_B_BYTES;

template <int P_OUT>
__global__ void __launch_bounds__(NT, 1)
k_net_dw(Geom g, LinkView<float2> u, const unsigned char* __restrict__ signs, const __nv_bfloat162* __restrict__ act_in,
         const float2* __restrict__ g_out, float* __restrict__ partials, int* err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  __shared__ float part[NET_K][NET_C];
  const int tid = threadIdx.x, warp = tid >> 5;
  const long sh = g.sizeh;
  unsigned char* A = smem;
  unsigned char* B = smem + 3 * DW_A_BYTES;
  if (warp == 0) tc::tmem_alloc(&tslot, 32);
  if (tid == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = tslot;
  const int ntiles = (g.sizeh + NT - 1) / NT;
  int done_tiles = 0;
  bool ok = true;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int idx = t * NT + tid;
    const bool valid = idx < g.sizeh;
    int fwd[4] = {0, 0, 0, 0}, bwd[4] = {0, 0, 0, 0};
    if (valid) {
      Site s = site_of(g, idx, P_OUT);
      neighbours(g, s, fwd, bwd);
    }
    // A: transported inputs, transposed (row = k, column = site)
#pragma unroll 1
    for (int d = 0; d < 8; ++d) {
      float h[6][NET_C];
      if (valid) transport8(u, signs, sh, hop_ctx(fwd, bwd, idx, d, P_OUT), act_in, h);
      else {
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
          for (int c = 0; c < NET_C; ++c) h[a][c] = 0.f;
      }
#pragma unroll
      for (int a = 0; a < 6; ++a) {
        unsigned char* tile = A + (a >> 1) * DW_A_BYTES;
        const int row0 = (a & 1) * 64 + d * NET_C;
#pragma unroll
        for (int c = 0; c < NET_C; ++c)
          *reinterpret_cast<__nv_bfloat16*>(tile + tc::kmajor_offset(row0 + c, tid, NT)) = __float2bfloat16_rn(h[a][c]);
      }
    }
    // B: output gradients, transposed (row = channel, column = site)
#pragma unroll
    for (int col = 0; col < 3; ++col)
#pragma unroll
      for (int c = 0; c < NET_C; ++c) {
        float2 gv = valid ? g_out[(long(c) * 3 + col) * sh + idx] : make_float2(0.f, 0.f);
        unsigned char* tile = B + col * DW_B_BYTES;
        *reinterpret_cast<__nv_bfloat16*>(tile + tc::kmajor_offset(c, tid, NT)) = __float2bfloat16_rn(gv.x);
        *reinterpret_cast<__nv_bfloat16*>(tile + tc::kmajor_offset(8 + c, tid, NT)) = __float2bfloat16_rn(gv.y);
      }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      const uint32_t idesc = tc::idesc_bf16(128, NET_N);
      for (int pr = 0; pr < 3; ++pr)
        for (int ks = 0; ks < NT / 16; ++ks) {
          uint64_t ad = tc::make_desc(tc::smem_u32(A + pr * DW_A_BYTES) + ks * 256, 128, NT * 16);
          uint64_t bd = tc::make_desc(tc::smem_u32(B + pr * DW_B_BYTES) + ks * 256, 128, NT * 16);
          tc::mma_bf16(taddr, ad, bd, idesc, (done_tiles > 0 || pr > 0 || ks > 0) ? 1 : 0);
        }
      tc::mma_commit(&mbar);
    }
    // the tiles are rewritten next round: wait for the MMAs that read them
    ok = ok && tc::mbar_wait_bounded(&mbar, done_tiles & 1, WAIT_LIMIT);
    tc::fence_after_sync();
    __syncthreads();
    ++done_tiles;
  }
  if (!ok && (tid & 31) == 0) atomicExch(err, 1);
  float dv[16];
  if (done_tiles > 0) tc::tmem_ld16(taddr + (uint32_t(warp * 32) << 16), dv);
  else {
#pragma unroll
    for (int i = 0; i < 16; ++i) dv[i] = 0.f;
  }
  const int m = tid;   // TMEM lane = D row
  if (m < 64) {
#pragma unroll
    for (int n = 0; n < NET_C; ++n) part[m][n] = dv[n];
  }
  __syncthreads();
  if (m >= 64) {
#pragma unroll
    for (int n = 0; n < NET_C; ++n) part[m - 64][n] += dv[8 + n];
  }
  __syncthreads();
  for (int e = tid; e < NET_K * NET_C; e += NT) partials[long(blockIdx.x) * NET_K * NET_C + e] = (&part[0][0])[e];
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, 32);
}

__global__ void k_net_dw_sum(const float* __restrict__ partials, int nblocks, float* dw) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= NET_K * NET_C) return;
  float s = 0.f;
  for (int b = 0; b < nblocks; ++b) s += partials[long(b) * NET_K * NET_C + e];
  dw[e] += s;
}

// ---- input gradient: g_in(y) = sum_d T_d^+ (W_d^T g_out) (adjoint of the hops) ----
template <int P_IN>
__global__ void __launch_bounds__(128)
k_net_bwd_in(Geom g, LinkView<float2> u, const unsigned char* __restrict__ signs, const float2* __restrict__ g_out,
             const float* __restrict__ w /* [64][8] */, float2* __restrict__ g_in) {
  __shared__ float ws[NET_K][NET_C];
  for (int e = threadIdx.x; e < NET_K * NET_C; e += blockDim.x) (&ws[0][0])[e] = w[e];
  __syncthreads();
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= g.sizeh) return;
  const int P_OUT = 1 - P_IN;
  const long sh = g.sizeh;
  Site s = site_of(g, y, P_IN);
  int fwd[4], bwd[4];
  neighbours(g, s, fwd, bwd);
  float2 acc[NET_C][3];
#pragma unroll
  for (int c = 0; c < NET_C; ++c)
#pragma unroll
    for (int col = 0; col < 3; ++col) acc[c][col] = make_float2(0.f, 0.f);
#pragma unroll 1
  for (int e = 0; e < 8; ++e) {
    const int mu = e & 3;
    // e < 4: the output site x = y - mu read y through its forward hop mu (link U_mu(x));
    // e >= 4: x = y + mu read y through its backward hop 4+mu (link U_mu(y))
    const bool fwd_hop = e < 4;
    const int x = fwd_hop ? bwd[mu] : fwd[mu];
    const int dir = fwd_hop ? 2 * mu + P_OUT : 2 * mu + P_IN;
    const int li = fwd_hop ? x : y;
    const int d = fwd_hop ? mu : 4 + mu;
    float2 m[6];
    load_two_rows(u, dir, li, m);
    const unsigned mask = __ldg(signs + long(dir) * sh + li) ? 0x80000000u : 0u;
    float2 go[NET_C][3];
#pragma unroll
    for (int n = 0; n < NET_C; ++n)
#pragma unroll
      for (int col = 0; col < 3; ++col) go[n][col] = g_out[(long(n) * 3 + col) * sh + x];
#pragma unroll
    for (int c = 0; c < NET_C; ++c) {
      float2 dh[3];
#pragma unroll
      for (int col = 0; col < 3; ++col) {
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int n = 0; n < NET_C; ++n) {
          const float wv = ws[d * NET_C + c][n];
          re = fmaf(wv, go[n][col].x, re);
          im = fmaf(wv, go[n][col].y, im);
        }
        dh[col] = make_float2(flip_sign(re, mask), flip_sign(im, mask));
      }
      // forward hop used U: its adjoint applies U^+; backward hop used U^+: adjoint applies U
      if (fwd_hop) mac_Udag(acc[c], m, dh);
      else mac_U(acc[c], m, dh);
    }
  }
#pragma unroll
  for (int c = 0; c < NET_C; ++c)
#pragma unroll
    for (int col = 0; col < 3; ++col) g_in[(long(c) * 3 + col) * sh + y] = acc[c][col];
}

// ---- small kernels ----
__global__ void k_net_input(const float2* __restrict__ r, __nv_bfloat162* __restrict__ act, long sh) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < 3 * sh; i += long(gridDim.x) * blockDim.x) {
    act[i] = __float22bfloat162_rn(r[i]);                      // channel 0
    for (int c = 1; c < NET_C; ++c) act[long(c) * 3 * sh + i] = __floats2bfloat162_rn(0.f, 0.f);
  }
}

// Residual loss of one pair: with w = A (z - x) and aw = A w (A the
// Hermitian operator the network preconditions), L = |w|^2 / |b|^2 and
// dL/dz = 2 A w / |b|^2.  Writes dL/dz into channel 0 of g (channels 1..7
// zeroed) and accumulates L * scale into loss[0].
__global__ void k_net_res_loss(const float2* __restrict__ w, const float2* __restrict__ aw, float2* __restrict__ gbuf,
                               long sh, double scale, ReduceWs ws, double* loss, int accumulate) {
  double v[1] = {0.0};
  const float g2 = float(2.0 * scale);
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < 3 * sh; i += long(gridDim.x) * blockDim.x) {
    const float2 a = w[i], b = aw[i];
    v[0] += double(a.x) * a.x + double(a.y) * a.y;
    gbuf[i] = make_float2(g2 * b.x, g2 * b.y);
    for (int c = 1; c < NET_C; ++c) gbuf[long(c) * 3 * sh + i] = make_float2(0.f, 0.f);
  }
  double tot[1];
  if (grid_reduce<1>(v, ws, tot)) loss[0] = (accumulate ? loss[0] : 0.0) + tot[0] * scale;
}

__global__ void k_net_adam(float* w, float* m, float* v, const float* dw, int n, float lr, float b1, float b2,
                           float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = dw[i];
  const float mi = b1 * m[i] + (1.f - b1) * g;
  const float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// master [L][64][8] -> MMA operand source [L][16][64] (n >= 8 zero)
__global__ void k_net_sync(const float* __restrict__ w, __nv_bfloat16* __restrict__ wm) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= NET_LAYERS * NET_N * NET_K) return;
  const int l = e / (NET_N * NET_K), r = e % (NET_N * NET_K), n = r / NET_K, k = r % NET_K;
  wm[e] = __float2bfloat16_rn(n < NET_C ? w[(l * NET_K + k) * NET_C + n] : 0.f);
}

// ---- launchers ----
static bool g_attr_set = false;
static void set_attrs() {
  if (g_attr_set) return;
  OST_CUDA(cudaFuncSetAttribute(k_net_fwd<0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, FWD_SMEM));
  OST_CUDA(cudaFuncSetAttribute(k_net_fwd<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, FWD_SMEM));
  OST_CUDA(cudaFuncSetAttribute(k_net_fwd<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, FWD_SMEM));
  OST_CUDA(cudaFuncSetAttribute(k_net_fwd<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, FWD_SMEM));
  OST_CUDA(cudaFuncSetAttribute(k_net_dw<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, DW_SMEM));
  OST_CUDA(cudaFuncSetAttribute(k_net_dw<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, DW_SMEM));
  g_attr_set = true;
}

static __nv_bfloat162* act_of(const NetBuffers& nb, int l) {
  return nb.act + size_t(l) * NET_C * 3 * size_t(rt().g.sizeh);
}

void net_load_input(const NetBuffers& nb, const float2* r, cudaStream_t st) {
  k_net_input<<<8 * rt().num_sms, 256, 0, st>>>(r, act_of(nb, 0), rt().g.sizeh);
  OST_LAUNCH_CHECK();
}

void net_layer_forward(const NetBuffers& nb, int layer, const float2* u32, const unsigned char* signs,
                       float2* out_f32, cudaStream_t st) {
  set_attrs();
  const Geom& g = rt().g;
  LinkView<float2> u{u32, g.sizeh, 6};
  const int nb_ = blocks_for(g.sizeh, NT);
  const int p_out = (layer & 1) ? 0 : 1;   // even -> odd -> even -> odd -> even
  const __nv_bfloat16* w = nb.w_mma + size_t(layer) * NET_N * NET_K;
  const bool last = layer == NET_LAYERS - 1;
  __nv_bfloat162* out = last ? nullptr : act_of(nb, layer + 1);
  if (p_out == 1 && !last) k_net_fwd<1, false><<<nb_, FWD_THREADS, FWD_SMEM, st>>>(g, u, signs, act_of(nb, layer), w, out, out_f32, nb.err);
  else if (p_out == 0 && !last) k_net_fwd<0, false><<<nb_, FWD_THREADS, FWD_SMEM, st>>>(g, u, signs, act_of(nb, layer), w, out, out_f32, nb.err);
  else k_net_fwd<0, true><<<nb_, FWD_THREADS, FWD_SMEM, st>>>(g, u, signs, act_of(nb, layer), w, out, out_f32, nb.err);
  OST_LAUNCH_CHECK();
}

void net_residual_loss_grad(const NetBuffers& nb, const float2* w, const float2* aw, double scale, int accumulate,
                            cudaStream_t st) {
  const long sh = rt().g.sizeh;
  const int gr = reduce_grid(3 * sh);
  k_net_res_loss<<<gr, RED_THREADS, 0, st>>>(w, aw, reinterpret_cast<float2*>(nb.grad_a), sh, scale,
                                             reduce_ws(1, gr), nb.loss, accumulate);
  OST_LAUNCH_CHECK();
}

void net_layer_backward(const NetBuffers& nb, int layer, const float2* u32, const unsigned char* signs,
                        const float* g_out, float* g_in, int need_g_in, cudaStream_t st) {
  set_attrs();
  const Geom& g = rt().g;
  LinkView<float2> u{u32, g.sizeh, 6};
  const int p_out = (layer & 1) ? 0 : 1;
  const int ntiles = blocks_for(g.sizeh, NT);
  const int grid = ntiles < 2 * rt().num_sms ? ntiles : 2 * rt().num_sms;
  if (p_out == 1)
    k_net_dw<1><<<grid, NT, DW_SMEM, st>>>(g, u, signs, act_of(nb, layer), reinterpret_cast<const float2*>(g_out),
                                           nb.dw_partials, nb.err);
  else
    k_net_dw<0><<<grid, NT, DW_SMEM, st>>>(g, u, signs, act_of(nb, layer), reinterpret_cast<const float2*>(g_out),
                                           nb.dw_partials, nb.err);
  OST_LAUNCH_CHECK();
  k_net_dw_sum<<<(NET_K * NET_C + 255) / 256, 256, 0, st>>>(nb.dw_partials, grid, nb.dw + size_t(layer) * NET_K * NET_C);
  OST_LAUNCH_CHECK();
  if (need_g_in) {
    const float* w = nb.w_master + size_t(layer) * NET_K * NET_C;
    if (p_out == 1)   // input parity even
      k_net_bwd_in<0><<<blocks_for(g.sizeh, 128), 128, 0, st>>>(g, u, signs, reinterpret_cast<const float2*>(g_out), w,
                                                                 reinterpret_cast<float2*>(g_in));
    else
      k_net_bwd_in<1><<<blocks_for(g.sizeh, 128), 128, 0, st>>>(g, u, signs, reinterpret_cast<const float2*>(g_out), w,
                                                                 reinterpret_cast<float2*>(g_in));
    OST_LAUNCH_CHECK();
  }
}

void net_adam_step(const NetBuffers& nb, float lr, float b1, float b2, float eps, int t, cudaStream_t st) {
  const int n = NET_LAYERS * NET_K * NET_C;
  const float c1 = 1.f - powf(b1, float(t)), c2 = 1.f - powf(b2, float(t));
  k_net_adam<<<(n + 255) / 256, 256, 0, st>>>(nb.w_master, nb.adam_m, nb.adam_v, nb.dw, n, lr, b1, b2, eps, c1, c2);
  OST_LAUNCH_CHECK();
  net_sync_weights(nb, st);
}

void net_sync_weights(const NetBuffers& nb, cudaStream_t st) {
  const int n = NET_LAYERS * NET_N * NET_K;
  k_net_sync<<<(n + 255) / 256, 256, 0, st>>>(nb.w_master, nb.w_mma);
  OST_LAUNCH_CHECK();
}

void net_zero_dw(const NetBuffers& nb, cudaStream_t st) {
  OST_CUDA(cudaMemsetAsync(nb.dw, 0, sizeof(float) * NET_LAYERS * NET_K * NET_C, st));
}

}  // namespace ost

namespace ost {

// Self-test of the bounded-wait path used by every tensor-core kernel: one
// thread initialises an mbarrier for one arrival, arrives on it or not, and
// waits with the same bounded poll as the MMA completion waits.  Without the
// arrival the wait runs out after `polls` polls and the error word is set,
// exactly as a lost MMA completion would; the kernel returns normally.
__global__ void k_wait_selftest(int signal, long polls, int* err) {
  __shared__ __align__(8) uint64_t mbar;
  if (threadIdx.x != 0) return;
  tc::mbar_init(&mbar, 1);
  if (signal) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(tc::smem_u32(&mbar)) : "memory");
  if (!tc::mbar_wait_bounded(&mbar, 0, polls)) atomicExch(err, 1);
}

void net_wait_selftest(const NetBuffers& nb, int signal, long polls, cudaStream_t st) {
  k_wait_selftest<<<1, 32, 0, st>>>(signal, polls, nb.err);
  OST_LAUNCH_CHECK();
}

}  // namespace ost
