// dslash_df.cu -- the staggered hop term and M^+M in double-float arithmetic
// (see dslash_df.cuh).  Same operator as the FP64 kernels -- backward hops
// first, then forward hops, each e^{i theta} U v with the third link row
// rebuilt as conj(r0 x r1) (fermion_matrix.c:47-157, matvecmul.h:88-172) --
// restricted to phases of 0 or pi, which become sign flips.
#include "dslash_df.cuh"
#include "dslash.cuh"
#include "runtime.cuh"

namespace ost {

namespace {

constexpr int DF_THREADS = 128;

// The transformations below rely on every operation being rounded on its
// own: the _rn intrinsics are never contracted into an FMA by the compiler
// (a fused a*b + c inside two_sum would count the product's error twice).

// Knuth's two-sum: s + e = a + b exactly.
OST_D void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// Dekker's fast two-sum (|a| >= |b|): s + e = a + b exactly.
OST_D void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

// A real double-float accumulator hi + lo; lo collects the rounding errors
// of the products and of the running sum and is folded in at the end.
struct DfAcc {
  float hi, lo;
};

// acc += (ah + al) * (bh + bl), dropping al*bl (below 2^-46 of the product)
OST_D void df_fma(DfAcc& acc, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  float e = fmaf(ah, bh, -p);          // exact error of p
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  float s, t;
  two_sum(acc.hi, p, s, t);
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(t, e));
}

// Complex double-float number (hi.x + lo.x) + i (hi.y + lo.y).
struct DfC {
  float2 hi, lo;
};

OST_D DfC df_norm(const DfAcc& re, const DfAcc& im) {
  DfC z;
  fast_two_sum(re.hi, re.lo, z.hi.x, z.lo.x);
  fast_two_sum(im.hi, im.lo, z.hi.y, z.lo.y);
  return z;
}

// conj(a*b - c*d): the third link row from rows 0 and 1
OST_D DfC df_conj_cross(const DfC& a, const DfC& b, const DfC& c, const DfC& d) {
  DfAcc re{0.f, 0.f}, im{0.f, 0.f};
  df_fma(re, a.hi.x, a.lo.x, b.hi.x, b.lo.x);
  df_fma(re, -a.hi.y, -a.lo.y, b.hi.y, b.lo.y);
  df_fma(re, -c.hi.x, -c.lo.x, d.hi.x, d.lo.x);
  df_fma(re, c.hi.y, c.lo.y, d.hi.y, d.lo.y);
  df_fma(im, a.hi.x, a.lo.x, b.hi.y, b.lo.y);
  df_fma(im, a.hi.y, a.lo.y, b.hi.x, b.lo.x);
  df_fma(im, -c.hi.x, -c.lo.x, d.hi.y, d.lo.y);
  df_fma(im, -c.hi.y, -c.lo.y, d.hi.x, d.lo.x);
  DfC z = df_norm(re, im);
  z.hi.y = -z.hi.y;
  z.lo.y = -z.lo.y;
  return z;
}

// acc += m * v (CONJ: conj(m) * v)
template <bool CONJ>
OST_D void df_cmac(DfAcc& re, DfAcc& im, const DfC& m, const DfC& v) {
  const float sh = CONJ ? -m.hi.y : m.hi.y, sl = CONJ ? -m.lo.y : m.lo.y;
  df_fma(re, m.hi.x, m.lo.x, v.hi.x, v.lo.x);
  df_fma(re, -sh, -sl, v.hi.y, v.lo.y);
  df_fma(im, m.hi.x, m.lo.x, v.hi.y, v.lo.y);
  df_fma(im, sh, sl, v.hi.x, v.lo.x);
}

OST_D DfC ld_df(const float2* hi, const float2* lo, long i) {
  DfC z;
  z.hi = __ldg(hi + i);
  z.lo = __ldg(lo + i);
  return z;
}
OST_D DfC ld_df_stream(const float2* hi, const float2* lo, long i) {
  DfC z;
  z.hi = __ldcs(hi + i);
  z.lo = __ldcs(lo + i);
  return z;
}

// Hop term of parity P at idx: re/im accumulators of the three colours.
template <int P>
OST_D void df_hop(const Geom& g, const DfOperator& op, const float2* in_hi, const float2* in_lo, int idx,
                  DfAcc re[3], DfAcc im[3]) {
  const long sh = g.sizeh;
  Site s = site_of(g, idx, P);
  int fwd[4], bwd[4];
  neighbours(g, s, fwd, bwd);
#pragma unroll
  for (int c = 0; c < 3; ++c) { re[c] = DfAcc{0.f, 0.f}; im[c] = DfAcc{0.f, 0.f}; }
#pragma unroll
  for (int hm = 0; hm < 8; ++hm) {
    const bool back = hm < 4;        // backward hops first, as in the reference
    const int mu = hm & 3;
    const int dir = back ? 2 * mu + (1 - P) : 2 * mu + P;
    const int nb = back ? bwd[mu] : fwd[mu];
    const int li = back ? nb : idx;
    DfC m[6], v[3];
#pragma unroll
    for (int e = 0; e < 6; ++e) m[e] = ld_df_stream(op.u_hi, op.u_lo, (long(dir) * 6 + e) * sh + li);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = ld_df(in_hi, in_lo, c * sh + nb);
    // sign: staggered/boundary sign of the link, and -1 for a backward hop
    const bool neg = (__ldg(op.signs + long(dir) * sh + li) != 0) != back;
    if (neg) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        v[c].hi.x = -v[c].hi.x; v[c].hi.y = -v[c].hi.y;
        v[c].lo.x = -v[c].lo.x; v[c].lo.y = -v[c].lo.y;
      }
    }
    const DfC r20 = df_conj_cross(m[1], m[5], m[2], m[4]);
    const DfC r21 = df_conj_cross(m[2], m[3], m[0], m[5]);
    const DfC r22 = df_conj_cross(m[0], m[4], m[1], m[3]);
    if (back) {   // U^+ v
      df_cmac<true>(re[0], im[0], m[0], v[0]); df_cmac<true>(re[0], im[0], m[3], v[1]);
      df_cmac<true>(re[0], im[0], r20, v[2]);
      df_cmac<true>(re[1], im[1], m[1], v[0]); df_cmac<true>(re[1], im[1], m[4], v[1]);
      df_cmac<true>(re[1], im[1], r21, v[2]);
      df_cmac<true>(re[2], im[2], m[2], v[0]); df_cmac<true>(re[2], im[2], m[5], v[1]);
      df_cmac<true>(re[2], im[2], r22, v[2]);
    } else {      // U v
      df_cmac<false>(re[0], im[0], m[0], v[0]); df_cmac<false>(re[0], im[0], m[1], v[1]);
      df_cmac<false>(re[0], im[0], m[2], v[2]);
      df_cmac<false>(re[1], im[1], m[3], v[0]); df_cmac<false>(re[1], im[1], m[4], v[1]);
      df_cmac<false>(re[1], im[1], m[5], v[2]);
      df_cmac<false>(re[2], im[2], r20, v[0]); df_cmac<false>(re[2], im[2], r21, v[1]);
      df_cmac<false>(re[2], im[2], r22, v[2]);
    }
  }
}

// t = D_oe x (hi/lo out; the factor 1/2 is exact)
__global__ void __launch_bounds__(DF_THREADS)
k_df_doe(Geom g, DfOperator op, const float2* __restrict__ x_hi, const float2* __restrict__ x_lo,
         float2* __restrict__ t_hi, float2* __restrict__ t_lo) {
  const int idx = blockIdx.x * DF_THREADS + threadIdx.x;
  if (idx >= g.sizeh) return;
  DfAcc re[3], im[3];
  df_hop<1>(g, op, x_hi, x_lo, idx, re, im);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const DfC z = df_norm(re[c], im[c]);
    const long q = c * long(g.sizeh) + idx;
    t_hi[q] = make_float2(0.5f * z.hi.x, 0.5f * z.hi.y);
    t_lo[q] = make_float2(0.5f * z.lo.x, 0.5f * z.lo.y);
  }
}

// out = m2 x - D_eo t, with the last step in FP64
__global__ void __launch_bounds__(DF_THREADS)
k_df_deo_mdagm(Geom g, DfOperator op, const float2* __restrict__ t_hi, const float2* __restrict__ t_lo,
               const double2* __restrict__ x, double2* __restrict__ out, double m2) {
  const int idx = blockIdx.x * DF_THREADS + threadIdx.x;
  if (idx >= g.sizeh) return;
  DfAcc re[3], im[3];
  df_hop<0>(g, op, t_hi, t_lo, idx, re, im);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const long q = c * long(g.sizeh) + idx;
    const double2 xv = x[q];
    const double ar = double(re[c].hi) + double(re[c].lo);
    const double ai = double(im[c].hi) + double(im[c].lo);
    out[q] = make_double2(fma(m2, xv.x, -0.5 * ar), fma(m2, xv.y, -0.5 * ai));
  }
}

__global__ void k_df_split(const double2* __restrict__ x, float2* __restrict__ hi, float2* __restrict__ lo, long n) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    const double2 v = x[i];
    const float hx = float(v.x), hy = float(v.y);
    hi[i] = make_float2(hx, hy);
    lo[i] = make_float2(df_lo_part(v.x, hx), df_lo_part(v.y, hy));
  }
}

}  // namespace

bool df_prepare(const float2* u_hi, const float2* u_lo, const unsigned char* signs, DfOperator* op, DfWork* w) {
  const long sh = rt().g.sizeh;
  const size_t n = 3 * size_t(sh);
  float2* wk = static_cast<float2*>(workspace(WS_DF, sizeof(float2) * 4 * n));
  if (!wk || !u_hi || !u_lo) return false;
  op->u_hi = u_hi;
  op->u_lo = u_lo;
  op->signs = signs;
  w->x_hi = wk;
  w->x_lo = wk + n;
  w->t_hi = wk + 2 * n;
  w->t_lo = wk + 3 * n;
  return error_code() == 0;
}

void df_mdagm(const DfOperator& op, const DfWork& w, double2* out, const double2* in, double m2, cudaStream_t st) {
  const Geom& g = rt().g;
  const long n = 3L * g.sizeh;
  const int nb = int((g.sizeh + DF_THREADS - 1) / DF_THREADS);
  k_df_split<<<8 * rt().num_sms, 256, 0, st>>>(in, w.x_hi, w.x_lo, n);
  OST_LAUNCH_CHECK();
  k_df_doe<<<nb, DF_THREADS, 0, st>>>(g, op, w.x_hi, w.x_lo, w.t_hi, w.t_lo);
  OST_LAUNCH_CHECK();
  k_df_deo_mdagm<<<nb, DF_THREADS, 0, st>>>(g, op, w.t_hi, w.t_lo, in, out, m2);
  OST_LAUNCH_CHECK();
}

}  // namespace ost
