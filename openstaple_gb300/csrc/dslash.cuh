// dslash.cuh -- the staggered even/odd hopping term as a device function,
// shared by the plain Dirac kernels, the fused M^+M kernels and the solvers.
//
// For an output site x of parity P (P=0: D_eo, P=1: D_oe) it returns
//   aux = sum_mu [ e^{i th_f} U_f(x) in(x+mu) - e^{-i th_b} U_b(x-mu)^+ in(x-mu) ]
// with U_f = u[2mu+P] at snum(x), U_b = u[2mu+1-P] at snum(x-mu), and the
// third link row rebuilt as conj(r0 x r1), exactly as the reference's
// mat_vec_mul_arg / conjmat_vec_mul_arg (matvecmul.h:88-172) and
// acc_Deo_unsafe / acc_Doe_unsafe (fermion_matrix.c:47-157) define it.
// The reference subtracts the four backward terms first, then adds the four
// forward terms; the same order is kept here.
#pragma once
#include <cmath>
#include <type_traits>
#include "common.cuh"

namespace ost {

// How the U(1) phase of each link is given.
enum PhaseMode {
  PH_ANGLE = 0,   // reference double_soa/float_soa angle per link; e^{i th} = cos+i sin
  PH_SIGN8 = 1,   // one byte per link: 0 -> +1, 1 -> -1 (staggered phases + APBC)
  PH_NONE = 2     // no phase
};

template <typename T> struct PiBits;
template <> struct PiBits<double> {
  // 0.5 * (2*3.14159265358979323846) in double: the angle the reference stores
  // for a -1 phase (backfield.c:180-187).
  static OST_D unsigned long long bits() { return 0x400921FB54442D18ull; }
};
template <> struct PiBits<float> {
  static OST_D unsigned int bits() { return 0x40490FDBu; }   // (float)pi
};

OST_D double flip_sign(double v, unsigned long long m) {
  return __longlong_as_double(__double_as_longlong(v) ^ (long long)m);
}
OST_D float flip_sign(float v, unsigned int m) {
  return __int_as_float(__float_as_int(v) ^ (int)m);
}

template <typename T> struct SignMask;
template <> struct SignMask<double> { typedef unsigned long long type; static constexpr unsigned long long neg = 0x8000000000000000ull; };
template <> struct SignMask<float> { typedef unsigned int type; static constexpr unsigned int neg = 0x80000000u; };

// Applies the link phase (or its conjugate) to a colour vector.  The two
// exact cases 0 and pi become a sign flip done with integer operations;
// any other angle takes the general complex multiply.
template <typename T, bool CONJ>
OST_D void apply_angle_phase(typename cplx_t<T>::type v[3], T arg,
                             typename SignMask<T>::type extra_mask) {
  typedef typename cplx_t<T>::type C;
  typedef typename SignMask<T>::type M;
  M bits;
  if (sizeof(T) == 8) bits = (M)__double_as_longlong((double)arg);
  else bits = (M)__float_as_uint((float)arg);
  if (bits == 0 || bits == (M)PiBits<T>::bits()) {
    M mask = (bits == 0 ? M(0) : SignMask<T>::neg) ^ extra_mask;
#pragma unroll
    for (int c = 0; c < 3; ++c) { v[c].x = flip_sign(v[c].x, mask); v[c].y = flip_sign(v[c].y, mask); }
  } else {
    T s, co;
    sincos(arg, &s, &co);
    C ph = cmk<C>(co, CONJ ? -s : s);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      v[c] = cmul(v[c], ph);
      v[c].x = flip_sign(v[c].x, extra_mask); v[c].y = flip_sign(v[c].y, extra_mask);
    }
  }
}

// Link field access: 8 blocks, one per (mu, parity).  The reference layout
// (su3_soa) holds 9 complex arrays per block (rows r0,r1,r2 of columns
// c0,c1,c2; rows_per_dir = 9); the library's internal single-precision copy
// keeps only the two rows the kernels read (rows_per_dir = 6).
template <typename C>
struct LinkView {
  const C* base;
  long sizeh;
  int rows_per_dir;
  OST_D const C* at(int dir, int row, int col) const {
    return base + (long(dir) * rows_per_dir + row * 3 + col) * sizeh;
  }
};

template <typename C>
OST_D void load_two_rows(const LinkView<C>& u, int dir, int idx, C m[6]) {
#pragma unroll
  for (int k = 0; k < 6; ++k) m[k] = __ldcs(u.at(dir, k / 3, k % 3) + idx);
}

// Sloppy links in 16-bit fixed point: the first two rows of each link,
// every real and imaginary part q = rint(32768 x) (x rounded to FP32 first)
// clamped to +-32767 and stored biased as q + 32768 in 16 bits (real part in the low half of a
// 32-bit word, imaginary part in the high half).  SU(3) entries lie in
// [-1, 1], so the absolute error is at most 2^-16.  Per direction two
// planes over the half lattice: `a` holds elements 0-3 of rows 0-1
// (16 bytes), `b` elements 4-5 (8 bytes), so one link is 24 bytes against
// 48 for two FP32 rows.  Decoding: the bit pattern 0x4B000000 | u is the
// float 2^23 + u, and (2^23 + u) * 2^-15 - 257 = (u - 32768) / 32768 is exact
// in one FMA.
struct LinkQ16 {
  const uint4* a;
  const uint2* b;
  long sizeh;
};

OST_D float2 q16_decode(unsigned w) {
  const float lo = __int_as_float(int(0x4B000000u | (w & 0xFFFFu)));
  const float hi = __int_as_float(int(0x4B000000u | (w >> 16)));
  return make_float2(fmaf(lo, 3.0517578125e-05f, -257.0f), fmaf(hi, 3.0517578125e-05f, -257.0f));
}

// q = rint(32768 h) of the FP32 rounding h of a link entry, clamped to
// +-32767, biased by 32768 (the scaling is exact; the conversion rounds to
// nearest even).  No FP64 arithmetic: on this part it runs at 1/64 of FP32.
OST_HD unsigned q16_encode_f32(float h) {
  const float y = h * 32768.0f;
#ifdef __CUDA_ARCH__
  int q = __float2int_rn(y);
#else
  int q = int(nearbyintf(y));
#endif
  q = q > 32767 ? 32767 : (q < -32767 ? -32767 : q);
  return unsigned(q + 32768);
}

OST_D void load_two_rows(const LinkQ16& u, int dir, int idx, float2 m[6]) {
  const long k = long(dir) * u.sizeh + idx;
  const uint4 a = __ldcs(u.a + k);
  const uint2 b = __ldcs(u.b + k);
  m[0] = q16_decode(a.x); m[1] = q16_decode(a.y); m[2] = q16_decode(a.z);
  m[3] = q16_decode(a.w); m[4] = q16_decode(b.x); m[5] = q16_decode(b.y);
}

// aux += U v (U rebuilt from two rows)
template <typename C>
OST_D void mac_U(C aux[3], const C m[6], const C v[3]) {
  C r20 = conj_cross(m[1], m[5], m[2], m[4]);
  C r21 = conj_cross(m[2], m[3], m[0], m[5]);
  C r22 = conj_cross(m[0], m[4], m[1], m[3]);
  cmac(aux[0], m[0], v[0]); cmac(aux[0], m[1], v[1]); cmac(aux[0], m[2], v[2]);
  cmac(aux[1], m[3], v[0]); cmac(aux[1], m[4], v[1]); cmac(aux[1], m[5], v[2]);
  cmac(aux[2], r20, v[0]); cmac(aux[2], r21, v[1]); cmac(aux[2], r22, v[2]);
}

// aux += U^+ v
template <typename C>
OST_D void mac_Udag(C aux[3], const C m[6], const C v[3]) {
  C r20 = conj_cross(m[1], m[5], m[2], m[4]);
  C r21 = conj_cross(m[2], m[3], m[0], m[5]);
  C r22 = conj_cross(m[0], m[4], m[1], m[3]);
  cmacc(aux[0], m[0], v[0]); cmacc(aux[0], m[3], v[1]); cmacc(aux[0], r20, v[2]);
  cmacc(aux[1], m[1], v[0]); cmacc(aux[1], m[4], v[1]); cmacc(aux[1], r21, v[2]);
  cmacc(aux[2], m[2], v[0]); cmacc(aux[2], m[5], v[1]); cmacc(aux[2], r22, v[2]);
}

template <typename C>
OST_D void load_vec(const C* v, long sizeh, int idx, C out[3]) {
  out[0] = __ldg(v + idx);
  out[1] = __ldg(v + sizeh + idx);
  out[2] = __ldg(v + 2 * sizeh + idx);
}

// Phase source for one link direction at one index.
template <typename T, int PH>
struct PhaseView {
  const void* p;
  long sizeh;
};

// An empty asm statement that consumes a value: the value must be
// available at this point of the program.
OST_D void pin_value(float v) { asm volatile("" ::"f"(v)); }
OST_D void pin_value(double v) { asm volatile("" ::"d"(v)); }
OST_D void pin_value(float2 v) { asm volatile("" ::"f"(v.x), "f"(v.y)); }
OST_D void pin_value(double2 v) { asm volatile("" ::"d"(v.x), "d"(v.y)); }
OST_D void pin_value(unsigned char v) { asm volatile("" ::"r"(unsigned(v))); }

// Raw link words as loaded (before decoding), per link view type.
template <typename LV> struct LinkRaw;
template <typename C> struct LinkRaw<LinkView<C>> {
  C m[6];
  OST_D void load(const LinkView<C>& u, int dir, int idx) { load_two_rows(u, dir, idx, m); }
  OST_D void rows(C out[6]) const {
#pragma unroll
    for (int k = 0; k < 6; ++k) out[k] = m[k];
  }
  OST_D void pin() const {
#pragma unroll
    for (int k = 0; k < 6; ++k) pin_value(m[k]);
  }
};
template <> struct LinkRaw<LinkQ16> {
  uint4 a;
  uint2 b;
  OST_D void load(const LinkQ16& u, int dir, int idx) {
    const long k = long(dir) * u.sizeh + idx;
    a = __ldcs(u.a + k);
    b = __ldcs(u.b + k);
  }
  OST_D void rows(float2 m[6]) const {
    m[0] = q16_decode(a.x); m[1] = q16_decode(a.y); m[2] = q16_decode(a.z);
    m[3] = q16_decode(a.w); m[4] = q16_decode(b.x); m[5] = q16_decode(b.y);
  }
  OST_D void pin() const { asm volatile("" ::"r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b.x), "r"(b.y)); }
};

// The hop term at output index idx of parity P: aux = sum over the four
// backward hops -e^{-i th} U_b(x-mu)^+ in(x-mu), then the four forward hops
// e^{i th} U_f(x) in(x+mu), accumulated in that order.  The loads (link,
// input, phase) of HB consecutive hops are issued before their arithmetic;
// HB changes how many loads a thread keeps in flight, never the arithmetic
// or its order, so every HB gives the same bits.  LV is LinkView<C> (FP64
// or FP32 rows) or LinkQ16 (FP32 arithmetic only).
template <typename T, int P, int PH, typename LV, int HB = 1>
OST_D void hop(const Geom& g, const LV& u, const typename cplx_t<T>::type* in, const void* phases, int idx,
               typename cplx_t<T>::type aux[3]) {
  static_assert(8 % HB == 0, "hops in flight must divide 8");
  typedef typename cplx_t<T>::type C;
  typedef typename SignMask<T>::type M;
  const long sh = g.sizeh;
  Site s = site_of(g, idx, P);
  int fwd[4], bwd[4];
  neighbours(g, s, fwd, bwd);
#pragma unroll
  for (int c = 0; c < 3; ++c) aux[c] = cmk<C>(T(0), T(0));
#pragma unroll
  for (int h0 = 0; h0 < 8; h0 += HB) {
    LinkRaw<LV> raw[HB];
    C v[HB][3];
    T arg[HB];
    unsigned char sb[HB];
#pragma unroll
    for (int k = 0; k < HB; ++k) {
      const int hm = h0 + k;
      const bool back = hm < 4;                 // backward hops first, as in the reference
      const int mu = hm & 3;
      const int dir = back ? 2 * mu + (1 - P) : 2 * mu + P;
      const int j = back ? bwd[mu] : fwd[mu];   // input site
      const int l = back ? j : idx;             // link site
      raw[k].load(u, dir, l);
      load_vec(in, sh, j, v[k]);
      if (PH == PH_ANGLE) arg[k] = __ldcs(static_cast<const T*>(phases) + long(dir) * sh + l);
      else if (PH == PH_SIGN8) sb[k] = __ldg(static_cast<const unsigned char*>(phases) + long(dir) * sh + l);
    }
    // the batch's loaded values all pass through one empty asm statement, so
    // every load of the batch is issued before the first hop's arithmetic
    // (otherwise the compiler may sink each load to its first use)
    if (HB > 1) {
#pragma unroll
      for (int k = 0; k < HB; ++k) {
        raw[k].pin();
#pragma unroll
        for (int c = 0; c < 3; ++c) pin_value(v[k][c]);
        if (PH == PH_ANGLE) pin_value(arg[k]);
        else if (PH == PH_SIGN8) pin_value(sb[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < HB; ++k) {
      const bool back = h0 + k < 4;
      if (PH == PH_ANGLE) {
        if (back) apply_angle_phase<T, true>(v[k], arg[k], SignMask<T>::neg);
        else apply_angle_phase<T, false>(v[k], arg[k], M(0));
      } else if (PH == PH_SIGN8) {
        const M mask = back ? (sb[k] ? M(0) : SignMask<T>::neg) : (sb[k] ? SignMask<T>::neg : M(0));
#pragma unroll
        for (int c = 0; c < 3; ++c) { v[k][c].x = flip_sign(v[k][c].x, mask); v[k][c].y = flip_sign(v[k][c].y, mask); }
      } else if (back) {
#pragma unroll
        for (int c = 0; c < 3; ++c) { v[k][c].x = -v[k][c].x; v[k][c].y = -v[k][c].y; }
      }
      C m[6];
      raw[k].rows(m);
      if (back) mac_Udag(aux, m, v[k]);
      else mac_U(aux, m, v[k]);
    }
  }
}

// ---- FP32 hop term with the backward and forward sums kept apart ----
//
// aux = B + F with B = sum over the four backward hops and F over the four
// forward hops, each accumulated in hop order (two independent FMA chains
// instead of one).  A backward hop adds U^+ v as sum_j cmac(conj(U_ji), v_j),
// which is exactly mac_Udag's cmacc(U_ji, v_j).  Every HB gives the same
// bits.

// the phase of a hop applied to v (back: the conjugate phase and the minus
// sign of the backward term)
template <int PH>
OST_D void apply_hop_phase(float2 v[3], bool back, float arg, unsigned char sb) {
  typedef SignMask<float>::type M;
  if (PH == PH_ANGLE) {
    const M extra = back ? SignMask<float>::neg : M(0);
    const M bits = __float_as_uint(arg);
    if (bits == 0 || bits == PiBits<float>::bits()) {
      const M mask = (bits == 0 ? M(0) : SignMask<float>::neg) ^ extra;
#pragma unroll
      for (int c = 0; c < 3; ++c) { v[c].x = flip_sign(v[c].x, mask); v[c].y = flip_sign(v[c].y, mask); }
    } else {
      float sn, co;
      sincosf(arg, &sn, &co);
      const float2 ph = make_float2(co, back ? -sn : sn);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        v[c] = cmul(v[c], ph);
        v[c].x = flip_sign(v[c].x, extra); v[c].y = flip_sign(v[c].y, extra);
      }
    }
  } else {
    M mask;
    if (PH == PH_SIGN8) mask = back ? (sb ? M(0) : SignMask<float>::neg) : (sb ? SignMask<float>::neg : M(0));
    else mask = back ? SignMask<float>::neg : M(0);
#pragma unroll
    for (int c = 0; c < 3; ++c) { v[c].x = flip_sign(v[c].x, mask); v[c].y = flip_sign(v[c].y, mask); }
  }
}

// acc += W v with W = U (forward) or U^+ (backward), U rebuilt from rows m
OST_D void mac_hop(float2 acc[3], const float2 m[6], const float2 v[3], bool back) {
  const float2 r20 = conj_cross(m[1], m[5], m[2], m[4]);
  const float2 r21 = conj_cross(m[2], m[3], m[0], m[5]);
  const float2 r22 = conj_cross(m[0], m[4], m[1], m[3]);
  const float2 u[3][3] = {{m[0], m[1], m[2]}, {m[3], m[4], m[5]}, {r20, r21, r22}};
  const SignMask<float>::type cm = back ? SignMask<float>::neg : 0u;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float2 w = back ? u[j][i] : u[i][j];
      w.y = flip_sign(w.y, cm);
      cmac(acc[i], w, v[j]);
    }
}

// the four hops of one kind (back: hops 0-3, else 4-7) added to acc,
// HB hops' loads issued before their arithmetic
template <int P, int PH, typename LV, int HB>
OST_D void hop4(const LV& u, const float2* in, const void* phases, long sh, int idx, const int fwd[4],
                const int bwd[4], bool back, float2 acc[3]) {
  static_assert(4 % HB == 0, "hops in flight must divide 4");
#pragma unroll
  for (int h0 = 0; h0 < 4; h0 += HB) {
    LinkRaw<LV> raw[HB];
    float2 v[HB][3];
    float arg[HB];
    unsigned char sb[HB];
#pragma unroll
    for (int k = 0; k < HB; ++k) {
      const int mu = h0 + k;
      const int dir = back ? 2 * mu + (1 - P) : 2 * mu + P;
      const int j = back ? bwd[mu] : fwd[mu];   // input site
      const int l = back ? j : idx;             // link site
      raw[k].load(u, dir, l);
      load_vec(in, sh, j, v[k]);
      arg[k] = 0.f;
      sb[k] = 0;
      if (PH == PH_ANGLE) arg[k] = __ldcs(static_cast<const float*>(phases) + long(dir) * sh + l);
      else if (PH == PH_SIGN8) sb[k] = __ldg(static_cast<const unsigned char*>(phases) + long(dir) * sh + l);
    }
    if (HB > 1) {
#pragma unroll
      for (int k = 0; k < HB; ++k) {
        raw[k].pin();
#pragma unroll
        for (int c = 0; c < 3; ++c) pin_value(v[k][c]);
        if (PH == PH_ANGLE) pin_value(arg[k]);
        else if (PH == PH_SIGN8) pin_value(sb[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < HB; ++k) {
      apply_hop_phase<PH>(v[k], back, arg[k], sb[k]);
      float2 m[6];
      raw[k].rows(m);
      mac_hop(acc, m, v[k], back);
    }
  }
}

OST_D void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// L2 prefetches of the eight links the hop term of site idx (parity P) reads
// (no data returns to the thread)
template <int P, typename LV>
OST_D void prefetch_links(const Geom& g, const LV& u, int idx) {
  const long sh = g.sizeh;
  Site s = site_of(g, idx, P);
  int fwd[4], bwd[4];
  neighbours(g, s, fwd, bwd);
#pragma unroll
  for (int hm = 0; hm < 8; ++hm) {
    const bool back = hm < 4;
    const int mu = hm & 3;
    const int dir = back ? 2 * mu + (1 - P) : 2 * mu + P;
    const int l = back ? bwd[mu] : idx;
    if constexpr (std::is_same<LV, LinkQ16>::value) {
      prefetch_l2(u.a + long(dir) * sh + l);
      prefetch_l2(u.b + long(dir) * sh + l);
    } else {
#pragma unroll
      for (int e = 0; e < 6; ++e) prefetch_l2(u.at(dir, e / 3, e % 3) + l);
    }
  }
}

template <int P, int PH, typename LV, int HB>
OST_D void hop_fb(const Geom& g, const LV& u, const float2* in, const void* phases, int idx, float2 aux[3]) {
  const long sh = g.sizeh;
  Site s = site_of(g, idx, P);
  int fwd[4], bwd[4];
  neighbours(g, s, fwd, bwd);
  float2 accb[3], accf[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) accb[c] = accf[c] = make_float2(0.f, 0.f);
  hop4<P, PH, LV, HB>(u, in, phases, sh, idx, fwd, bwd, true, accb);
  hop4<P, PH, LV, HB>(u, in, phases, sh, idx, fwd, bwd, false, accf);
#pragma unroll
  for (int c = 0; c < 3; ++c) aux[c] = cadd(accb[c], accf[c]);
}

}  // namespace ost
