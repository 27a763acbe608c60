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

// The hop term at output index idx of parity P.
template <typename T, int P, int PH>
OST_D void hop(const Geom& g, const LinkView<typename cplx_t<T>::type>& u,
               const typename cplx_t<T>::type* in, const void* phases, int idx,
               typename cplx_t<T>::type aux[3]) {
  typedef typename cplx_t<T>::type C;
  typedef typename SignMask<T>::type M;
  const long sh = g.sizeh;
  Site s = site_of(g, idx, P);
  int fwd[4], bwd[4];
  neighbours(g, s, fwd, bwd);
#pragma unroll
  for (int c = 0; c < 3; ++c) aux[c] = cmk<C>(T(0), T(0));

  // backward hops: aux -= e^{-i th} U_b(x-mu)^+ in(x-mu)
#pragma unroll
  for (int mu = 0; mu < 4; ++mu) {
    const int dir = 2 * mu + (1 - P);
    const int j = bwd[mu];
    C m[6], v[3];
    load_two_rows(u, dir, j, m);
    load_vec(in, sh, j, v);
    if (PH == PH_ANGLE) {
      T arg = __ldcs(static_cast<const T*>(phases) + long(dir) * sh + j);
      apply_angle_phase<T, true>(v, arg, SignMask<T>::neg);
    } else if (PH == PH_SIGN8) {
      unsigned char sb = __ldg(static_cast<const unsigned char*>(phases) + long(dir) * sh + j);
      M mask = (sb ? M(0) : SignMask<T>::neg);
#pragma unroll
      for (int c = 0; c < 3; ++c) { v[c].x = flip_sign(v[c].x, mask); v[c].y = flip_sign(v[c].y, mask); }
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) { v[c].x = -v[c].x; v[c].y = -v[c].y; }
    }
    mac_Udag(aux, m, v);
  }
  // forward hops: aux += e^{i th} U_f(x) in(x+mu)
#pragma unroll
  for (int mu = 0; mu < 4; ++mu) {
    const int dir = 2 * mu + P;
    const int j = fwd[mu];
    C m[6], v[3];
    load_two_rows(u, dir, idx, m);
    load_vec(in, sh, j, v);
    if (PH == PH_ANGLE) {
      T arg = __ldcs(static_cast<const T*>(phases) + long(dir) * sh + idx);
      apply_angle_phase<T, false>(v, arg, M(0));
    } else if (PH == PH_SIGN8) {
      unsigned char sb = __ldg(static_cast<const unsigned char*>(phases) + long(dir) * sh + idx);
      M mask = (sb ? SignMask<T>::neg : M(0));
#pragma unroll
      for (int c = 0; c < 3; ++c) { v[c].x = flip_sign(v[c].x, mask); v[c].y = flip_sign(v[c].y, mask); }
    }
    mac_U(aux, m, v);
  }
}

}  // namespace ost
