// dslash_df.cuh -- M^+M in double-float arithmetic: every FP64 number is
// carried as an unevaluated sum hi + lo of two FP32 numbers (about 48
// significant bits) and products and sums use error-free transformations
// (Dekker's product via FMA, Knuth's two-sum; Dekker 1971, Knuth TAOCP vol. 2
// 4.2.2).  GB300 executes FP64 at 1/62 of its FP32 rate and the FP64 Dslash
// is bound by that rate (0.42 ms per half application at 32^4, 96% of the
// FP64 peak); in double-float the same operator becomes memory bound.  The
// mixed-precision solvers use it for their intermediate reliable updates,
// where a relative accuracy of ~1e-14 is ample; every final (true) residual
// is still computed in native FP64.
#pragma once
#include <cuda_runtime.h>
#include <cstring>
#include "common.cuh"

namespace ost {

// Double-float operand set for D_eo / D_oe: links split into FP32 hi and lo
// parts (rows 0-1, compact layout [dir][6][sizeh]) and one sign byte per link.
struct DfOperator {
  const float2* u_hi;
  const float2* u_lo;
  const unsigned char* signs;
};

// Work fields of one double-float M^+M application: the input and the
// odd-parity intermediate in hi/lo form (3*sizeh complex each).
struct DfWork {
  float2* x_hi;
  float2* x_lo;
  float2* t_hi;
  float2* t_lo;
};

// lo = (float)(x - (double)hi) for hi = (float)x, without FP64 arithmetic
// (1/64 of the FP32 rate on this part): with x = m 2^(e-1075) (m the 53-bit
// mantissa) and hi = mh 2^(eh-150), the difference d = m - mh 2^(eh-e+925)
// is an exact integer of at most 30 bits; lo = (float)d 2^(e-1075) rounds
// once, like the FP64 expression, and the power of two is exact while
// 2^(e-1075) is a normal float.  Zero, tiny and huge x take the FP64 route.
OST_HD float df_lo_part(double x, float hi) {
  unsigned long long b;
  unsigned hb;
#ifdef __CUDA_ARCH__
  b = (unsigned long long)__double_as_longlong(x);
  hb = __float_as_uint(hi);
#else
  memcpy(&b, &x, sizeof(b));
  memcpy(&hb, &hi, sizeof(hb));
#endif
  const int e = int((b >> 52) & 0x7FF);
  if (e < 1075 - 126 + 30 || e > 1023 + 100) return float(x - double(hi));
  const long long m = (long long)((b & 0xFFFFFFFFFFFFFull) | (1ull << 52));
  const int eh = int((hb >> 23) & 0xFF);
  const long long mh = (long long)((hb & 0x7FFFFFu) | 0x800000u);
  const long long d = m - (mh << (eh - e + 925));
  if (d == 0) return 0.0f;   // x - hi = +0 in FP64, whatever the sign of x
  const unsigned pb = unsigned(e - 1075 + 127) << 23;   // 2^(e-1075) as a float
  float p2;
#ifdef __CUDA_ARCH__
  p2 = __uint_as_float(pb);
#else
  memcpy(&p2, &pb, sizeof(p2));
#endif
  const float lo = float(int(d)) * p2;
  return (b >> 63) ? -lo : lo;
}

// Operator and work fields (workspace slot WS_DF) for a solve on the current
// lattice.  u_hi / u_lo: the compact FP32 links and their lo parts, both
// written by links_to_f32_compact; signs: one sign byte per link.
bool df_prepare(const float2* u_hi, const float2* u_lo, const unsigned char* signs, DfOperator* op, DfWork* w);

// out = (m2 + shift) in - D_eo D_oe in, in double-float arithmetic; in and
// out are FP64 vec3 fields on the even sites.  Needs exact phases (signs).
void df_mdagm(const DfOperator& op, const DfWork& w, double2* out, const double2* in, double m2,
              cudaStream_t st);

}  // namespace ost
