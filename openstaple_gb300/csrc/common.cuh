// common.cuh -- geometry, complex arithmetic and error plumbing shared by the
// sm_103a kernels of the staggered-fermion hot path.
//
// Memory layout (identical to the reference so that its buffers can be used in
// place): every field is structure-of-arrays over the half lattice of
// sizeh = V/2 sites.
//   vec3_soa  : c0[sizeh], c1[sizeh], c2[sizeh]           complex   (struct_c_def.h:16-20)
//   su3_soa   : r0, r1, r2, each a vec3_soa                (struct_c_def.h:37-44)
//   links     : su3_soa[8], link (mu, parity) at 2*mu+parity (geometry_multidev.h:284-296)
//   double_soa: d[sizeh]                                   (struct_c_def.h:25-27)
//   tamat_soa : c01,c02,c12 complex, ic00,ic11 real        (struct_c_def.h:47-53)
//   thmat_soa : c01,c02,c12 complex, rc00,rc11 real        (struct_c_def.h:54-60)
// The half-lattice index of site (d0,d1,d2,d3) is
//   snum = (d0 + d1*n0 + d2*n0*n1 + d3*n0*n1*n2) / 2      (geometry_multidev.h:219-229)
// so the even and the odd site of each x-pair share one index.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define OST_HD __host__ __device__ __forceinline__
#define OST_D __device__ __forceinline__

namespace ost {

// Unsigned division by a runtime constant via multiply-high (Granlund &
// Montgomery 1994, "Division by invariant integers using multiplication").
// Valid for numerators below 2^31.
struct FastDiv {
  uint32_t d, m, s;
  FastDiv() : d(1), m(0), s(0) {}
  explicit FastDiv(uint32_t div) : d(div) {
    if (div == 1) { m = 0; s = 0; return; }
    uint32_t l = 0;
    while ((1u << l) < div) ++l;               // l = ceil(log2 d)
    uint64_t mm = ((uint64_t(1) << 32) * ((uint64_t(1) << l) - div)) / div + 1;
    m = uint32_t(mm);
    s = l - 1;
  }
  OST_HD uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
    if (d == 1) return n;
    uint32_t t = __umulhi(n, m);
    return (t + ((n - t) >> 1)) >> s;
#else
    return n / d;
#endif
  }
};

// Lattice geometry at run time (the reference fixes it at compile time).
struct Geom {
  int n0, n1, n2, n3;
  int nh0;                  // n0/2
  int sizeh;                // V/2
  int vol1, vol2, vol3;     // lexicographic strides of d1, d2, d3
  FastDiv fnh0, fn1, fn2;
};

// Coordinates of half-lattice index idx on the sub-lattice of parity par
// (0 even, 1 odd); follows the d0 = 2*hd0 + parity-bit rule of
// fermion_matrix.c:67,120.
struct Site { int d0, d1, d2, d3, lex; };

OST_D Site site_of(const Geom& g, int idx, int par) {
  Site s;
  uint32_t r = g.fnh0.div(uint32_t(idx));
  int hd0 = idx - int(r) * g.nh0;
  uint32_t r2 = g.fn1.div(r);
  s.d1 = int(r) - int(r2) * g.n1;
  uint32_t r3 = g.fn2.div(r2);
  s.d2 = int(r2) - int(r3) * g.n2;
  s.d3 = int(r3);
  s.d0 = 2 * hd0 + ((s.d1 + s.d2 + s.d3 + par) & 1);
  s.lex = s.d0 + s.d1 * g.vol1 + s.d2 * g.vol2 + s.d3 * g.vol3;
  return s;
}

// Half-lattice indices of the 8 neighbours (periodic wrap in every direction,
// geometry.c:14-100).  fwd[mu] = snum(x+mu), bwd[mu] = snum(x-mu).
OST_D void neighbours(const Geom& g, const Site& s, int fwd[4], int bwd[4]) {
  const int l = s.lex;
  fwd[0] = (s.d0 == g.n0 - 1 ? l - (g.n0 - 1) : l + 1) >> 1;
  bwd[0] = (s.d0 == 0 ? l + (g.n0 - 1) : l - 1) >> 1;
  fwd[1] = (s.d1 == g.n1 - 1 ? l - (g.n1 - 1) * g.vol1 : l + g.vol1) >> 1;
  bwd[1] = (s.d1 == 0 ? l + (g.n1 - 1) * g.vol1 : l - g.vol1) >> 1;
  fwd[2] = (s.d2 == g.n2 - 1 ? l - (g.n2 - 1) * g.vol2 : l + g.vol2) >> 1;
  bwd[2] = (s.d2 == 0 ? l + (g.n2 - 1) * g.vol2 : l - g.vol2) >> 1;
  fwd[3] = (s.d3 == g.n3 - 1 ? l - (g.n3 - 1) * g.vol3 : l + g.vol3) >> 1;
  bwd[3] = (s.d3 == 0 ? l + (g.n3 - 1) * g.vol3 : l - g.vol3) >> 1;
}

// ---- complex helpers over CUDA's double2 / float2 ----
template <typename T> struct cplx_t;
template <> struct cplx_t<double> { typedef double2 type; };
template <> struct cplx_t<float> { typedef float2 type; };

// Device side of a programmatic dependent launch (launch_pdl): wait until
// the previous kernel on the stream has completed and its writes are
// visible; allow the next kernel to be scheduled.
OST_D void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
OST_D void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename C> OST_HD C cmk(decltype(C().x) r, decltype(C().x) i) { C z; z.x = r; z.y = i; return z; }

// a*b and a*conj(b), conj(a)*b with explicit FMA contraction order.
template <typename C> OST_D C cmul(C a, C b) {
  return cmk<C>(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
template <typename C> OST_D C conjmul(C a, C b) {     // conj(a) * b
  return cmk<C>(fma(a.x, b.x, a.y * b.y), fma(a.x, b.y, -a.y * b.x));
}
template <typename C> OST_D C cadd(C a, C b) { return cmk<C>(a.x + b.x, a.y + b.y); }
template <typename C> OST_D C csub(C a, C b) { return cmk<C>(a.x - b.x, a.y - b.y); }
template <typename C> OST_D C cconj(C a) { return cmk<C>(a.x, -a.y); }
template <typename C> OST_D C cscale(C a, decltype(C().x) s) { return cmk<C>(a.x * s, a.y * s); }
// acc += a*b
template <typename C> OST_D void cmac(C& acc, C a, C b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a)*b
template <typename C> OST_D void cmacc(C& acc, C a, C b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(-a.y, b.x, acc.y);
}
// conj(a*b - c*d): third row of an SU(3) matrix from its first two rows
// (matvecmul.h:115-118).
template <typename C> OST_D C conj_cross(C a, C b, C c, C d) {
  decltype(C().x) re = a.x * b.x;
  re = fma(-a.y, b.y, re); re = fma(-c.x, d.x, re); re = fma(c.y, d.y, re);
  decltype(C().x) im = a.x * b.y;
  im = fma(a.y, b.x, im); im = fma(-c.x, d.y, im); im = fma(-c.y, d.x, im);
  return cmk<C>(re, -im);
}

// Streaming loads that bypass L1 allocation for single-use data.
OST_D double2 ldg_stream(const double2* p) { return __ldcs(p); }
OST_D float2 ldg_stream(const float2* p) { return __ldcs(p); }

}  // namespace ost
