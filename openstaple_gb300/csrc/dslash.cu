// dslash.cu -- sm_103a kernels for the staggered D_eo / D_oe operator and the
// fused M^+M = (m^2 + shift) - D_eo D_oe application.
//
// One thread per output site of the half lattice.  Consecutive threads own
// consecutive half-lattice indices, so each of the 6 complex link loads and
// the output store of a warp touch 32 consecutive 16-byte (FP64) or 8-byte
// (FP32) elements: fully coalesced.  Neighbour spinors are read through the
// read-only path so that the eight-fold reuse of every input spinor across
// the eight hops is served from L1/L2.  Links are single-use per application
// and streamed (evict-first).
#include "dslash.cuh"
#include "kernels.cuh"
#include "runtime.cuh"

namespace ost {

static constexpr int DSLASH_THREADS = 128;

// out = 0.5 * hop(in)                                        (EPI_PLAIN)
// out = mass2 * in0 - 0.5 * hop(in)                          (EPI_MDAGM)
template <typename T, int P, int PH, int EPI>
__global__ void __launch_bounds__(DSLASH_THREADS)
dslash_kernel(Geom g, LinkView<typename cplx_t<T>::type> u, typename cplx_t<T>::type* __restrict__ out,
              const typename cplx_t<T>::type* __restrict__ in, const void* __restrict__ phases,
              const typename cplx_t<T>::type* __restrict__ in0, T mass2) {
  typedef typename cplx_t<T>::type C;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.sizeh) return;
  C aux[3];
  hop<T, P, PH>(g, u, in, phases, idx, aux);
  const long sh = g.sizeh;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    C r = cscale(aux[c], T(0.5));
    if (EPI == EPI_MDAGM) {
      C a = in0[c * sh + idx];
      r = cmk<C>(fma(a.x, mass2, -r.x), fma(a.y, mass2, -r.y));
    }
    __stcs(out + c * sh + idx, r);
  }
}

template <typename T, int P, int PH, int EPI>
static void launch_one(const DslashArgs<T>& a) {
  const Geom& g = rt().g;
  LinkView<typename cplx_t<T>::type> u{a.u, g.sizeh, a.compact_links ? 6 : 9};
  dslash_kernel<T, P, PH, EPI><<<blocks_for(g.sizeh, DSLASH_THREADS), DSLASH_THREADS, 0, a.stream>>>(
      g, u, a.out, a.in, a.phases, a.in0, a.mass2);
  OST_LAUNCH_CHECK();
}

template <typename T>
void launch_dslash(const DslashArgs<T>& a) {
#define OST_DSL(P, PH, E) \
  if (a.parity == P && a.phase_mode == PH && a.epilogue == E) { launch_one<T, P, PH, E>(a); return; }
  OST_DSL(0, PH_ANGLE, EPI_PLAIN) OST_DSL(1, PH_ANGLE, EPI_PLAIN)
  OST_DSL(0, PH_ANGLE, EPI_MDAGM) OST_DSL(1, PH_ANGLE, EPI_MDAGM)
  OST_DSL(0, PH_SIGN8, EPI_PLAIN) OST_DSL(1, PH_SIGN8, EPI_PLAIN)
  OST_DSL(0, PH_SIGN8, EPI_MDAGM) OST_DSL(1, PH_SIGN8, EPI_MDAGM)
#undef OST_DSL
  set_error(-10, "launch_dslash: unsupported combination parity=%d phase=%d epilogue=%d", a.parity,
            a.phase_mode, a.epilogue);
}

template void launch_dslash<double>(const DslashArgs<double>&);
template void launch_dslash<float>(const DslashArgs<float>&);

}  // namespace ost
