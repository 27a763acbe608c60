// hmc.cuh -- launch interface of the pure-gauge tree-level Symanzik HMC
// kernels (hmc.cu).  Every kernel is instantiated for double (the
// reference-named FP64 entry points) and float (the FP32 molecular dynamics
// of the link generator).
//
// Link views: `rows` complex arrays per direction, the first two rows of
// every link stored (rows = 9: the reference su3_soa layout; rows = 6: a
// compact two-row copy), or rows = 0: an array of structures with the six
// complex numbers of rows 0-1 of each link contiguous (the link generator's
// FP32 copy).  Momenta and forces are thmat_soa[8] /
// tamat_soa[8] in the reference layout (per direction 3 complex then 2 real
// arrays of sizeh) in the kernel's precision.
#pragma once
#include <cuda_runtime.h>
#include "common.cuh"

namespace ost {

template <typename R> struct HmcLinks {
  typename cplx_t<R>::type* p;
  int rows;   // complex arrays per direction: 9 or 6
};

// What the gauge-force kernel does with TA(U dS/dU) of each link.
enum GaugeForceMode {
  GF_IPDOT = 0,        // write tipdot (and the staples dS/dU if a buffer is given)
  GF_MOM = 1,          // mom -= i fact TA(U dS/dU) (complex), += on the real diagonals
  GF_STAPLES = 2       // only add the staple parts to the staples buffer (FP64 layout)
};
// staple parts (rectangles.c / plaquettes.c split the staple into four
// launches; the reference-named entry points use the same split)
enum StapleParts { SP_PLAQ = 1, SP_RECT_A = 2, SP_RECT_B = 4, SP_RECT_C = 8, SP_ALL = 15 };

template <typename R>
void launch_gauge_force(HmcLinks<R> u, int parts, int mode, typename cplx_t<R>::type* stap_addto,
                        R* ipdot_or_mom, double fact, cudaStream_t st);
// tipdot = TA(U staples) for given staples (su3_utilities.c:146-175)
void launch_conf_times_staples_ta(HmcLinks<double> u, const double2* stap, double* ipdot, cudaStream_t st);
// mom += factor x ipdot in the reference's convention (su3_utilities.c:241-270)
template <typename R>
void launch_mom_sum_mult(R* mom, const R* ipdot, double fact, cudaStream_t st);
// U = exp(i delta P) U, rows 0-1 reunitarised (su3_utilities.c:272-305)
template <typename R>
void launch_mom_exp_times_conf(HmcLinks<R> u, const R* mom, double delta, cudaStream_t st);
// dst[0] = sum of Re tr plaquettes, dst[1] = sum of Re tr 2x1 + 1x2 rectangles
// (planes mu < nu); which: 1 plaquettes only, 2 rectangles only, 3 both
template <typename R>
void launch_gauge_action(HmcLinks<R> u, int which, double* dst, cudaStream_t st);
// dst[0] = sum over the links of directions [d0, d1) of 1/2 tr P^2
template <typename R>
void launch_momenta_action(const R* mom, int d0, int d1, double* dst, cudaStream_t st);
// Gaussian momenta from the counter-based generator (seed, stream): the
// reference's composition of 8 normal deviates of variance 1/2 per link
// (random_assignement.c:145-185)
template <typename R>
void launch_gen_momenta(R* mom, unsigned long long seed, unsigned long long stream, cudaStream_t st);
// Gaussian vec3_soa (3*sizeh complex numbers, real and imaginary parts of
// variance 1/2) from the same generator
void launch_gen_vec3_gauss(double2* v, unsigned long long seed, unsigned long long stream, cudaStream_t st);
// FP64 reference-layout links <-> the FP32 array-of-structures copy (rows
// 0-1 of a link contiguous); the way back reunitarises rows 0-1 in FP64
void launch_links_64_to_32(const double2* u64, int rows64, float2* u32, cudaStream_t st);
void launch_links_32_to_64(const float2* u32, double2* u64, int rows64, cudaStream_t st);
void launch_alg_64_to_32(const double* a64, float* a32, cudaStream_t st);
void launch_alg_32_to_64(const float* a32, double* a64, cudaStream_t st);

}  // namespace ost
