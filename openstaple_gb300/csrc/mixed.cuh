// mixed.cuh -- single-precision solver engine with FP64 reliable updates.
#pragma once
#include "dslash.cuh"
#include <cuda_runtime.h>
#include "common.cuh"
#include "dslash_df.cuh"

namespace ost {

// Device-resident scalars of the mixed-precision CG.  Every kernel of the
// iteration reads what it needs from here, so the host never waits on a
// reduction inside an iteration.
struct MixScal {
  double delta;      // |r|^2 entering the iteration
  double pAp;
  double alpha;
  double lambda;
  double beta;
  double last_max;   // largest |r|^2 since the last reliable update
  double target2;    // the FP32 recursion stops at lambda <= target2
  double frac;       // reliable update when delta < frac * last_max (every == 0)
  double m2;         // mass^2 + shift
  double true_r2;    // |b - A x|^2 from the last FP64 residual
  double bnorm2;
  int iter;
  int max_iter;
  int done;
  int need_rel;
  int every;         // > 0: reliable update every `every` iterations
  int n_rel;
};

struct MixedOptions {
  double mass2;            // mass^2 + shift
  double res;              // target relative residual
  double safety;           // the FP32 recursion aims at safety*res (reference: 0.9)
  int max_iter;
  int reliable_every;      // 0: reference delta criterion
  double delta_frac;       // reference mixedPrecisionDelta (0.1)
  int guarantee;           // 1: iterate until the FP64 true residual <= res
  int chunk;               // iterations per captured graph launch
};

struct MixedResult {
  int iters;
  int n_reliable;
  double true_res;         // sqrt(|b - A x|^2 / |b|^2), FP64
  int converged;
};

struct MixedBuffers {
  const double2* u64;      // reference su3_soa[8]
  const void* ph64;        // double angles [8][sizeh]
  const float2* u32;       // single-precision links
  int u32_compact;         // 1: two rows per direction
  int q16;                 // 1: the FP32 iteration reads the 16-bit links uq instead of u32
  LinkQ16 uq;
  const void* ph32;        // sign bytes or float angles
  int ph32_mode;           // PhaseMode for the FP32 kernels
  double2* x;              // solution (in: guess, out: result)
  const double2* b;
  double2* r64;            // FP64 work
  double2* t64;            // FP64 work
  double2* t64b;           // FP64 work (odd-parity temporary)
  float2* r;               // FP32 work
  float2* p;
  float2* s;
  float2* xf;
  float2* t;               // odd-parity temporary
  int use_df;              // reliable updates in double-float arithmetic (exact phases only)
  DfOperator df;
  DfWork dfw;
};

// Converts the first two rows of FP64 su3_soa[8] links to a compact FP32 copy
// ([dir][6][sizeh]); with u_lo (same layout) also the lo parts
// (float)(u - (double)(float)u) of the double-float links.
void links_to_f32_compact(const double2* u64, float2* u32, long sizeh, cudaStream_t st, float2* u_lo = nullptr);
// Converts the compact FP32 links (links_to_f32_compact) to the 16-bit
// fixed-point planes of LinkQ16 (a: 8 x sizeh uint4, b: 8 x sizeh uint2).
void links_to_q16(const float2* u32, uint4* a, uint2* b, long sizeh, cudaStream_t st);
// Sign bytes from FP64 phase angles; *all_exact (device int) is cleared when
// some angle is neither 0 nor pi.
void phases_to_signs(const double* ph64, unsigned char* sg, int* all_exact, long sizeh, cudaStream_t st);
void phases_to_f32(const double* ph64, float* ph32, long sizeh, cudaStream_t st);

// Solves (M^+M + shift) x = b.
MixedResult mixed_cg(const MixedBuffers& B, const MixedOptions& o, MixScal* scal_dev, cudaStream_t st);

double time_mixed_kernel(const MixedBuffers& B, MixScal* sc, int which, int reps, cudaStream_t st);

// out = m2 in - D_eo D_oe in with the FP32 iteration kernels and B's links.
void sloppy_mdagm(const MixedBuffers& B, double m2, const double2* in, double2* out, MixScal* sc, cudaStream_t st);

// Link format of the FP32 iteration when the library converts the links
// itself: 1 (default) 16-bit fixed point (LinkQ16), 0 two FP32 rows.
int sloppy_links_q16();

}  // namespace ost
