// batched.cuh -- several systems (right-hand sides and/or shifts) solved
// together: every FP32 Dslash application reads each link once for all of
// them.
#pragma once
#include <cuda_runtime.h>
#include "common.cuh"
#include "mixed.cuh"

namespace ost {

static constexpr int BATCH_MAX = 8;          // systems per batched launch
static constexpr int CGM_MAX_SHIFTS = 25;    // MAX_APPROX_ORDER (rationalapprox.h:8)

// Device-resident scalars of a batch of independent mixed-precision CG
// systems (M^+M + m2_s) x_s = b_s.
struct BatchScal {
  double delta[BATCH_MAX], pAp[BATCH_MAX], alpha[BATCH_MAX], lambda[BATCH_MAX], beta[BATCH_MAX];
  double last_max[BATCH_MAX], target2[BATCH_MAX], m2[BATCH_MAX], true_r2[BATCH_MAX], bnorm2[BATCH_MAX];
  double frac;
  int iter[BATCH_MAX], done[BATCH_MAX], need_rel[BATCH_MAX], n_rel[BATCH_MAX];
  int max_iter, every, nsys;
};

struct BatchBuffers {
  const double2* u64;       // reference su3_soa[8]
  const void* ph64;         // double angles
  const float2* u32;        // compact FP32 links
  int q16;                  // 1: the FP32 iteration reads the 16-bit links uq instead of u32
  LinkQ16 uq;
  const void* ph32;         // sign bytes or float angles
  int ph32_mode;
  int nsys;
  double2* x;               // nsys FP64 solutions (contiguous vec3 fields)
  const double2* b;         // nsys FP64 sources
  double2* r64;             // FP64 work (one field, reused per system)
  double2* t64;
  double2* t64b;
  float2* r;                // nsys FP32 fields each
  float2* p;
  float2* s;
  float2* xf;
  float2* t;
  int use_df;               // reliable updates in double-float arithmetic (exact phases only)
  DfOperator df;
  DfWork dfw;
};

struct BatchResult {
  int iters[BATCH_MAX];
  int n_reliable[BATCH_MAX];
  double true_res[BATCH_MAX];
  int converged[BATCH_MAX];
};

// Solves (M^+M + m2[k]) x_k = b_k for k < B.nsys (nsys <= BATCH_MAX); every
// system reaches its own FP64 true residual <= res (or max_iter).
BatchResult batched_mixed_cg(const BatchBuffers& B, const double* m2, double res, int max_iter, double delta_frac,
                             BatchScal* sc_dev, cudaStream_t st);

// Multi-shift CG in FP32 for nrhs right-hand sides at once (CG-M,
// inverter_multishift_full.c:23-252, with the per-shift recurrences on the
// device).  xs[r*nshift + k] receives the solution of (M^+M + shift_k) x = b_r.
struct CgmBatchBuffers {
  const float2* u32;
  const void* ph32;
  int ph32_mode;
  int nrhs;
  int nshift;
  const float2* b;          // nrhs FP32 sources
  float2* xs;               // nrhs*nshift FP32 solutions
  float2* ps;               // nrhs*nshift FP32 shifted directions
  float2* r;                // nrhs
  float2* p;                // nrhs
  float2* s;                // nrhs
  float2* t;                // nrhs
};

struct CgmBatchResult {
  int iters[BATCH_MAX];
  bool device_loop;   // the iterations ran as one graph launch with a device-side while loop
};

CgmBatchResult batched_cgm_f32(const CgmBatchBuffers& B, double mass2, const double* shifts, double res,
                               int max_iter, cudaStream_t st);

// All `order` shifts for nrhs <= 4 right-hand sides (device FP64 fields,
// xs64[r*order + k]): an FP32 CG-M for all right-hand sides together to the
// relative residual res_cgm, then (refine != 0) every system refined to an
// FP64 true residual <= res by the batched mixed solver.  Returns
// INVERTER_SUCCESS / INVERTER_FAILURE (capi_batched.cu).
int multishift_two_phase(const double2* u64, const double* ph64, double mass, const double* shifts, int order,
                         int nrhs, const double2* b64, double2* xs64, double res_cgm, double res, int max_iter,
                         double delta_frac, int refine, int* iters_cgm, int* iters_refine, double* true_res);

}  // namespace ost
