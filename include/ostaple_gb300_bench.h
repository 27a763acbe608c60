/* ostaple_gb300_bench.h -- measurement entry points of the benchmark library
 * libostaple_gb300_bench.so (linked against libostaple_gb300.so).  They are
 * not part of the drop-in and have no reference counterpart. */
#ifndef OSTAPLE_GB300_BENCH_H
#define OSTAPLE_GB300_BENCH_H

#include "ostaple_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Mean milliseconds of one launch of a hot kernel, timed with CUDA events on
 * the library stream (launched as in the solve, after one untimed pass):
 * which = 0 FP64 D_eo (as acc_Deo), 1 FP32 D_oe of the mixed solver, 2 FP32
 * fused D_eo + M^+M epilogue + <p,Ap>, 3 double-float M^+M.  Returns the
 * library's error code. */
int ostaple_time_kernel(int which, const su3_soa *u, const double_soa *phases, int reps, double *ms);

/* Measured FMA throughput of this device in TFLOP/s (fp64 != 0: FP64, else
 * FP32); the ceiling of the compute-bound FP64 kernels. */
int ostaple_probe_fma_tflops(int fp64, double *tflops);

#ifdef __cplusplus
}
#endif

#endif
