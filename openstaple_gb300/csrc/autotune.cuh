// autotune.cuh -- launch-shape autotuner for the FP32 hop kernels.
//
// Only kernels whose results do not depend on their launch shape are tuned:
// the D_oe hops of the mixed, batched and multi-shift solvers, which have no
// reduction and compute every output with the same arithmetic whatever the
// block size or the number of systems a thread carries.  Tuning therefore
// never changes a single bit of a solve.  The first time a (kernel, lattice,
// variant) key is seen, each candidate is launched once to warm up and three
// times under CUDA events on the caller's stream; the fastest is kept for
// the life of the process.  Callers tune before they capture a CUDA graph
// (nothing may be timed inside a capture).  OSTAPLE_AUTOTUNE=0 in the
// environment or ostaple_autotune(0) selects candidate 0 (the default shape)
// everywhere.
#pragma once
#include <cuda_runtime.h>
#include <functional>

namespace ost {

enum TuneKernel { TUNE_MX_DOE = 0, TUNE_B_DOE = 1, TUNE_CGM_DOE = 2, TUNE_MX_DEO = 3 };

bool autotune_enabled();

// Index of the chosen candidate for (kernel, sizeh, variant); `launch(c)`
// enqueues candidate c on stream st.  Returns 0 when tuning is disabled.
int autotune_pick(int kernel, long sizeh, int variant, int ncand, const std::function<void(int)>& launch,
                  cudaStream_t st);

// The cached choice, or -1 if the key has not been tuned.
int autotune_cached(int kernel, long sizeh, int variant);

// A device copy of the host bytes [host, host + bytes) (at most 64 KiB) for
// the solver scalars of a tuning launch: the tuned kernels return at once when
// their scalars say every system has converged, so they are timed against a
// copy that marks every system active rather than the caller's live state.
void* autotune_scalars(const void* host, size_t bytes, cudaStream_t st);

}  // namespace ost
