// runtime.cuh -- library-internal runtime: geometry, stream, device
// residency registry, error state, and a growable device workspace.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include "common.cuh"

namespace ost {

struct Runtime {
  bool initialized = false;
  int device = 0;
  int num_sms = 0;
  Geom g{};
  cudaStream_t stream = nullptr;
  bool own_stream = false;
};

Runtime& rt();
// The lattice of the last ostaple_init call with valid extents, also when no
// device could be initialised (host-only functions such as the configuration
// files use it).
const Geom& host_geom();

// Error state: the reference's void entry points report through printf; this
// library records the first failure and returns failure codes where the
// reference signature has one.
void set_error(int code, const char* fmt, ...);
int error_code();
const char* error_message();
void clear_error();

#define OST_CUDA(call)                                                       \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      ::ost::set_error(int(e_), "%s:%d %s -> %s", __FILE__, __LINE__, #call, \
                       cudaGetErrorString(e_));                              \
    }                                                                        \
  } while (0)

// Every kernel launch of the library goes through OST_LAUNCH_CHECK, which
// also counts it (graph replays add the kernels they contain).
extern unsigned long long g_kernel_launches;
#define OST_LAUNCH_CHECK()          \
  do {                              \
    ++::ost::g_kernel_launches;     \
    OST_CUDA(cudaGetLastError());   \
  } while (0)

bool require_init(const char* who);

// Programmatic dependent launch.  A kernel launched by launch_pdl may start
// while the kernel before it on the stream is still running (its blocks are
// scheduled once every block of that kernel has started or passed
// pdl_trigger).  Such a kernel calls pdl_wait() before it reads anything the
// previous kernel writes; it may read earlier before the wait only what
// kernels at least two launches back wrote, and it calls pdl_trigger() only
// after its own pdl_wait(), so a kernel two launches on finds every earlier
// kernel complete.  Both are no-ops for a kernel launched without the
// attribute.  OSTAPLE_PDL=0 in the environment launches without it.
bool pdl_enabled();

// Solvers run their iteration as one graph launch with a device-side loop
// (conditional graph nodes) unless this is off: ostaple_device_loop(0), or
// OSTAPLE_DEVICE_LOOP=0 in the environment.
bool device_loop_enabled();

template <typename... P, typename... A>
void launch_pdl(void (*kernel)(P...), int grid, int block, cudaStream_t st, A&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(unsigned(grid));
  cfg.blockDim = dim3(unsigned(block));
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  OST_CUDA(cudaLaunchKernelEx(&cfg, kernel, static_cast<P>(args)...));
}

// Host pointer -> device mirror (the OpenACC `present` table).  A pointer that
// is not registered but already addresses device memory is used as is.
// Returns nullptr (and records an error) if the pointer is neither.
void* resolve(const void* p, const char* what);
template <typename T> T* dev(const T* p, const char* what) {
  return static_cast<T*>(resolve(static_cast<const void*>(p), what));
}

// Growable named device workspace; buffers persist until finalize.
void* workspace(int slot, size_t bytes);
// Changes whenever the geometry is set or any workspace buffer is allocated
// or freed.  State derived from workspace contents or addresses (a zeroed
// ticket counter, a captured CUDA graph) is valid only for the epoch it was
// made in: fresh cudaMalloc memory holds whatever was there before.
unsigned long long runtime_epoch();
enum WorkspaceSlot {
  WS_REDUCE = 0,   // block partial sums
  WS_SCALARS,      // device-resident solver scalars
  WS_VEC0, WS_VEC1, WS_VEC2, WS_VEC3, WS_VEC4, WS_VEC5,
  WS_LINKS_F32,    // FP32 copy of links for the mixed/batched solvers
  WS_SIGNS,        // per-link staggered sign bytes
  WS_MULTI,        // multi-shift / multi-RHS vectors
  WS_MULTI2,
  WS_FORCE0, WS_FORCE1, WS_FORCE2, WS_FORCE3,
  WS_NET,          // learned preconditioner weights and activations
  WS_NET2,
  WS_CGM,          // batched multi-shift scalars
  WS_BATCH,        // batched solver vectors
  WS_BATCH64,
  WS_LINKS_LO,     // lo parts of the double-float links
  WS_DF,           // double-float M^+M work fields
  WS_LINKS_Q16,    // 16-bit fixed-point sloppy links
  WS_HMC_MOM,      // link generator: FP64 momenta
  WS_HMC_BKP,      // link generator: links before the trajectory (Metropolis reject)
  WS_HMC_F32,      // link generator: FP32 links and momenta of the molecular dynamics
  WS_RHMC,         // RHMC trajectory: smeared levels, parking fields, pseudofermions, momenta
  WS_NSLOTS
};

inline int blocks_for(long n, int threads) { return int((n + threads - 1) / threads); }

}  // namespace ost
