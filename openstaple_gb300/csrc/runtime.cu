// runtime.cu -- library runtime: initialisation with run-time lattice
// geometry, the device-residency registry that stands in for OpenACC's
// `enter data` / `update device|host` / `present` semantics
// (alloc_vars.c:94-284, memory_wrapper.c:14-57 in the reference), error
// reporting and the device workspace.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <cstdlib>
#include "runtime.cuh"
#include "../../include/ostaple_gb300.h"

namespace ost {

static Runtime g_rt;
static Geom g_host_geom{};
unsigned long long g_kernel_launches = 0;

int g_device_loop = -1;   // -1: the environment decides

bool device_loop_enabled() {
  if (g_device_loop < 0) {
    const char* e = std::getenv("OSTAPLE_DEVICE_LOOP");
    g_device_loop = (e && std::strcmp(e, "0") == 0) ? 0 : 1;
  }
  return g_device_loop != 0;
}

bool pdl_enabled() {
  static int on = -1;
  if (on < 0) {
    const char* e = getenv("OSTAPLE_PDL");
    on = (e && e[0] == '0' && e[1] == 0) ? 0 : 1;
  }
  return on == 1;
}
Runtime& rt() { return g_rt; }
const Geom& host_geom() { return g_host_geom; }

static int g_err = 0;
static char g_msg[512] = "";

void set_error(int code, const char* fmt, ...) {
  if (g_err != 0) return;  // keep the first failure
  g_err = code ? code : -1;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
  va_end(ap);
  fprintf(stderr, "[ostaple] error: %s\n", g_msg);
}
int error_code() { return g_err; }
const char* error_message() { return g_msg; }
void clear_error() { g_err = 0; g_msg[0] = 0; }

bool require_init(const char* who) {
  if (!g_rt.initialized) {
    set_error(-2, "%s called before ostaple_init()", who);
    return false;
  }
  return true;
}

// ---- residency registry ----
struct Mirror { size_t bytes; void* dptr; };
static std::map<uintptr_t, Mirror> g_reg;
static std::mutex g_reg_mu;

static bool lookup(uintptr_t a, uintptr_t* base, Mirror* m) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  auto it = g_reg.upper_bound(a);
  if (it == g_reg.begin()) return false;
  --it;
  if (a >= it->first && a < it->first + it->second.bytes) {
    *base = it->first;
    *m = it->second;
    return true;
  }
  return false;
}

void* resolve(const void* p, const char* what) {
  if (p == nullptr) {
    set_error(-3, "null pointer for %s", what);
    return nullptr;
  }
  uintptr_t a = reinterpret_cast<uintptr_t>(p), base;
  Mirror m;
  if (lookup(a, &base, &m)) return static_cast<char*>(m.dptr) + (a - base);
  cudaPointerAttributes attr;
  cudaError_t e = cudaPointerGetAttributes(&attr, p);
  if (e == cudaSuccess && (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged))
    return const_cast<void*>(p);
  cudaGetLastError();
  set_error(-4, "%s: pointer %p is neither registered with ostaple_enter_data nor device memory",
            what, p);
  return nullptr;
}

// ---- workspace ----
struct Slot { void* p = nullptr; size_t bytes = 0; };
static Slot g_ws[WS_NSLOTS];
static unsigned long long g_epoch = 1;
unsigned long long runtime_epoch() { return g_epoch; }

void* workspace(int slot, size_t bytes) {
  Slot& s = g_ws[slot];
  if (bytes <= s.bytes) return s.p;
  if (s.p) { cudaStreamSynchronize(g_rt.stream); cudaFree(s.p); s.p = nullptr; s.bytes = 0; }
  size_t want = (bytes + 255) & ~size_t(255);
  ++g_epoch;
  if (cudaMalloc(&s.p, want) != cudaSuccess) {
    cudaGetLastError();
    set_error(-5, "workspace slot %d: cudaMalloc(%zu) failed", slot, want);
    return nullptr;
  }
  s.bytes = want;
  return s.p;
}

static void free_workspace() {
  ++g_epoch;
  for (auto& s : g_ws) { if (s.p) cudaFree(s.p); s.p = nullptr; s.bytes = 0; }
}

}  // namespace ost

using namespace ost;

extern "C" {

int ostaple_device_loop(int enable) {
  ost::g_device_loop = enable ? 1 : 0;
  return 0;
}

int ostaple_init(int n0, int n1, int n2, int n3) {
  clear_error();
  if (n0 < 2 || n1 < 2 || n2 < 2 || n3 < 2 || (n0 & 1) || (n1 & 1) || (n2 & 1) || (n3 & 1)) {
    set_error(-6, "ostaple_init: every lattice extent must be even and >= 2 (got %d %d %d %d)",
              n0, n1, n2, n3);
    return -6;
  }
  long vol = long(n0) * n1 * n2 * n3;
  if (vol / 2 > (1L << 30)) {
    set_error(-6, "ostaple_init: lattice too large");
    return -6;
  }
  // the lattice is known to the host-only functions (configuration files)
  // even when no device can be initialised
  g_host_geom = Geom{};
  g_host_geom.n0 = n0; g_host_geom.n1 = n1; g_host_geom.n2 = n2; g_host_geom.n3 = n3;
  g_host_geom.nh0 = n0 / 2;
  g_host_geom.sizeh = int(vol / 2);
  g_host_geom.vol1 = n0; g_host_geom.vol2 = n0 * n1; g_host_geom.vol3 = n0 * n1 * n2;
  Runtime& r = g_rt;
  if (!r.initialized) {
    if (cudaGetDevice(&r.device) != cudaSuccess) { cudaGetLastError(); r.device = 0; }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, r.device) != cudaSuccess) {
      cudaGetLastError();
      set_error(-7, "ostaple_init: no CUDA device available");
      return -7;
    }
    r.num_sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&r.stream, cudaStreamNonBlocking) != cudaSuccess) {
      set_error(-7, "ostaple_init: stream creation failed");
      return -7;
    }
    r.own_stream = true;
  }
  Geom& g = r.g;
  g.n0 = n0; g.n1 = n1; g.n2 = n2; g.n3 = n3;
  g.nh0 = n0 / 2;
  g.sizeh = int(vol / 2);
  g.vol1 = n0; g.vol2 = n0 * n1; g.vol3 = n0 * n1 * n2;
  g.fnh0 = FastDiv(uint32_t(g.nh0));
  g.fn1 = FastDiv(uint32_t(n1));
  g.fn2 = FastDiv(uint32_t(n2));
  ++g_epoch;
  r.initialized = true;
  return 0;
}

int ostaple_finalize(void) {
  Runtime& r = g_rt;
  if (!r.initialized) return 0;
  cudaStreamSynchronize(r.stream);
  {
    std::lock_guard<std::mutex> lk(g_reg_mu);
    for (auto& kv : g_reg) cudaFree(kv.second.dptr);
    g_reg.clear();
  }
  free_workspace();
  if (r.own_stream) cudaStreamDestroy(r.stream);
  r.stream = nullptr;
  r.initialized = false;
  return 0;
}

int ostaple_sizeh(void) { return g_rt.initialized ? g_rt.g.sizeh : 0; }

int ostaple_set_stream(void* stream) {
  if (!require_init("ostaple_set_stream")) return -2;
  Runtime& r = g_rt;
  cudaStreamSynchronize(r.stream);
  if (r.own_stream) cudaStreamDestroy(r.stream);
  r.stream = static_cast<cudaStream_t>(stream);
  r.own_stream = false;
  return 0;
}

int ostaple_synchronize(void) {
  if (!g_rt.initialized) return 0;
  OST_CUDA(cudaStreamSynchronize(g_rt.stream));
  return g_err;
}

int ostaple_get_error(void) { return g_err; }
const char* ostaple_last_error(void) { return g_msg; }
void ostaple_clear_error(void) { clear_error(); }

int ostaple_enter_data(const void* host, size_t bytes) {
  if (!require_init("ostaple_enter_data")) return -2;
  uintptr_t a = reinterpret_cast<uintptr_t>(host), base;
  Mirror m;
  if (lookup(a, &base, &m)) {
    if (a == base && bytes <= m.bytes) return 0;  // already present
    set_error(-8, "ostaple_enter_data: %p overlaps an existing mirror", host);
    return -8;
  }
  void* d = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) {
    cudaGetLastError();
    set_error(-5, "ostaple_enter_data: cudaMalloc(%zu) failed", bytes);
    return -5;
  }
  OST_CUDA(cudaMemsetAsync(d, 0, bytes, g_rt.stream));
  std::lock_guard<std::mutex> lk(g_reg_mu);
  g_reg[a] = Mirror{bytes, d};
  return 0;
}

int ostaple_exit_data(const void* host) {
  if (!require_init("ostaple_exit_data")) return -2;
  uintptr_t a = reinterpret_cast<uintptr_t>(host);
  std::lock_guard<std::mutex> lk(g_reg_mu);
  auto it = g_reg.find(a);
  if (it == g_reg.end()) return -9;
  cudaStreamSynchronize(g_rt.stream);
  cudaFree(it->second.dptr);
  g_reg.erase(it);
  return 0;
}

int ostaple_update_device(const void* host, size_t bytes) {
  if (!require_init("ostaple_update_device")) return -2;
  uintptr_t a = reinterpret_cast<uintptr_t>(host), base;
  Mirror m;
  if (!lookup(a, &base, &m) || a + bytes > base + m.bytes) {
    set_error(-9, "ostaple_update_device: %p (+%zu) is not present", host, bytes);
    return -9;
  }
  OST_CUDA(cudaMemcpyAsync(static_cast<char*>(m.dptr) + (a - base), host, bytes,
                           cudaMemcpyHostToDevice, g_rt.stream));
  OST_CUDA(cudaStreamSynchronize(g_rt.stream));
  return g_err;
}

int ostaple_update_host(void* host, size_t bytes) {
  if (!require_init("ostaple_update_host")) return -2;
  uintptr_t a = reinterpret_cast<uintptr_t>(host), base;
  Mirror m;
  if (!lookup(a, &base, &m) || a + bytes > base + m.bytes) {
    set_error(-9, "ostaple_update_host: %p (+%zu) is not present", host, bytes);
    return -9;
  }
  OST_CUDA(cudaMemcpyAsync(host, static_cast<char*>(m.dptr) + (a - base), bytes,
                           cudaMemcpyDeviceToHost, g_rt.stream));
  OST_CUDA(cudaStreamSynchronize(g_rt.stream));
  return g_err;
}

unsigned long long ostaple_kernel_launches(void) { return g_kernel_launches; }

int ostaple_pin_host(void* host, size_t bytes) {
  cudaError_t e = cudaHostRegister(host, bytes, cudaHostRegisterDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(int(e), "ostaple_pin_host: %s", cudaGetErrorString(e));
    return int(e);
  }
  return 0;
}

int ostaple_unpin_host(void* host) {
  cudaError_t e = cudaHostUnregister(host);
  if (e != cudaSuccess) { cudaGetLastError(); return int(e); }
  return 0;
}

void* ostaple_deviceptr(const void* host) {
  uintptr_t a = reinterpret_cast<uintptr_t>(host), base;
  Mirror m;
  if (lookup(a, &base, &m)) return static_cast<char*>(m.dptr) + (a - base);
  return nullptr;
}

}  // extern "C"
