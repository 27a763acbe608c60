// autotune.cu -- the launch-shape cache and its timing (see autotune.cuh).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include "autotune.cuh"
#include "runtime.cuh"
#include "../../include/ostaple_gb300.h"

namespace ost {

namespace {

struct Entry {
  int choice;
  float us[12];
  int ncand;
};

std::map<std::tuple<int, long, int>, Entry>& table() {
  static std::map<std::tuple<int, long, int>, Entry> t;
  return t;
}

int g_enabled = -1;   // -1: read the environment on first use
int g_forced = -1;    // >= 0: every tuned launch uses this candidate (tests)

const char* kernel_name(int k) {
  switch (k) {
    case TUNE_MX_DOE:
      return "k_mx_doe (threads per block, hops in flight) {128/1, 256/1, 64/1, 128/2, 128/4, 256/2, 64/2}";
    case TUNE_MX_DEO: return "k_mx_deo_dot hops in flight {1, 2, 4}";
    case TUNE_B_DOE: return "k_b_doe systems per thread {default, 1, 2, 4}";
    default: return "k_cgm_doe systems per thread {default, 1, 2, 4}";
  }
}

}  // namespace

bool autotune_enabled() {
  if (g_enabled < 0) {
    const char* e = getenv("OSTAPLE_AUTOTUNE");
    g_enabled = (e && strcmp(e, "0") == 0) ? 0 : 1;
  }
  return g_enabled == 1;
}

int autotune_cached(int kernel, long sizeh, int variant) {
  if (g_forced >= 0) return g_forced;
  auto it = table().find(std::make_tuple(kernel, sizeh, variant));
  return it == table().end() ? -1 : it->second.choice;
}

void* autotune_scalars(const void* host, size_t bytes, cudaStream_t st) {
  static void* buf = nullptr;
  const size_t cap = 64 << 10;
  if (bytes > cap) {
    set_error(-1, "autotune_scalars: %zu bytes exceed the %zu-byte buffer", bytes, cap);
    return nullptr;
  }
  if (!buf) OST_CUDA(cudaMalloc(&buf, cap));
  if (!buf) return nullptr;
  OST_CUDA(cudaMemcpyAsync(buf, host, bytes, cudaMemcpyHostToDevice, st));
  OST_CUDA(cudaStreamSynchronize(st));
  return buf;
}

int autotune_pick(int kernel, long sizeh, int variant, int ncand, const std::function<void(int)>& launch,
                  cudaStream_t st) {
  if (g_forced >= 0) return g_forced < ncand ? g_forced : 0;
  if (!autotune_enabled() || ncand <= 1) return 0;
  const auto key = std::make_tuple(kernel, sizeh, variant);
  auto it = table().find(key);
  if (it != table().end()) return it->second.choice;
  Entry e{};
  e.ncand = ncand < 12 ? ncand : 12;
  cudaEvent_t a, b;
  OST_CUDA(cudaEventCreate(&a));
  OST_CUDA(cudaEventCreate(&b));
  int best = 0;
  const bool clean = error_code() == 0;
  for (int c = 0; c < e.ncand; ++c) {
    launch(c);
    if (c > 0 && clean && error_code() != 0) {
      // a candidate that this device refuses to launch (a launch-configuration
      // error: nothing ran, the context is intact) is never picked
      const cudaError_t le = cudaGetLastError();
      if (le == cudaErrorInvalidValue || le == cudaErrorInvalidConfiguration ||
          le == cudaErrorLaunchOutOfResources) {
        clear_error();
        e.us[c] = INFINITY;
        continue;
      }
    }
    OST_CUDA(cudaEventRecord(a, st));
    for (int r = 0; r < 3; ++r) launch(c);
    OST_CUDA(cudaEventRecord(b, st));
    OST_CUDA(cudaEventSynchronize(b));
    float ms = 0.f;
    OST_CUDA(cudaEventElapsedTime(&ms, a, b));
    e.us[c] = ms * 1e3f / 3.f;
    // a candidate must beat the default by 2 % to replace it
    if (c > 0 && e.us[c] < 0.98f * e.us[best]) best = c;
  }
  OST_CUDA(cudaEventDestroy(a));
  OST_CUDA(cudaEventDestroy(b));
  e.choice = error_code() ? 0 : best;
  table()[key] = e;
  return e.choice;
}

}  // namespace ost

using namespace ost;

extern "C" {

int ostaple_autotune(int enable) {
  g_enabled = enable ? 1 : 0;
  g_forced = enable >= 2 ? enable - 2 : -1;
  return 0;
}

int ostaple_autotune_report(char* buf, int len) {
  std::string s;
  char line[256];
  for (const auto& kv : table()) {
    const Entry& e = kv.second;
    snprintf(line, sizeof(line), "%s, sizeh %ld, variant %d: choice %d (us:", kernel_name(std::get<0>(kv.first)),
             std::get<1>(kv.first), std::get<2>(kv.first), e.choice);
    s += line;
    for (int c = 0; c < e.ncand; ++c) {
      snprintf(line, sizeof(line), " %.2f", e.us[c]);
      s += line;
    }
    s += ")\n";
  }
  if (buf && len > 0) {
    strncpy(buf, s.c_str(), size_t(len) - 1);
    buf[len - 1] = 0;
  }
  return int(s.size());
}

}  // extern "C"
