// capi_learned.cu -- C entry points of the learned preconditioner: weight
// initialisation and exchange, application, gradients, training on
// (source, solution) pairs, and flexible CG preconditioned by the network.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>
#include "dslash.cuh"
#include "kernels.cuh"
#include "learned.cuh"
#include "mixed.cuh"
#include "runtime.cuh"
#include "../../include/ostaple_gb300.h"

using namespace ost;

namespace {

typedef double2 Z;

struct NetState {
  bool ready = false;
  long sizeh = 0;
  NetBuffers nb{};
  float2* z = nullptr;      // network output (FP32 vec3)
  float2* in32 = nullptr;   // network input staging (FP32 vec3)
  float2* x32 = nullptr;    // training target staging
  float2* e32 = nullptr;    // residual loss: z - x, A (z - x), A A (z - x), operator temporary
  float2* w32 = nullptr;
  float2* aw32 = nullptr;
  float2* t32 = nullptr;
  int adam_t = 0;
};
NetState g_net;

void free_net() {
  NetBuffers& b = g_net.nb;
  for (void* p : {(void*)b.act, (void*)b.grad_a, (void*)b.grad_b, (void*)b.w_master, (void*)b.adam_m,
                  (void*)b.adam_v, (void*)b.dw, (void*)b.dw_partials, (void*)b.w_mma, (void*)b.err, (void*)b.loss,
                  (void*)g_net.z, (void*)g_net.in32, (void*)g_net.x32, (void*)g_net.e32, (void*)g_net.w32,
                  (void*)g_net.aw32, (void*)g_net.t32})
    if (p) cudaFree(p);
  g_net = NetState();
}

bool ensure_net() {
  const long sh = rt().g.sizeh;
  if (g_net.ready && g_net.sizeh == sh) return true;
  std::vector<float> keep;
  if (g_net.ready) {   // keep the weights across a geometry change
    keep.resize(NET_LAYERS * NET_K * NET_C);
    cudaMemcpy(keep.data(), g_net.nb.w_master, keep.size() * sizeof(float), cudaMemcpyDeviceToHost);
    free_net();
  }
  NetBuffers& b = g_net.nb;
  const size_t nw = NET_LAYERS * NET_K * NET_C;
  const size_t nch = size_t(NET_C) * 3 * sh;
  bool ok = cudaMalloc(&b.act, NET_LAYERS * nch * sizeof(__nv_bfloat162)) == cudaSuccess &&
            cudaMalloc(&b.grad_a, nch * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&b.grad_b, nch * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&b.w_master, nw * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&b.adam_m, nw * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&b.adam_v, nw * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&b.dw, nw * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&b.dw_partials, 4 * size_t(rt().num_sms) * NET_K * NET_C * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&b.w_mma, NET_LAYERS * NET_N * NET_K * sizeof(__nv_bfloat16)) == cudaSuccess &&
            cudaMalloc(&b.err, 64) == cudaSuccess && cudaMalloc(&b.loss, 64) == cudaSuccess &&
            cudaMalloc(&g_net.z, 3 * sh * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&g_net.in32, 3 * sh * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&g_net.x32, 3 * sh * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&g_net.e32, 3 * sh * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&g_net.w32, 3 * sh * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&g_net.aw32, 3 * sh * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&g_net.t32, 3 * sh * sizeof(float2)) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    set_error(-5, "learned preconditioner: out of device memory");
    free_net();
    return false;
  }
  cudaMemset(b.err, 0, 64);
  cudaMemset(b.adam_m, 0, nw * sizeof(float));
  cudaMemset(b.adam_v, 0, nw * sizeof(float));
  cudaMemset(b.w_master, 0, nw * sizeof(float));
  if (!keep.empty()) cudaMemcpy(b.w_master, keep.data(), nw * sizeof(float), cudaMemcpyHostToDevice);
  g_net.sizeh = sh;
  g_net.ready = true;
  net_sync_weights(b, rt().stream);
  return true;
}

struct Prep {
  const float2* u32;
  const unsigned char* sg;
};

// FP32 compact links and sign bytes; the network needs phases of 0 or pi
bool prep(const su3_soa* u, const double_soa* phases, Prep* p, const Z** u64_out = nullptr,
          const void** ph_out = nullptr) {
  cudaStream_t st = rt().stream;
  const long sh = rt().g.sizeh;
  const Z* u64 = dev(reinterpret_cast<const Z*>(u), "u");
  const void* ph = resolve(phases, "phases");
  if (!u64 || !ph) return false;
  float2* u32 = static_cast<float2*>(workspace(WS_LINKS_F32, sizeof(float2) * 48 * size_t(sh)));
  char* sg = static_cast<char*>(workspace(WS_SIGNS, 256 + 8 * size_t(sh) * sizeof(float)));
  if (!u32 || !sg) return false;
  links_to_f32_compact(u64, u32, sh, st);
  int* flag = reinterpret_cast<int*>(sg);
  const int one = 1;
  OST_CUDA(cudaMemcpyAsync(flag, &one, sizeof(int), cudaMemcpyHostToDevice, st));
  phases_to_signs(static_cast<const double*>(ph), reinterpret_cast<unsigned char*>(sg + 256), flag, sh, st);
  int exact = 0;
  OST_CUDA(cudaMemcpyAsync(&exact, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  OST_CUDA(cudaStreamSynchronize(st));
  if (!exact) {
    set_error(-12, "learned preconditioner: phases must be 0 or pi (staggered phases and boundary signs)");
    return false;
  }
  p->u32 = u32;
  p->sg = reinterpret_cast<const unsigned char*>(sg + 256);
  if (u64_out) *u64_out = u64;
  if (ph_out) *ph_out = ph;
  return true;
}

void apply_net(const Prep& p, const float2* r, float2* z, cudaStream_t st) {
  net_load_input(g_net.nb, r, st);
  for (int l = 0; l < NET_LAYERS; ++l) net_layer_forward(g_net.nb, l, p.u32, p.sg, z, st);
}

bool check_err(const char* who) {
  int e = 0;
  OST_CUDA(cudaMemcpyAsync(&e, g_net.nb.err, sizeof(int), cudaMemcpyDeviceToHost, rt().stream));
  OST_CUDA(cudaStreamSynchronize(rt().stream));
  if (e) {
    set_error(-13, "%s: a tensor-core MMA did not complete within its wait limit", who);
    cudaMemsetAsync(g_net.nb.err, 0, sizeof(int), rt().stream);
    return false;
  }
  return error_code() == 0;
}

double norm2_f(const float2* v, long n, cudaStream_t st) {
  double* d = static_cast<double*>(workspace(WS_SCALARS, 64 * sizeof(double) + 4 * sizeof(MixScal) + 256));
  blas_norm2<float>(v, n, d + 40, st);
  double h;
  OST_CUDA(cudaMemcpyAsync(&h, d + 40, sizeof(double), cudaMemcpyDeviceToHost, st));
  OST_CUDA(cudaStreamSynchronize(st));
  return h;
}
double rdot_f(const float2* a, const float2* b, long n, cudaStream_t st) {
  double* d = static_cast<double*>(workspace(WS_SCALARS, 64 * sizeof(double) + 4 * sizeof(MixScal) + 256));
  blas_rdot<float>(a, b, n, d + 41, st);
  double h;
  OST_CUDA(cudaMemcpyAsync(&h, d + 41, sizeof(double), cudaMemcpyDeviceToHost, st));
  OST_CUDA(cudaStreamSynchronize(st));
  return h;
}

void mdagm_f32(const Prep& p, float2* out, const float2* in, float2* tmp, double m2, cudaStream_t st) {
  DslashArgs<float> a;
  a.phase_mode = PH_SIGN8; a.u = p.u32; a.phases = p.sg; a.stream = st; a.compact_links = 1;
  a.parity = 1; a.epilogue = EPI_PLAIN; a.out = tmp; a.in = in; a.in0 = nullptr; a.mass2 = 0.f;
  launch_dslash<float>(a);
  a.parity = 0; a.epilogue = EPI_MDAGM; a.out = out; a.in = tmp; a.in0 = in; a.mass2 = float(m2);
  launch_dslash<float>(a);
}

void mdagm_f64(const Z* u64, const void* ph, Z* out, const Z* in, Z* tmp, double m2, cudaStream_t st) {
  DslashArgs<double> a;
  a.phase_mode = PH_ANGLE; a.u = u64; a.phases = ph; a.stream = st; a.compact_links = 0;
  a.parity = 1; a.epilogue = EPI_PLAIN; a.out = tmp; a.in = in; a.in0 = nullptr; a.mass2 = 0;
  launch_dslash<double>(a);
  a.parity = 0; a.epilogue = EPI_MDAGM; a.out = out; a.in = tmp; a.in0 = in; a.mass2 = m2;
  launch_dslash<double>(a);
}

// Forward + backward of one (source b, solution x) pair; dW accumulates.
// The loss is the residual of the preconditioned source, |A (N(b) - x)|^2 =
// |A N(b) - b|^2, scaled by `scale`: it weights the error by A^2, so the
// network learns A^{-1} where CG needs it (the large eigenvalues, which a
// few hops can reach) instead of chasing the low modes that dominate x, and
// the trained map comes out close to Hermitian.
void pair_grad(const Prep& p, const float2* b32, const float2* x32, double scale, double m2, int accumulate_loss,
               cudaStream_t st) {
  NetBuffers& nb = g_net.nb;
  const long n = 3L * rt().g.sizeh;
  apply_net(p, b32, g_net.z, st);
  blas_axpy<float>(x32, -1.0, g_net.z, g_net.e32, n, st);        // e = z - x
  mdagm_f32(p, g_net.w32, g_net.e32, g_net.t32, m2, st);         // w = A e
  mdagm_f32(p, g_net.aw32, g_net.w32, g_net.t32, m2, st);        // A w
  net_residual_loss_grad(nb, g_net.w32, g_net.aw32, scale, accumulate_loss, st);
  float* gout = nb.grad_a;
  float* gin = nb.grad_b;
  for (int l = NET_LAYERS - 1; l >= 0; --l) {
    net_layer_backward(nb, l, p.u32, p.sg, gout, gin, l > 0, st);
    float* t = gout; gout = gin; gin = t;
  }
}

}  // namespace

extern "C" {

int ostaple_selftest_bounded_wait(int signal) {
  if (!require_init("ostaple_selftest_bounded_wait")) return -2;
  if (!ensure_net()) return -5;
  net_wait_selftest(g_net.nb, signal ? 1 : 0, 1024, rt().stream);
  return check_err("ostaple_selftest_bounded_wait") ? 0 : -13;
}

// ---- weight files: magic, version, shape, FP32 weights, FNV-1a 64 checksum ----
namespace {
constexpr char kNetMagic[8] = {'O', 'S', 'T', 'N', 'E', 'T', 'W', 'T'};
constexpr uint32_t kNetVersion = 1;

uint64_t fnv1a64(const unsigned char* p, size_t n, uint64_t h = 0xcbf29ce484222325ull) {
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 0x100000001b3ull;
  }
  return h;
}

struct NetFileHeader {
  char magic[8];
  uint32_t version, layers, rows, cols;
};
}  // namespace

int ostaple_net_weights_save(const char* path, const float* w) {
  NetFileHeader h;
  memcpy(h.magic, kNetMagic, 8);
  h.version = kNetVersion;
  h.layers = NET_LAYERS;
  h.rows = NET_K;
  h.cols = NET_C;
  const size_t nw = size_t(NET_LAYERS) * NET_K * NET_C;
  uint64_t sum = fnv1a64(reinterpret_cast<const unsigned char*>(&h), sizeof(h));
  sum = fnv1a64(reinterpret_cast<const unsigned char*>(w), nw * sizeof(float), sum);
  FILE* f = fopen(path, "wb");
  if (!f) {
    set_error(-17, "ostaple_net_weights_save: cannot open %s", path);
    return -17;
  }
  const bool ok = fwrite(&h, sizeof(h), 1, f) == 1 && fwrite(w, sizeof(float), nw, f) == nw &&
                  fwrite(&sum, sizeof(sum), 1, f) == 1;
  if (fclose(f) != 0 || !ok) {
    set_error(-17, "ostaple_net_weights_save: write to %s failed", path);
    return -17;
  }
  return 0;
}

int ostaple_net_weights_load(const char* path, float* w) {
  FILE* f = fopen(path, "rb");
  if (!f) {
    set_error(-17, "ostaple_net_weights_load: cannot open %s", path);
    return -17;
  }
  NetFileHeader h;
  const size_t nw = size_t(NET_LAYERS) * NET_K * NET_C;
  std::vector<float> buf(nw);
  uint64_t stored = 0;
  const bool ok = fread(&h, sizeof(h), 1, f) == 1 && fread(buf.data(), sizeof(float), nw, f) == nw &&
                  fread(&stored, sizeof(stored), 1, f) == 1;
  fclose(f);
  if (!ok) {
    set_error(-18, "ostaple_net_weights_load: %s is truncated", path);
    return -18;
  }
  if (memcmp(h.magic, kNetMagic, 8) != 0 || h.version != kNetVersion || h.layers != uint32_t(NET_LAYERS) ||
      h.rows != uint32_t(NET_K) || h.cols != uint32_t(NET_C)) {
    set_error(-18, "ostaple_net_weights_load: %s is not a version-%u weight file of shape %dx%dx%d", path,
              kNetVersion, NET_LAYERS, NET_K, NET_C);
    return -18;
  }
  uint64_t sum = fnv1a64(reinterpret_cast<const unsigned char*>(&h), sizeof(h));
  sum = fnv1a64(reinterpret_cast<const unsigned char*>(buf.data()), nw * sizeof(float), sum);
  if (sum != stored) {
    set_error(-19, "ostaple_net_weights_load: checksum mismatch in %s", path);
    return -19;
  }
  memcpy(w, buf.data(), nw * sizeof(float));
  return 0;
}

int ostaple_net_init(unsigned seed, double scale) {
  if (!require_init("ostaple_net_init")) return -2;
  if (!ensure_net()) return -5;
  const size_t nw = NET_LAYERS * NET_K * NET_C;
  std::vector<float> w(nw);
  uint64_t s = 0x9E3779B97F4A7C15ull ^ seed;
  for (size_t i = 0; i < nw; ++i) {   // uniform in [-scale, scale], splitmix64
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    w[i] = float(scale * (2.0 * (double(z >> 11) / 9007199254740992.0) - 1.0));
  }
  OST_CUDA(cudaMemcpy(g_net.nb.w_master, w.data(), nw * sizeof(float), cudaMemcpyHostToDevice));
  OST_CUDA(cudaMemset(g_net.nb.adam_m, 0, nw * sizeof(float)));
  OST_CUDA(cudaMemset(g_net.nb.adam_v, 0, nw * sizeof(float)));
  g_net.adam_t = 0;
  net_sync_weights(g_net.nb, rt().stream);
  OST_CUDA(cudaStreamSynchronize(rt().stream));
  return error_code();
}

int ostaple_net_set_weights(const float* w) {
  if (!require_init("ostaple_net_set_weights")) return -2;
  if (!ensure_net()) return -5;
  OST_CUDA(cudaMemcpy(g_net.nb.w_master, w, NET_LAYERS * NET_K * NET_C * sizeof(float), cudaMemcpyHostToDevice));
  net_sync_weights(g_net.nb, rt().stream);
  OST_CUDA(cudaStreamSynchronize(rt().stream));
  return error_code();
}

int ostaple_net_get_weights(float* w) {
  if (!require_init("ostaple_net_get_weights")) return -2;
  if (!ensure_net()) return -5;
  OST_CUDA(cudaMemcpy(w, g_net.nb.w_master, NET_LAYERS * NET_K * NET_C * sizeof(float), cudaMemcpyDeviceToHost));
  return error_code();
}

int ostaple_net_apply(const su3_soa* u, const double_soa* phases, const vec3_soa* in, vec3_soa* out) {
  if (!require_init("ostaple_net_apply")) return -2;
  if (!ensure_net()) return -5;
  cudaStream_t st = rt().stream;
  Prep p;
  if (!prep(u, phases, &p)) return -3;
  const long n = 3L * rt().g.sizeh;
  const Z* din = dev(reinterpret_cast<const Z*>(in), "in");
  Z* dout = dev(reinterpret_cast<Z*>(out), "out");
  if (!din || !dout) return -3;
  conv_d2f(din, g_net.in32, n, st);
  apply_net(p, g_net.in32, g_net.z, st);
  conv_f2d(g_net.z, dout, n, st);
  return check_err("ostaple_net_apply") ? 0 : -13;
}

int ostaple_net_gradient(const su3_soa* u, const double_soa* phases, double mass, double shift,
                         const vec3_soa* source, const vec3_soa* target, float* dw, double* loss) {
  if (!require_init("ostaple_net_gradient")) return -2;
  if (!ensure_net()) return -5;
  cudaStream_t st = rt().stream;
  Prep p;
  if (!prep(u, phases, &p)) return -3;
  const long n = 3L * rt().g.sizeh;
  const Z* b = dev(reinterpret_cast<const Z*>(source), "source");
  const Z* x = dev(reinterpret_cast<const Z*>(target), "target");
  if (!b || !x) return -3;
  conv_d2f(b, g_net.in32, n, st);
  conv_d2f(x, g_net.x32, n, st);
  const double bn = norm2_f(g_net.in32, n, st);
  net_zero_dw(g_net.nb, st);
  pair_grad(p, g_net.in32, g_net.x32, 1.0 / bn, mass * mass + shift, 0, st);
  OST_CUDA(cudaMemcpyAsync(dw, g_net.nb.dw, NET_LAYERS * NET_K * NET_C * sizeof(float), cudaMemcpyDeviceToHost, st));
  OST_CUDA(cudaMemcpyAsync(loss, g_net.nb.loss, sizeof(double), cudaMemcpyDeviceToHost, st));
  return check_err("ostaple_net_gradient") ? 0 : -13;
}

int ostaple_net_train(const su3_soa* u, const double_soa* phases, double mass, double shift, int npairs,
                      const vec3_soa* sources, const vec3_soa* solutions, int epochs, double lr,
                      double* loss_history) {
  if (!require_init("ostaple_net_train")) return -2;
  if (!ensure_net()) return -5;
  cudaStream_t st = rt().stream;
  Prep p;
  if (!prep(u, phases, &p)) return -3;
  const long n = 3L * rt().g.sizeh;
  const Z* b = dev(reinterpret_cast<const Z*>(sources), "sources");
  const Z* x = dev(reinterpret_cast<const Z*>(solutions), "solutions");
  if (!b || !x || npairs < 1) return -3;
  const double m2 = mass * mass + shift;
  std::vector<double> bn(npairs);
  for (int i = 0; i < npairs; ++i) {
    conv_d2f(b + i * n, g_net.in32, n, st);
    bn[i] = norm2_f(g_net.in32, n, st);
  }
  for (int e = 0; e < epochs; ++e) {
    net_zero_dw(g_net.nb, st);
    for (int i = 0; i < npairs; ++i) {
      conv_d2f(b + i * n, g_net.in32, n, st);
      conv_d2f(x + i * n, g_net.x32, n, st);
      pair_grad(p, g_net.in32, g_net.x32, 1.0 / (bn[i] * npairs), m2, i > 0, st);
    }
    ++g_net.adam_t;
    net_adam_step(g_net.nb, float(lr), 0.9f, 0.999f, 1e-8f, g_net.adam_t, st);
    if (loss_history) {
      OST_CUDA(cudaMemcpyAsync(&loss_history[e], g_net.nb.loss, sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    if (!check_err("ostaple_net_train")) return -13;
  }
  OST_CUDA(cudaStreamSynchronize(st));
  return error_code();
}

// Flexible CG (Notay's FCG with one stored direction) on (M^+M + shift) x = b,
// preconditioned by the network: FP32 iteration, FP64 solution, reliable
// updates of the residual in FP64, stop when the FP64 true residual is <= res.
// If the preconditioned iteration does not converge within max_iter, stalls
// (no new minimum of the residual for 500 iterations) or produces non-finite
// numbers, the plain mixed-precision CG finishes the solve and
// *used_fallback is set.
int ostaple_invert_learned(const su3_soa* u, const double_soa* phases, double mass, double shift, vec3_soa* solution,
                           const vec3_soa* in, double res, int max_iter, int* iters, double* true_res,
                           int* used_fallback) {
  if (!require_init("ostaple_invert_learned")) return INVERTER_FAILURE;
  if (!ensure_net()) return INVERTER_FAILURE;
  cudaStream_t st = rt().stream;
  Prep p;
  const Z* u64;
  const void* ph;
  if (!prep(u, phases, &p, &u64, &ph)) return INVERTER_FAILURE;
  const long n = 3L * rt().g.sizeh;
  Z* x = dev(reinterpret_cast<Z*>(solution), "solution");
  const Z* b = dev(reinterpret_cast<const Z*>(in), "in");
  if (!x || !b) return INVERTER_FAILURE;
  Z* r64 = static_cast<Z*>(workspace(WS_VEC0, 3 * n * sizeof(Z)));
  float2* f = static_cast<float2*>(workspace(WS_VEC1, 6 * n * sizeof(float2)));
  if (!r64 || !f) return INVERTER_FAILURE;
  Z* t64 = r64 + n;
  Z* t64b = r64 + 2 * n;
  float2 *r = f, *z = f + n, *pv = f + 2 * n, *s = f + 3 * n, *xf = f + 4 * n, *t = f + 5 * n;
  const double m2 = mass * mass + shift;
  double bn;
  {
    double* d = static_cast<double*>(workspace(WS_SCALARS, 64 * sizeof(double) + 4 * sizeof(MixScal) + 256));
    blas_norm2<double>(b, n, d + 42, st);
    OST_CUDA(cudaMemcpyAsync(&bn, d + 42, sizeof(double), cudaMemcpyDeviceToHost, st));
    OST_CUDA(cudaStreamSynchronize(st));
  }
  const double target2 = res * res * bn;
  auto reliable = [&]() -> double {   // x += x_f ; r = b - A x in FP64 ; returns |r|^2
    acc_f2d(xf, x, n, st);
    blas_zero<float>(xf, n, st);
    mdagm_f64(u64, ph, t64, x, t64b, m2, st);
    blas_axmy<double>(b, 1.0, t64, r64, n, st);
    conv_d2f(r64, r, n, st);
    double* d = static_cast<double*>(workspace(WS_SCALARS, 64 * sizeof(double) + 4 * sizeof(MixScal) + 256));
    blas_norm2<double>(r64, n, d + 43, st);
    double h;
    OST_CUDA(cudaMemcpyAsync(&h, d + 43, sizeof(double), cudaMemcpyDeviceToHost, st));
    OST_CUDA(cudaStreamSynchronize(st));
    return h;
  };
  blas_zero<float>(xf, n, st);
  double tr2 = reliable();
  double rr_ref = tr2;
  int it = 0;
  bool converged = tr2 <= target2, broke = false;
  apply_net(p, r, z, st);
  blas_copy<float>(z, pv, n, st);
  mdagm_f32(p, s, pv, t, m2, st);
  double pAp = rdot_f(pv, s, n, st);
  // stagnation guard: a preconditioner that does not help (an untrained or
  // zero network) leaves the residual above its best value for long
  // stretches; hand over to plain CG after STALL iterations without a new best
  constexpr int STALL = 500;
  double rr_best = tr2;
  int it_best = 0;
  while (!converged && it < max_iter) {
    const double pr = rdot_f(pv, r, n, st);
    const double alpha = pr / pAp;
    if (!std::isfinite(alpha)) { broke = true; break; }
    blas_axpy<float>(pv, alpha, xf, xf, n, st);
    blas_axpy<float>(s, -alpha, r, r, n, st);
    ++it;
    double rr = norm2_f(r, n, st);
    if (!std::isfinite(rr)) { broke = true; break; }
    if (rr < rr_best) { rr_best = rr; it_best = it; }
    else if (it - it_best > STALL) break;
    if (rr <= 0.81 * target2 || rr < 1e-4 * rr_ref) {
      tr2 = reliable();
      rr_ref = tr2;
      if (tr2 <= target2) { converged = true; break; }
    }
    apply_net(p, r, z, st);
    const double beta = -rdot_f(z, s, n, st) / pAp;     // A-orthogonalise against the previous direction
    blas_axpy<float>(pv, beta, z, pv, n, st);           // p = z + beta p
    mdagm_f32(p, s, pv, t, m2, st);
    pAp = rdot_f(pv, s, n, st);
    if (error_code()) break;
  }
  if (!check_err("ostaple_invert_learned")) broke = true;
  int fallback = 0;
  if (!converged) {
    // plain mixed-precision CG from the current solution
    acc_f2d(xf, x, n, st);
    blas_zero<float>(xf, n, st);
    ostaple_clear_error();
    int it2 = 0, nrel = 0;
    double trr = 0;
    ostaple_invert_mixed(u, phases, mass, shift, solution, in, res, max_iter, 0, 0.0, &it2, &trr, &nrel);
    it += it2;
    tr2 = trr * trr * bn;
    converged = trr <= res;
    fallback = 1;
  }
  (void)broke;
  if (iters) *iters = it;
  if (true_res) *true_res = std::sqrt(tr2 / bn);
  if (used_fallback) *used_fallback = fallback;
  if (error_code()) return INVERTER_FAILURE;
  return converged ? INVERTER_SUCCESS : INVERTER_FAILURE;
}

}  // extern "C"
