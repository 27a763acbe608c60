// capi_mixed.cu -- C entry points of the mixed-precision solver and the
// inverter dispatch wrappers (inverter_mixedp.c:41-181,
// inverter_wrappers.c:24-160).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include "dslash.cuh"
#include "dslash_df.cuh"
#include "kernels.cuh"
#include "mixed.cuh"
#include "runtime.cuh"
#include "../../include/ostaple_gb300.h"

using namespace ost;

namespace {

typedef double2 Z;
typedef float2 Zf;

struct PreparedF32 {
  const float2* u32;
  int compact;
  const void* ph;
  int mode;
  int q16;
  LinkQ16 uq;
  const float2* lo;   // lo parts of the double-float links (library-converted links only)
};

int g_sloppy_q16 = 1;

// FP32 links and phases for the single-precision kernels.  Links: the
// caller's su3_soa_f if given, else a compact conversion of the FP64 links.
// Phases: one sign byte per link when every angle is 0 or pi, else float
// angles.
bool prepare_f32(const Z* u64, const void* u_f, const double* ph64, PreparedF32* out, cudaStream_t st) {
  const long sh = rt().g.sizeh;
  out->q16 = 0;
  out->uq = LinkQ16{nullptr, nullptr, sh};
  out->lo = nullptr;
  if (u_f) {
    out->u32 = static_cast<const float2*>(resolve(u_f, "u_f"));
    if (!out->u32) return false;
    out->compact = 0;
  } else {
    float2* u32 = static_cast<float2*>(workspace(WS_LINKS_F32, sizeof(float2) * 48 * size_t(sh)));
    float2* lo = static_cast<float2*>(workspace(WS_LINKS_LO, sizeof(float2) * 48 * size_t(sh)));
    if (!u32 || !lo) return false;
    links_to_f32_compact(u64, u32, sh, st, lo);
    out->u32 = u32;
    out->lo = lo;
    out->compact = 1;
    if (g_sloppy_q16) {
      // 8 directions x (16 + 8) bytes per half-lattice site
      char* q = static_cast<char*>(workspace(WS_LINKS_Q16, 8 * 24 * size_t(sh)));
      if (!q) return false;
      uint4* a = reinterpret_cast<uint4*>(q);
      uint2* b = reinterpret_cast<uint2*>(q + 8 * 16 * size_t(sh));
      links_to_q16(u32, a, b, sh, st);
      out->q16 = 1;
      out->uq = LinkQ16{a, b, sh};
    }
  }
  char* sg = static_cast<char*>(workspace(WS_SIGNS, 256 + 8 * size_t(sh) * sizeof(float)));
  if (!sg) return false;
  int* flag = reinterpret_cast<int*>(sg);
  const int one = 1;
  OST_CUDA(cudaMemcpyAsync(flag, &one, sizeof(int), cudaMemcpyHostToDevice, st));
  phases_to_signs(ph64, reinterpret_cast<unsigned char*>(sg + 256), flag, sh, st);
  int exact = 0;
  OST_CUDA(cudaMemcpyAsync(&exact, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  OST_CUDA(cudaStreamSynchronize(st));
  if (exact) {
    out->ph = sg + 256;
    out->mode = PH_SIGN8;
  } else {
    phases_to_f32(ph64, reinterpret_cast<float*>(sg + 256), sh, st);
    out->ph = sg + 256;
    out->mode = PH_ANGLE;
  }
  return error_code() == 0;
}

// Double-float operator for the reliable updates: the lo parts of the
// compact links and four work fields.  Only with exact phases (sign bytes)
// and the library's own compact FP32 links.
bool prepare_df(const Z* u64, const PreparedF32& pf, DfOperator* op, DfWork* w, cudaStream_t st) {
  if (pf.mode != PH_SIGN8 || !pf.compact) return false;
  return df_prepare(pf.u32, pf.lo, static_cast<const unsigned char*>(pf.ph), op, w);
}

template <typename T>
T* ws_vec(int slot, int k, int nvec) {
  const size_t n = 3 * size_t(rt().g.sizeh);
  char* base = static_cast<char*>(workspace(slot, nvec * n * sizeof(T)));
  return base ? reinterpret_cast<T*>(base) + k * n : nullptr;
}

MixScal* mix_scalars() {
  char* p = static_cast<char*>(workspace(WS_SCALARS, 64 * sizeof(double) + 4 * sizeof(MixScal) + 256));
  return p ? reinterpret_cast<MixScal*>(p + 64 * sizeof(double)) : nullptr;
}

}  // namespace

namespace ost {
int sloppy_links_q16() { return g_sloppy_q16; }
}  // namespace ost

extern "C" {

// Host runs of the device encoders (same source), for tests without a GPU.
int ostaple_q16_encode_host(const float* h, long n, unsigned* q) {
  for (long i = 0; i < n; ++i) q[i] = q16_encode_f32(h[i]);
  return 0;
}

int ostaple_df_split_host(const double* x, long n, float* hi, float* lo) {
  for (long i = 0; i < n; ++i) {
    hi[i] = float(x[i]);
    lo[i] = df_lo_part(x[i], hi[i]);
  }
  return 0;
}

int ostaple_set_sloppy_links(int fmt) {
  const int prev = g_sloppy_q16;
  g_sloppy_q16 = fmt ? 1 : 0;
  return prev;
}

int ostaple_mdagm_sloppy(const su3_soa* u, const double_soa* phases, double mass, double shift, vec3_soa* out,
                         const vec3_soa* in) {
  if (!require_init("ostaple_mdagm_sloppy")) return -2;
  cudaStream_t st = rt().stream;
  const Z* u64 = dev(reinterpret_cast<const Z*>(u), "u");
  const void* ph = resolve(phases, "phases");
  const Z* din = dev(reinterpret_cast<const Z*>(in), "in");
  Z* dout = dev(reinterpret_cast<Z*>(out), "out");
  if (!u64 || !ph || !din || !dout) return -3;
  MixedBuffers B{};
  B.u64 = u64;
  B.ph64 = ph;
  B.t = ws_vec<Zf>(WS_VEC1, 1, 5);
  B.s = ws_vec<Zf>(WS_VEC1, 2, 5);
  B.p = ws_vec<Zf>(WS_VEC1, 3, 5);
  if (!B.t || !B.s || !B.p) return -4;
  PreparedF32 pf;
  if (!prepare_f32(u64, nullptr, static_cast<const double*>(ph), &pf, st)) return -4;
  B.u32 = pf.u32;
  B.u32_compact = pf.compact;
  B.q16 = pf.q16;
  B.uq = pf.uq;
  B.ph32 = pf.ph;
  B.ph32_mode = pf.mode;
  MixScal* sc = mix_scalars();
  if (!sc) return -4;
  sloppy_mdagm(B, mass * mass + shift, din, dout, sc + 1, st);
  return error_code();
}

int inverter_mixed_precision(inverter_package ip, ferm_param* pars, vec3_soa* solution, const vec3_soa* in,
                             double res, const int max_cg, double shift, int* cg_return) {
  if (!require_init("inverter_mixed_precision")) return INVERTER_FAILURE;
  cudaStream_t st = rt().stream;
  MixedBuffers B{};
  B.u64 = dev(reinterpret_cast<const Z*>(ip.u), "ip.u");
  B.ph64 = resolve(pars->phases, "phases");
  B.x = dev(reinterpret_cast<Z*>(solution), "solution");
  B.b = dev(reinterpret_cast<const Z*>(in), "in");
  if (!B.u64 || !B.ph64 || !B.x || !B.b) return INVERTER_FAILURE;
  // FP64 parking vectors of the package, else workspace
  B.r64 = ip.loc_r ? dev(reinterpret_cast<Z*>(ip.loc_r), "loc_r") : ws_vec<Z>(WS_VEC0, 0, 3);
  B.t64 = ip.loc_s ? dev(reinterpret_cast<Z*>(ip.loc_s), "loc_s") : ws_vec<Z>(WS_VEC0, 1, 3);
  B.t64b = ip.loc_h ? dev(reinterpret_cast<Z*>(ip.loc_h), "loc_h") : ws_vec<Z>(WS_VEC0, 2, 3);
  // FP32 parking vectors of the package, else workspace
  B.r = ip.loc_r_f ? dev(reinterpret_cast<Zf*>(ip.loc_r_f), "loc_r_f") : ws_vec<Zf>(WS_VEC1, 0, 5);
  B.t = ip.loc_h_f ? dev(reinterpret_cast<Zf*>(ip.loc_h_f), "loc_h_f") : ws_vec<Zf>(WS_VEC1, 1, 5);
  B.s = ip.loc_s_f ? dev(reinterpret_cast<Zf*>(ip.loc_s_f), "loc_s_f") : ws_vec<Zf>(WS_VEC1, 2, 5);
  B.p = ip.loc_p_f ? dev(reinterpret_cast<Zf*>(ip.loc_p_f), "loc_p_f") : ws_vec<Zf>(WS_VEC1, 3, 5);
  B.xf = ip.out_f ? dev(reinterpret_cast<Zf*>(ip.out_f), "out_f") : ws_vec<Zf>(WS_VEC1, 4, 5);
  if (!B.r64 || !B.t64 || !B.t64b || !B.r || !B.t || !B.s || !B.p || !B.xf) return INVERTER_FAILURE;
  PreparedF32 pf;
  if (!prepare_f32(B.u64, ip.u_f, static_cast<const double*>(B.ph64), &pf, st)) return INVERTER_FAILURE;
  B.u32 = pf.u32;
  B.u32_compact = pf.compact;
  B.q16 = pf.q16;
  B.uq = pf.uq;
  B.ph32 = pf.ph;
  B.ph32_mode = pf.mode;
  B.use_df = prepare_df(B.u64, pf, &B.df, &B.dfw, st) ? 1 : 0;
  MixedOptions o;
  o.mass2 = pars->ferm_mass * pars->ferm_mass + shift;
  o.res = res;
  o.safety = 0.9;                      // inverter_mixedp.c:39
  o.max_iter = max_cg;
  o.reliable_every = 0;
  o.delta_frac = inverter_tricks.mixedPrecisionDelta;
  o.guarantee = 0;
  o.chunk = 8;
  MixScal* sc = mix_scalars();
  if (!sc) return INVERTER_FAILURE;
  MixedResult r = mixed_cg(B, o, sc, st);
  *cg_return = r.iters;
  if (r.iters >= max_cg) printf("WARNING: maximum number of iterations reached in invert\n");
  if (error_code()) return INVERTER_FAILURE;
  return r.converged ? INVERTER_SUCCESS : INVERTER_FAILURE;
}

int ostaple_invert_mixed(const su3_soa* u, const double_soa* phases, double mass, double shift, vec3_soa* solution,
                         const vec3_soa* in, double res, int max_iter, int reliable_every, double delta_frac,
                         int* iters, double* true_res, int* n_reliable) {
  if (!require_init("ostaple_invert_mixed")) return INVERTER_FAILURE;
  cudaStream_t st = rt().stream;
  MixedBuffers B{};
  B.u64 = dev(reinterpret_cast<const Z*>(u), "u");
  B.ph64 = resolve(phases, "phases");
  B.x = dev(reinterpret_cast<Z*>(solution), "solution");
  B.b = dev(reinterpret_cast<const Z*>(in), "in");
  if (!B.u64 || !B.ph64 || !B.x || !B.b) return INVERTER_FAILURE;
  B.r64 = ws_vec<Z>(WS_VEC0, 0, 3);
  B.t64 = ws_vec<Z>(WS_VEC0, 1, 3);
  B.t64b = ws_vec<Z>(WS_VEC0, 2, 3);
  B.r = ws_vec<Zf>(WS_VEC1, 0, 5);
  B.t = ws_vec<Zf>(WS_VEC1, 1, 5);
  B.s = ws_vec<Zf>(WS_VEC1, 2, 5);
  B.p = ws_vec<Zf>(WS_VEC1, 3, 5);
  B.xf = ws_vec<Zf>(WS_VEC1, 4, 5);
  if (!B.r64 || !B.t64 || !B.t64b || !B.r || !B.t || !B.s || !B.p || !B.xf) return INVERTER_FAILURE;
  PreparedF32 pf;
  if (!prepare_f32(B.u64, nullptr, static_cast<const double*>(B.ph64), &pf, st)) return INVERTER_FAILURE;
  B.u32 = pf.u32;
  B.u32_compact = pf.compact;
  B.q16 = pf.q16;
  B.uq = pf.uq;
  B.ph32 = pf.ph;
  B.ph32_mode = pf.mode;
  B.use_df = prepare_df(B.u64, pf, &B.df, &B.dfw, st) ? 1 : 0;
  MixedOptions o;
  o.mass2 = mass * mass + shift;
  o.res = res;
  o.safety = 0.9;
  o.max_iter = max_iter;
  o.reliable_every = reliable_every;
  o.delta_frac = delta_frac > 0 ? delta_frac : inverter_tricks.mixedPrecisionDelta;
  o.guarantee = 1;
  o.chunk = 8;
  MixScal* sc = mix_scalars();
  if (!sc) return INVERTER_FAILURE;
  MixedResult r = mixed_cg(B, o, sc, st);
  if (iters) *iters = r.iters;
  if (true_res) *true_res = r.true_res;
  if (n_reliable) *n_reliable = r.n_reliable;
  if (error_code()) return INVERTER_FAILURE;
  return r.converged ? INVERTER_SUCCESS : INVERTER_FAILURE;
}

int ostaple_mdagm_df(const su3_soa* u, const double_soa* phases, double mass, double shift, vec3_soa* out,
                     const vec3_soa* in) {
  if (!require_init("ostaple_mdagm_df")) return -2;
  cudaStream_t st = rt().stream;
  const Z* u64 = dev(reinterpret_cast<const Z*>(u), "u");
  const void* ph = resolve(phases, "phases");
  const Z* din = dev(reinterpret_cast<const Z*>(in), "in");
  Z* dout = dev(reinterpret_cast<Z*>(out), "out");
  if (!u64 || !ph || !din || !dout) return -3;
  PreparedF32 pf;
  if (!prepare_f32(u64, nullptr, static_cast<const double*>(ph), &pf, st)) return -4;
  DfOperator op;
  DfWork w;
  if (!prepare_df(u64, pf, &op, &w, st)) {
    set_error(-12, "ostaple_mdagm_df: phases must be 0 or pi (staggered phases and boundary signs)");
    return -12;
  }
  df_mdagm(op, w, dout, din, mass * mass + shift, st);
  OST_CUDA(cudaStreamSynchronize(st));
  return error_code();
}

// Exits on a failure in a critical region, as the reference does
// (inverter_wrappers.c:24-39).
void convergence_messages(int conv_importance, int inverter_status) {
  if (inverter_status == INVERTER_FAILURE) {
    if (conv_importance == CONVERGENCE_CRITICAL) {
      printf("\n\n\t\tERROR : inverter failed to converge in a critical region of the code. Exiting now!!\n\n");
      exit(1);
    }
    printf("\n\t\tWARNING : inverter failed to converge.\n");
  }
}

int inverter_wrapper(inverter_package ip, ferm_param* pars, vec3_soa* out, const vec3_soa* in, double res,
                     int max_cg, double shift, int convergence_importance) {
  int cg = 0, st;
  if (inverter_tricks.useMixedPrecision)
    st = inverter_mixed_precision(ip, pars, out, in, res, max_cg, shift, &cg);
  else
    st = ker_invert_openacc(ip.u, pars, out, in, res, ip.loc_r, ip.loc_h, ip.loc_s, ip.loc_p, max_cg, shift, &cg);
  convergence_messages(convergence_importance, st);
  return cg;
}

}  // extern "C"

namespace ost {

// Mean duration (ms) of one launch of a hot kernel, timed with CUDA events on
// the stream it is launched on: which = 0: FP64 D_eo (reference layout and
// angle phases, as acc_Deo); 1: FP32 D_oe of the mixed solver; 2: FP32 fused
// D_eo + M^+M epilogue + <p, Ap> of the mixed solver; 3: double-float M^+M.
// Internal: the benchmark library's ostaple_time_kernel calls it.
int time_hot_kernel(int which, const su3_soa* u, const double_soa* phases, int reps, double* ms) {
  if (!require_init("ostaple_time_kernel")) return -2;
  cudaStream_t st = rt().stream;
  const Z* u64 = dev(reinterpret_cast<const Z*>(u), "u");
  const void* ph = resolve(phases, "phases");
  if (!u64 || !ph) return -3;
  Z* a = ws_vec<Z>(WS_VEC0, 0, 3);
  Z* b = ws_vec<Z>(WS_VEC0, 1, 3);
  if (!a || !b) return -5;
  if (which == 0) {
    DslashArgs<double> d;
    d.parity = 0; d.phase_mode = PH_ANGLE; d.epilogue = EPI_PLAIN; d.u = u64; d.out = a; d.in = b;
    d.phases = ph; d.in0 = nullptr; d.mass2 = 0; d.stream = st; d.compact_links = 0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float t = 0;
    for (int pass = 0; pass < 2; ++pass) {
      cudaEventRecord(e0, st);
      for (int k = 0; k < reps; ++k) launch_dslash<double>(d);
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      cudaEventElapsedTime(&t, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = double(t) / reps;
    return error_code();
  }
  if (which == 3) {   // double-float M^+M (split + D_oe + D_eo)
    PreparedF32 pf;
    if (!prepare_f32(u64, nullptr, static_cast<const double*>(ph), &pf, st)) return -4;
    DfOperator op;
    DfWork w;
    if (!prepare_df(u64, pf, &op, &w, st)) return -12;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float t = 0;
    for (int pass = 0; pass < 2; ++pass) {
      cudaEventRecord(e0, st);
      for (int k = 0; k < reps; ++k) df_mdagm(op, w, a, b, 0.01, st);
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      cudaEventElapsedTime(&t, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = double(t) / reps;
    return error_code();
  }
  MixedBuffers B{};
  B.u64 = u64;
  B.ph64 = ph;
  B.r = ws_vec<Zf>(WS_VEC1, 0, 5);
  B.t = ws_vec<Zf>(WS_VEC1, 1, 5);
  B.s = ws_vec<Zf>(WS_VEC1, 2, 5);
  B.p = ws_vec<Zf>(WS_VEC1, 3, 5);
  B.xf = ws_vec<Zf>(WS_VEC1, 4, 5);
  PreparedF32 pf;
  if (!prepare_f32(u64, nullptr, static_cast<const double*>(ph), &pf, st)) return -4;
  B.u32 = pf.u32;
  B.u32_compact = pf.compact;
  B.q16 = pf.q16;
  B.uq = pf.uq;
  B.ph32 = pf.ph;
  B.ph32_mode = pf.mode;
  MixScal* sc = mix_scalars();
  *ms = time_mixed_kernel(B, sc + 1, which, reps, st);
  return error_code();
}

}  // namespace ost
