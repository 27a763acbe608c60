// capi_f32.cu -- the reference's single-precision twins of the hot path.
//
// The reference generates them from the double-precision files
// (double_to_single_transformer.py): the names gain "_f", the SoA types
// become su3_soa_f / vec3_soa_f / float_soa (float complex, the same
// structure-of-arrays layouts with 8-byte elements).  In fermion_matrix.c,
// which the generator converts wholesale, `double` becomes `float` too (so
// fermion_matrix_multiplication_shifted_f takes a float shift); the solver
// and BLAS files keep double scalars (sp_inverter_full.c,
// sp_inverter_multishift_full.c, sp_fermionic_utilities.c).  The reference's
// own benchmark drivers call these (deo_doe_test.c:296-345,
// inverter_multishift_test.c:334-356), together with the float <-> double
// conversions of float_double_conv.c:9-150, which are here as well.
//
// Arithmetic: FP32 links and vectors, FP64 scalars and FP64 accumulation in
// every global reduction.  Phases are the float angles of
// ferm_param.phases_f (exactly 0 or pi take the sign path, as in FP64).
#include <cmath>
#include "dslash.cuh"
#include "kernels.cuh"
#include "runtime.cuh"
#include "solver_kernels.cuh"
#include "solvers_fp.cuh"
#include "../../include/ostaple_gb300.h"

using namespace ost;

namespace {

typedef float2 Zf;
typedef double2 Zd;

inline long vlen() { return 3L * rt().g.sizeh; }
inline cudaStream_t S() { return rt().stream; }

#define DF(p, name) dev(reinterpret_cast<const Zf*>(p), name)
#define DFW(p, name) dev(reinterpret_cast<Zf*>(p), name)

void dslash32(int parity, const su3_soa_f* u, vec3_soa_f* out, const vec3_soa_f* in, const float_soa* bf,
              const char* who) {
  if (!require_init(who)) return;
  const Zf* du = DF(u, "u");
  Zf* o = DFW(out, "out");
  const Zf* i = DF(in, "in");
  const void* ph = resolve(bf, "backfield");
  if (!du || !o || !i || !ph) return;
  fp::dslash<float>(parity, du, o, i, ph, EPI_PLAIN, nullptr, 0.0);
}

__global__ void k_d2f(const double* __restrict__ d, float* f, long n) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x)
    f[i] = float(d[i]);
}
__global__ void k_f2d(const float* __restrict__ f, double* d, long n) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x)
    d[i] = double(f[i]);
}

// element-wise real conversions of n doubles / floats (complex arrays are
// pairs of reals with the same rounding)
void convert(const void* src, void* dst, long nreal, bool to_float, const char* who) {
  if (!require_init(who)) return;
  const void* s = resolve(src, "source");
  void* d = resolve(dst, "destination");
  if (!s || !d) return;
  const long cap = 8L * rt().num_sms;
  const long b = (nreal + 255) / 256;
  const int grid = int(b < cap ? (b < 1 ? 1 : b) : cap);
  if (to_float) k_d2f<<<grid, 256, 0, S()>>>(static_cast<const double*>(s), static_cast<float*>(d), nreal);
  else k_f2d<<<grid, 256, 0, S()>>>(static_cast<const float*>(s), static_cast<double*>(d), nreal);
  OST_LAUNCH_CHECK();
}

}  // namespace

extern "C" {

// ---- Dirac operator (sp_fermion_matrix.c) ----
void acc_Deo_f(const su3_soa_f* u, vec3_soa_f* out, const vec3_soa_f* in, const float_soa* bf) {
  dslash32(0, u, out, in, bf, "acc_Deo_f");
}
void acc_Doe_f(const su3_soa_f* u, vec3_soa_f* out, const vec3_soa_f* in, const float_soa* bf) {
  dslash32(1, u, out, in, bf, "acc_Doe_f");
}
void acc_Deo_unsafe_f(const su3_soa_f* u, vec3_soa_f* out, const vec3_soa_f* in, const float_soa* bf) {
  dslash32(0, u, out, in, bf, "acc_Deo_unsafe_f");
}
void acc_Doe_unsafe_f(const su3_soa_f* u, vec3_soa_f* out, const vec3_soa_f* in, const float_soa* bf) {
  dslash32(1, u, out, in, bf, "acc_Doe_unsafe_f");
}

void fermion_matrix_multiplication_shifted_f(const su3_soa_f* u, vec3_soa_f* out, const vec3_soa_f* in,
                                             vec3_soa_f* temp1, ferm_param* pars, float shift) {
  if (!require_init("fermion_matrix_multiplication_f")) return;
  const Zf* du = DF(u, "u");
  Zf* o = DFW(out, "out");
  const Zf* i = DF(in, "in");
  Zf* t = DFW(temp1, "temp1");
  const void* ph = resolve(pars->phases_f, "phases_f");
  if (!du || !o || !i || !t || !ph) return;
  // temp1 = D_oe in ; out = (m^2 + shift) in - D_eo temp1
  fp::mdagm<float>(du, o, i, t, ph, float(pars->ferm_mass * pars->ferm_mass) + shift);
}

void fermion_matrix_multiplication_f(const su3_soa_f* u, vec3_soa_f* out, const vec3_soa_f* in, vec3_soa_f* temp1,
                                     ferm_param* pars) {
  fermion_matrix_multiplication_shifted_f(u, out, in, temp1, pars, 0.0f);
}

// ---- BLAS and reductions (sp_fermionic_utilities.c) ----
double l2norm2_global_f(const vec3_soa_f* a) {
  if (!require_init("l2norm2_global_f")) return NAN;
  const Zf* da = DF(a, "in_vect1");
  if (!da) return NAN;
  blas_norm2<float>(da, vlen(), fp::dscal(0), S());
  return fp::readback(fp::dscal(0));
}
double real_scal_prod_global_f(const vec3_soa_f* a, const vec3_soa_f* b) {
  if (!require_init("real_scal_prod_global_f")) return NAN;
  const Zf *da = DF(a, "in_vect1"), *db = DF(b, "in_vect2");
  if (!da || !db) return NAN;
  blas_rdot<float>(da, db, vlen(), fp::dscal(0), S());
  return fp::readback(fp::dscal(0));
}
void set_vec3_soa_to_zero_f(vec3_soa_f* f) {
  if (!require_init("set_vec3_soa_to_zero_f")) return;
  Zf* a = DFW(f, "fermion");
  if (a) blas_zero<float>(a, vlen(), S());
}
void assign_in_to_out_f(const vec3_soa_f* in1, vec3_soa_f* out) {
  if (!require_init("assign_in_to_out_f")) return;
  const Zf* a = DF(in1, "in");
  Zf* o = DFW(out, "out");
  if (a && o) blas_copy<float>(a, o, vlen(), S());
}
void combine_in1xfactor_plus_in2_f(const vec3_soa_f* in1, const double factor, const vec3_soa_f* in2,
                                   vec3_soa_f* out) {
  if (!require_init("combine_in1xfactor_plus_in2_f")) return;
  const Zf *a = DF(in1, "in1"), *b = DF(in2, "in2");
  Zf* o = DFW(out, "out");
  if (a && b && o) blas_axpy<float>(a, factor, b, o, vlen(), S());
}
void combine_add_factor_x_in2_to_in1_f(vec3_soa_f* in1, const vec3_soa_f* in2, double factor) {
  if (!require_init("combine_add_factor_x_in2_to_in1_f")) return;
  Zf* a = DFW(in1, "in1");
  const Zf* b = DF(in2, "in2");
  if (a && b) blas_axpy<float>(b, factor, a, a, vlen(), S());
}
void combine_in1xferm_mass_minus_in2_f(const vec3_soa_f* in1, double m2, vec3_soa_f* in2) {
  if (!require_init("combine_in1xferm_mass_minus_in2_f")) return;
  const Zf* a = DF(in1, "in1");
  Zf* b = DFW(in2, "in2");
  if (a && b) blas_axmy<float>(a, m2, b, b, vlen(), S());
}
void combine_in1_minus_in2_f(const vec3_soa_f* in1, const vec3_soa_f* in2, vec3_soa_f* out) {
  if (!require_init("combine_in1_minus_in2_f")) return;
  const Zf *a = DF(in1, "in1"), *b = DF(in2, "in2");
  Zf* o = DFW(out, "out");
  if (a && b && o) blas_axmy<float>(a, 1.0, b, o, vlen(), S());
}
void multiply_fermion_x_doublefactor_f(vec3_soa_f* in1, const double factor) {
  if (!require_init("multiply_fermion_x_doublefactor_f")) return;
  Zf* a = DFW(in1, "in1");
  if (a) blas_scale<float>(a, factor, vlen(), S());
}

// ---- solvers (sp_inverter_full.c, sp_inverter_multishift_full.c) ----
int ker_invert_openacc_f(const su3_soa_f* u, ferm_param* pars, vec3_soa_f* solution, const vec3_soa_f* in,
                         double res, vec3_soa_f* loc_r, vec3_soa_f* loc_h, vec3_soa_f* loc_s, vec3_soa_f* loc_p,
                         const int max_cg, double shift, int* cg_return) {
  if (!require_init("ker_invert_openacc_f")) return INVERTER_FAILURE;
  const Zf* du = DF(u, "u");
  Zf* x = DFW(solution, "solution");
  const Zf* b = DF(in, "in");
  Zf *r = DFW(loc_r, "loc_r"), *h = DFW(loc_h, "loc_h"), *s = DFW(loc_s, "loc_s"), *p = DFW(loc_p, "loc_p");
  const void* ph = resolve(pars->phases_f, "phases_f");
  if (!du || !x || !b || !r || !h || !s || !p || !ph) return INVERTER_FAILURE;
  return fp::cg<float>(du, ph, pars->ferm_mass, x, b, res, r, h, s, p, max_cg, shift,
                       inverter_tricks.restartingEvery, cg_return);
}

int multishift_invert_f(const su3_soa_f* u, ferm_param* pars, RationalApprox* approx, vec3_soa_f* out,
                        const vec3_soa_f* in, double residuo, vec3_soa_f* loc_r, vec3_soa_f* loc_h,
                        vec3_soa_f* loc_s, vec3_soa_f* loc_p, vec3_soa_f* shiftferm, const int max_cg,
                        int* cg_return) {
  if (!require_init("multishift_invert_f")) return INVERTER_FAILURE;
  const int order = approx->approx_order;
  if (order < 1 || order > OST_MAX_SHIFTS) {
    set_error(-11, "multishift_invert_f: approx_order %d outside [1,%d]", order, OST_MAX_SHIFTS);
    return INVERTER_FAILURE;
  }
  const Zf* du = DF(u, "u");
  Zf* xs = DFW(out, "out");
  const Zf* b = DF(in, "in");
  Zf *r = DFW(loc_r, "loc_r"), *h = DFW(loc_h, "loc_h"), *s = DFW(loc_s, "loc_s"), *p = DFW(loc_p, "loc_p");
  Zf* ps = DFW(shiftferm, "shiftferm");
  const void* ph = resolve(pars->phases_f, "phases_f");
  if (!du || !xs || !b || !r || !h || !s || !p || !ps || !ph) return INVERTER_FAILURE;
  return fp::cgm<float>(du, ph, pars->ferm_mass, approx->RA_b, order, xs, b, residuo, r, h, s, p, ps, max_cg,
                        cg_return);
}

void recombine_shifted_vec3_to_vec3_f(const vec3_soa_f* in_shifted, const vec3_soa_f* in, vec3_soa_f* out,
                                      const RationalApprox* approx) {
  if (!require_init("recombine_shifted_vec3_to_vec3_f")) return;
  const Zf* xs = DF(in_shifted, "in_shifted");
  const Zf* b = DF(in, "in");
  Zf* o = DFW(out, "out");
  if (!xs || !b || !o) return;
  RecombCoeffs rc;
  rc.order = approx->approx_order;
  rc.a0 = approx->RA_a0;
  for (int k = 0; k < rc.order && k < OST_MAX_SHIFTS; ++k) rc.a[k] = approx->RA_a[k];
  recombine<float>(xs, vlen(), b, o, rc, vlen(), S());
}

// ---- float <-> double conversions (float_double_conv.c:9-150) ----
void convert_double_to_float_vec3_soa(const vec3_soa* d, vec3_soa_f* f) {
  convert(d, f, 2 * vlen(), true, "convert_double_to_float_vec3_soa");
}
void convert_float_to_double_vec3_soa(const vec3_soa_f* f, vec3_soa* d) {
  convert(f, d, 2 * vlen(), false, "convert_float_to_double_vec3_soa");
}
void convert_double_to_float_real_soa(const double_soa* d, float_soa* f) {
  convert(d, f, rt().g.sizeh, true, "convert_double_to_float_real_soa");
}
void convert_float_to_double_real_soa(const float_soa* f, double_soa* d) {
  convert(f, d, rt().g.sizeh, false, "convert_float_to_double_real_soa");
}
// all 8 link directions, 3 rows each
void convert_double_to_float_su3_soa(const su3_soa* d, su3_soa_f* f) {
  convert(d, f, 8L * 2 * 9 * rt().g.sizeh, true, "convert_double_to_float_su3_soa");
}
void convert_float_to_double_su3_soa(const su3_soa_f* f, su3_soa* d) {
  convert(f, d, 8L * 2 * 9 * rt().g.sizeh, false, "convert_float_to_double_su3_soa");
}

}  // extern "C"
