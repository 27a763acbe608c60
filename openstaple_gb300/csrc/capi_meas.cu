// capi_meas.cu -- the full-D inversion of the fermionic measurements
// (Meas/ferm_meas.c:50-71): the chiral condensate, quark number and
// susceptibility estimators of the reference call it once per noise vector.
//
// D = [[m, D_eo], [D_oe, m]] on (even, odd) is inverted through its even
// Schur complement m^2 - D_eo D_oe = M^+M, so the solve itself is the
// library's single-shift solver chosen by inverter_wrapper (FP64 CG or the
// mixed-precision CG, by inverter_tricks.useMixedPrecision); the rest is two
// hops and two vector combinations on the device.
#include "runtime.cuh"
#include "../../include/ostaple_gb300.h"

extern "C" {

void eo_inversion(inverter_package ip, ferm_param* fp, double res, int max_cg, vec3_soa* in_e, vec3_soa* in_o,
                  vec3_soa* out_e, vec3_soa* out_o, vec3_soa* phi_e, vec3_soa* phi_o) {
  if (!ost::require_init("eo_inversion")) return;
  if (!fp || fp->ferm_mass == 0.0) {
    ost::set_error(-3, "eo_inversion: the even/odd reduction needs a nonzero mass");
    return;
  }
  // phi_e = m in_e - D_eo in_o
  acc_Deo(ip.u, phi_e, in_o, fp->phases);
  combine_in1_x_fact1_minus_in2_back_into_in2(in_e, fp->ferm_mass, phi_e);
  // out_e = (m^2 - D_eo D_oe)^-1 phi_e
  set_vec3_soa_to_zero(out_e);
  inverter_wrapper(ip, fp, out_e, phi_e, res, max_cg, 0.0, CONVERGENCE_CRITICAL);
  // out_o = (in_o - D_oe out_e) / m
  acc_Doe(ip.u, phi_o, out_e, fp->phases);
  combine_in1_minus_in2_allxfact(in_o, phi_o, 1.0 / fp->ferm_mass, out_o);
}

}  // extern "C"
