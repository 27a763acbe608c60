/* abi_layout.c -- prints the size and field offsets of the plain structs
 * that cross the C ABI (RationalApprox, ferm_param, inv_tricks,
 * inverter_package, action_param, md_param) and the element sizes of the SoA types.
 *
 * Built twice by tests/test_abi_reference.py:
 *   -DWITH_REFERENCE_HEADERS: with the reference's own headers
 *      (struct_c_def.h, fermion_parameters.h, inverter_package.h, action.h,
 *      rationalapprox.h, inverter_tricks.h, md_parameters.h and the hot-path
 *      and gauge-HMC function headers)
 *      included BEFORE ostaple_gb300.h with OSTAPLE_HAVE_REFERENCE_TYPES, so
 *      the compiler also checks that every prototype the library declares is
 *      compatible with the reference's declaration of the same function;
 *   without it: with ostaple_gb300.h alone.
 * Both outputs must be identical. */
#include <stddef.h>
#include <stdio.h>

#ifdef WITH_REFERENCE_HEADERS
#include "struct_c_def.h"
#include "sp_struct_c_def.h"
#include "../Include/fermion_parameters.h"
#include "../Include/inverter_tricks.h"
#include "../RationalApprox/rationalapprox.h"
#include "action.h"
#include "inverter_package.h"
#include "fermion_matrix.h"
#include "fermionic_utilities.h"
#include "inverter_full.h"
#include "inverter_multishift_full.h"
#include "inverter_wrappers.h"
#include "stouting.h"
#include "fermion_force.h"
#include "fermion_force_utilities.h"
#include "find_min_max.h"
#include "float_double_conv.h"
#include "ipdot_gauge.h"
#include "plaquettes.h"
#include "rectangles.h"
#include "su3_utilities.h"
#include "su3_measurements.h"
#include "md_parameters.h"
#include "md_integrator.h"
#include "random_assignement.h"
#include "io.h"
#include "../Include/setting_file_parser.h"
#define OSTAPLE_HAVE_REFERENCE_TYPES
#endif
#include "ostaple_gb300.h"

#define F(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))

int main(void)
{
  printf("RationalApprox %zu\n", sizeof(RationalApprox));
  F(RationalApprox, exponent_num); F(RationalApprox, approx_order); F(RationalApprox, lambda_min);
  F(RationalApprox, gmp_remez_precision); F(RationalApprox, error); F(RationalApprox, RA_a0);
  F(RationalApprox, RA_a); F(RationalApprox, RA_b);
  printf("ferm_param %zu\n", sizeof(ferm_param));
  F(ferm_param, ferm_mass); F(ferm_param, degeneracy); F(ferm_param, number_of_ps); F(ferm_param, name);
  F(ferm_param, ferm_charge); F(ferm_param, ferm_im_chem_pot); F(ferm_param, index_of_the_first_ps);
  F(ferm_param, index_of_the_first_shift); F(ferm_param, phases); F(ferm_param, mag_re); F(ferm_param, mag_im);
  F(ferm_param, printed_bf_dbg_info); F(ferm_param, phases_f); F(ferm_param, approx_fi_mother);
  F(ferm_param, approx_md_mother); F(ferm_param, approx_li_mother); F(ferm_param, approx_fi);
  F(ferm_param, approx_md); F(ferm_param, approx_li);
  printf("inv_tricks %zu\n", sizeof(inv_tricks));
  F(inv_tricks, singlePInvAccelMultiInv); F(inv_tricks, useMixedPrecision); F(inv_tricks, mixedPrecisionDelta);
  F(inv_tricks, restartingEvery);
  printf("inverter_package %zu\n", sizeof(inverter_package));
  F(inverter_package, u); F(inverter_package, u_f); F(inverter_package, ferm_shift_temp);
  F(inverter_package, ferm_shift_temp_f); F(inverter_package, nshifts); F(inverter_package, loc_r);
  F(inverter_package, loc_p); F(inverter_package, loc_r_f); F(inverter_package, loc_p_f); F(inverter_package, out_f);
  printf("md_param %zu\n", sizeof(md_param));
  F(md_param, no_md); F(md_param, gauge_scale); F(md_param, t); F(md_param, residue_metro);
  F(md_param, expected_max_eigenvalue); F(md_param, singlePrecMD); F(md_param, residue_md);
  F(md_param, max_cg_iterations); F(md_param, recycleInvsForce); F(md_param, extrapolateInvsForce);
  printf("action_param %zu\n", sizeof(action_param));
  F(action_param, beta); F(action_param, stout_steps); F(action_param, stout_rho); F(action_param, topo_action);
  F(action_param, barrier); F(action_param, width); F(action_param, topo_file_path);
  F(action_param, topo_stout_steps); F(action_param, topo_rho);
#ifdef WITH_REFERENCE_HEADERS
  /* the SoA types: per-site element sizes the library's kernels assume */
  printf("vec3_soa_per_site %zu\n", sizeof(vec3_soa) / LNH_SIZEH);
  printf("su3_soa_per_site %zu\n", sizeof(su3_soa) / LNH_SIZEH);
  printf("double_soa_per_site %zu\n", sizeof(double_soa) / LNH_SIZEH);
  printf("tamat_soa_per_site %zu\n", sizeof(tamat_soa) / LNH_SIZEH);
  printf("thmat_soa_per_site %zu\n", sizeof(thmat_soa) / LNH_SIZEH);
  printf("vec3_soa_f_per_site %zu\n", sizeof(vec3_soa_f) / LNH_SIZEH);
  printf("su3_soa_f_per_site %zu\n", sizeof(su3_soa_f) / LNH_SIZEH);
  printf("float_soa_per_site %zu\n", sizeof(float_soa) / LNH_SIZEH);
#else
  printf("vec3_soa_per_site %d\n", 48);   /* 3 complex double      */
  printf("su3_soa_per_site %d\n", 144);   /* 3 rows of vec3_soa    */
  printf("double_soa_per_site %d\n", 8);
  printf("tamat_soa_per_site %d\n", 64);  /* 3 complex + 2 double  */
  printf("thmat_soa_per_site %d\n", 64);
  printf("vec3_soa_f_per_site %d\n", 24); /* 3 complex float       */
  printf("su3_soa_f_per_site %d\n", 72);
  printf("float_soa_per_site %d\n", 4);
#endif
  return 0;
}
