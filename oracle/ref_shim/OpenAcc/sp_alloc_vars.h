/* Build shim: the single-precision globals the reference's DP force file
 * names (src/OpenAcc/fermion_force.c:214).  Oracle build infrastructure only. */
#ifndef SP_ALLOC_VARS_H_
#define SP_ALLOC_VARS_H_
#include "sp_struct_c_def.h"
extern su3_soa_f *conf_acc_f;
extern vec3_soa_f *ferm_shiftmulti_acc_f;
extern vec3_soa_f *aux1_f;
#endif
