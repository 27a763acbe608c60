/* Build shim for compiling the reference's double-precision sources with gcc.
 * The reference generates its single-precision headers with a Python-2 script
 * (src/double_to_single_transformer.py) that cannot run here.  The DP files
 * on the fermion hot path only need the float type NAMES to exist (they
 * appear in inverter_package and a few prototypes), so this header declares
 * float twins of the reference's SoA types (src/OpenAcc/struct_c_def.h:16-58).
 * Oracle build infrastructure only. */
#ifndef SP_STRUCT_C_DEF_H_
#define SP_STRUCT_C_DEF_H_
#include "struct_c_def.h"
#include <complex.h>
typedef float complex f_complex;
typedef struct vec3_soa_f_t { f_complex c0[sizeh]; f_complex c1[sizeh]; f_complex c2[sizeh]; } vec3_soa_f;
typedef struct vec3_f_t { f_complex c0; f_complex c1; f_complex c2; } vec3_f;
typedef struct fcomplex_soa_t { f_complex c[sizeh]; } fcomplex_soa;
typedef struct float_soa_t { float d[sizeh]; } float_soa;
typedef struct su3_soa_f_t { vec3_soa_f r0; vec3_soa_f r1; vec3_soa_f r2; } su3_soa_f;
typedef struct tamat_soa_f_t { f_complex c01[sizeh]; f_complex c02[sizeh]; f_complex c12[sizeh]; float ic00[sizeh]; float ic11[sizeh]; } tamat_soa_f;
typedef struct thmat_soa_f_t { f_complex c01[sizeh]; f_complex c02[sizeh]; f_complex c12[sizeh]; float rc00[sizeh]; float rc11[sizeh]; } thmat_soa_f;
#endif
