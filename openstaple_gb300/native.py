"""ctypes binding of the in-tree CUDA library ``libostaple_gb300.so``.

The library is the product: every hot-path call below goes to a hand-written
sm_103a kernel.  There is no fallback: if the shared library is missing or
cannot be loaded, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libostaple_gb300.so"
BENCH_LIB_PATH = Path(__file__).resolve().parent / "libostaple_gb300_bench.so"
MAX_APPROX_ORDER = 25  # rationalapprox.h:8
INVERTER_SUCCESS = 1
INVERTER_FAILURE = 0


class RationalApprox(C.Structure):
    """Layout of the reference's RationalApprox (rationalapprox.h:15-26)."""
    _fields_ = [
        ("exponent_num", C.c_int),
        ("exponent_den", C.c_int),
        ("approx_order", C.c_int),
        ("lambda_min", C.c_double),
        ("lambda_max", C.c_double),
        ("gmp_remez_precision", C.c_int),
        ("error", C.c_double),
        ("RA_a0", C.c_double),
        ("RA_a", C.c_double * MAX_APPROX_ORDER),
        ("RA_b", C.c_double * MAX_APPROX_ORDER),
    ]


class FermParam(C.Structure):
    """Layout of the reference's ferm_param (Include/fermion_parameters.h:9-41)."""
    _fields_ = [
        ("ferm_mass", C.c_double),
        ("degeneracy", C.c_int),
        ("number_of_ps", C.c_int),
        ("name", C.c_char * 30),
        ("ferm_charge", C.c_double),
        ("ferm_im_chem_pot", C.c_double),
        ("index_of_the_first_ps", C.c_int),
        ("index_of_the_first_shift", C.c_int),
        ("phases", C.c_void_p),
        ("mag_re", C.c_void_p),
        ("mag_im", C.c_void_p),
        ("printed_bf_dbg_info", C.c_int),
        ("phases_f", C.c_void_p),
        ("approx_fi_mother", RationalApprox),
        ("approx_md_mother", RationalApprox),
        ("approx_li_mother", RationalApprox),
        ("approx_fi", RationalApprox),
        ("approx_md", RationalApprox),
        ("approx_li", RationalApprox),
    ]


class InvTricks(C.Structure):
    """Layout of the reference's inv_tricks (Include/inverter_tricks.h:4-11)."""
    _fields_ = [
        ("singlePInvAccelMultiInv", C.c_int),
        ("useMixedPrecision", C.c_int),
        ("mixedPrecisionDelta", C.c_double),
        ("restartingEvery", C.c_int),
    ]


class InverterPackage(C.Structure):
    """Layout of the reference's inverter_package (OpenAcc/inverter_package.h:13-31)."""
    _fields_ = [
        ("u", C.c_void_p), ("u_f", C.c_void_p),
        ("ferm_shift_temp", C.c_void_p), ("ferm_shift_temp_f", C.c_void_p),
        ("nshifts", C.c_int),
        ("loc_r", C.c_void_p), ("loc_h", C.c_void_p), ("loc_s", C.c_void_p), ("loc_p", C.c_void_p),
        ("loc_r_f", C.c_void_p), ("loc_h_f", C.c_void_p), ("loc_s_f", C.c_void_p), ("loc_p_f", C.c_void_p),
        ("out_f", C.c_void_p),
    ]


_P = C.c_void_p
_D = C.c_double
_I = C.c_int

# name -> (restype, argtypes)
SIGNATURES = {
    "ostaple_init": (_I, [_I, _I, _I, _I]),
    "ostaple_finalize": (_I, []),
    "ostaple_sizeh": (_I, []),
    "ostaple_set_stream": (_I, [_P]),
    "ostaple_synchronize": (_I, []),
    "ostaple_get_error": (_I, []),
    "ostaple_last_error": (C.c_char_p, []),
    "ostaple_clear_error": (None, []),
    "ostaple_enter_data": (_I, [_P, C.c_size_t]),
    "ostaple_exit_data": (_I, [_P]),
    "ostaple_update_device": (_I, [_P, C.c_size_t]),
    "ostaple_update_host": (_I, [_P, C.c_size_t]),
    "ostaple_deviceptr": (_P, [_P]),
    "ostaple_kernel_launches": (C.c_ulonglong, []),
    "ostaple_pin_host": (_I, [_P, C.c_size_t]),
    "ostaple_unpin_host": (_I, [_P]),
    "ostaple_autotune": (_I, [_I]),
    "ostaple_autotune_report": (_I, [C.c_char_p, _I]),
    "acc_Deo": (None, [_P, _P, _P, _P]),
    "acc_Doe": (None, [_P, _P, _P, _P]),
    "acc_Deo_unsafe": (None, [_P, _P, _P, _P]),
    "acc_Doe_unsafe": (None, [_P, _P, _P, _P]),
    "fermion_matrix_multiplication": (None, [_P, _P, _P, _P, C.POINTER(FermParam)]),
    "fermion_matrix_multiplication_shifted": (None, [_P, _P, _P, _P, C.POINTER(FermParam), _D]),
    "scal_prod_global_ri": (None, [_P, _P, C.POINTER(_D)]),
    "real_scal_prod_global": (_D, [_P, _P]),
    "l2norm2_global": (_D, [_P]),
    "ostaple_mdagm_df": (_I, [_P, _P, _D, _D, _P, _P]),
    "ostaple_set_sloppy_links": (_I, [_I]),
    "ostaple_q16_encode_host": (_I, [_P, C.c_long, _P]),
    "ostaple_df_split_host": (_I, [_P, C.c_long, _P, _P]),
    "ostaple_mdagm_sloppy": (_I, [_P, _P, _D, _D, _P, _P]),
    "ostaple_net_weights_save": (_I, [C.c_char_p, _P]),
    "ostaple_net_weights_load": (_I, [C.c_char_p, _P]),
    "ostaple_selftest_bounded_wait": (_I, [_I]),
    "ostaple_real_scal_prod_global_noalloc": (_D, [_P, _P]),
    "combine_in1xfactor_plus_in2": (None, [_P, _D, _P, _P]),
    "multiply_fermion_x_doublefactor": (None, [_P, _D]),
    "combine_add_factor_x_in2_to_in1": (None, [_P, _P, _D]),
    "combine_in1xferm_mass2_minus_in2_minus_in3": (None, [_P, _D, _P, _P, _P]),
    "combine_inside_loop": (None, [_P, _P, _P, _P, _D]),
    "combine_in1xferm_mass_minus_in2": (None, [_P, _D, _P]),
    "combine_in1_minus_in2": (None, [_P, _P, _P]),
    "assign_in_to_out": (None, [_P, _P]),
    "set_vec3_soa_to_zero": (None, [_P]),
    "multiple_combine_in1_minus_in2x_factor_back_into_in1": (None, [_P, _P, _I, C.POINTER(_I), C.POINTER(_D)]),
    "multiple1_combine_in1_x_fact1_plus_in2_x_fact2_back_into_in1":
        (None, [_P, _I, C.POINTER(_I), C.POINTER(_D), _P, C.POINTER(_D)]),
    "combine_in1_x_fact1_minus_in2_back_into_in2": (None, [_P, _D, _P]),
    "combine_in1_minus_in2_allxfact": (None, [_P, _P, _D, _P]),
    "ker_invert_openacc": (_I, [_P, C.POINTER(FermParam), _P, _P, _D, _P, _P, _P, _P, _I, _D, C.POINTER(_I)]),
    "multishift_invert": (_I, [_P, C.POINTER(FermParam), C.POINTER(RationalApprox), _P, _P, _D, _P, _P, _P, _P,
                               _P, _I, C.POINTER(_I)]),
    "recombine_shifted_vec3_to_vec3": (None, [_P, _P, _P, C.POINTER(RationalApprox)]),
    "ker_find_max_eigenvalue_openacc": (_D, [_P, C.POINTER(FermParam), _P, _P, _P]),
    "rational_approx_filename": (C.c_void_p, [_D, _I, _I, _D]),
    "rational_approx_filename_old": (C.c_void_p, [_I, _I, _I, _D]),
    "rationalapprox_read": (_I, [C.POINTER(RationalApprox)]),
    "rationalapprox_read_custom_nomefile": (_I, [C.POINTER(RationalApprox), C.c_char_p]),
    "rationalapprox_save": (None, [C.c_char_p, C.POINTER(RationalApprox)]),
    "rescale_rational_approximation": (None, [C.POINTER(RationalApprox), C.POINTER(RationalApprox), _P]),
    "renormalize_rational_approximation": (None, [C.POINTER(RationalApprox), C.POINTER(RationalApprox)]),
    "rational_approx_evaluate": (_D, [C.POINTER(RationalApprox), _D]),
    "ostaple_remez_approximation": (_I, [C.POINTER(RationalApprox)]),
    "ostaple_remez_generate": (_I, [C.POINTER(RationalApprox), _D, _I]),
    "ker_find_min_eigenvalue_openacc": (_D, [_P, C.POINTER(FermParam), _P, _P, _P, _D]),
    "find_min_max_eigenvalue_soloopenacc": (None, [_P, C.POINTER(FermParam), _P, _P, _P, _P, _P]),
    "inverter_mixed_precision": (_I, [InverterPackage, C.POINTER(FermParam), _P, _P, _D, _I, _D, C.POINTER(_I)]),
    "inverter_wrapper": (_I, [InverterPackage, C.POINTER(FermParam), _P, _P, _D, _I, _D, _I]),
    "eo_inversion": (None, [InverterPackage, C.POINTER(FermParam), _D, _I, _P, _P, _P, _P, _P, _P]),
    "ostaple_gaussian_vec3": (_I, [_P, C.c_ulonglong, C.c_ulonglong]),
    "ostaple_device_loop": (_I, [_I]),
    "convergence_messages": (None, [_I, _I]),
    "ostaple_invert_mixed": (_I, [_P, _P, _D, _D, _P, _P, _D, _I, _I, _D, C.POINTER(_I), C.POINTER(_D),
                                  C.POINTER(_I)]),
    "ostaple_invert_mixed_batch": (_I, [_P, _P, _D, _I, _P, _P, _P, _D, _I, _D, _P, _P, _P]),
    "ostaple_multishift_batch": (_I, [_P, _P, _D, C.POINTER(RationalApprox), _I, _P, _P, _D, _I, _D, _P, _P, _P]),
    "ostaple_net_init": (_I, [C.c_uint, _D]),
    "ostaple_net_set_weights": (_I, [_P]),
    "ostaple_net_get_weights": (_I, [_P]),
    "ostaple_net_apply": (_I, [_P, _P, _P, _P]),
    "ostaple_net_gradient": (_I, [_P, _P, _D, _D, _P, _P, _P, C.POINTER(_D)]),
    "ostaple_net_train": (_I, [_P, _P, _D, _D, _I, _P, _P, _I, _D, _P]),
    "ostaple_invert_learned": (_I, [_P, _P, _D, _D, _P, _P, _D, _I, C.POINTER(_I), C.POINTER(_D), C.POINTER(_I)]),
    "stout_isotropic": (None, [_P, _P, _P, _P, _P, _I]),
    "stout_wrapper": (None, [_P, _P, _I]),
    "exp_minus_QA_times_conf": (None, [_P, _P, _P, _P]),
    "compute_lambda": (None, [_P, _P, _P, _P, _P]),
    "compute_sigma": (None, [_P, _P, _P, _P, _P, _I]),
    "compute_sigma_from_sigma_prime_backinto_sigma_prime": (None, [_P, _P, _P, _P, _P, _I]),
    "set_su3_soa_to_zero": (None, [_P]),
    "set_tamat_soa_to_zero": (None, [_P]),
    "direct_product_of_fermions_into_auxmat": (None, [_P, _P, _P, C.POINTER(RationalApprox), _I]),
    "ker_openacc_compute_fermion_force": (None, [_P, _P, _P, _P, _P, C.POINTER(FermParam)]),
    "multiply_backfield_times_force": (None, [C.POINTER(FermParam), _P, _P]),
    "multiply_conf_times_force_and_take_ta_nophase": (None, [_P, _P, _P]),
    "fermion_force_soloopenacc": (None, [_P, _P, _P, _P, C.POINTER(FermParam), _I, _P, _D, _P, _P,
                                         InverterPackage, _I]),
    "inverter_multishift_wrapper": (_I, [InverterPackage, C.POINTER(FermParam), C.POINTER(RationalApprox), _P, _P,
                                         _D, _I, _I]),
    # pure-gauge tree-level Symanzik HMC
    "calc_loc_staples_nnptrick_all": (None, [_P, _P]),
    "calc_loc_improved_staples_typeA_nnptrick_all": (None, [_P, _P]),
    "calc_loc_improved_staples_typeB_nnptrick_all": (None, [_P, _P]),
    "calc_loc_improved_staples_typeC_nnptrick_all": (None, [_P, _P]),
    "conf_times_staples_ta_part": (None, [_P, _P, _P]),
    "calc_ipdot_gauge_soloopenacc": (None, [_P, _P, _P]),
    "calc_plaquette_soloopenacc": (_D, [_P, _P, _P]),
    "calc_rettangolo_soloopenacc": (_D, [_P, _P, _P]),
    "calc_momenta_action": (_D, [_P, _P, _I]),
    "mom_sum_mult": (None, [_P, _P, C.POINTER(_D), _I]),
    "mom_exp_times_conf_soloopenacc": (None, [_P, _P, C.POINTER(_D), _I]),
    "multistep_2MN_gauge": (None, [_P, _P, _P, _P]),
    "generate_Momenta_gauss": (None, [_P]),
    "ostaple_set_momenta_seed": (None, [C.c_ulonglong]),
    "ostaple_pure_gauge_hmc": (_I, [_P, _D, _I, _I, _I, _D, C.c_ulonglong, _I, _I, _I, C.POINTER(_I), _P, _P]),
    "ostaple_gauge_momenta": (_I, [_P, C.c_ulonglong, C.c_ulonglong]),
    "ostaple_gauge_action": (_I, [_P, _D, C.POINTER(_D), C.POINTER(_D), C.POINTER(_D)]),
    "multistep_2MN_SOLOOPENACC": (None, [_P, _P, _P, _P, _P, C.POINTER(FermParam), _I, _P, _P, InverterPackage, _P, _P,
                                         _D, _I]),
    "ostaple_rhmc_trajectory": (_I, [_P, C.POINTER(FermParam), _I, _D, _I, _I, _D, _D, _D, _I, C.c_ulonglong, _I,
                                     _I, C.POINTER(_I), C.POINTER(_D), _P]),
    # configuration files
    "print_su3_soa_ASCII": (_I, [_P, C.c_char_p, _I, _P]),
    "read_su3_soa_ASCII": (_I, [_P, C.c_char_p, C.POINTER(_I)]),
    "print_su3_soa_ildg_binary": (_I, [_P, C.c_char_p, _I]),
    "read_su3_soa_ildg_binary": (_I, [_P, C.c_char_p, C.POINTER(_I)]),
    # single-precision twins (sp_*.c) and float <-> double conversions
    "acc_Deo_f": (None, [_P, _P, _P, _P]),
    "acc_Doe_f": (None, [_P, _P, _P, _P]),
    "acc_Deo_unsafe_f": (None, [_P, _P, _P, _P]),
    "acc_Doe_unsafe_f": (None, [_P, _P, _P, _P]),
    "fermion_matrix_multiplication_f": (None, [_P, _P, _P, _P, C.POINTER(FermParam)]),
    "fermion_matrix_multiplication_shifted_f": (None, [_P, _P, _P, _P, C.POINTER(FermParam), C.c_float]),
    "l2norm2_global_f": (_D, [_P]),
    "real_scal_prod_global_f": (_D, [_P, _P]),
    "set_vec3_soa_to_zero_f": (None, [_P]),
    "assign_in_to_out_f": (None, [_P, _P]),
    "combine_in1xfactor_plus_in2_f": (None, [_P, _D, _P, _P]),
    "combine_add_factor_x_in2_to_in1_f": (None, [_P, _P, _D]),
    "combine_in1xferm_mass_minus_in2_f": (None, [_P, _D, _P]),
    "combine_in1_minus_in2_f": (None, [_P, _P, _P]),
    "multiply_fermion_x_doublefactor_f": (None, [_P, _D]),
    "ker_invert_openacc_f": (_I, [_P, C.POINTER(FermParam), _P, _P, _D, _P, _P, _P, _P, _I, _D, C.POINTER(_I)]),
    "multishift_invert_f": (_I, [_P, C.POINTER(FermParam), C.POINTER(RationalApprox), _P, _P, _D, _P, _P, _P, _P,
                                 _P, _I, C.POINTER(_I)]),
    "recombine_shifted_vec3_to_vec3_f": (None, [_P, _P, _P, C.POINTER(RationalApprox)]),
    "convert_double_to_float_vec3_soa": (None, [_P, _P]),
    "convert_float_to_double_vec3_soa": (None, [_P, _P]),
    "convert_double_to_float_real_soa": (None, [_P, _P]),
    "convert_float_to_double_real_soa": (None, [_P, _P]),
    "convert_double_to_float_su3_soa": (None, [_P, _P]),
    "convert_float_to_double_su3_soa": (None, [_P, _P]),
}

_lib = None


def lib() -> C.CDLL:
    """Loads the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(LIB_PATH), mode=C.RTLD_LOCAL)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        L.initialize_md_global_variables.restype = None
        L.initialize_md_global_variables.argtypes = [MdParam]
        _lib = L
    return _lib


_bench_lib = None


def bench_lib() -> C.CDLL:
    """Loads the benchmark's measurement library (kernel timing, FMA probe)."""
    global _bench_lib
    if _bench_lib is None:
        lib()
        if not BENCH_LIB_PATH.exists():
            raise RuntimeError(f"{BENCH_LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; "
                               "g.build()'`")
        L = C.CDLL(str(BENCH_LIB_PATH), mode=C.RTLD_LOCAL)
        L.ostaple_probe_fma_tflops.restype = C.c_int
        L.ostaple_probe_fma_tflops.argtypes = [C.c_int, C.POINTER(C.c_double)]
        L.ostaple_time_kernel.restype = C.c_int
        L.ostaple_time_kernel.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_double)]
        _bench_lib = L
    return _bench_lib


class MdParam(C.Structure):
    """Layout of the reference's md_param (OpenAcc/md_parameters.h:7-20)."""
    _fields_ = [
        ("no_md", C.c_int), ("gauge_scale", C.c_int), ("t", C.c_double), ("residue_metro", C.c_double),
        ("expected_max_eigenvalue", C.c_double), ("singlePrecMD", C.c_int), ("residue_md", C.c_double),
        ("max_cg_iterations", C.c_int), ("recycleInvsForce", C.c_int), ("extrapolateInvsForce", C.c_int),
    ]


def md_parameters() -> "MdParam":
    """The library's `md_parameters` global (writable)."""
    return MdParam.in_dll(lib(), "md_parameters")


def deltas_omelyan():
    """The library's `deltas_Omelyan[7]` global."""
    return (C.c_double * 7).in_dll(lib(), "deltas_Omelyan")


class ActionParam(C.Structure):
    """Layout of the reference's action_param (OpenAcc/action.h:8-20)."""
    _fields_ = [
        ("beta", C.c_double), ("stout_steps", C.c_int), ("stout_rho", C.c_double), ("topo_action", C.c_int),
        ("barrier", C.c_double), ("width", C.c_double), ("topo_file_path", C.c_char * 20),
        ("topo_stout_steps", C.c_int), ("topo_rho", C.c_double),
    ]


def act_params() -> ActionParam:
    """The library's `act_params` global (writable)."""
    return ActionParam.in_dll(lib(), "act_params")


def set_stout_rho(rho: float) -> None:
    C.c_double.in_dll(lib(), "gl_stout_rho").value = float(rho)


def inverter_tricks() -> InvTricks:
    """The library's `inverter_tricks` global (writable)."""
    return InvTricks.in_dll(lib(), "inverter_tricks")


def check(ret: int = 0, what: str = "") -> None:
    L = lib()
    code = L.ostaple_get_error()
    if code != 0 or (isinstance(ret, int) and ret < 0):
        msg = L.ostaple_last_error().decode()
        L.ostaple_clear_error()
        raise RuntimeError(f"ostaple error in {what}: {msg} (code {code}, ret {ret})")
