"""Python mirror of the reference's hot-path interface.

Functions carry the reference's names and argument order
(fermion_matrix.h, fermionic_utilities.h, inverter_full.h,
inverter_multishift_full.h) and take numpy arrays in the reference's SoA
layouts.  Host arrays are made present on the device with
:meth:`Lattice.present` (the OpenACC ``enter data`` + ``update device``
pair) and read back with :meth:`Lattice.update_host`; every compute call goes
to the CUDA library.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from .native import FermParam, InverterPackage, RationalApprox, check, inverter_tricks, lib, set_stout_rho  # noqa: F401


def ptr(a) -> int:
    """Address of a numpy array or a CUDA tensor (``data_ptr``)."""
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if isinstance(a, int):
        return a
    raise TypeError(f"cannot take the address of {type(a)}")


class Lattice:
    """Initialises the library for one lattice and tracks device mirrors."""

    def __init__(self, dims: Sequence[int]):
        self.dims = tuple(int(d) for d in dims)
        self.L = lib()
        rc = self.L.ostaple_init(*self.dims)
        check(rc, "ostaple_init")
        self.sizeh = self.L.ostaple_sizeh()
        self._present: dict[int, int] = {}

    def present(self, arr: np.ndarray, copy: bool = True) -> np.ndarray:
        if not arr.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous")
        p = arr.ctypes.data
        if p in self._present and self._present[p] != arr.nbytes:
            # the mapping of a freed array that lay at the same host address
            self.L.ostaple_exit_data(p)
            del self._present[p]
        if p not in self._present:
            check(self.L.ostaple_enter_data(p, arr.nbytes), "enter_data")
            self._present[p] = arr.nbytes
        if copy:
            check(self.L.ostaple_update_device(p, arr.nbytes), "update_device")
        return arr

    def update_device(self, arr: np.ndarray) -> None:
        check(self.L.ostaple_update_device(arr.ctypes.data, arr.nbytes), "update_device")

    def update_host(self, arr: np.ndarray) -> np.ndarray:
        check(self.L.ostaple_update_host(arr.ctypes.data, arr.nbytes), "update_host")
        return arr

    def release(self, arr: np.ndarray) -> None:
        p = arr.ctypes.data
        if p in self._present:
            self.L.ostaple_exit_data(p)
            del self._present[p]

    def release_all(self) -> None:
        for p in list(self._present):
            self.L.ostaple_exit_data(p)
        self._present.clear()

    def sync(self) -> None:
        check(self.L.ostaple_synchronize(), "synchronize")

    # --- field constructors in the reference layouts ---
    def vec3(self, n: int | None = None) -> np.ndarray:
        shape = (3, self.sizeh) if n is None else (n, 3, self.sizeh)
        return np.zeros(shape, dtype=np.complex128)

    def close(self) -> None:
        self.release_all()
        self.L.ostaple_finalize()


def make_ferm_param(mass: float, phases: np.ndarray | int) -> FermParam:
    fp = FermParam()
    fp.ferm_mass = float(mass)
    fp.degeneracy = 1
    fp.number_of_ps = 1
    fp.phases = ptr(phases)
    return fp


def make_approx(a0: float, a: Sequence[float], b: Sequence[float]) -> RationalApprox:
    ra = RationalApprox()
    ra.approx_order = len(a)
    ra.RA_a0 = float(a0)
    for i, (ai, bi) in enumerate(zip(a, b)):
        ra.RA_a[i] = float(ai)
        ra.RA_b[i] = float(bi)
    return ra


# ---- reference-named calls ----
def acc_Deo(u, out, inp, backfield) -> None:
    lib().acc_Deo(ptr(u), ptr(out), ptr(inp), ptr(backfield))
    check(0, "acc_Deo")


def acc_Doe(u, out, inp, backfield) -> None:
    lib().acc_Doe(ptr(u), ptr(out), ptr(inp), ptr(backfield))
    check(0, "acc_Doe")


def fermion_matrix_multiplication_shifted(u, out, inp, temp1, pars: FermParam, shift: float) -> None:
    lib().fermion_matrix_multiplication_shifted(ptr(u), ptr(out), ptr(inp), ptr(temp1), C.byref(pars), shift)
    check(0, "fermion_matrix_multiplication_shifted")


def fermion_matrix_multiplication(u, out, inp, temp1, pars: FermParam) -> None:
    lib().fermion_matrix_multiplication(ptr(u), ptr(out), ptr(inp), ptr(temp1), C.byref(pars))
    check(0, "fermion_matrix_multiplication")


def mdagm_df(u, phases, mass: float, out, inp, shift: float = 0.0) -> None:
    """out = (m^2 + shift) inp - D_eo D_oe inp in double-float arithmetic."""
    check(lib().ostaple_mdagm_df(ptr(u), ptr(phases), mass, shift, ptr(out), ptr(inp)), "ostaple_mdagm_df")


def set_sloppy_links(fmt: str) -> str:
    """Link format of the FP32 iteration: "q16" (16-bit fixed point, the
    default) or "f32"; returns the previous one."""
    if fmt not in ("q16", "f32"):
        raise ValueError(f"sloppy link format must be 'q16' or 'f32', not {fmt!r}")
    prev = lib().ostaple_set_sloppy_links(1 if fmt == "q16" else 0)
    return "q16" if prev else "f32"


def mdagm_sloppy(u, phases, mass: float, out, inp, shift: float = 0.0) -> None:
    """out = (m^2 + shift) inp - D_eo D_oe inp through the FP32 iteration kernels."""
    check(lib().ostaple_mdagm_sloppy(ptr(u), ptr(phases), mass, shift, ptr(out), ptr(inp)), "ostaple_mdagm_sloppy")


def l2norm2_global(v) -> float:
    r = lib().l2norm2_global(ptr(v))
    check(0, "l2norm2_global")
    return r


def real_scal_prod_global(a, b) -> float:
    r = lib().real_scal_prod_global(ptr(a), ptr(b))
    check(0, "real_scal_prod_global")
    return r


def scal_prod_global(a, b) -> complex:
    out = (C.c_double * 2)()
    lib().scal_prod_global_ri(ptr(a), ptr(b), out)
    check(0, "scal_prod_global")
    return complex(out[0], out[1])


def ker_invert_openacc(u, pars: FermParam, solution, inp, res: float, loc_r, loc_h, loc_s, loc_p, max_cg: int,
                       shift: float) -> tuple[int, int]:
    cg = C.c_int(0)
    st = lib().ker_invert_openacc(ptr(u), C.byref(pars), ptr(solution), ptr(inp), res, ptr(loc_r), ptr(loc_h),
                                  ptr(loc_s), ptr(loc_p), max_cg, shift, C.byref(cg))
    check(0, "ker_invert_openacc")
    return st, cg.value


def multishift_invert(u, pars: FermParam, approx: RationalApprox, out, inp, residuo: float, loc_r, loc_h, loc_s,
                      loc_p, shiftferm, max_cg: int) -> tuple[int, int]:
    cg = C.c_int(0)
    st = lib().multishift_invert(ptr(u), C.byref(pars), C.byref(approx), ptr(out), ptr(inp), residuo, ptr(loc_r),
                                 ptr(loc_h), ptr(loc_s), ptr(loc_p), ptr(shiftferm), max_cg, C.byref(cg))
    check(0, "multishift_invert")
    return st, cg.value


def recombine_shifted_vec3_to_vec3(in_shifted, inp, out, approx: RationalApprox) -> None:
    lib().recombine_shifted_vec3_to_vec3(ptr(in_shifted), ptr(inp), ptr(out), C.byref(approx))
    check(0, "recombine_shifted_vec3_to_vec3")


def find_min_max_eigenvalue_soloopenacc(u, pars: FermParam, loc_r, loc_h, loc_p1, loc_p2) -> np.ndarray:
    """[m^2, largest eigenvalue of M^+M] by power iteration from the start vector in loc_p1."""
    mm = np.zeros(2)
    lib().find_min_max_eigenvalue_soloopenacc(ptr(u), C.byref(pars), ptr(loc_r), ptr(loc_h), ptr(loc_p1),
                                              ptr(loc_p2), mm.ctypes.data)
    check(0, "find_min_max_eigenvalue_soloopenacc")
    return mm


def ker_find_min_eigenvalue_openacc(u, pars: FermParam, loc_r, loc_h, loc_p, max_eig: float) -> float:
    v = lib().ker_find_min_eigenvalue_openacc(ptr(u), C.byref(pars), ptr(loc_r), ptr(loc_h), ptr(loc_p), max_eig)
    check(0, "ker_find_min_eigenvalue_openacc")
    return v


def set_restarting_every(n: int) -> None:
    inverter_tricks().restartingEvery = int(n)


def make_inverter_package(u, loc_r=None, loc_h=None, loc_s=None, loc_p=None, u_f=None, loc_r_f=None, loc_h_f=None,
                          loc_s_f=None, loc_p_f=None, out_f=None, ferm_shift_temp=None, nshifts=0) -> InverterPackage:
    """setup_inverter_package_dp/_sp (inverter_package.c:17-77) in one call;
    unset parking vectors make the library use its own workspace."""
    ip = InverterPackage()
    ip.u = ptr(u)
    opt = lambda a: None if a is None else ptr(a)  # noqa: E731
    ip.u_f = opt(u_f)
    ip.loc_r, ip.loc_h, ip.loc_s, ip.loc_p = opt(loc_r), opt(loc_h), opt(loc_s), opt(loc_p)
    ip.loc_r_f, ip.loc_h_f, ip.loc_s_f, ip.loc_p_f = opt(loc_r_f), opt(loc_h_f), opt(loc_s_f), opt(loc_p_f)
    ip.out_f = opt(out_f)
    ip.ferm_shift_temp = opt(ferm_shift_temp)
    ip.nshifts = nshifts
    return ip


def inverter_mixed_precision(ip: InverterPackage, pars: FermParam, solution, inp, res: float, max_cg: int,
                             shift: float) -> tuple[int, int]:
    cg = C.c_int(0)
    st = lib().inverter_mixed_precision(ip, C.byref(pars), ptr(solution), ptr(inp), res, max_cg, shift, C.byref(cg))
    check(0, "inverter_mixed_precision")
    return st, cg.value


def invert_mixed(u, phases, mass: float, shift: float, solution, inp, res: float = 1e-10, max_iter: int = 100000,
                 reliable_every: int = 0, delta_frac: float = 0.0) -> dict:
    """Mixed-precision solve to an FP64 true residual <= res."""
    it, nrel, tr = C.c_int(0), C.c_int(0), C.c_double(0)
    st = lib().ostaple_invert_mixed(ptr(u), ptr(phases), mass, shift, ptr(solution), ptr(inp), res, max_iter,
                                    reliable_every, delta_frac, C.byref(it), C.byref(tr), C.byref(nrel))
    check(0, "ostaple_invert_mixed")
    return dict(status=st, iters=it.value, true_res=tr.value, n_reliable=nrel.value)


# ---- stout smearing and fermion force (stouting.h, fermion_force_utilities.h) ----
def su3_field(sizeh: int, n: int = 8) -> np.ndarray:
    """su3_soa[n] in the reference layout: complex128 (n, 3, 3, sizeh)."""
    return np.zeros((n, 3, 3, sizeh), np.complex128)


def alg_field(sizeh: int) -> np.ndarray:
    """tamat_soa[8] / thmat_soa[8]: float64 (8, 8*sizeh) (3 complex + 2 real arrays per direction)."""
    return np.zeros((8, 8 * sizeh))


def stout_isotropic(u, uprime, local_staples, auxiliary, tipdot, istopo: int = 0) -> None:
    lib().stout_isotropic(ptr(u), ptr(uprime), None if local_staples is None else ptr(local_staples),
                          None if auxiliary is None else ptr(auxiliary), ptr(tipdot), istopo)
    check(0, "stout_isotropic")


def stout_wrapper(u, stout_levels, istopo: int = 0) -> None:
    lib().stout_wrapper(ptr(u), ptr(stout_levels), istopo)
    check(0, "stout_wrapper")


def compute_sigma_from_sigma_prime_backinto_sigma_prime(sigma, lam, qa, u, tmp, istopo: int = 0) -> None:
    lib().compute_sigma_from_sigma_prime_backinto_sigma_prime(ptr(sigma), ptr(lam), ptr(qa), ptr(u), ptr(tmp),
                                                              istopo)
    check(0, "compute_sigma_from_sigma_prime_backinto_sigma_prime")


def ker_openacc_compute_fermion_force(u, aux_u, in_shiftmulti, loc_s, loc_h, pars: FermParam) -> None:
    lib().ker_openacc_compute_fermion_force(ptr(u), ptr(aux_u), ptr(in_shiftmulti), ptr(loc_s), ptr(loc_h),
                                            C.byref(pars))
    check(0, "ker_openacc_compute_fermion_force")


def multiply_backfield_times_force(pars: FermParam, auxmat, pseudo_ipdot) -> None:
    lib().multiply_backfield_times_force(C.byref(pars), ptr(auxmat), ptr(pseudo_ipdot))
    check(0, "multiply_backfield_times_force")


def multiply_conf_times_force_and_take_ta_nophase(u, auxmat, ipdot) -> None:
    lib().multiply_conf_times_force_and_take_ta_nophase(ptr(u), ptr(auxmat), ptr(ipdot))
    check(0, "multiply_conf_times_force_and_take_ta_nophase")


# ---- pure-gauge tree-level Symanzik HMC ----
def calc_ipdot_gauge_soloopenacc(u, local_staples, tipdot) -> None:
    lib().calc_ipdot_gauge_soloopenacc(ptr(u), None if local_staples is None else ptr(local_staples), ptr(tipdot))
    check(0, "calc_ipdot_gauge_soloopenacc")


def calc_plaquette_soloopenacc(u) -> float:
    v = lib().calc_plaquette_soloopenacc(ptr(u), None, None)
    check(0, "calc_plaquette_soloopenacc")
    return v


def calc_rettangolo_soloopenacc(u) -> float:
    v = lib().calc_rettangolo_soloopenacc(ptr(u), None, None)
    check(0, "calc_rettangolo_soloopenacc")
    return v


def momenta_action(mom) -> float:
    """sum over the 8 directions of calc_momenta_action (1/2 tr P^2 over all links)."""
    v = sum(lib().calc_momenta_action(ptr(mom), None, mu) for mu in range(8))
    check(0, "calc_momenta_action")
    return v


def mom_sum_mult(mom, ipdot, factor: float) -> None:
    f = (C.c_double * 1)(factor)
    lib().mom_sum_mult(ptr(mom), ptr(ipdot), f, 0)
    check(0, "mom_sum_mult")


def mom_exp_times_conf_soloopenacc(u, mom, delta: float) -> None:
    f = (C.c_double * 1)(delta)
    lib().mom_exp_times_conf_soloopenacc(ptr(u), ptr(mom), f, 0)
    check(0, "mom_exp_times_conf_soloopenacc")


def multistep_2MN_gauge(u, local_staples, tipdot, mom, beta: float, no_md: int, gauge_scale: int, t: float,
                        ncalls: int = 1) -> None:
    """ncalls x multistep_2MN_gauge with deltas_Omelyan set by
    initialize_md_global_variables for (beta, no_md, gauge_scale, t)."""
    from .native import MdParam, act_params, md_parameters
    act_params().beta = float(beta)
    mp = md_parameters()
    mp.no_md, mp.gauge_scale, mp.t = int(no_md), int(gauge_scale), float(t)
    lib().initialize_md_global_variables(mp)
    for _ in range(ncalls):
        lib().multistep_2MN_gauge(ptr(u), ptr(local_staples), ptr(tipdot), ptr(mom))
    check(0, "multistep_2MN_gauge")


def pure_gauge_hmc(u, beta: float, ntraj: int, no_md: int = 18, gauge_scale: int = 4, traj_len: float = 1.0,
                   seed: int = 1, first_traj: int = 0, precision: str = "fp64", metropolis: bool = True) -> dict:
    """ntraj pure-gauge tree-level Symanzik HMC trajectories on the links u
    (updated in place on the device); precision "fp64" or "fp32" (FP32
    molecular dynamics, FP64 actions and Metropolis)."""
    acc = C.c_int(0)
    plaq = np.zeros(max(ntraj, 1))
    ds = np.zeros(max(ntraj, 1))
    rc = lib().ostaple_pure_gauge_hmc(ptr(u), beta, ntraj, no_md, gauge_scale, traj_len, seed, first_traj,
                                      {"fp64": 0, "fp32": 1}[precision], int(metropolis), C.byref(acc),
                                      plaq.ctypes.data, ds.ctypes.data)
    check(rc, "ostaple_pure_gauge_hmc")
    return dict(accepted=acc.value, plaquette=plaq[:ntraj], delta_s=ds[:ntraj])


def rhmc_trajectory(u, fpars, beta: float, no_md: int, gauge_scale: int, traj_len: float = 1.0,
                    res_metro: float = 1e-10, res_md: float = 1e-8, max_cg: int = 10000, seed: int = 1, traj: int = 0,
                    metropolis: bool = True) -> dict:
    """One RHMC update of the links u (device-resident) with the flavours
    fpars (a ctypes array of FermParam with their mother approximations)."""
    acc, ds = C.c_int(0), C.c_double(0)
    act = np.zeros(6)
    rc = lib().ostaple_rhmc_trajectory(ptr(u), fpars, len(fpars), beta, no_md, gauge_scale, traj_len, res_metro, res_md,
                                       max_cg, seed, traj, int(metropolis), C.byref(acc), C.byref(ds),
                                       act.ctypes.data)
    check(rc, "ostaple_rhmc_trajectory")
    return dict(accepted=acc.value, delta_s=ds.value, action=act)


def gauge_momenta(mom, seed: int, stream: int) -> None:
    check(lib().ostaple_gauge_momenta(ptr(mom), seed, stream), "ostaple_gauge_momenta")


def gauge_action(u, beta: float) -> dict:
    p, r, s = C.c_double(0), C.c_double(0), C.c_double(0)
    check(lib().ostaple_gauge_action(ptr(u), beta, C.byref(p), C.byref(r), C.byref(s)), "ostaple_gauge_action")
    return dict(plaq_sum=p.value, rect_sum=r.value, action=s.value)


# ---- batched solvers ----
def remez(exponent_num: int, exponent_den: int, lambda_min: float, order: int = 0,
          goal_error: float | None = None) -> RationalApprox:
    """The best relative-error rational approximation of x^(num/den) on
    [lambda_min, 1] from the library's generator: of the given order, or of
    the smallest order (starting from the reference driver's guess) whose
    error is at most goal_error.  Returns the filled RationalApprox."""
    ra = RationalApprox()
    ra.exponent_num, ra.exponent_den, ra.lambda_min = int(exponent_num), int(exponent_den), float(lambda_min)
    if goal_error is None:
        ra.approx_order = int(order)
        rc = lib().ostaple_remez_approximation(C.byref(ra))
    else:
        rc = lib().ostaple_remez_generate(C.byref(ra), float(goal_error), int(order))
    check(rc, "ostaple_remez")
    return ra


def eo_inversion(ip, fp, res: float, max_cg: int, in_e, in_o, out_e, out_o, phi_e, phi_o) -> None:
    """Full-D inversion by even/odd reduction (Meas/ferm_meas.c:50-71)."""
    lib().eo_inversion(ip, C.byref(fp), res, max_cg, ptr(in_e), ptr(in_o), ptr(out_e), ptr(out_o), ptr(phi_e),
                       ptr(phi_o))
    check(0, "eo_inversion")


def chiral_condensate(in_e, in_o, out_e, out_o, degeneracy: int, volume: int) -> complex:
    """The chiral condensate estimator of one noise vector,
    degeneracy / 4 / V * (<in_e, out_e> + <in_o, out_o>) with out = D^-1 in
    (Meas/ferm_meas.c:295, 314-321), from the library's global scalar
    products (the fields must be present)."""
    L = lib()
    a = np.zeros(2)
    b = np.zeros(2)
    L.scal_prod_global_ri(ptr(in_e), ptr(out_e), a.ctypes.data_as(C.POINTER(C.c_double)))
    L.scal_prod_global_ri(ptr(in_o), ptr(out_o), b.ctypes.data_as(C.POINTER(C.c_double)))
    check(0, "scal_prod_global_ri")
    return degeneracy * 0.25 / volume * complex(a[0] + b[0], a[1] + b[1])


def invert_mixed_batch(u, phases, mass: float, solutions, sources, shifts=None, res: float = 1e-10,
                       max_iter: int = 100000, delta_frac: float = 0.0) -> dict:
    """(M^+M + shift_k) x_k = b_k for all k at once (links read once per Dslash per batch of 8)."""
    nsys = solutions.shape[0]
    sh = None if shifts is None else np.ascontiguousarray(shifts, dtype=np.float64)
    it = np.zeros(nsys, np.int32)
    tr = np.zeros(nsys)
    nr = np.zeros(nsys, np.int32)
    st = lib().ostaple_invert_mixed_batch(ptr(u), ptr(phases), mass, nsys, None if sh is None else sh.ctypes.data,
                                          ptr(solutions), ptr(sources), res, max_iter, delta_frac, it.ctypes.data,
                                          tr.ctypes.data, nr.ctypes.data)
    check(0, "ostaple_invert_mixed_batch")
    return dict(status=st, iters=it, true_res=tr, n_reliable=nr)


def multishift_batch(u, phases, mass: float, approx: RationalApprox, sources, solutions, res: float = 1e-10,
                     max_iter: int = 100000, delta_frac: float = 0.0) -> dict:
    """All shifts of `approx` for every source: FP32 CG-M then FP64-guaranteed refinement."""
    nrhs = sources.shape[0]
    order = approx.approx_order
    ic = np.zeros(nrhs, np.int32)
    ir = np.zeros(nrhs * order, np.int32)
    tr = np.zeros(nrhs * order)
    st = lib().ostaple_multishift_batch(ptr(u), ptr(phases), mass, C.byref(approx), nrhs, ptr(sources),
                                        ptr(solutions), res, max_iter, delta_frac, ic.ctypes.data, ir.ctypes.data,
                                        tr.ctypes.data)
    check(0, "ostaple_multishift_batch")
    return dict(status=st, iters_cgm=ic, iters_refine=ir.reshape(nrhs, order), true_res=tr.reshape(nrhs, order))


# ---- learned preconditioner ----
NET_SHAPE = (4, 64, 8)   # [layer][hop*8 + in_channel][out_channel]


def net_init(seed: int = 1, scale: float = 0.05) -> None:
    check(lib().ostaple_net_init(seed, scale), "ostaple_net_init")


def net_set_weights(w: np.ndarray) -> None:
    w = np.ascontiguousarray(w, dtype=np.float32).reshape(NET_SHAPE)
    check(lib().ostaple_net_set_weights(w.ctypes.data), "ostaple_net_set_weights")


def net_get_weights() -> np.ndarray:
    w = np.zeros(NET_SHAPE, np.float32)
    check(lib().ostaple_net_get_weights(w.ctypes.data), "ostaple_net_get_weights")
    return w


def net_weights_save(path, w: np.ndarray) -> None:
    w = np.ascontiguousarray(w, dtype=np.float32).reshape(NET_SHAPE)
    check(lib().ostaple_net_weights_save(str(path).encode(), w.ctypes.data), "ostaple_net_weights_save")


def net_weights_load(path) -> np.ndarray:
    w = np.zeros(NET_SHAPE, np.float32)
    check(lib().ostaple_net_weights_load(str(path).encode(), w.ctypes.data), "ostaple_net_weights_load")
    return w


def net_apply(u, phases, inp, out) -> None:
    check(lib().ostaple_net_apply(ptr(u), ptr(phases), ptr(inp), ptr(out)), "ostaple_net_apply")


def net_gradient(u, phases, mass: float, source, target, shift: float = 0.0) -> tuple[np.ndarray, float]:
    """Residual loss |A (N(source) - target)|^2 / |source|^2 of one pair and its
    weight gradient, A = M^+M + shift."""
    dw = np.zeros(NET_SHAPE, np.float32)
    loss = C.c_double(0)
    check(lib().ostaple_net_gradient(ptr(u), ptr(phases), mass, shift, ptr(source), ptr(target), dw.ctypes.data,
                                     C.byref(loss)), "ostaple_net_gradient")
    return dw, loss.value


def net_train(u, phases, mass: float, sources, solutions, epochs: int, lr: float, shift: float = 0.0) -> np.ndarray:
    """Full-batch Adam on (source, solution) pairs of A = M^+M + shift; returns the loss per epoch."""
    hist = np.zeros(epochs)
    check(lib().ostaple_net_train(ptr(u), ptr(phases), mass, shift, sources.shape[0], ptr(sources), ptr(solutions),
                                  epochs, lr, hist.ctypes.data), "ostaple_net_train")
    return hist


def invert_learned(u, phases, mass: float, shift: float, solution, inp, res: float = 1e-10,
                   max_iter: int = 20000) -> dict:
    it, tr, fb = C.c_int(0), C.c_double(0), C.c_int(0)
    st = lib().ostaple_invert_learned(ptr(u), ptr(phases), mass, shift, ptr(solution), ptr(inp), res, max_iter,
                                      C.byref(it), C.byref(tr), C.byref(fb))
    check(0, "ostaple_invert_learned")
    return dict(status=st, iters=it.value, true_res=tr.value, used_fallback=fb.value)


def autotune(enable: bool) -> None:
    """Switch the launch-shape autotuner of the FP32 D_oe hops on or off."""
    lib().ostaple_autotune(1 if enable else 0)


def autotune_force(candidate: int) -> None:
    """Every tuned launch uses candidate shape `candidate` (0 = the default;
    a kernel with fewer candidates uses its default): for tests."""
    lib().ostaple_autotune(2 + int(candidate))


def autotune_report() -> str:
    """One line per tuned (kernel, lattice, variant): the chosen candidate and
    each candidate's microseconds per launch."""
    n = lib().ostaple_autotune_report(None, 0)
    buf = C.create_string_buffer(n + 1)
    lib().ostaple_autotune_report(buf, n + 1)
    return buf.value.decode()
