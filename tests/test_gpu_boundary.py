"""The rest of the reference-named boundary through the C ABI on the GPU:

* the single-precision twins (acc_Deo_f, acc_Doe_f,
  fermion_matrix_multiplication(_shifted)_f, ker_invert_openacc_f,
  multishift_invert_f, the _f BLAS) and the float <-> double conversions
  (float_double_conv.c), against the FP64 oracle on the same FP32-rounded
  inputs: 5e-6 relative for one operator application (FP32 arithmetic over
  8 hops), solver iteration counts within 10 % of the FP64 recursion;
* the whole fermion BLAS set (fermionic_utilities.c:180-377) against numpy,
  1e-15 relative (one FP64 rounding per element);
* inverter_multishift_wrapper in its three modes (inverter_wrappers.c:41-114)
  and a fermion force whose pseudofermions are solved together, against the
  oracle and against the sequential FP64 force: every shift at an FP64 true
  residual <= the target, solutions within 1e-8 of the FP64 oracle CG-M.
"""
import ctypes as C
import json

import numpy as np
import pytest

from conftest import GOLDEN, relerr
from openstaple_gb300 import api, fields as F

pytestmark = pytest.mark.gpu


@pytest.fixture
def lat_factory(gpu):
    made = []

    def make(dims):
        lat = api.Lattice(dims)
        made.append(lat)
        return lat
    yield make
    for lat in made:
        lat.close()
    t = api.inverter_tricks()
    t.singlePInvAccelMultiInv, t.useMixedPrecision, t.mixedPrecisionDelta, t.restartingEvery = 0, 0, 0.1, 10000
    from openstaple_gb300.native import act_params
    act_params().stout_steps = 2
    api.set_stout_rho(0.15)


def approx8_rescaled():
    ap = json.loads((GOLDEN / "ratapprox.json").read_text())["order8"]
    mx = 64.0 * 1.05
    eps = mx ** (ap["exponent_num"] / ap["exponent_den"])
    return ap["a0"] * eps, np.array(ap["a"]) * mx * eps, np.array(ap["b"]) * mx


def f32(a):
    """The FP32 copy of an FP64 field, as convert_double_to_float_* makes it."""
    return np.ascontiguousarray(a.astype(np.complex64 if np.iscomplexobj(a) else np.float32))


def f64(a):
    return np.ascontiguousarray(a.astype(np.complex128 if np.iscomplexobj(a) else np.float64))


def test_conversions_round_like_a_cast(lat_factory):
    from openstaple_gb300.native import lib
    L = lib()
    dims = (4, 6, 8, 10)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 301)
    v = F.gaussian_vec3(dims, 302)
    ph = F.staggered_phases(dims)
    uf, vf, phf = np.zeros_like(f32(u)), np.zeros_like(f32(v)), np.zeros_like(f32(ph[0]))
    ub, vb, phb = np.zeros_like(u), np.zeros_like(v), np.zeros_like(ph[0])
    ph0 = np.ascontiguousarray(ph[1])
    for a in (u, v, ph0, uf, vf, phf, ub, vb, phb):
        lat.present(a)
    L.convert_double_to_float_su3_soa(u.ctypes.data, uf.ctypes.data)
    L.convert_double_to_float_vec3_soa(v.ctypes.data, vf.ctypes.data)
    L.convert_double_to_float_real_soa(ph0.ctypes.data, phf.ctypes.data)
    assert np.array_equal(lat.update_host(uf), f32(u))
    assert np.array_equal(lat.update_host(vf), f32(v))
    assert np.array_equal(lat.update_host(phf), f32(ph0))
    L.convert_float_to_double_su3_soa(uf.ctypes.data, ub.ctypes.data)
    L.convert_float_to_double_vec3_soa(vf.ctypes.data, vb.ctypes.data)
    L.convert_float_to_double_real_soa(phf.ctypes.data, phb.ctypes.data)
    assert np.array_equal(lat.update_host(ub), f64(f32(u)))
    assert np.array_equal(lat.update_host(vb), f64(f32(v)))
    assert np.array_equal(lat.update_host(phb), f64(f32(ph0)))
    api.check(0, "conversions")


@pytest.mark.parametrize("dims", [(8, 8, 8, 8), (4, 6, 8, 10)])
def test_single_precision_operator_twins(lat_factory, dims):
    from oracle import Oracle
    from openstaple_gb300.native import lib
    L = lib()
    o = Oracle(dims)
    lat = lat_factory(dims)
    u, v = F.random_su3_links(dims, 311), F.gaussian_vec3(dims, 312)
    ph = F.staggered_phases(dims)
    uf, vf, phf = f32(u), f32(v), f32(ph)
    out, tmp = np.zeros_like(vf), np.zeros_like(vf)
    for a in (uf, vf, phf, out, tmp):
        lat.present(a)
    # the oracle on the same FP32-rounded inputs, in FP64
    u64, v64, ph64 = f64(uf), f64(vf), f64(phf)
    L.acc_Deo_f(uf.ctypes.data, out.ctypes.data, vf.ctypes.data, phf.ctypes.data)
    assert relerr(lat.update_host(out), o.Deo(u64, v64, ph64)) <= 5e-6
    L.acc_Doe_f(uf.ctypes.data, out.ctypes.data, vf.ctypes.data, phf.ctypes.data)
    assert relerr(lat.update_host(out), o.Doe(u64, v64, ph64)) <= 5e-6
    L.acc_Deo_unsafe_f(uf.ctypes.data, out.ctypes.data, vf.ctypes.data, phf.ctypes.data)
    assert relerr(lat.update_host(out), o.Deo(u64, v64, ph64)) <= 5e-6
    fp = api.make_ferm_param(0.1, ph)
    fp.phases_f = phf.ctypes.data
    L.fermion_matrix_multiplication_f(uf.ctypes.data, out.ctypes.data, vf.ctypes.data, tmp.ctypes.data, C.byref(fp))
    assert relerr(lat.update_host(out), o.mdagm(u64, v64, ph64, 0.01)) <= 5e-6
    assert relerr(lat.update_host(tmp), o.Doe(u64, v64, ph64)) <= 5e-6
    L.fermion_matrix_multiplication_shifted_f(uf.ctypes.data, out.ctypes.data, vf.ctypes.data, tmp.ctypes.data,
                                              C.byref(fp), C.c_float(0.37))
    m2 = float(np.float32(np.float32(0.01) + np.float32(0.37)))
    assert relerr(lat.update_host(out), o.mdagm(u64, v64, ph64, m2)) <= 5e-6
    # the _f reductions accumulate in FP64
    n2 = float(np.sum(np.abs(v64) ** 2))
    assert abs(L.l2norm2_global_f(vf.ctypes.data) - n2) <= 1e-12 * n2
    api.check(0, "single-precision operator")


def test_single_precision_solver_twins(lat_factory):
    from oracle import Oracle
    from openstaple_gb300.native import lib
    L = lib()
    dims = (8, 8, 8, 8)
    o = Oracle(dims)
    lat = lat_factory(dims)
    u, b = F.random_su3_links(dims, 321), F.gaussian_vec3(dims, 322)
    ph = F.staggered_phases(dims)
    uf, bf, phf = f32(u), f32(b), f32(ph)
    u64, b64, ph64 = f64(uf), f64(bf), f64(phf)
    x = np.zeros_like(bf)
    work = [np.zeros_like(bf) for _ in range(4)]
    for a in (uf, bf, phf, x, *work):
        lat.present(a)
    fp = api.make_ferm_param(0.1, ph)
    fp.phases_f = phf.ctypes.data
    res = 1e-5
    cg = C.c_int(0)
    st = L.ker_invert_openacc_f(uf.ctypes.data, C.byref(fp), x.ctypes.data, bf.ctypes.data, res,
                                *[w.ctypes.data for w in work], 10000, 0.0, C.byref(cg))
    api.check(0, "ker_invert_openacc_f")
    st_o, n_o, x_o = o.cg(u64, ph64, 0.1, b64, res)
    assert st == 1 and st_o == 1
    assert abs(cg.value - n_o) <= 0.1 * n_o
    xd = f64(lat.update_host(x))
    r = b64 - o.mdagm(u64, xd, ph64, 0.01)
    assert np.sqrt(o.norm2(np.ascontiguousarray(r)) / o.norm2(b64)) <= 2 * res
    # multi-shift twin (the reference runs it to 8e-7 sqrt(sizeh) in its
    # accelerated wrapper, inverter_wrappers.c:57-60)
    a0, a, bsh = approx8_rescaled()
    approx = api.make_approx(a0, a, bsh)
    xs = np.zeros((len(a),) + bf.shape, np.complex64)
    ps = np.zeros_like(xs)
    for arr in (xs, ps):
        lat.present(arr)
    st = L.multishift_invert_f(uf.ctypes.data, C.byref(fp), C.byref(approx), xs.ctypes.data, bf.ctypes.data, res,
                               *[w.ctypes.data for w in work], ps.ctypes.data, 10000, C.byref(cg))
    api.check(0, "multishift_invert_f")
    st_o, n_o, xs_o = o.cgm(u64, ph64, 0.1, bsh, b64, res)
    assert st == 1 and st_o == 1
    assert abs(cg.value - n_o) <= 0.1 * n_o
    xs64 = f64(lat.update_host(xs))
    for k in range(len(a)):
        r = b64 - o.mdagm(u64, np.ascontiguousarray(xs64[k]), ph64, 0.01 + bsh[k])
        assert np.sqrt(o.norm2(np.ascontiguousarray(r)) / o.norm2(b64)) <= 3 * res, k
    assert relerr(xs64, xs_o) <= 1e-3
    rec = np.zeros_like(bf)
    lat.present(rec)
    L.recombine_shifted_vec3_to_vec3_f(xs.ctypes.data, bf.ctypes.data, rec.ctypes.data, C.byref(approx))
    assert relerr(f64(lat.update_host(rec)), o.recombine(xs64, b64, a0, a)) <= 1e-6


def test_fermion_blas_family(lat_factory):
    """Every reference-named vector operation, FP64 and FP32, against numpy."""
    from openstaple_gb300.native import lib
    L = lib()
    dims = (4, 4, 4, 8)
    lat = lat_factory(dims)
    a, b, c, d = (F.gaussian_vec3(dims, 330 + k) for k in range(4))
    out = lat.vec3()
    for arr in (a, b, c, d, out):
        lat.present(arr)

    def fresh(*arrs):
        for x in arrs:
            lat.update_device(x)

    P = lambda x: x.ctypes.data  # noqa: E731
    a0, b0, c0, d0 = a.copy(), b.copy(), c.copy(), d.copy()
    L.multiply_fermion_x_doublefactor(P(a), 0.7)
    assert relerr(lat.update_host(a), 0.7 * a0) <= 1e-15
    a[:] = a0; fresh(a)
    L.combine_add_factor_x_in2_to_in1(P(a), P(b), -1.3)
    assert relerr(lat.update_host(a), a0 - 1.3 * b0) <= 1e-15
    a[:] = a0; fresh(a)
    L.combine_in1xferm_mass_minus_in2(P(a), 0.25, P(b))
    assert relerr(lat.update_host(b), 0.25 * a0 - b0) <= 1e-15
    b[:] = b0; fresh(b)
    L.combine_in1_minus_in2(P(a), P(b), P(out))
    assert relerr(lat.update_host(out), a0 - b0) <= 1e-15
    L.assign_in_to_out(P(c), P(out))
    assert np.array_equal(lat.update_host(out), c0)
    L.set_vec3_soa_to_zero(P(out))
    assert not np.any(lat.update_host(out))
    L.combine_in1_x_fact1_minus_in2_back_into_in2(P(a), 0.9, P(b))
    assert relerr(lat.update_host(b), 0.9 * a0 - b0) <= 1e-15
    b[:] = b0; fresh(b)
    # combine_inside_loop: out += w p ; r -= w s
    o0 = F.gaussian_vec3(dims, 339)
    out[:] = o0; fresh(out)
    L.combine_inside_loop(P(out), P(a), P(b), P(c), 0.6)
    assert relerr(lat.update_host(out), o0 + 0.6 * c0) <= 1e-15
    assert relerr(lat.update_host(a), a0 - 0.6 * b0) <= 1e-15
    a[:] = a0; fresh(a)
    # multi-shift updates over 4 shifts, shift 1 frozen (flag 0)
    xs = np.stack([F.gaussian_vec3(dims, 350 + k) for k in range(4)])
    pk = np.stack([F.gaussian_vec3(dims, 360 + k) for k in range(4)])
    lat.present(xs)
    lat.present(pk)
    xs0, pk0 = xs.copy(), pk.copy()
    flag = (C.c_int * 4)(1, 0, 1, 1)
    om = (C.c_double * 4)(0.1, 0.2, 0.3, 0.4)
    ga = (C.c_double * 4)(1.1, 1.2, 1.3, 1.4)
    ze = (C.c_double * 4)(0.5, 0.6, 0.7, 0.8)
    L.multiple_combine_in1_minus_in2x_factor_back_into_in1(P(xs), P(pk), 4, flag, om)
    want = xs0.copy()
    for k in (0, 2, 3):
        want[k] = xs0[k] - om[k] * pk0[k]
    assert relerr(lat.update_host(xs), want) <= 1e-15
    L.multiple1_combine_in1_x_fact1_plus_in2_x_fact2_back_into_in1(P(pk), 4, flag, ga, P(a), ze)
    want = pk0.copy()
    for k in (0, 2, 3):
        want[k] = ga[k] * pk0[k] + ze[k] * a0
    assert relerr(lat.update_host(pk), want) <= 1e-15
    # FP32 twins of the family
    af, bf, of = f32(a0), f32(b0), np.zeros_like(f32(a0))
    for arr in (af, bf, of):
        lat.present(arr)
    L.combine_in1xfactor_plus_in2_f(P(af), 0.3, P(bf), P(of))
    assert relerr(f64(lat.update_host(of)), 0.3 * f64(af) + f64(bf)) <= 1e-7
    L.combine_in1_minus_in2_f(P(af), P(bf), P(of))
    assert relerr(f64(lat.update_host(of)), f64(af) - f64(bf)) <= 1e-7
    L.assign_in_to_out_f(P(bf), P(of))
    assert np.array_equal(lat.update_host(of), bf)
    rd = float(np.sum(f64(af).real * f64(bf).real + f64(af).imag * f64(bf).imag))
    assert abs(L.real_scal_prod_global_f(P(af), P(bf)) - rd) <= 1e-12 * abs(rd) + 1e-12
    api.check(0, "BLAS family")


def _true_res(o, u, ph, mass, shift, x, b):
    r = np.ascontiguousarray(b - o.mdagm(u, np.ascontiguousarray(x), ph, mass * mass + shift))
    return np.sqrt(o.norm2(r) / o.norm2(b))


@pytest.mark.parametrize("accel,mixed", [(0, 0), (1, 0), (1, 1)])
def test_inverter_multishift_wrapper_modes(lat_factory, accel, mixed):
    """Default: the FP64 multishift_invert.  singlePInvAccelMultiInv: FP32
    CG-M to max(8e-7 sqrt(sizeh), res), then every shift refined in FP64
    (per shift by ker_invert_openacc, or all together by the batched mixed
    solver with useMixedPrecision)."""
    from oracle import Oracle
    from openstaple_gb300.native import lib
    L = lib()
    dims = (8, 8, 8, 8)
    o = Oracle(dims)
    lat = lat_factory(dims)
    u, b = F.random_su3_links(dims, 341), F.gaussian_vec3(dims, 342)
    ph = F.staggered_phases(dims)
    mass, res = 0.05, 1e-10
    a0, a, bsh = approx8_rescaled()
    approx = api.make_approx(a0, a, bsh)
    xs, ps = lat.vec3(len(a)), lat.vec3(len(a))
    work = [lat.vec3() for _ in range(4)]
    for arr in (u, ph, b, xs, ps, *work):
        lat.present(arr)
    t = api.inverter_tricks()
    t.singlePInvAccelMultiInv, t.useMixedPrecision = accel, mixed
    fp = api.make_ferm_param(mass, ph)
    ip = api.make_inverter_package(u, *work, ferm_shift_temp=ps, nshifts=len(a))
    total = L.inverter_multishift_wrapper(ip, C.byref(fp), C.byref(approx), xs.ctypes.data, b.ctypes.data, res, 10000,
                                          0)
    api.check(0, "inverter_multishift_wrapper")
    lat.update_host(xs)
    st_o, n_o, xs_o = o.cgm(u, ph, mass, bsh, b, res)
    assert total >= n_o if accel == 0 else total > 0
    if accel == 0:
        assert total == n_o
    for k in range(len(a)):
        tr = _true_res(o, u, ph, mass, bsh[k], xs[k], b)
        # the FP64 CG-M's last shifts stop on their recursed residual; the
        # refined modes guarantee the true one
        assert tr <= (5 * res if accel == 0 else res), (k, tr)
    assert relerr(xs, xs_o) <= 1e-8


@pytest.mark.parametrize("accel,mixed", [(1, 0), (1, 1)])
def test_force_with_batched_pseudofermions_equals_sequential(lat_factory, accel, mixed):
    """fermion_force_soloopenacc with three pseudofermions: solved together in
    the accelerated modes, one after the other by the FP64 CG-M by default;
    the forces agree to the solvers' tolerance."""
    from openstaple_gb300.native import act_params, lib
    dims = (4, 6, 8, 10)
    lat = lat_factory(dims)
    a0, a, bsh = approx8_rescaled()
    mass, res = 0.1, 1e-11
    u = F.random_su3_links(dims, 351, eps=0.3)
    ph = F.staggered_phases(dims)
    phis = np.stack([F.gaussian_vec3(dims, 352 + k) for k in range(3)])
    order = len(a)

    def force():
        stout_levels = api.su3_field(lat.sizeh, 16)
        gl3, taux = api.su3_field(lat.sizeh), api.su3_field(lat.sizeh)
        ipdot = api.alg_field(lat.sizeh)
        shiftmulti, shifttemp = lat.vec3(order), lat.vec3(order)
        r, h, s, p = (lat.vec3() for _ in range(4))
        for arr in (u, ph, phis, stout_levels, gl3, ipdot, taux, shiftmulti, shifttemp, r, h, s, p):
            lat.present(arr)
        act_params().stout_steps = 2
        fp = api.make_ferm_param(mass, ph)
        fp.number_of_ps = len(phis)
        fp.approx_md.approx_order = order
        for k in range(order):
            fp.approx_md.RA_a[k] = a[k]
            fp.approx_md.RA_b[k] = bsh[k]
        ip = api.make_inverter_package(u, r, h, s, p, ferm_shift_temp=shifttemp, nshifts=order)
        lib().fermion_force_soloopenacc(u.ctypes.data, stout_levels.ctypes.data, gl3.ctypes.data,
                                        ipdot.ctypes.data, C.byref(fp), 1, phis.ctypes.data, res,
                                        taux.ctypes.data, shiftmulti.ctypes.data, ip, 10000)
        api.check(0, "fermion_force_soloopenacc")
        lat.update_host(shiftmulti)
        out = lat.update_host(ipdot).copy(), shiftmulti.copy(), lat.update_host(s).copy()
        # the per-call arrays are freed on return: drop their device mirrors
        for arr in (stout_levels, gl3, ipdot, taux, shiftmulti, shifttemp, r, h, s, p):
            lat.release(arr)
        return out

    t = api.inverter_tricks()
    t.singlePInvAccelMultiInv, t.useMixedPrecision = 0, 0
    ref, sm_ref, s_ref = force()
    t.singlePInvAccelMultiInv, t.useMixedPrecision = accel, mixed
    got, sm, s_last = force()
    assert relerr(got, ref) <= 1e-8
    # the last pseudofermion's solutions stay in the shift buffer, its last shift in loc_s
    assert relerr(sm, sm_ref) <= 1e-8
    assert relerr(s_last, s_ref) <= 1e-8
