"""GPU parity of stout smearing and the rational fermion force chain through
the C ABI, against the CPU oracle (itself pinned to the reference's compiled
code).  FP64 throughout; tolerances (relative, max-norm): 1e-13 for a stout
step and the outer products, 1e-12 for the Sigma chain, whose Lambda
coefficients divide by (9u^2 - w^2)^2."""
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
    api.set_stout_rho(0.15)


@pytest.mark.parametrize("dims,eps", [((4, 4, 4, 4), 0.3), ((4, 6, 8, 10), 0.05), ((8, 8, 8, 8), 0.3),
                                      ((4, 4, 4, 4), 0.01)])
def test_stout_step(lat_factory, dims, eps):
    from oracle import Oracle
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 101, eps=eps)
    up = api.su3_field(lat.sizeh)
    stap = api.su3_field(lat.sizeh)
    qa = api.alg_field(lat.sizeh)
    for a in (u, up, stap, qa):
        lat.present(a)
    api.stout_isotropic(u, up, stap, None, qa, 0)
    for a in (up, stap, qa):
        lat.update_host(a)
    assert relerr(stap, o.staples(u)) <= 1e-13
    assert relerr(qa, o.rho_ta(u, o.staples(u), 0.15)) <= 1e-13
    assert relerr(up[:, :2], o.stout(u, 0.15)[:, :2]) <= 1e-13


def test_stout_wrapper_two_levels(lat_factory):
    from oracle import Oracle
    dims = (4, 4, 8, 4)
    o = Oracle(dims)
    lat = lat_factory(dims)
    api.set_stout_rho(0.12)
    u = F.random_su3_links(dims, 7, eps=0.4)
    levels = api.su3_field(lat.sizeh, 16)
    lat.present(u)
    lat.present(levels)
    api.stout_wrapper(u, levels, 0)
    lat.update_host(levels)
    l1 = o.stout(u, 0.12)
    l2 = o.stout(l1, 0.12)
    assert relerr(levels[:8, :2], l1[:, :2]) <= 1e-13
    assert relerr(levels[8:, :2], l2[:, :2]) <= 1e-13


@pytest.mark.parametrize("dims,eps", [((4, 4, 4, 4), 0.3), ((4, 6, 8, 10), 0.05), ((4, 4, 4, 4), 0.01)])
def test_sigma_chain(lat_factory, dims, eps):
    from oracle import Oracle
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 17, eps=eps)
    sig = F.random_su3_links(dims, 18, eps=1.0) * 0.7
    lam, qa, tmp = api.alg_field(lat.sizeh), api.alg_field(lat.sizeh), api.su3_field(lat.sizeh)
    s_dev = sig.copy()
    for a in (u, s_dev, lam, qa, tmp):
        lat.present(a)
    api.compute_sigma_from_sigma_prime_backinto_sigma_prime(s_dev, lam, qa, u, tmp, 0)
    lat.update_host(s_dev)
    lat.update_host(lam)
    ref = o.sigma_prime_to_sigma(sig, u, 0.15)
    assert relerr(s_dev, ref) <= 1e-12
    qa_o = o.rho_ta(u, o.staples(u), 0.15)
    assert relerr(lam, o.lambda_(sig, u, qa_o)) <= 1e-12


def test_force_pieces(lat_factory):
    from oracle import Oracle
    dims = (4, 4, 6, 8)
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 27)
    ph = F.staggered_phases(dims)
    a = [0.31, 0.21, 0.11, 0.07]
    xs = np.stack([F.gaussian_vec3(dims, 40 + k) for k in range(len(a))])
    aux = api.su3_field(lat.sizeh)
    pip = F.random_su3_links(dims, 29)
    ip = np.zeros((8, 8 * lat.sizeh))
    s, h = lat.vec3(), lat.vec3()
    for arr in (u, ph, xs, aux, pip, ip, s, h):
        lat.present(arr)
    fp = api.make_ferm_param(0.05, ph)
    fp.approx_md.approx_order = len(a)
    for k, v in enumerate(a):
        fp.approx_md.RA_a[k] = v
    api.ker_openacc_compute_fermion_force(u, aux, xs, s, h, fp)
    aux_o = o.force_outer(u, xs, ph, a)
    assert relerr(lat.update_host(aux), aux_o) <= 1e-13
    pip0 = pip.copy()
    api.multiply_backfield_times_force(fp, aux, pip)
    pip_o = o.backfield_times_force(ph, aux_o, pip0)
    assert relerr(lat.update_host(pip), pip_o) <= 1e-13
    api.multiply_conf_times_force_and_take_ta_nophase(u, pip, ip)
    assert relerr(lat.update_host(ip), o.conf_times_force_ta(u, pip_o, np.zeros_like(ip))) <= 1e-13
    # the parking vectors hold the last shift's X and D_oe X
    assert relerr(lat.update_host(s), xs[-1]) == 0.0
    assert relerr(lat.update_host(h), o.Doe(u, np.ascontiguousarray(xs[-1]), ph)) <= 1e-13


def test_full_fermion_force(lat_factory):
    """fermion_force_soloopenacc: 2 stout levels, multi-shift solve with
    approx_md, outer products, phases, Sigma chain, TA projection -- against
    the same chain assembled from oracle pieces."""
    from oracle import Oracle
    from openstaple_gb300.native import act_params
    dims = (4, 4, 4, 8)
    o = Oracle(dims)
    lat = lat_factory(dims)
    ap = json.loads((GOLDEN / "ratapprox.json").read_text())["order8"]
    mx = 64.0 * 1.05
    eps = mx ** (ap["exponent_num"] / ap["exponent_den"])
    a = np.array(ap["a"]) * mx * eps
    b = np.array(ap["b"]) * mx
    mass = 0.1
    u = F.random_su3_links(dims, 51, eps=0.3)
    ph = F.staggered_phases(dims)
    phi = F.gaussian_vec3(dims, 52)
    stout_levels = api.su3_field(lat.sizeh, 16)
    gl3 = api.su3_field(lat.sizeh)
    ipdot = api.alg_field(lat.sizeh)
    taux = api.su3_field(lat.sizeh)
    shiftmulti = lat.vec3(len(a))
    shifttemp = lat.vec3(len(a))
    r, h, s, p = (lat.vec3() for _ in range(4))
    for arr in (u, ph, phi, stout_levels, gl3, ipdot, taux, shiftmulti, shifttemp, r, h, s, p):
        lat.present(arr)
    act_params().stout_steps = 2
    api.set_stout_rho(0.15)
    fp = api.make_ferm_param(mass, ph)
    fp.number_of_ps = 1
    fp.index_of_the_first_ps = 0
    fp.approx_md.approx_order = len(a)
    for k in range(len(a)):
        fp.approx_md.RA_a[k] = a[k]
        fp.approx_md.RA_b[k] = b[k]
    ip = api.make_inverter_package(u, r, h, s, p, ferm_shift_temp=shifttemp, nshifts=len(a))
    import ctypes as C
    from openstaple_gb300.native import lib
    lib().fermion_force_soloopenacc(u.ctypes.data, stout_levels.ctypes.data, gl3.ctypes.data, ipdot.ctypes.data,
                                    C.byref(fp), 1, phi.ctypes.data, 1e-12, taux.ctypes.data,
                                    shiftmulti.ctypes.data, ip, 10000)
    lat.update_host(ipdot)
    # oracle chain
    u1 = o.stout(u, 0.15)
    u2 = o.stout(u1, 0.15)
    st, n, xs = o.cgm(u2, ph, mass, b, phi, 1e-12)
    aux = o.force_outer(u2, xs, ph, a)
    sig = o.backfield_times_force(ph, aux, np.zeros_like(aux))
    sig = o.sigma_prime_to_sigma(sig, u1, 0.15)
    sig = o.sigma_prime_to_sigma(sig, u, 0.15)
    ref = o.conf_times_force_ta(u, sig, np.zeros_like(ipdot))
    # the solver tolerance (1e-12) bounds the agreement
    assert relerr(ipdot, ref) <= 1e-9
