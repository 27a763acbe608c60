"""GPU parity of the stout and fermion-force entry points against fixtures
written by the reference's own compiled C (tests/golden/make_golden.py):
every kernel of the chain is called through the C ABI on the fixture's
seeded inputs and compared at the fixture's sites.

Tolerances (relative, max-norm): 1e-13 for the staples, Q_A, the stout
levels, exp(-Q_A) U, the outer products, the backfield and TA steps; 1e-12
for Lambda and Sigma (their Cayley-Hamilton derivative coefficients divide
by (9u^2 - w^2)^2); 1e-9 for a whole force, whose multi-shift solves stop at
a residual of 1e-12; for the 16^4 configuration 1e-9 for the CG-M solutions
(both stop at 1e-10 after the same number of iterations) and 1e-8 for its
force."""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN, load_gauge_fixture, relerr, sample_alg, sample_sites
from openstaple_gb300 import api, fields as F

pytestmark = pytest.mark.gpu

GAUGE_TAGS = ["4x4x4x4_e0.3", "4x4x4x4_e0.01", "4x6x8x10_e0.05"]


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
    from openstaple_gb300.native import act_params
    act_params().stout_steps = 2


def _force(lat, u, ph, mass, a, b, phis, res, steps=2):
    """fermion_force_soloopenacc of one flavour with len(phis) pseudofermions
    through the C ABI; returns ipdot (tamat_soa[8])."""
    from openstaple_gb300.native import act_params, lib
    order = len(a)
    stout_levels = api.su3_field(lat.sizeh, 8 * steps)
    gl3, taux = api.su3_field(lat.sizeh), api.su3_field(lat.sizeh)
    ipdot = api.alg_field(lat.sizeh)
    shiftmulti, shifttemp = lat.vec3(order), lat.vec3(order)
    r, h, s, p = (lat.vec3() for _ in range(4))
    phis = np.ascontiguousarray(phis)
    for arr in (u, ph, phis, stout_levels, gl3, ipdot, taux, shiftmulti, shifttemp, r, h, s, p):
        lat.present(arr)
    act_params().stout_steps = steps
    fp = api.make_ferm_param(mass, ph)
    fp.number_of_ps = len(phis)
    fp.index_of_the_first_ps = 0
    fp.approx_md.approx_order = order
    for k in range(order):
        fp.approx_md.RA_a[k] = a[k]
        fp.approx_md.RA_b[k] = b[k]
    ip = api.make_inverter_package(u, r, h, s, p, ferm_shift_temp=shifttemp, nshifts=order)
    lib().fermion_force_soloopenacc(u.ctypes.data, stout_levels.ctypes.data, gl3.ctypes.data, ipdot.ctypes.data,
                                    C.byref(fp), 1, phis.ctypes.data, res, taux.ctypes.data,
                                    shiftmulti.ctypes.data, ip, 10000)
    api.check(0, "fermion_force_soloopenacc")
    return lat.update_host(ipdot)


@pytest.mark.parametrize("tag", GAUGE_TAGS)
def test_gauge_kernels_match_reference_fixture(lat_factory, tag):
    from openstaple_gb300.native import lib
    L = lib()
    g, dims, u, sig, xs, phis = load_gauge_fixture(tag)
    lat = lat_factory(dims)
    rho = float(g["rho"])
    api.set_stout_rho(rho)
    sh = lat.sizeh
    ph = F.staggered_phases(dims)
    up, stap, tmp = api.su3_field(sh), api.su3_field(sh), api.su3_field(sh)
    qa, lam = api.alg_field(sh), api.alg_field(sh)
    levels = api.su3_field(sh, 16)
    expo = api.su3_field(sh)
    s_sig = sig.copy()
    s_chain = sig.copy()
    for a in (u, sig, ph, up, stap, tmp, qa, lam, levels, expo, s_sig, s_chain):
        lat.present(a)
    # stout_isotropic: staples (C_0-weighted), Q_A and one smeared level
    api.stout_isotropic(u, up, stap, None, qa, 0)
    assert relerr(sample_sites(lat.update_host(stap), g), g["staples"]) <= 1e-13
    assert relerr(sample_alg(lat.update_host(qa), g), g["qa"]) <= 1e-13
    assert relerr(sample_sites(lat.update_host(up)[:, :2], g), g["stout1"]) <= 1e-13
    # stout_wrapper: two levels
    api.stout_wrapper(u, levels, 0)
    lat.update_host(levels)
    assert relerr(sample_sites(levels[:8, :2], g), g["stout1"]) <= 1e-13
    assert relerr(sample_sites(levels[8:, :2], g), g["stout2"]) <= 1e-13
    # exp(-Q_A) U with the Q_A computed above
    L.exp_minus_QA_times_conf(u.ctypes.data, qa.ctypes.data, expo.ctypes.data, tmp.ctypes.data)
    assert relerr(sample_sites(lat.update_host(expo)[:, :2], g), g["exp_qa_u"]) <= 1e-13
    # Lambda, then Sigma from Lambda, one by one
    L.compute_lambda(lam.ctypes.data, sig.ctypes.data, u.ctypes.data, qa.ctypes.data, tmp.ctypes.data)
    assert relerr(sample_alg(lat.update_host(lam), g), g["lambda"]) <= 1e-12
    L.compute_sigma(lam.ctypes.data, u.ctypes.data, s_sig.ctypes.data, qa.ctypes.data, tmp.ctypes.data, 0)
    assert relerr(sample_sites(lat.update_host(s_sig), g), g["sigma"]) <= 1e-12
    # the whole Sigma' -> Sigma step of one level
    api.compute_sigma_from_sigma_prime_backinto_sigma_prime(s_chain, lam, qa, u, tmp, 0)
    assert relerr(sample_sites(lat.update_host(s_chain), g), g["sigma_prime_to_sigma"]) <= 1e-12
    api.check(0, "gauge chain")


@pytest.mark.parametrize("tag", GAUGE_TAGS)
def test_force_pieces_match_reference_fixture(lat_factory, tag):
    g, dims, u, sig, xs, phis = load_gauge_fixture(tag)
    lat = lat_factory(dims)
    sh = lat.sizeh
    ph = F.staggered_phases(dims)
    aux, pip = api.su3_field(sh), api.su3_field(sh)
    ip = api.alg_field(sh)
    s, h = lat.vec3(), lat.vec3()
    xs = np.ascontiguousarray(xs)
    for arr in (u, ph, xs, aux, pip, ip, s, h):
        lat.present(arr)
    a = g["force_a"]
    fp = api.make_ferm_param(float(g["force_mass"]), ph)
    fp.approx_md.approx_order = len(a)
    for k, v in enumerate(a):
        fp.approx_md.RA_a[k] = v
    api.ker_openacc_compute_fermion_force(u, aux, xs, s, h, fp)
    assert relerr(sample_sites(lat.update_host(aux), g), g["force_outer"]) <= 1e-13
    api.multiply_backfield_times_force(fp, aux, pip)
    assert relerr(sample_sites(lat.update_host(pip), g), g["backfield"]) <= 1e-13
    api.multiply_conf_times_force_and_take_ta_nophase(u, pip, ip)
    assert relerr(sample_alg(lat.update_host(ip), g), g["conf_force_ta"]) <= 1e-13


@pytest.mark.parametrize("tag", GAUGE_TAGS)
def test_fermion_force_matches_reference_fixture(lat_factory, tag):
    """fermion_force_soloopenacc with two pseudofermions and the order-8
    approx_md against the reference's own run of it."""
    g, dims, u, sig, xs, phis = load_gauge_fixture(tag)
    lat = lat_factory(dims)
    api.set_stout_rho(float(g["rho"]))
    ph = F.staggered_phases(dims)
    ip = _force(lat, u, ph, float(g["force_mass"]), g["md_a"], g["md_b"], phis, 1e-12)
    assert relerr(sample_alg(ip, g), g["fermion_force"]) <= 1e-9


def test_config2_16x16x16x16_matches_reference_fixture(lat_factory):
    """The 16^4 configuration: seeded links after 2 stout steps of
    rho = 0.15, m = 0.05, order-8 x^(-1/4) CG-M to 1e-10 per shift (same
    iteration count as the reference), the recombined result, the FP32/FP64
    batched multi-shift solver on the same system, and the rational force."""
    g = dict(np.load(GOLDEN / "config2_16x16x16x16.npz"))
    dims = tuple(int(d) for d in g["dims"])
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, int(g["link_seed"]))
    phi = F.gaussian_vec3(dims, int(g["src_seed"]))
    assert np.isclose(np.sum(np.abs(u) ** 2), float(g["u_checksum"]), rtol=1e-14)
    rho, mass, res = float(g["rho"]), float(g["mass"]), float(g["res"])
    api.set_stout_rho(rho)
    ph = F.staggered_phases(dims)
    levels = api.su3_field(lat.sizeh, 16)
    for arr in (u, ph, phi, levels):
        lat.present(arr)
    api.stout_wrapper(u, levels, 0)
    lat.update_host(levels)
    assert relerr(sample_sites(levels[8:, :2], g), g["stout2"]) <= 1e-13
    u2 = levels[8:].copy()   # its own buffer: a view would alias the registered levels
    lat.present(u2)
    order = len(g["a"])
    approx = api.make_approx(float(g["a0"]), g["a"], g["b"])
    xs = lat.vec3(order)
    ps = lat.vec3(order)
    work = [lat.vec3() for _ in range(4)]
    for arr in (xs, ps, *work):
        lat.present(arr)
    st, n = api.multishift_invert(u2, api.make_ferm_param(mass, ph), approx, xs, phi, res, *work, ps, 10000)
    assert st == int(g["cgm_status"]) == 1
    assert n == int(g["cgm_iters"])
    lat.update_host(xs)
    assert relerr(sample_sites(xs, g), g["cgm_xs"]) <= 1e-9
    rec = lat.vec3()
    lat.present(rec)
    api.recombine_shifted_vec3_to_vec3(xs, phi, rec, approx)
    assert relerr(sample_sites(lat.update_host(rec), g), g["recombined"]) <= 1e-9
    # the batched FP32 CG-M + FP64-guaranteed refinement on the same system
    xb = lat.vec3(order)
    lat.present(xb)
    info = api.multishift_batch(u2, ph, mass, approx, phi[None], xb[None], res=res)
    assert info["status"] == 1
    assert np.max(info["true_res"]) <= res
    lat.update_host(xb)
    assert relerr(sample_sites(xb, g), g["cgm_xs"]) <= 1e-8
    ip = _force(lat, u, ph, mass, g["a"], g["b"], phi[None], res)
    assert relerr(sample_alg(ip, g), g["fermion_force"]) <= 1e-8
