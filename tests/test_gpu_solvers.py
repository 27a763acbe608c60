"""GPU parity of the FP64 solvers (ker_invert_openacc, multishift_invert,
recombine_shifted_vec3_to_vec3) through the C ABI.

Bar: same INVERTER_SUCCESS/FAILURE status and the same iteration count as the
reference (golden vectors from its compiled code) or the oracle; solutions
within 1e-9 relative of theirs (a CG solution to a 1e-10 residual is only
defined to that level); and an FP64 true residual <= the target, recomputed
on the CPU by the oracle."""
import json

import numpy as np
import pytest

from conftest import GOLDEN, load_golden, relerr
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
    api.set_restarting_every(10000)


def approx8_rescaled():
    ap = json.loads((GOLDEN / "ratapprox.json").read_text())["order8"]
    mx = 64.0 * 1.05
    eps = mx ** (ap["exponent_num"] / ap["exponent_den"])
    return ap["a0"] * eps, np.array(ap["a"]) * mx * eps, np.array(ap["b"]) * mx


def true_residual(o, u, ph, mass, x, b, shift=0.0):
    r = b - o.mdagm(u, x, ph, mass * mass + shift)
    return np.sqrt(o.norm2(np.ascontiguousarray(r)) / o.norm2(b))


@pytest.mark.parametrize("tag", ["4x4x4x4", "4x6x8x10", "8x8x8x8"])
def test_cg_matches_reference(lat_factory, tag):
    from oracle import Oracle
    g = load_golden(tag)
    dims = tuple(int(d) for d in g["dims"])
    lat = lat_factory(dims)
    o = Oracle(dims)
    u = F.random_su3_links(dims, int(g["link_seed"]))
    b = F.gaussian_vec3(dims, int(g["src_seed"]))
    ph = F.staggered_phases(dims)
    m = float(g["mass"])
    x = lat.vec3()
    work = [lat.vec3() for _ in range(4)]
    for a in (u, b, ph, x, *work):
        lat.present(a)
    st, n = api.ker_invert_openacc(u, api.make_ferm_param(m, ph), x, b, 1e-10, *work, 10000, 0.0)
    lat.update_host(x)
    assert st == 1 and n == int(g["cg_iters"])
    assert relerr(x, g["cg_x"]) <= 1e-9
    assert true_residual(o, u, ph, m, x, b) <= 1e-10


@pytest.mark.parametrize("tag", ["4x4x4x4", "4x6x8x10", "8x8x8x8"])
def test_eigenvalue_bounds_match_reference(lat_factory, tag):
    """find_min_max_eigenvalue_soloopenacc and ker_find_min_eigenvalue_openacc
    against the reference's own outputs (golden): the power iteration
    stops at the same step, so the bound and the last product agree to
    rounding."""
    g = load_golden(tag)
    dims = tuple(int(d) for d in g["dims"])
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, int(g["link_seed"]))
    p1 = F.gaussian_vec3(dims, int(g["src_seed"]))
    ph = F.staggered_phases(dims)
    m = float(g["mass"])
    r, h, p2 = lat.vec3(), lat.vec3(), lat.vec3()
    for a in (u, ph, p1, r, h, p2):
        lat.present(a)
    pars = api.make_ferm_param(m, ph)
    mm = api.find_min_max_eigenvalue_soloopenacc(u, pars, r, h, p1, p2)
    lat.update_host(p1)
    assert mm[0] == m * m
    assert abs(mm[1] - g["eig_minmax"][1]) <= 1e-12 * mm[1]
    assert relerr(p1, g["eig_p"]) <= 1e-10
    p = F.gaussian_vec3(dims, int(g["src_seed"]))
    lat.present(p)
    mn = api.ker_find_min_eigenvalue_openacc(u, pars, r, h, p, mm[1])
    assert abs(mn - float(g["eig_min"])) <= 1e-12 * abs(mn)


def test_cg_restarts_and_shift(lat_factory):
    from oracle import Oracle
    dims = (4, 4, 8, 8)
    lat = lat_factory(dims)
    o = Oracle(dims)
    u = F.random_su3_links(dims, 51)
    b = F.gaussian_vec3(dims, 52)
    ph = F.staggered_phases(dims)
    x0 = F.gaussian_vec3(dims, 53) * 0.01          # non-zero initial guess is used
    api.set_restarting_every(17)
    st_o, n_o, x_o = o.cg(u, ph, 0.05, b, 1e-10, shift=0.2, restart=17, x0=x0)
    x = x0.copy()
    work = [lat.vec3() for _ in range(4)]
    for a in (u, b, ph, x, *work):
        lat.present(a)
    st, n = api.ker_invert_openacc(u, api.make_ferm_param(0.05, ph), x, b, 1e-10, *work, 10000, 0.2)
    lat.update_host(x)
    assert (st, n) == (st_o, n_o) == (1, n_o)
    assert relerr(x, x_o) <= 1e-9
    assert true_residual(o, u, ph, 0.05, x, b, 0.2) <= 1e-10


def test_cg_max_iterations_reports_failure(lat_factory):
    dims = (4, 4, 4, 4)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 61)
    b = F.gaussian_vec3(dims, 62)
    ph = F.staggered_phases(dims)
    x = lat.vec3()
    work = [lat.vec3() for _ in range(4)]
    for a in (u, b, ph, x, *work):
        lat.present(a)
    api.set_restarting_every(5)
    st, n = api.ker_invert_openacc(u, api.make_ferm_param(0.1, ph), x, b, 1e-10, *work, 5, 0.0)
    assert (st, n) == (0, 5)


@pytest.mark.parametrize("tag", ["4x4x4x4", "4x6x8x10", "8x8x8x8"])
def test_multishift_matches_reference(lat_factory, tag):
    from oracle import Oracle
    g = load_golden(tag)
    dims = tuple(int(d) for d in g["dims"])
    lat = lat_factory(dims)
    o = Oracle(dims)
    u = F.random_su3_links(dims, int(g["link_seed"]))
    b = F.gaussian_vec3(dims, int(g["src_seed"]))
    ph = F.staggered_phases(dims)
    m = float(g["mass"])
    a0, a, sh = approx8_rescaled()
    ra = api.make_approx(a0, a, sh)
    xs = lat.vec3(len(a))
    ps = lat.vec3(len(a))
    work = [lat.vec3() for _ in range(4)]
    rec = lat.vec3()
    for arr in (u, b, ph, xs, ps, rec, *work):
        lat.present(arr)
    st, n = api.multishift_invert(u, api.make_ferm_param(m, ph), ra, xs, b, 1e-10, *work, ps, 10000)
    lat.update_host(xs)
    assert st == 1 and n == int(g["cgm_iters"])
    assert relerr(xs, g["cgm_xs"]) <= 1e-9
    for k in range(len(a)):
        assert true_residual(o, u, ph, m, np.ascontiguousarray(xs[k]), b, sh[k]) <= 1e-10 * 1.2
    api.recombine_shifted_vec3_to_vec3(xs, b, rec, ra)
    lat.update_host(rec)
    assert relerr(rec, g["cgm_recombined"]) <= 1e-9


def test_blas_and_reductions(lat_factory):
    dims = (8, 4, 4, 4)
    lat = lat_factory(dims)
    a = F.gaussian_vec3(dims, 71)
    b = F.gaussian_vec3(dims, 72)
    out = lat.vec3()
    for arr in (a, b, out):
        lat.present(arr)
    assert abs(api.l2norm2_global(a) - np.sum(np.abs(a) ** 2)) <= 1e-12 * np.sum(np.abs(a) ** 2)
    rd = np.sum(a.real * b.real + a.imag * b.imag)
    assert abs(api.real_scal_prod_global(a, b) - rd) <= 1e-12 * abs(rd) + 1e-12
    cd = np.sum(np.conj(a) * b)
    assert abs(api.scal_prod_global(a, b) - cd) <= 1e-12 * abs(cd)
    from openstaple_gb300.native import lib
    L = lib()
    L.combine_in1xfactor_plus_in2(a.ctypes.data, 0.3, b.ctypes.data, out.ctypes.data)
    assert relerr(lat.update_host(out), 0.3 * a + b) <= 1e-15
    L.combine_in1_minus_in2_allxfact(a.ctypes.data, b.ctypes.data, 1.7, out.ctypes.data)
    assert relerr(lat.update_host(out), 1.7 * (a - b)) <= 1e-15
    L.combine_in1xferm_mass2_minus_in2_minus_in3(a.ctypes.data, 0.4, b.ctypes.data, a.ctypes.data,
                                                 out.ctypes.data)
    assert relerr(lat.update_host(out), 0.4 * a - b - a) <= 1e-15
    # reductions are deterministic (bitwise equal on repeat)
    assert api.l2norm2_global(a) == api.l2norm2_global(a)
