"""Pins the CPU oracle (oracle/ostaple_oracle.c) to the reference.

* against the golden vectors produced by the reference's own compiled C code
  (tests/golden/, made by tests/golden/make_golden.py);
* against the reference compiled from source (oracle/_ref) where it is
  available (this is skipped on machines without the reference tree).
"""
import numpy as np
import pytest

from conftest import load_golden, relerr
from openstaple_gb300 import fields as F

GOLDEN_TAGS = ["4x4x4x4", "4x6x8x10", "8x8x8x8"]


def _inputs(g):
    dims = tuple(int(d) for d in g["dims"])
    u = F.random_su3_links(dims, int(g["link_seed"]))
    v = F.gaussian_vec3(dims, int(g["src_seed"]))
    # the generator must still produce the fixture's inputs
    assert np.isclose(np.sum(np.abs(u) ** 2), float(g["u_checksum"]), rtol=1e-14)
    assert np.isclose(np.sum(np.abs(v) ** 2), float(g["src_checksum"]), rtol=1e-14)
    return dims, u, v


@pytest.mark.parametrize("tag", GOLDEN_TAGS)
def test_oracle_matches_golden_dirac(built, tag):
    from oracle import Oracle
    g = load_golden(tag)
    dims, u, v = _inputs(g)
    o = Oracle(dims)
    ph = o.phases()
    assert np.array_equal(ph, F.staggered_phases(dims))
    assert relerr(o.Deo(u, v, ph), g["Deo"]) <= 1e-15
    assert relerr(o.Doe(u, v, ph), g["Doe"]) <= 1e-15
    m = float(g["mass"])
    assert relerr(o.mdagm(u, v, ph, m * m), g["mdagm"]) <= 1e-14
    assert relerr(o.mdagm(u, v, ph, m * m + 0.37), g["mdagm_shift"]) <= 1e-14


@pytest.mark.parametrize("tag", GOLDEN_TAGS)
def test_oracle_matches_golden_solvers(built, tag):
    import json
    from conftest import GOLDEN
    from oracle import Oracle
    g = load_golden(tag)
    dims, u, v = _inputs(g)
    o = Oracle(dims)
    ph = o.phases()
    m = float(g["mass"])
    st, n, x = o.cg(u, ph, m, v, 1e-10)
    assert st == int(g["cg_status"]) == 1
    assert n == int(g["cg_iters"])
    assert relerr(x, g["cg_x"]) <= 1e-12
    ap = json.loads((GOLDEN / "ratapprox.json").read_text())["order8"]
    mx = 64.0 * 1.05
    eps = mx ** (ap["exponent_num"] / ap["exponent_den"])
    a0, a, b = ap["a0"] * eps, np.array(ap["a"]) * mx * eps, np.array(ap["b"]) * mx
    st, n, xs = o.cgm(u, ph, m, b, v, 1e-10)
    assert st == int(g["cgm_status"]) == 1
    assert n == int(g["cgm_iters"])
    assert relerr(xs, g["cgm_xs"]) <= 1e-12
    assert relerr(o.recombine(xs, v, a0, a), g["cgm_recombined"]) <= 1e-12


@pytest.mark.parametrize("tag", GOLDEN_TAGS)
def test_oracle_matches_golden_eigenvalue_bounds(built, tag):
    from oracle import Oracle
    g = load_golden(tag)
    dims, u, v = _inputs(g)
    o = Oracle(dims)
    ph = o.phases()
    m = float(g["mass"])
    mx, loops, p, _ = o.find_max(u, ph, m, v)
    assert loops > 1
    assert g["eig_minmax"][0] == m * m
    assert abs(mx - g["eig_minmax"][1]) <= 1e-13 * mx
    assert relerr(p, g["eig_p"]) <= 1e-12
    mn, _, _, _ = o.find_min(u, ph, m, v, mx)
    assert abs(mn - float(g["eig_min"])) <= 1e-12 * abs(mn)


REF_DIMS = [(4, 4, 4, 4), (8, 8, 8, 8), (4, 6, 8, 10)]


@pytest.mark.parametrize("dims", REF_DIMS)
def test_oracle_matches_compiled_reference(built, dims):
    from oracle import Oracle, Reference, ref_available
    if not ref_available(dims):
        pytest.skip("reference not compiled here (no reference source tree)")
    r, o = Reference(dims), Oracle(dims)
    ph = r.phases()
    assert np.array_equal(o.phases(), ph)
    u = F.random_su3_links(dims, 101)
    v = F.gaussian_vec3(dims, 102)
    # same arithmetic up to the compiler's FMA contraction choices
    assert relerr(o.Deo(u, v, ph), r.Deo(u, v, ph)) <= 2e-16
    assert relerr(o.Doe(u, v, ph), r.Doe(u, v, ph)) <= 2e-16
    # a generic (imaginary chemical potential) phase exercises the cos/sin path
    ph2 = r.phases(0.3)
    assert np.array_equal(o.phases(0.3), ph2)
    assert relerr(o.Deo(u, v, ph2), r.Deo(u, v, ph2)) <= 1e-15
    st1, n1, x1 = o.cg(u, ph, 0.05, v, 1e-10, restart=40)
    st2, n2, x2 = r.cg(u, ph, 0.05, v, 1e-10, restart=40)
    assert (st1, n1) == (st2, n2)
    assert relerr(x1, x2) <= 1e-12
    mm, p2, _ = r.find_min_max(u, ph, 0.05, v)
    mx, _, p1, _ = o.find_max(u, ph, 0.05, v)
    assert mm[0] == 0.05 * 0.05
    assert abs(mx - mm[1]) <= 1e-13 * mx
    assert relerr(p1, p2) <= 1e-12


def test_oracle_cg_max_iterations_failure(built):
    """max_cg exhaustion reports INVERTER_FAILURE like the reference."""
    from oracle import Oracle
    dims = (4, 4, 4, 4)
    o = Oracle(dims)
    ph = o.phases()
    u = F.random_su3_links(dims, 3)
    v = F.gaussian_vec3(dims, 4)
    st, n, _ = o.cg(u, ph, 0.1, v, 1e-10, max_cg=5, restart=5)
    assert st == 0 and n == 5
