"""Batched solvers: several systems sharing the links in every Dslash.  Each
system must meet its own FP64 true residual (recomputed by the CPU oracle)
and agree with the oracle's FP64 solution to 1e-8 relative."""
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


def true_residual(o, u, ph, mass, x, b, shift=0.0):
    r = np.ascontiguousarray(b - o.mdagm(u, np.ascontiguousarray(x), ph, mass * mass + shift))
    return np.sqrt(o.norm2(r) / o.norm2(np.ascontiguousarray(b)))


@pytest.mark.parametrize("nsys", [1, 3, 8, 11])
def test_mixed_batch(lat_factory, nsys):
    from oracle import Oracle
    dims = (8, 8, 4, 8)
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 301)
    ph = F.staggered_phases(dims)
    b = np.stack([F.gaussian_vec3(dims, 310 + k) for k in range(nsys)])
    shifts = np.linspace(0.0, 0.3, nsys)
    x = lat.vec3(nsys)
    for a in (u, ph, b, x):
        lat.present(a)
    info = api.invert_mixed_batch(u, ph, 0.03, x, b, shifts, 1e-10)
    lat.update_host(x)
    assert info["status"] == 1, info
    for k in range(nsys):
        assert info["true_res"][k] <= 1e-10
        assert true_residual(o, u, ph, 0.03, x[k], b[k], shifts[k]) <= 1e-10
        _, _, xo = o.cg(u, ph, 0.03, np.ascontiguousarray(b[k]), 1e-10, shift=shifts[k])
        assert relerr(x[k], xo) <= 1e-8


def test_batched_generic_phases(lat_factory):
    from oracle import Oracle
    dims = (8, 4, 4, 8)
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 321)
    ph = F.staggered_phases(dims, im_chem_pot=0.2)
    b = np.stack([F.gaussian_vec3(dims, 330 + k) for k in range(2)])
    x = lat.vec3(2)
    for a in (u, ph, b, x):
        lat.present(a)
    info = api.invert_mixed_batch(u, ph, 0.05, x, b, None, 1e-10)
    lat.update_host(x)
    assert info["status"] == 1
    for k in range(2):
        assert true_residual(o, u, ph, 0.05, x[k], b[k]) <= 1e-10


@pytest.mark.parametrize("nrhs", [1, 3])
def test_multishift_batch(lat_factory, nrhs):
    from oracle import Oracle
    dims = (8, 8, 8, 4)
    o = Oracle(dims)
    lat = lat_factory(dims)
    ap = json.loads((GOLDEN / "ratapprox.json").read_text())["order8"]
    mx = 64.0 * 1.05
    eps = mx ** (ap["exponent_num"] / ap["exponent_den"])
    ra = api.make_approx(ap["a0"] * eps, np.array(ap["a"]) * mx * eps, np.array(ap["b"]) * mx)
    shifts = np.array(ap["b"]) * mx
    u = F.random_su3_links(dims, 341)
    ph = F.staggered_phases(dims)
    b = np.stack([F.gaussian_vec3(dims, 350 + k) for k in range(nrhs)])
    xs = lat.vec3(nrhs * len(shifts))
    for a in (u, ph, b, xs):
        lat.present(a)
    info = api.multishift_batch(u, ph, 0.05, ra, b, xs, 1e-10)
    lat.update_host(xs)
    assert info["status"] == 1, info
    xs = xs.reshape(nrhs, len(shifts), 3, -1)
    for r in range(nrhs):
        _, _, xo = o.cgm(u, ph, 0.05, shifts, np.ascontiguousarray(b[r]), 1e-10)
        for k in range(len(shifts)):
            assert info["true_res"][r, k] <= 1e-10
            assert true_residual(o, u, ph, 0.05, xs[r, k], b[r], shifts[k]) <= 1e-10
            assert relerr(xs[r, k], xo[k]) <= 1e-8


@pytest.mark.parametrize("fmt", ["f32", "q16"])
def test_mixed_batch_link_formats(lat_factory, fmt):
    """Both sloppy link formats of the batched FP32 iteration reach every
    system's FP64 target at a light mass."""
    from oracle import Oracle
    dims = (8, 8, 8, 8)
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 361)
    ph = F.staggered_phases(dims)
    b = np.stack([F.gaussian_vec3(dims, 370 + k) for k in range(4)])
    x = lat.vec3(4)
    for a in (u, ph, b, x):
        lat.present(a)
    prev = api.set_sloppy_links(fmt)
    try:
        info = api.invert_mixed_batch(u, ph, 0.01, x, b, None, 1e-10, 100000, 1e-4)
    finally:
        api.set_sloppy_links(prev)
    lat.update_host(x)
    assert info["status"] == 1, info
    for k in range(4):
        assert true_residual(o, u, ph, 0.01, x[k], b[k]) <= 1e-10
