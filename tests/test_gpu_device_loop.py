"""The solvers' iteration as one graph launch with its loop on the device
(conditional graph nodes: a while node around the captured iterations, an
if node for reliable updates) against the host-driven chunk loop: the same
kernels in the same order, so the solutions, iteration counts and residuals
are the same bits; the reliable-update path is exercised by an update every
20 iterations and by the default delta criterion."""
import json

import numpy as np
import pytest

from conftest import GOLDEN
from openstaple_gb300 import api, fields as F
from openstaple_gb300.native import lib

pytestmark = pytest.mark.gpu

DIMS = (8, 8, 8, 16)


@pytest.fixture
def lat(gpu):
    lat = api.Lattice(DIMS)
    yield lat
    lib().ostaple_device_loop(1)
    lat.close()


def _mixed(lat, u, ph, b, every):
    x = lat.vec3()
    lat.present(x)
    info = api.invert_mixed(u, ph, 0.02, 0.0, x, b, 1e-10, 100000, every, 1e-4)
    out = lat.update_host(x).copy()
    lat.release(x)
    return info, out


@pytest.mark.parametrize("every", [0, 20])
def test_mixed_device_loop_matches_host_loop(lat, every):
    u = F.random_su3_links(DIMS, 1301, eps=0.5)
    ph = F.staggered_phases(DIMS)
    b = F.gaussian_vec3(DIMS, 1302)
    for a in (u, ph, b):
        lat.present(a)
    L = lib()
    L.ostaple_device_loop(0)
    ih, xh = _mixed(lat, u, ph, b, every)
    L.ostaple_device_loop(1)
    idv, xd = _mixed(lat, u, ph, b, every)
    assert ih["status"] == 1 and idv["status"] == 1
    assert ih["iters"] == idv["iters"] and ih["n_reliable"] == idv["n_reliable"] > 0
    assert ih["true_res"] == idv["true_res"] <= 1e-10
    assert np.array_equal(xh.view(np.uint64), xd.view(np.uint64))
    # and again with the cached graph
    idv2, xd2 = _mixed(lat, u, ph, b, every)
    assert np.array_equal(xd2.view(np.uint64), xd.view(np.uint64)) and idv2["iters"] == idv["iters"]


def test_multishift_device_loop_matches_host_loop(lat):
    u = F.random_su3_links(DIMS, 1311, eps=0.5)
    ph = F.staggered_phases(DIMS)
    ap = json.loads((GOLDEN / "ratapprox.json").read_text())["order8"]
    mx = 64.0 * 1.05
    eps = mx ** (ap["exponent_num"] / ap["exponent_den"])
    ra = api.make_approx(ap["a0"] * eps, np.array(ap["a"]) * mx * eps, np.array(ap["b"]) * mx)
    bs = np.stack([F.gaussian_vec3(DIMS, 1312 + k) for k in range(3)])
    for a in (u, ph, bs):
        lat.present(a)
    L = lib()
    out = []
    for loop in (0, 1):
        L.ostaple_device_loop(loop)
        xs = lat.vec3(3 * ra.approx_order)
        lat.present(xs)
        info = api.multishift_batch(u, ph, 0.02, ra, bs, xs, 1e-10)
        assert info["status"] == 1 and info["true_res"].max() <= 1e-10
        out.append((info, lat.update_host(xs).copy()))
        lat.release(xs)
    (ih, xh), (idv, xd) = out
    assert np.array_equal(ih["iters_cgm"], idv["iters_cgm"])
    assert np.array_equal(xh.view(np.uint64), xd.view(np.uint64))
