"""Launch-shape autotuner: every candidate shape of the tuned FP32 D_oe hops
(block size of the mixed solver, systems per thread of the batched and
multi-shift solvers) must give bitwise the same solutions, since the tuner
is only allowed to change speed."""
import json

import numpy as np
import pytest

from conftest import GOLDEN
from openstaple_gb300 import api, fields as F

pytestmark = pytest.mark.gpu

DIMS = (8, 8, 8, 8)
MASS = 0.03


@pytest.fixture
def lat(gpu):
    lat = api.Lattice(DIMS)
    yield lat
    api.autotune(True)
    lat.close()


def _approx():
    ap = json.loads((GOLDEN / "ratapprox.json").read_text())["order8"]
    mx = 64.0 * 1.05
    eps = mx ** (ap["exponent_num"] / ap["exponent_den"])
    return api.make_approx(ap["a0"] * eps, np.array(ap["a"]) * mx * eps, np.array(ap["b"]) * mx)


def _solve_all(lat, u, ph, b):
    """Mixed single solve, batched solve of 3 and of 8 systems, multi-shift
    of 3 sources; returns the solutions as host copies."""
    out = []
    x = lat.vec3()
    b0 = b[0].copy()
    lat.present(x)
    lat.present(b0)
    info = api.invert_mixed(u, ph, MASS, 0.0, x, b0, 1e-10)
    assert info["status"] == 1, info
    out.append(lat.update_host(x).copy())
    for nsys in (3, 8):
        xb = lat.vec3(nsys)
        lat.present(xb)
        bb = b[:nsys].copy()
        lat.present(bb)
        info = api.invert_mixed_batch(u, ph, MASS, xb, bb, np.linspace(0.0, 0.2, nsys), 1e-10)
        assert info["status"] == 1, info
        out.append(lat.update_host(xb).copy())
        lat.release(xb)
        lat.release(bb)
    ra = _approx()
    xs = lat.vec3(3 * ra.approx_order)
    bb = b[:3].copy()
    lat.present(xs)
    lat.present(bb)
    info = api.multishift_batch(u, ph, MASS, ra, bb, xs, 1e-10)
    assert info["status"] == 1, info
    out.append(lat.update_host(xs).copy())
    lat.release(xs)
    lat.release(bb)
    lat.release(x)
    lat.release(b0)
    return out


def test_every_shape_gives_the_same_bits(lat):
    u = F.random_su3_links(DIMS, 901)
    ph = F.staggered_phases(DIMS)
    b = np.stack([F.gaussian_vec3(DIMS, 910 + k) for k in range(8)])
    for a in (u, ph, b):
        lat.present(a)
    api.autotune(False)
    base = _solve_all(lat, u, ph, b)
    for cand in (1, 2, 3, 4, 5, 6):
        api.autotune_force(cand)
        got = _solve_all(lat, u, ph, b)
        for k, (g, r) in enumerate(zip(got, base)):
            assert np.array_equal(g.view(np.uint64), r.view(np.uint64)), (cand, k)
    api.autotune(True)
    got = _solve_all(lat, u, ph, b)
    for g, r in zip(got, base):
        assert np.array_equal(g.view(np.uint64), r.view(np.uint64))
    rep = api.autotune_report()
    for name in ("k_mx_doe", "k_b_doe", "k_cgm_doe"):
        assert name in rep, rep
