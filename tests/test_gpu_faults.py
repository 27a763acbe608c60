"""Fault injection on the GPU path, made on the host (no kernel is made to
fault, trap or hang): non-finite sources and guesses, iteration-limit
exhaustion, a learned preconditioner corrupted host-side, and a bounded
device wait that is made to run out.  Every case ends in the reference's
INVERTER_FAILURE or in a plain-CG fallback, quickly, and leaves the library
usable."""
import time

import numpy as np
import pytest

from conftest import relerr
from openstaple_gb300 import api, fields as F

pytestmark = pytest.mark.gpu


@pytest.fixture
def setup(gpu):
    dims = (8, 8, 8, 8)
    lat = api.Lattice(dims)
    u = F.random_su3_links(dims, 601)
    ph = F.staggered_phases(dims)
    b = F.gaussian_vec3(dims, 602)
    x = lat.vec3()
    for a in (u, ph, b, x):
        lat.present(a)
    yield dims, lat, u, ph, b, x
    lat.close()


def _healthy_solve(lat, u, ph, b, x):
    x[:] = 0
    lat.update_device(x)
    info = api.invert_mixed(u, ph, 0.05, 0.0, x, b, 1e-10, 20000, 0, 1e-4)
    assert info["status"] == 1 and info["true_res"] <= 1e-10


def test_nan_source_fails_fast(setup):
    dims, lat, u, ph, b, x = setup
    bad = b.copy()
    bad[1, 17] = np.nan
    lat.present(bad)
    t0 = time.time()
    info = api.invert_mixed(u, ph, 0.05, 0.0, x, bad, 1e-10, 20000, 0, 1e-4)
    assert info["status"] == 0 and not np.isfinite(info["true_res"])
    assert time.time() - t0 < 5.0
    st, n = api.ker_invert_openacc(u, api.make_ferm_param(0.05, ph), x, bad, 1e-10,
                                   *[lat.present(lat.vec3()) for _ in range(4)], 1000, 0.0)
    assert st == 0
    _healthy_solve(lat, u, ph, b, x)


def test_inf_guess_fails_fast(setup):
    dims, lat, u, ph, b, x = setup
    x[:] = 0
    x[0, 3] = np.inf
    lat.update_device(x)
    info = api.invert_mixed(u, ph, 0.05, 0.0, x, b, 1e-10, 20000, 0, 1e-4)
    assert info["status"] == 0
    _healthy_solve(lat, u, ph, b, x)


def test_batched_nonfinite_system_fails_alone(setup):
    dims, lat, u, ph, b, x = setup
    bs = np.stack([F.gaussian_vec3(dims, 610 + k) for k in range(3)])
    bs[1, 2, 5] = np.inf
    xs = lat.vec3(3)
    lat.present(bs)
    lat.present(xs)
    info = api.invert_mixed_batch(u, ph, 0.05, xs, bs, None, 1e-10)
    assert info["status"] == 0
    tr = info["true_res"]
    assert not np.isfinite(tr[1])
    assert tr[0] <= 1e-10 and tr[2] <= 1e-10


def test_iteration_limit_exhaustion(setup):
    dims, lat, u, ph, b, x = setup
    x[:] = 0
    lat.update_device(x)
    info = api.invert_mixed(u, ph, 0.01, 0.0, x, b, 1e-10, 20, 0, 1e-4)
    assert info["status"] == 0 and info["iters"] <= 28


def test_corrupted_network_falls_back_to_plain_cg(setup):
    dims, lat, u, ph, b, x = setup
    api.net_init(1, 0.05)
    w = api.net_get_weights()
    w[2, 10, 3] = np.nan                       # corrupted host-side, then uploaded
    api.net_set_weights(w)
    x[:] = 0
    lat.update_device(x)
    res = api.invert_learned(u, ph, 0.05, 0.0, x, b, 1e-10, 500)
    assert res["used_fallback"] == 1
    assert res["status"] == 1 and res["true_res"] <= 1e-10


def test_bounded_wait_runs_out_and_reports(setup):
    dims, lat, u, ph, b, x = setup
    from openstaple_gb300.native import lib
    L = lib()
    assert L.ostaple_selftest_bounded_wait(1) == 0
    with pytest.raises(RuntimeError, match="did not complete within its wait limit"):
        api.check(L.ostaple_selftest_bounded_wait(0), "ostaple_selftest_bounded_wait")
    # the context is intact: the next operator application matches the oracle
    from oracle import Oracle
    out = lat.vec3()
    lat.present(out)
    api.acc_Deo(u, out, b, ph)
    lat.update_host(out)
    assert relerr(out, Oracle(dims).Deo(u, b, ph)) <= 1e-13
    _healthy_solve(lat, u, ph, b, x)
