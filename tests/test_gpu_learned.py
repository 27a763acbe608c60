"""Learned preconditioner on the GPU (tcgen05 BF16 forward/backward) against
the CPU oracle (oracle/learned_ref.py).

Tolerances: the forward pass is compared with the oracle that rounds
weights, transported vectors and hidden activations to BF16 at the same
points (FP32 accumulation order and FP32 links remain): 2e-2 relative in the
2-norm.  Gradients of the residual loss |A (N(b) - x)|^2 / |b|^2 use BF16
tensor-core operands and the FP32 operator against the oracle's exact FP64
gradient: 5e-2 relative in the 2-norm.  The flexible CG is judged by
the FP64 true residual recomputed by the CPU oracle (<= 1e-10)."""
import numpy as np
import pytest

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


def nrel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _weights(seed, scale=0.2):
    return np.random.default_rng(seed).uniform(-scale, scale, (4, 64, 8)).astype(np.float32)


@pytest.mark.parametrize("dims", [(8, 8, 8, 8), (4, 6, 8, 10), (16, 8, 4, 4)])
def test_forward_matches_oracle(lat_factory, dims):
    from oracle import learned_ref as R
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 401)
    ph = F.staggered_phases(dims)
    r = F.gaussian_vec3(dims, 402)
    z = lat.vec3()
    for a in (u, ph, r, z):
        lat.present(a)
    W = _weights(403)
    api.net_set_weights(W)
    api.net_apply(u, ph, r, z)
    lat.update_host(z)
    geo = R.Geometry(dims)
    zo = R.forward(geo, R.full_links(u), R.signs_of(ph), W.astype(np.float64), r, bf16=True)
    assert nrel(z, zo) <= 2e-2
    # and the network is linear: N(2r) = 2 N(r) exactly up to rounding
    r2 = 2.0 * r
    z2 = lat.vec3()
    lat.present(r2)
    lat.present(z2)
    api.net_apply(u, ph, r2, z2)
    lat.update_host(z2)
    assert nrel(z2, 2.0 * z) <= 1e-6


def test_gradient_matches_oracle(lat_factory):
    from oracle import Oracle
    from oracle import learned_ref as R
    dims = (8, 8, 4, 8)
    mass = 0.1
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 411)
    ph = F.staggered_phases(dims)
    b = F.gaussian_vec3(dims, 412)
    x = F.gaussian_vec3(dims, 413) * 0.3
    for a in (u, ph, b, x):
        lat.present(a)
    W = _weights(414)
    api.net_set_weights(W)
    dw, loss = api.net_gradient(u, ph, mass, b, x)
    geo = R.Geometry(dims)
    A = lambda v: o.mdagm(u, np.ascontiguousarray(v), ph, mass * mass)
    lo, dwo = R.loss_and_grad(geo, R.full_links(u), R.signs_of(ph), W.astype(np.float64), b, x, A)
    assert abs(loss - lo) <= 3e-2 * lo
    assert nrel(dw, dwo) <= 5e-2
    for layer in range(4):
        assert nrel(dw[layer], dwo[layer]) <= 5e-2


def test_training_reduces_loss_and_flexible_cg_converges(lat_factory):
    """Pairs from the solver itself, GPU training, then the preconditioned
    solve to an FP64 true residual of 1e-10 (checked on the CPU)."""
    from oracle import Oracle
    dims = (8, 8, 8, 8)
    mass = 0.05
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 421)
    ph = F.staggered_phases(dims)
    npairs = 8
    b = np.stack([F.gaussian_vec3(dims, 430 + k) for k in range(npairs)])
    x = lat.vec3(npairs)
    for a in (u, ph, b, x):
        lat.present(a)
    info = api.invert_mixed_batch(u, ph, mass, x, b, None, 1e-10)
    assert info["status"] == 1
    api.net_init(7, 0.05)
    hist = api.net_train(u, ph, mass, b, x, 60, 3e-3)
    assert np.all(np.isfinite(hist))
    assert hist[-1] < 0.8 * hist[0]
    src = F.gaussian_vec3(dims, 499)
    sol = lat.vec3()
    lat.present(src)
    lat.present(sol)
    res = api.invert_learned(u, ph, mass, 0.0, sol, src, 1e-10, 5000)
    lat.update_host(sol)
    assert res["status"] == 1
    r = np.ascontiguousarray(src - o.mdagm(u, sol, ph, mass * mass))
    assert np.sqrt(o.norm2(r) / o.norm2(src)) <= 1e-10


def test_zero_network_falls_back_to_plain_cg(lat_factory):
    """A zero network is no preconditioner at all (its output vanishes): the
    flexible CG must detect it and the plain CG must finish the solve."""
    dims = (8, 8, 4, 4)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 441)
    ph = F.staggered_phases(dims)
    src = F.gaussian_vec3(dims, 442)
    sol = lat.vec3()
    z = lat.vec3()
    for a in (u, ph, src, sol, z):
        lat.present(a)
    api.net_init(3, 0.1)
    api.net_set_weights(np.zeros((4, 64, 8), np.float32))
    assert np.abs(api.net_get_weights()).max() == 0.0
    api.net_apply(u, ph, src, z)
    assert np.abs(lat.update_host(z)).max() == 0.0
    res = api.invert_learned(u, ph, 0.1, 0.0, sol, src, 1e-10, 200)
    assert res["used_fallback"] == 1, res
    assert res["status"] == 1 and res["true_res"] <= 1e-10, res


def test_trained_network_gains_over_plain_cg(lat_factory):
    """What training buys: the network trained on solver-produced pairs cuts
    the flexible-CG iteration count well below plain CG's on a new source,
    without falling back, while the untrained (initial) network does not."""
    from oracle import Oracle
    dims = (8, 8, 8, 8)
    mass = 0.02
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 451)
    ph = F.staggered_phases(dims)
    npairs = 8
    b = np.stack([F.gaussian_vec3(dims, 460 + k) for k in range(npairs)])
    x = lat.vec3(npairs)
    src = F.gaussian_vec3(dims, 470)
    sol = lat.vec3()
    for a in (u, ph, b, x, src, sol):
        lat.present(a)
    info = api.invert_mixed_batch(u, ph, mass, x, b, None, 1e-10)
    assert info["status"] == 1
    plain_iters = int(info["iters"].max())
    api.net_init(11, 0.05)
    before = api.invert_learned(u, ph, mass, 0.0, sol, src, 1e-10, 3000)
    sol[:] = 0
    lat.update_device(sol)
    api.net_init(11, 0.05)
    hist = api.net_train(u, ph, mass, b, x, 200, 3e-3)
    after = api.invert_learned(u, ph, mass, 0.0, sol, src, 1e-10, 3000)
    lat.update_host(sol)
    print(f"plain CG {plain_iters} iterations; loss {hist[0]:.4f} -> {hist[-1]:.4f}; "
          f"flexible CG untrained {before}, trained {after}")
    assert after["status"] == 1 and after["used_fallback"] == 0, after
    r = np.ascontiguousarray(src - o.mdagm(u, sol, ph, mass * mass))
    assert np.sqrt(o.norm2(r) / o.norm2(src)) <= 1e-10
    assert after["iters"] <= 0.75 * plain_iters
    untrained_cost = before["iters"] if not before["used_fallback"] else 10 ** 9
    assert after["iters"] < untrained_cost
