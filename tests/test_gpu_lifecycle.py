"""Library life cycle: finalize followed by a new ostaple_init, and a change
of geometry without finalize, must leave every reduction and every cached
CUDA graph valid.  Fresh device allocations hold whatever the previous owner
wrote, so the device memory is dirtied (all bits set) between the two
lattices; state derived from the old workspace (the reduction ticket counter,
captured iteration graphs keyed by buffer addresses) must be rebuilt."""
import numpy as np
import pytest

from openstaple_gb300 import api, fields as F

pytestmark = pytest.mark.gpu


def true_residual(o, u, ph, mass, x, b):
    r = np.ascontiguousarray(b - o.mdagm(u, x, ph, mass * mass))
    return np.sqrt(o.norm2(r) / o.norm2(b))


def solve_and_check(lat, dims, seed, mass=0.05):
    from oracle import Oracle
    o = Oracle(dims)
    u = F.random_su3_links(dims, seed)
    b = F.gaussian_vec3(dims, seed + 1)
    ph = F.staggered_phases(dims)
    x = lat.vec3()
    for a in (u, b, ph, x):
        lat.present(a)
    exact = float(np.sum(np.abs(b) ** 2))
    assert abs(api.l2norm2_global(b) - exact) <= 1e-12 * exact
    info = api.invert_mixed(u, ph, mass, 0.0, x, b, 1e-10, 20000, 0)
    lat.update_host(x)
    assert info["status"] == 1, info
    assert true_residual(o, u, ph, mass, x, b) <= 1e-10
    return info["iters"]


def dirty_device_memory():
    torch = pytest.importorskip("torch")
    t = torch.full((256 << 20,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    del t
    torch.cuda.empty_cache()


def test_reinit_after_finalize(gpu):
    dims = (8, 8, 8, 8)
    lat = api.Lattice(dims)
    n1 = solve_and_check(lat, dims, 301)
    lat.close()
    dirty_device_memory()
    lat = api.Lattice(dims)
    try:
        assert solve_and_check(lat, dims, 301) == n1
    finally:
        lat.close()


def test_geometry_change_without_finalize(gpu):
    big, small = (8, 8, 8, 16), (4, 4, 8, 8)
    lat = api.Lattice(big)
    try:
        solve_and_check(lat, big, 311)
        lat.release_all()
        lat2 = api.Lattice(small)     # same workspace buffers, smaller lattice
        solve_and_check(lat2, small, 321)
        lat2.release_all()
        lat3 = api.Lattice(big)
        solve_and_check(lat3, big, 331)
        lat3.release_all()
    finally:
        lat.close()
