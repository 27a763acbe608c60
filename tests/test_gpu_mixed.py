"""Mixed-precision CG (FP32 iteration, FP64 reliable updates): the FP64 true
residual recomputed by the CPU oracle must meet the 1e-10 target, and the
solution must agree with the FP64 oracle solution to the accuracy that target
implies (1e-8 relative here)."""
import numpy as np
import pytest

from conftest import quantise_links, relerr
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
    r = np.ascontiguousarray(b - o.mdagm(u, x, ph, mass * mass + shift))
    return np.sqrt(o.norm2(r) / o.norm2(b))


@pytest.mark.parametrize("dims,mass,every", [((8, 8, 8, 8), 0.05, 0), ((8, 8, 8, 8), 0.01, 50),
                                              ((4, 6, 8, 10), 0.1, 0), ((16, 8, 8, 8), 0.02, 25)])
def test_mixed_reaches_fp64_target(lat_factory, dims, mass, every):
    from oracle import Oracle
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 81)
    b = F.gaussian_vec3(dims, 82)
    ph = F.staggered_phases(dims)
    x = lat.vec3()
    for a in (u, b, ph, x):
        lat.present(a)
    info = api.invert_mixed(u, ph, mass, 0.0, x, b, 1e-10, 20000, every)
    lat.update_host(x)
    assert info["status"] == 1, info
    assert info["true_res"] <= 1e-10
    assert true_residual(o, u, ph, mass, x, b) <= 1e-10
    st, n, x_o = o.cg(u, ph, mass, b, 1e-10)
    assert relerr(x, x_o) <= 1e-8
    # the FP32 recursion needs at least as many iterations as FP64 CG, but not
    # wildly more
    assert n * 0.8 <= info["iters"] <= 3 * n + 50


def test_reference_mixed_entry_point(lat_factory):
    """inverter_mixed_precision with the reference's semantics: the caller's
    parking vectors, the delta criterion, success iff the FP64 true residual
    meets the target."""
    from oracle import Oracle
    dims = (8, 8, 4, 4)
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 91)
    b = F.gaussian_vec3(dims, 92)
    ph = F.staggered_phases(dims)
    x = lat.vec3()
    r, h, s, p = (lat.vec3() for _ in range(4))
    rf, hf, sf, pf, of = (np.zeros((3, lat.sizeh), np.complex64) for _ in range(5))
    for a in (u, b, ph, x, r, h, s, p, rf, hf, sf, pf, of):
        lat.present(a)
    ip = api.make_inverter_package(u, r, h, s, p, None, rf, hf, sf, pf, of)
    fp = api.make_ferm_param(0.05, ph)
    st, n = api.inverter_mixed_precision(ip, fp, x, b, 1e-9, 10000, 0.0)
    lat.update_host(x)
    tr = true_residual(o, u, ph, 0.05, x, b)
    assert st == (1 if tr <= 1e-9 else 0)
    assert tr <= 1e-9 * 1.5
    # the wrapper dispatches on inverter_tricks.useMixedPrecision
    from openstaple_gb300.native import inverter_tricks, lib
    import ctypes
    inverter_tricks().useMixedPrecision = 1
    try:
        x[:] = 0
        lat.update_device(x)
        n2 = lib().inverter_wrapper(ip, ctypes.byref(fp), x.ctypes.data, b.ctypes.data, 1e-9, 10000, 0.0, 0)
        assert n2 == n
    finally:
        inverter_tricks().useMixedPrecision = 0


def test_mixed_with_generic_phases(lat_factory):
    """Non-0/pi phases switch the FP32 kernels to angle mode."""
    from oracle import Oracle
    dims = (8, 4, 4, 8)
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 93)
    b = F.gaussian_vec3(dims, 94)
    ph = F.staggered_phases(dims, im_chem_pot=0.25)
    x = lat.vec3()
    for a in (u, b, ph, x):
        lat.present(a)
    info = api.invert_mixed(u, ph, 0.05, 0.1, x, b, 1e-10, 20000, 0)
    lat.update_host(x)
    assert info["status"] == 1
    assert true_residual(o, u, ph, 0.05, x, b, 0.1) <= 1e-10


@pytest.mark.parametrize("fmt", ["f32", "q16"])
@pytest.mark.parametrize("im_chem_pot", [0.0, 0.2])
def test_sloppy_operator(lat_factory, fmt, im_chem_pot):
    """The FP32 iteration's M^+M with each sloppy link format: against the
    FP64 oracle on the links the kernels see (FP32 arithmetic, 2e-6), and for
    the 16-bit links against the exact links (quantisation, 1e-4)."""
    from oracle import Oracle
    dims = (8, 4, 6, 8)
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 91)
    ph = F.staggered_phases(dims, im_chem_pot=im_chem_pot)
    b = F.gaussian_vec3(dims, 92)
    out = lat.vec3()
    for a in (u, ph, b, out):
        lat.present(a)
    prev = api.set_sloppy_links(fmt)
    try:
        api.mdagm_sloppy(u, ph, 0.03, out, b, shift=0.01)
    finally:
        api.set_sloppy_links(prev)
    lat.update_host(out)
    m2 = 0.03 ** 2 + 0.01
    seen = quantise_links(u, "q16") if fmt == "q16" else u
    assert relerr(out, o.mdagm(seen, b, ph, m2)) <= 2e-6
    if fmt == "q16":
        assert relerr(out, o.mdagm(u, b, ph, m2)) <= 1e-4


def test_q16_links_converge_like_f32(lat_factory):
    """Both sloppy link formats reach the FP64 target; the 16-bit links cost
    at most a few per cent more iterations."""
    from oracle import Oracle
    dims = (16, 8, 8, 8)
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 93)
    b = F.gaussian_vec3(dims, 94)
    ph = F.staggered_phases(dims)
    x = lat.vec3()
    for a in (u, b, ph, x):
        lat.present(a)
    iters = {}
    for fmt in ("f32", "q16"):
        prev = api.set_sloppy_links(fmt)
        try:
            x[:] = 0
            lat.update_device(x)
            info = api.invert_mixed(u, ph, 0.01, 0.0, x, b, 1e-10, 20000, 0, 1e-4)
        finally:
            api.set_sloppy_links(prev)
        lat.update_host(x)
        assert info["status"] == 1, (fmt, info)
        assert true_residual(o, u, ph, 0.01, x, b) <= 1e-10
        iters[fmt] = info["iters"]
    assert iters["q16"] <= 1.1 * iters["f32"] + 5, iters
