"""GPU parity of the staggered Dirac operator and M^+M through the C ABI,
against the CPU oracle on identical inputs.  Tolerance (FP64): 1e-13 relative
(max-norm), as stated for the Dslash parity."""
import numpy as np
import pytest

from conftest import load_golden, relerr
from openstaple_gb300 import api, fields as F

pytestmark = pytest.mark.gpu
TOL = 1e-13


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


@pytest.mark.parametrize("dims", [(4, 4, 4, 4), (8, 8, 8, 8), (4, 6, 8, 10), (2, 2, 2, 2), (16, 8, 4, 6)])
def test_deo_doe_host_buffers(lat_factory, dims):
    from oracle import Oracle
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 21)
    v = F.gaussian_vec3(dims, 22)
    ph = F.staggered_phases(dims)
    out = lat.vec3()
    for a in (u, v, ph, out):
        lat.present(a)
    api.acc_Deo(u, out, v, ph)
    lat.update_host(out)
    assert relerr(out, o.Deo(u, v, ph)) <= TOL
    api.acc_Doe(u, out, v, ph)
    lat.update_host(out)
    assert relerr(out, o.Doe(u, v, ph)) <= TOL


def test_generic_phases_take_the_sincos_path(lat_factory):
    from oracle import Oracle
    dims = (4, 4, 4, 8)
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 31)
    v = F.gaussian_vec3(dims, 32)
    ph = F.staggered_phases(dims, im_chem_pot=0.37)
    assert not np.all((ph == 0) | (ph == np.pi))
    out = lat.vec3()
    for a in (u, v, ph, out):
        lat.present(a)
    api.acc_Deo(u, out, v, ph)
    lat.update_host(out)
    assert relerr(out, o.Deo(u, v, ph)) <= TOL


@pytest.mark.parametrize("tag", ["4x4x4x4", "4x6x8x10", "8x8x8x8"])
def test_dirac_against_reference_golden(lat_factory, tag):
    g = load_golden(tag)
    dims = tuple(int(d) for d in g["dims"])
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, int(g["link_seed"]))
    v = F.gaussian_vec3(dims, int(g["src_seed"]))
    ph = F.staggered_phases(dims)
    out, tmp = lat.vec3(), lat.vec3()
    for a in (u, v, ph, out, tmp):
        lat.present(a)
    api.acc_Deo(u, out, v, ph)
    assert relerr(lat.update_host(out), g["Deo"]) <= TOL
    api.acc_Doe(u, out, v, ph)
    assert relerr(lat.update_host(out), g["Doe"]) <= TOL
    m = float(g["mass"])
    fp = api.make_ferm_param(m, ph)
    api.fermion_matrix_multiplication(u, out, v, tmp, fp)
    assert relerr(lat.update_host(out), g["mdagm"]) <= TOL
    api.fermion_matrix_multiplication_shifted(u, out, v, tmp, fp, 0.37)
    assert relerr(lat.update_host(out), g["mdagm_shift"]) <= TOL


def test_device_pointers_from_torch(lat_factory):
    """Device buffers (no registration) are used in place."""
    import torch
    from oracle import Oracle
    dims = (8, 4, 4, 4)
    o = Oracle(dims)
    lat_factory(dims)
    u = F.random_su3_links(dims, 41)
    v = F.gaussian_vec3(dims, 42)
    ph = F.staggered_phases(dims)
    tu = torch.from_numpy(u.view(np.float64)).cuda()
    tv = torch.from_numpy(v.view(np.float64)).cuda()
    tp = torch.from_numpy(ph).cuda()
    to = torch.zeros_like(tv)
    torch.cuda.synchronize()
    api.acc_Doe(tu, to, tv, tp)
    from openstaple_gb300.native import lib
    lib().ostaple_synchronize()
    out = to.cpu().numpy().view(np.complex128)
    assert relerr(out, o.Doe(u, v, ph)) <= TOL


def test_unregistered_host_pointer_is_an_error(lat_factory):
    dims = (4, 4, 4, 4)
    lat_factory(dims)
    u = F.random_su3_links(dims, 1)
    v = F.gaussian_vec3(dims, 2)
    ph = F.staggered_phases(dims)
    out = np.zeros_like(v)
    with pytest.raises(RuntimeError, match="neither registered"):
        api.acc_Deo(u, out, v, ph)


@pytest.mark.parametrize("dims", [(4, 4, 4, 4), (8, 8, 8, 8), (4, 6, 8, 10)])
def test_double_float_mdagm_matches_fp64(lat_factory, dims):
    """M^+M in double-float arithmetic (the operator of the mixed solvers'
    intermediate reliable updates) against the FP64 oracle: 1e-13 relative,
    the FP64 Dslash tolerance; in practice ~1e-14."""
    from oracle import Oracle
    o = Oracle(dims)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 31)
    v = F.gaussian_vec3(dims, 32)
    ph = F.staggered_phases(dims)
    out = lat.vec3()
    for a in (u, v, ph, out):
        lat.present(a)
    for mass, shift in ((0.05, 0.0), (0.01, 0.37)):
        api.mdagm_df(u, ph, mass, out, v, shift)
        lat.update_host(out)
        assert relerr(out, o.mdagm(u, v, ph, mass * mass + shift)) <= TOL


def test_double_float_mdagm_needs_exact_phases(lat_factory):
    dims = (4, 4, 4, 4)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 33)
    v = F.gaussian_vec3(dims, 34)
    ph = F.staggered_phases(dims, 0.3)
    out = lat.vec3()
    for a in (u, v, ph, out):
        lat.present(a)
    with pytest.raises(RuntimeError, match="phases must be 0 or pi"):
        api.mdagm_df(u, ph, 0.05, out, v)
