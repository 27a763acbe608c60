"""GPU parity of the pure-gauge tree-level Symanzik HMC through the C ABI.

* Against fixtures written by the reference's own compiled code
  (tests/golden/hmc_*.npz): the gauge staples and force (1e-13 relative,
  max-norm), the plaquette, rectangle and momentum sums (1e-13), the momentum
  kick and the link update (1e-13), two multistep_2MN_gauge calls with
  initialize_md_global_variables (1e-12).
* The device momentum and Gaussian-vector generators against the host field
  helpers (1e-15).
* Properties of whole trajectories of the link generator (FP64 and FP32
  molecular dynamics): reversibility of the FP64 integrator to 1e-11, energy
  conservation improving with the step size, FP32 against FP64 molecular
  dynamics, and a short thermalisation from a cold start.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN, relerr, sample_alg, sample_sites
from openstaple_gb300 import api, fields as F

pytestmark = pytest.mark.gpu

HMC_TAGS = ["4x4x4x4", "4x6x8x10"]


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


def _fixture(tag):
    g = dict(np.load(GOLDEN / f"hmc_{tag}.npz"))
    dims = tuple(int(d) for d in g["dims"])
    u = F.random_su3_links(dims, int(g["link_seed"]), eps=float(g["eps"]))
    mom = F.gauge_momenta(dims, int(g["mom_seed"]), int(g["mom_stream"]))
    assert np.isclose(np.sum(np.abs(u) ** 2), float(g["u_checksum"]), rtol=1e-14)
    return g, dims, u, mom


@pytest.mark.parametrize("tag", HMC_TAGS)
def test_gauge_hmc_pieces_match_reference_fixture(lat_factory, tag):
    from openstaple_gb300.native import lib
    L = lib()
    g, dims, u, mom = _fixture(tag)
    lat = lat_factory(dims)
    sh = lat.sizeh
    stap, stap_parts = api.su3_field(sh), api.su3_field(sh)
    ip, ip2 = api.alg_field(sh), api.alg_field(sh)
    m = mom.copy()
    ue = u.copy()
    for a in (u, stap, stap_parts, ip, ip2, m, ue):
        lat.present(a)
    api.calc_ipdot_gauge_soloopenacc(u, stap, ip)
    assert relerr(sample_sites(lat.update_host(stap), g), g["staples"]) <= 1e-13
    assert relerr(sample_alg(lat.update_host(ip), g), g["ipdot"]) <= 1e-13
    # the same staples from the four reference-named parts, then TA(U S)
    for f in (L.calc_loc_staples_nnptrick_all, L.calc_loc_improved_staples_typeA_nnptrick_all,
              L.calc_loc_improved_staples_typeB_nnptrick_all, L.calc_loc_improved_staples_typeC_nnptrick_all):
        f(u.ctypes.data, stap_parts.ctypes.data)
    L.conf_times_staples_ta_part(u.ctypes.data, stap_parts.ctypes.data, ip2.ctypes.data)
    assert relerr(sample_sites(lat.update_host(stap_parts), g), g["staples"]) <= 1e-13
    assert relerr(sample_alg(lat.update_host(ip2), g), g["ipdot"]) <= 1e-13
    pl, re = api.calc_plaquette_soloopenacc(u), api.calc_rettangolo_soloopenacc(u)
    assert abs(pl - float(g["plaq_sum"])) <= 1e-13 * abs(float(g["plaq_sum"]))
    assert abs(re - float(g["rect_sum"])) <= 1e-13 * abs(float(g["rect_sum"]))
    assert abs(api.momenta_action(m) - float(g["mom_action"])) <= 1e-13 * float(g["mom_action"])
    api.mom_sum_mult(m, ip, -0.02)
    assert relerr(sample_alg(lat.update_host(m), g), g["mom_sum_mult"]) <= 1e-13
    m[:] = mom
    lat.update_device(m)
    api.mom_exp_times_conf_soloopenacc(ue, m, 0.05)
    assert relerr(sample_sites(lat.update_host(ue)[:, :2], g), g["mom_exp"]) <= 1e-13
    # two gauge multisteps of the 2MN integrator
    api.multistep_2MN_gauge(u, stap, ip, m, float(g["md_beta"]), int(g["md_no_md"]), int(g["md_gauge_scale"]),
                            float(g["md_t"]), int(g["md_ncalls"]))
    from openstaple_gb300.native import deltas_omelyan
    assert np.array_equal(np.array(deltas_omelyan()[:]), g["deltas"])
    assert relerr(sample_sites(lat.update_host(u)[:, :2], g), g["md_u"]) <= 1e-12
    assert relerr(sample_alg(lat.update_host(m), g), g["md_mom"]) <= 1e-12


def test_device_momenta_equal_the_host_generator(lat_factory):
    dims = (4, 6, 8, 10)
    lat = lat_factory(dims)
    mom = api.alg_field(lat.sizeh)
    lat.present(mom)
    api.gauge_momenta(mom, 77, 5)
    assert relerr(lat.update_host(mom), F.gauge_momenta(dims, 77, 5)) <= 1e-15
    # 1/2 tr P^2 of Gaussian momenta: 4 per link on average (8 deviates of variance 1/2)
    assert abs(api.momenta_action(mom) / (8 * lat.sizeh) - 4.0) < 0.1


def test_device_gaussian_vectors_equal_the_host_generator(lat_factory):
    from openstaple_gb300.native import lib
    dims = (4, 6, 8, 10)
    lat = lat_factory(dims)
    v = lat.vec3()
    lat.present(v, copy=False)
    assert lib().ostaple_gaussian_vec3(v.ctypes.data, 123, 7) == 0
    assert relerr(lat.update_host(v), F.gaussian_vec3(dims, 123, 7)) <= 1e-15


def _md_trajectory(lat, u, mom, stap, ip, beta, no_md, gs, t):
    # a pure-gauge trajectory: 2 no_md gauge multisteps
    api.multistep_2MN_gauge(u, stap, ip, mom, beta, no_md, gs, t, ncalls=2 * no_md)


def test_fp64_integrator_is_reversible(lat_factory):
    """Integrate a trajectory, flip the momenta, integrate again: the links
    come back to 1e-11 (the integrator is time-reversible up to rounding)."""
    dims = (4, 4, 4, 8)
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 91, eps=0.6)
    u0 = u.copy()
    mom = F.gauge_momenta(dims, 92, 0)
    stap, ip = api.su3_field(lat.sizeh), api.alg_field(lat.sizeh)
    for a in (u, mom, stap, ip):
        lat.present(a)
    _md_trajectory(lat, u, mom, stap, ip, 3.75, 4, 2, 1.0)
    lat.update_host(mom)
    mom *= -1.0
    lat.update_device(mom)
    _md_trajectory(lat, u, mom, stap, ip, 3.75, 4, 2, 1.0)
    assert relerr(lat.update_host(u)[:, :2], u0[:, :2]) <= 1e-11


def test_hmc_energy_violation_falls_with_the_step(lat_factory):
    """|delta S| of the same trajectory (same links and momenta) with the
    2MN integrator at 4 and 8 steps: second order, so about 4x smaller."""
    dims = (4, 4, 4, 4)
    lat = lat_factory(dims)
    res = []
    for no_md in (4, 8):
        u = F.random_su3_links(dims, 95, eps=0.5)
        lat.present(u)
        out = api.pure_gauge_hmc(u, 3.75, 1, no_md=no_md, gauge_scale=1, seed=96, metropolis=False)
        res.append(abs(out["delta_s"][0]))
        lat.release(u)
    assert res[1] < res[0] / 2.5, res


def test_fp32_molecular_dynamics_follows_fp64(lat_factory):
    """The same trajectory in FP32 and FP64 molecular dynamics: links within
    1e-4 and delta S within 0.02 of each other."""
    dims = (8, 8, 8, 8)
    lat = lat_factory(dims)
    u64 = F.random_su3_links(dims, 97, eps=0.4)
    u32 = u64.copy()
    lat.present(u64)
    lat.present(u32)
    a = api.pure_gauge_hmc(u64, 3.75, 1, no_md=6, gauge_scale=2, seed=98, metropolis=False, precision="fp64")
    b = api.pure_gauge_hmc(u32, 3.75, 1, no_md=6, gauge_scale=2, seed=98, metropolis=False, precision="fp32")
    assert relerr(lat.update_host(u32)[:, :2], lat.update_host(u64)[:, :2]) <= 1e-4
    assert abs(a["delta_s"][0] - b["delta_s"][0]) <= 0.02, (a, b)
    # the generator's FP64 reunitarisation: rows orthonormal to FP64 precision
    r0, r1 = u32[:, 0], u32[:, 1]
    assert np.abs(np.sum(np.abs(r0) ** 2, axis=1) - 1).max() <= 1e-14
    assert np.abs(np.sum(np.conj(r0) * r1, axis=1)).max() <= 1e-14


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_thermalisation_from_a_cold_start(lat_factory, precision):
    """From unit links at beta = 3.75: six trajectories without the Metropolis
    test (from the identity the test fails for the first trajectories; the
    reference's ThermNtraj trajectories skip it, update_versatile.c:581),
    then eight with it.  The plaquette falls from 1, the Metropolis phase
    accepts most trajectories, and the action the library reports equals the
    one from the plaquette and rectangle sums."""
    dims = (8, 8, 8, 8)
    lat = lat_factory(dims)
    u = F.cold_links(dims)
    lat.present(u)
    therm = api.pure_gauge_hmc(u, 3.75, 6, no_md=8, gauge_scale=2, seed=7, precision=precision, metropolis=False)
    assert therm["accepted"] == 6
    assert therm["plaquette"][-1] < 0.9, therm["plaquette"]
    out = api.pure_gauge_hmc(u, 3.75, 8, no_md=8, gauge_scale=2, seed=7, first_traj=6, precision=precision)
    assert out["accepted"] >= 6, out
    assert 0.4 < out["plaquette"][-1] < 0.9, out["plaquette"]
    act = api.gauge_action(u, 3.75)
    pl = api.calc_plaquette_soloopenacc(u)
    assert abs(act["plaq_sum"] - pl) <= 1e-12 * abs(pl)
    want = -3.75 / 3 * (5 / 3 * act["plaq_sum"] - 1 / 12 * act["rect_sum"])
    assert abs(act["action"] - want) <= 1e-12 * abs(want)
    assert abs(act["plaq_sum"] / (18 * 2 * lat.sizeh) - out["plaquette"][-1]) <= 1e-12
