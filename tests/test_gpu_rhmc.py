"""GPU parity of the RHMC molecular dynamics and whole RHMC updates through
the C ABI.

* multistep_2MN_SOLOOPENACC (one flavour of two pseudofermions, stout 2 x
  0.15, order-8 approx_md, 2 steps x 2 gauge substeps) against the
  reference's own run of it (tests/golden/rhmc_md_4x4x4x4.npz): links and
  momenta within 1e-9 relative (the fermion forces' multi-shift solves stop
  at 1e-12).
* ostaple_rhmc_trajectory on seeded links (one flavour, x^(1/8) heatbath,
  x^(-1/4) molecular dynamics and last inversion, rescaled to the measured
  spectrum): small energy violations that shrink about fourfold when the
  step halves (second-order integrator), and the same dS with the
  accelerated solvers (FP32 multi-shift + FP64 refinement) as with the FP64
  ones, within 1e-6.
"""
import ctypes as C
import json

import numpy as np
import pytest

from conftest import GOLDEN, relerr
from openstaple_gb300 import api, fields as F
from openstaple_gb300.native import FermParam

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
    t = api.inverter_tricks()
    t.singlePInvAccelMultiInv, t.useMixedPrecision, t.mixedPrecisionDelta, t.restartingEvery = 0, 0, 0.1, 10000
    from openstaple_gb300.native import act_params
    act_params().stout_steps = 2
    api.set_stout_rho(0.15)


def test_fermion_md_matches_reference_fixture(lat_factory):
    from openstaple_gb300.native import act_params, lib, md_parameters
    g = dict(np.load(GOLDEN / "rhmc_md_4x4x4x4.npz"))
    dims = tuple(int(d) for d in g["dims"])
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, int(g["link_seed"]), eps=float(g["eps"]))
    mom = F.gauge_momenta(dims, *[int(v) for v in g["mom"]])
    chis = np.stack([F.gaussian_vec3(dims, int(k)) for k in g["chi_seeds"]])
    assert np.isclose(np.sum(np.abs(u) ** 2), float(g["u_checksum"]), rtol=1e-14)
    a, b = g["a"], g["b"]
    order, sh, steps = len(a), lat.sizeh, int(g["steps"])
    ph = F.staggered_phases(dims)
    levels = api.su3_field(sh, 8 * steps)
    auxbis, aux = api.su3_field(sh), api.su3_field(sh)
    ipdot = api.alg_field(sh)
    shiftmulti, shifttemp = lat.vec3(order), lat.vec3(order)
    r, h, s, p = (lat.vec3() for _ in range(4))
    for arr in (u, mom, chis, ph, levels, auxbis, aux, ipdot, shiftmulti, shifttemp, r, h, s, p):
        lat.present(arr)
    act_params().stout_steps = steps
    act_params().beta = float(g["beta"])
    api.set_stout_rho(float(g["rho"]))
    mp = md_parameters()
    mp.no_md, mp.gauge_scale, mp.t = int(g["no_md"]), int(g["gauge_scale"]), float(g["t"])
    lib().initialize_md_global_variables(mp)
    fp = api.make_ferm_param(float(g["mass"]), ph)
    fp.number_of_ps = len(chis)
    fp.approx_md.approx_order = order
    for k in range(order):
        fp.approx_md.RA_a[k] = a[k]
        fp.approx_md.RA_b[k] = b[k]
    ip = api.make_inverter_package(u, r, h, s, p, ferm_shift_temp=shifttemp, nshifts=order)
    lib().multistep_2MN_SOLOOPENACC(ipdot.ctypes.data, u.ctypes.data, levels.ctypes.data, auxbis.ctypes.data,
                                    aux.ctypes.data, C.byref(fp), 1, chis.ctypes.data, shiftmulti.ctypes.data, ip,
                                    mom.ctypes.data, None, float(g["res"]), 10000)
    api.check(0, "multistep_2MN_SOLOOPENACC")
    assert relerr(lat.update_host(u)[:, :2], g["md_u"]) <= 1e-9
    assert relerr(lat.update_host(mom), g["md_mom"]) <= 1e-9


def _approx(key):
    ap = json.loads((GOLDEN / "ratapprox.json").read_text())[key]
    ra = api.RationalApprox()
    ra.exponent_num, ra.exponent_den, ra.approx_order = ap["exponent_num"], ap["exponent_den"], ap["order"]
    ra.lambda_min, ra.lambda_max, ra.error, ra.RA_a0 = ap["lambda_min"], ap["lambda_max"], ap["error"], ap["a0"]
    for k in range(ap["order"]):
        ra.RA_a[k], ra.RA_b[k] = ap["a"][k], ap["b"][k]
    return ra


def _flavour(ph, mass, nps):
    fps = (FermParam * 1)()
    fp = fps[0]
    fp.ferm_mass, fp.degeneracy, fp.number_of_ps, fp.index_of_the_first_ps = mass, 1, nps, 0
    fp.phases = ph.ctypes.data
    fp.approx_fi_mother = _approx("fi_1_over_8")     # x^(+1/8): deg / (8 nps)
    fp.approx_md_mother = _approx("order8")          # x^(-1/4): -deg / (4 nps)
    fp.approx_li_mother = _approx("order19")         # x^(-1/4), more precise
    return fps


def _trajectory(lat_factory, dims, no_md, accel=0, mixed=0, nps=1, traj=0):
    lat = lat_factory(dims)
    u = F.random_su3_links(dims, 801, eps=0.25)
    ph = F.staggered_phases(dims)
    lat.present(u)
    lat.present(ph)
    t = api.inverter_tricks()
    t.singlePInvAccelMultiInv, t.useMixedPrecision = accel, mixed
    out = api.rhmc_trajectory(u, _flavour(ph, 0.1, nps), 5.0, no_md, 2, traj_len=0.5, res_metro=1e-11,
                              res_md=1e-10, seed=802, traj=traj, metropolis=True)
    lat.close()
    return out


def test_rhmc_energy_violation_is_second_order(lat_factory):
    dims = (4, 4, 4, 4)
    a = _trajectory(lat_factory, dims, 3)
    b = _trajectory(lat_factory, dims, 6)
    assert abs(a["delta_s"]) < 1.0, a
    assert abs(b["delta_s"]) < abs(a["delta_s"]) / 2.5, (a, b)
    # the fermion action before the update is |phi|^2: 3 sizeh on average
    assert abs(a["action"][2] / (3 * F.sizeh(dims)) - 1.0) < 0.2


@pytest.mark.parametrize("accel,mixed,nps", [(1, 0, 1), (1, 1, 2)])
def test_rhmc_accelerated_solvers_give_the_same_update(lat_factory, accel, mixed, nps):
    dims = (4, 4, 4, 4)
    ref = _trajectory(lat_factory, dims, 3, nps=nps)
    got = _trajectory(lat_factory, dims, 3, accel=accel, mixed=mixed, nps=nps)
    assert abs(got["delta_s"] - ref["delta_s"]) <= 1e-6, (ref, got)
    assert got["accepted"] == ref["accepted"]
