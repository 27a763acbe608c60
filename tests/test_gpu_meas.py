"""GPU parity of the full-D inversion of the fermionic measurements
(eo_inversion, Meas/ferm_meas.c:50-71) through the C ABI.

* Against the oracle's even/odd inversion (the oracle's D_eo, D_oe and FP64
  CG, each pinned to the compiled reference) on Z2 noise sources: solutions
  within 1e-8 relative, in the FP64 and in the mixed-precision mode of
  inverter_wrapper.
* The definition: D (out_e, out_o) = (in_e, in_o) with D = [[m, D_eo],
  [D_oe, m]], recomputed on the CPU with the oracle's hops, to 1e-8.
* The chiral condensate estimator of the reference (degeneracy / 4 / V times
  <noise, D^-1 noise>) from the library's global scalar products equals the
  oracle's to 1e-9.
"""
import numpy as np
import pytest

from conftest import relerr
from openstaple_gb300 import api, fields as F

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,mass", [((8, 8, 8, 8), 0.1), ((4, 6, 8, 10), 0.05)])
@pytest.mark.parametrize("mixed", [0, 1])
def test_eo_inversion_matches_oracle(gpu, dims, mass, mixed):
    from oracle import Oracle
    lat = api.Lattice(dims)
    try:
        u = F.random_su3_links(dims, 611, eps=0.3)
        ph = F.staggered_phases(dims)
        in_e, in_o = F.z2_noise_vec3(dims, 612, 1), F.z2_noise_vec3(dims, 612, 2)
        out_e, out_o, phi_e, phi_o = (lat.vec3() for _ in range(4))
        r, h, s, p = (lat.vec3() for _ in range(4))
        for a in (u, ph, in_e, in_o, out_e, out_o, phi_e, phi_o, r, h, s, p):
            lat.present(a)
        t = api.inverter_tricks()
        t.useMixedPrecision = mixed
        try:
            fp = api.make_ferm_param(mass, ph)
            ip = api.make_inverter_package(u, r, h, s, p)
            api.eo_inversion(ip, fp, 1e-10, 10000, in_e, in_o, out_e, out_o, phi_e, phi_o)
            cc = api.chiral_condensate(in_e, in_o, out_e, out_o, 4, 2 * lat.sizeh)
        finally:
            t.useMixedPrecision = 0
        lat.update_host(out_e)
        lat.update_host(out_o)
        o = Oracle(dims, threads=4)
        st, n, xe, xo = o.eo_inversion(u, ph, mass, in_e, in_o, 1e-10)
        assert st == 1 and n > 0
        assert relerr(out_e, xe) <= 1e-8
        assert relerr(out_o, xo) <= 1e-8
        # D x = noise, recomputed on the CPU
        re = mass * out_e + o.Deo(u, out_o, ph) - in_e
        ro = o.Doe(u, out_e, ph) + mass * out_o - in_o
        assert np.sqrt((np.sum(np.abs(re) ** 2) + np.sum(np.abs(ro) ** 2)) /
                       (np.sum(np.abs(in_e) ** 2) + np.sum(np.abs(in_o) ** 2))) <= 1e-8
        want = 4 * 0.25 / (2 * lat.sizeh) * (np.vdot(in_e, xe) + np.vdot(in_o, xo))
        assert abs(cc - want) <= 1e-9 * abs(want)
    finally:
        lat.close()
