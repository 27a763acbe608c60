"""The oracle's even/odd full-D inversion (Meas/ferm_meas.c:50-71) against
its definition on the CPU: D (out_e, out_o) = (in_e, in_o) with D = [[m,
D_eo], [D_oe, m]] to 1e-8, on Z2 noise (random_assignement.c:215-250
draws +-1 per colour with probability 1/2)."""
import numpy as np

from openstaple_gb300 import fields as F


def test_oracle_eo_inversion_solves_full_d(built):
    from oracle import Oracle
    dims, mass = (4, 4, 4, 4), 0.1
    o = Oracle(dims)
    u = F.random_su3_links(dims, 71, eps=0.4)
    ph = F.staggered_phases(dims)
    in_e, in_o = F.z2_noise_vec3(dims, 72, 1), F.z2_noise_vec3(dims, 72, 2)
    assert set(np.unique(in_e.real)) == {-1.0, 1.0} and not in_e.imag.any()
    st, n, xe, xo = o.eo_inversion(u, ph, mass, in_e, in_o, 1e-10)
    assert st == 1
    re = mass * xe + o.Deo(u, xo, ph) - in_e
    ro = o.Doe(u, xe, ph) + mass * xo - in_o
    rel = np.sqrt((np.sum(np.abs(re) ** 2) + np.sum(np.abs(ro) ** 2)) /
                  (np.sum(np.abs(in_e) ** 2) + np.sum(np.abs(in_o) ** 2)))
    assert rel <= 1e-8
