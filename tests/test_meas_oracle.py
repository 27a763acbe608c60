"""The oracle's even/odd full-D inversion (Meas/ferm_meas.c:50-71) against
its definition on the CPU: D (out_e, out_o) = (in_e, in_o) with D = [[m,
D_eo], [D_oe, m]] to 1e-8, on Z2 noise (random_assignement.c:215-250
draws +-1 per colour with probability 1/2); and against the same
composition of the reference's own compiled pieces."""
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


def test_oracle_eo_inversion_matches_the_reference_pieces(built):
    """The oracle's composition against the same composition of the
    reference's own compiled acc_Deo, ker_invert_openacc and acc_Doe
    (oracle/_ref): the same iteration count, solutions within 1e-12.
    ferm_meas.c itself needs the reference's generated single-precision
    headers and is not compiled."""
    import pytest
    from oracle import Oracle, Reference, ref_available
    dims, mass = (4, 6, 8, 10), 0.05
    if not ref_available(dims):
        pytest.skip("reference not compiled here (no reference source tree)")
    r, o = Reference(dims), Oracle(dims)
    ph = r.phases()
    u = F.random_su3_links(dims, 73, eps=0.3)
    in_e, in_o = F.z2_noise_vec3(dims, 74, 1), F.z2_noise_vec3(dims, 74, 2)
    phi_e = mass * in_e - r.Deo(u, in_o, ph)
    st_r, n_r, xe_r = r.cg(u, ph, mass, phi_e, 1e-10)
    xo_r = (in_o - r.Doe(u, xe_r, ph)) / mass
    st, n, xe, xo = o.eo_inversion(u, ph, mass, in_e, in_o, 1e-10)
    assert (st, n) == (st_r, n_r)
    for got, want in ((xe, xe_r), (xo, xo_r)):
        assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)
