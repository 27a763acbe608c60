"""Host-side generators and layout helpers."""
import numpy as np

from openstaple_gb300 import fields as F


def test_links_are_su3():
    u = F.random_su3_links((4, 4, 4, 4), 1)
    m = u.transpose(0, 3, 1, 2).reshape(-1, 3, 3)
    eye = np.eye(3)
    assert np.abs(m @ np.conj(np.swapaxes(m, 1, 2)) - eye).max() < 1e-13
    assert np.abs(np.linalg.det(m) - 1).max() < 1e-13
    # the third row equals conj(r0 x r1), the rebuild the kernels use
    r2 = np.conj(np.cross(m[:, 0], m[:, 1]))
    assert np.abs(r2 - m[:, 2]).max() < 1e-13


def test_generator_is_deterministic():
    a = F.gaussian_vec3((4, 4, 4, 4), 9)
    b = F.gaussian_vec3((4, 4, 4, 4), 9)
    c = F.gaussian_vec3((4, 4, 4, 4), 10)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    # variance 1/2 per real component (two_double_gauss)
    g = F.gaussians(3, 200000)
    assert abs(g.var() - 0.5) < 0.01


def test_phase_signs_cover_ks_and_apbc():
    dims = (4, 4, 4, 6)
    ph = F.staggered_phases(dims)
    s = F.sign_bytes(ph)
    lex, par, idx = F.site_parity_index(dims)
    n0, n1, n2, n3 = dims
    x = lex % n0
    y = (lex // n0) % n1
    z = (lex // (n0 * n1)) % n2
    t = lex // (n0 * n1 * n2)
    for mu, eta in enumerate([np.zeros_like(x), x & 1, (x + y) & 1, (x + y + z) & 1]):
        neg = eta.astype(bool)
        if mu == 3:
            neg = neg ^ (t == n3 - 1)
        assert np.array_equal(s[2 * mu + par, idx].astype(bool), neg)
