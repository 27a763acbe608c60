"""Seeded field generators and layout helpers (host side).

Fields are numpy arrays in the reference's SoA layouts over the half lattice
(``sizeh = V/2``):

* spinor ``vec3_soa``: complex128 ``(3, sizeh)``
* links ``su3_soa[8]``: complex128 ``(8, 3, 3, sizeh)``, index ``2*mu+parity``
* phases ``double_soa[8]``: float64 ``(8, sizeh)``

The random numbers come from a counter-based generator (splitmix64 of
``seed`` and the element counter, Box-Muller) so that the same seed gives the
same field on every machine and numpy version.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniforms(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """n uniforms in (0, 1) from (seed, stream, counter)."""
    base = _splitmix64(np.uint64(seed & 0xFFFFFFFF) * np.uint64(0x100000001) + np.uint64(stream))
    ctr = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        bits = _splitmix64(ctr * np.uint64(0xD1B54A32D192ED03) + base)
    return ((bits >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def gaussians(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """n normal deviates of variance 1/2 (the reference's two_double_gauss,
    random_assignement.c:44-55: radius sqrt(-log u))."""
    m = (n + 1) // 2
    u1 = uniforms(seed, m, 2 * stream)
    u2 = uniforms(seed, m, 2 * stream + 1)
    rad = np.sqrt(-np.log(u1))
    phi = 2 * np.pi * u2
    out = np.empty(2 * m)
    out[0::2] = rad * np.cos(phi)
    out[1::2] = rad * np.sin(phi)
    return out[:n]


def sizeh(dims) -> int:
    n0, n1, n2, n3 = dims
    return n0 * n1 * n2 * n3 // 2


def gaussian_vec3(dims, seed: int, stream: int = 7) -> np.ndarray:
    """Gaussian complex 3-vector per half-lattice site, complex128 (3, sizeh)."""
    sh = sizeh(dims)
    g = gaussians(seed, 6 * sh, stream)
    return (g[0::2] + 1j * g[1::2]).reshape(3, sh).copy()


def z2_noise_vec3(dims, seed: int, stream: int = 11) -> np.ndarray:
    """Z2 noise per half-lattice site and colour: +1 or -1 with probability
    1/2 each, imaginary part zero, as the noise vectors of the fermionic
    measurements (random_assignement.c:215-250).  complex128 (3, sizeh)."""
    sh = sizeh(dims)
    return np.where(uniforms(seed, 3 * sh, stream) < 0.5, 1.0, -1.0).reshape(3, sh).astype(np.complex128)


def random_su3_links(dims, seed: int, eps: float = 0.3, stream: int = 1, chunk: int = 1 << 20) -> np.ndarray:
    """U = exp(i eps H) per link, H Gaussian traceless Hermitian.

    Returns complex128 (8, 3, 3, sizeh) in su3_soa[8] layout (all three rows
    filled; the kernels read the first two)."""
    sh = sizeh(dims)
    nl = 8 * sh
    out = np.empty((nl, 3, 3), dtype=np.complex128)
    for s0 in range(0, nl, chunk):
        m = min(chunk, nl - s0)
        g = gaussians(seed, 18 * m, stream * 1000003 + s0 // chunk)
        a = (g[0::2] + 1j * g[1::2]).reshape(m, 3, 3)
        h = 0.5 * (a + np.conj(np.swapaxes(a, 1, 2)))
        tr = np.trace(h, axis1=1, axis2=2).real / 3.0
        h[:, 0, 0] -= tr
        h[:, 1, 1] -= tr
        h[:, 2, 2] -= tr
        w, v = np.linalg.eigh(h)
        ph = np.exp(1j * eps * w)
        out[s0:s0 + m] = np.einsum("nij,nj,nkj->nik", v, ph, np.conj(v))
    return np.ascontiguousarray(out.reshape(8, sh, 3, 3).transpose(0, 2, 3, 1))


def staggered_phases(dims, im_chem_pot: float = 0.0) -> np.ndarray:
    """Per-link phase angles: staggered eta phases and antiperiodic time
    boundary (backfield.c:20-187 with no external field), float64 (8, sizeh).

    angle = 2*pi*fold(0.5*[eta_mu(x) = -1] + mu_I/(2 N_t) [t-links]
                      + 0.5*[t = N_t - 1] [t-links]),  fold() into [-1/2, 1/2].
    """
    n0, n1, n2, n3 = dims
    sh = sizeh(dims)
    t, z, y, x = np.meshgrid(np.arange(n3), np.arange(n2), np.arange(n1), np.arange(n0), indexing="ij")
    lex = x + n0 * (y + n1 * (z + n2 * t))
    par = (x + y + z + t) % 2
    idx = lex // 2
    eta_neg = [np.zeros_like(x), x & 1, (x + y) & 1, (x + y + z) & 1]
    ph = np.zeros((8, sh))
    for mu in range(4):
        a = 0.5 * eta_neg[mu].astype(np.float64)
        if mu == 3:
            a = a + 0.5 * (im_chem_pot / n3) + 0.5 * (t == n3 - 1)
        while np.any(a > 0.5):
            a = np.where(a > 0.5, a - 1.0, a)
        while np.any(a < -0.5):
            a = np.where(a < -0.5, a + 1.0, a)
        a = a * (2 * 3.14159265358979323846)
        for p in (0, 1):
            m = par == p
            ph[2 * mu + p, idx[m]] = a[m]
    return ph


def sign_bytes(phases: np.ndarray) -> np.ndarray:
    """Phase angles in {0, pi} as one byte per link (1 = negative)."""
    neg = phases == np.float64(0.5 * (2 * 3.14159265358979323846))
    if not np.all(neg | (phases == 0.0)):
        raise ValueError("phases are not all 0 or pi")
    return neg.astype(np.uint8)


def site_parity_index(dims):
    """(lex, parity, idx) of every site, lexicographic order x fastest."""
    n0, n1, n2, n3 = dims
    t, z, y, x = np.meshgrid(np.arange(n3), np.arange(n2), np.arange(n1), np.arange(n0), indexing="ij")
    lex = (x + n0 * (y + n1 * (z + n2 * t))).ravel()
    par = ((x + y + z + t) % 2).ravel()
    return lex, par, lex // 2


def cold_links(dims) -> np.ndarray:
    """Every link the identity (a cold start), complex128 (8, 3, 3, sizeh)."""
    sh = sizeh(dims)
    u = np.zeros((8, 3, 3, sh), np.complex128)
    for r in range(3):
        u[:, r, r] = 1.0
    return u


def gauge_momenta(dims, seed: int, stream: int) -> np.ndarray:
    """The traceless Hermitian momenta thmat_soa[8], float64 (8, 8*sizeh),
    that the library's device generator makes from (seed, stream): per link
    eight normal deviates g of variance 1/2 (the counter-based generator of
    this module) composed as random_assignement.c:173-177:
    rc00 = g2 + g7/sqrt(3), rc11 = -g2 + g7/sqrt(3), c01 = g0 - i g1,
    c02 = g3 - i g4, c12 = g5 - i g6."""
    sh = sizeh(dims)
    g = gaussians(seed, 64 * sh, stream).reshape(8, sh, 8)
    r3 = 1.0 / np.sqrt(3.0)
    mom = np.zeros((8, 8 * sh))
    c = mom[:, :6 * sh].view(np.complex128).reshape(8, 3, sh)
    c[:, 0] = g[:, :, 0] - 1j * g[:, :, 1]
    c[:, 1] = g[:, :, 3] - 1j * g[:, :, 4]
    c[:, 2] = g[:, :, 5] - 1j * g[:, :, 6]
    mom[:, 6 * sh:7 * sh] = g[:, :, 2] + g[:, :, 7] * r3
    mom[:, 7 * sh:] = -g[:, :, 2] + g[:, :, 7] * r3
    return mom
