"""The CPU oracle of the learned preconditioner itself: its FP64 gradient
matches finite differences, and the network is gauge covariant."""
import numpy as np

from openstaple_gb300 import fields as F


def _setup(dims=(4, 4, 4, 4), seed=5):
    from oracle import learned_ref as R
    geo = R.Geometry(dims)
    u = F.random_su3_links(dims, seed)
    ph = F.staggered_phases(dims)
    U = R.full_links(u, fp32=False)
    sg = R.signs_of(ph)
    rng = np.random.default_rng(seed)
    W = rng.uniform(-0.2, 0.2, (4, 64, 8))
    return R, geo, u, ph, U, sg, W


def test_gradient_matches_finite_differences(built):
    """The residual loss |A (N(b) - x)|^2 / |b|^2, A = M^+M from the Dirac oracle."""
    from oracle import Oracle
    R, geo, u, ph, U, sg, W = _setup()
    o = Oracle(geo.dims)
    m2 = 0.1 ** 2
    A = lambda v: o.mdagm(u, np.ascontiguousarray(v), ph, m2)
    b = F.gaussian_vec3(geo.dims, 1)
    x = F.gaussian_vec3(geo.dims, 2) * 0.1
    loss, dW = R.loss_and_grad(geo, U, sg, W, b, x, A)
    bn = np.sum(np.abs(b) ** 2)

    def loss_of(Wv):
        w = A(R.forward(geo, U, sg, Wv, b, bf16=False) - x)
        return np.sum(np.abs(w) ** 2) / bn
    assert abs(loss_of(W) - loss) <= 1e-12 * loss
    rng = np.random.default_rng(0)
    for _ in range(6):
        l, k, n = rng.integers(4), rng.integers(64), rng.integers(8)
        e = 1e-6
        Wp, Wm = W.copy(), W.copy()
        Wp[l, k, n] += e
        Wm[l, k, n] -= e
        fd = (loss_of(Wp) - loss_of(Wm)) / (2 * e)
        assert abs(fd - dW[l, k, n]) <= 1e-6 * max(1.0, abs(fd))


def test_network_is_gauge_covariant():
    """N[U^Omega](Omega r) = Omega N[U](r) with U_mu(x) -> Omega(x) U_mu(x) Omega(x+mu)^+."""
    R, geo, u, ph, U, sg, W = _setup()
    dims = geo.dims
    sh = geo.sizeh
    # Omega per site: index [parity][sizeh]
    om = F.random_su3_links(dims, 77, eps=1.0)[:2]            # (2, 3, 3, sh) as (parity, row, col, idx)
    Om = np.transpose(om, (0, 3, 1, 2))                       # (2, sh, 3, 3)
    Ug = np.empty_like(U)
    for mu in range(4):
        for p in (0, 1):
            fwd, _ = geo.neighbours(p)
            d = 2 * mu + p
            Ug[d] = Om[p] @ U[d] @ np.conj(np.transpose(Om[1 - p][fwd[mu]], (0, 2, 1)))
    r = F.gaussian_vec3(dims, 3)
    rg = np.einsum("sab,bs->as", Om[0], r)
    z = R.forward(geo, U, sg, W, r, bf16=False)
    zg = R.forward(geo, Ug, sg, W, rg, bf16=False)
    assert np.abs(zg - np.einsum("sab,bs->as", Om[0], z)).max() <= 1e-12 * np.abs(z).max()
