"""CPU model of the mixed-precision CG's reliable update, on the oracle's
FP64 M^+M: why the solvers continue after a reliable update with the
Hestenes-Stiefel beta = -<r, A p>/<p, A p> rather than the reference's
beta = lambda/delta (inverter_mixedp.c:124-150).

The FP32 recursion runs on the 16-bit fixed-point links the solvers use for
it (the oracle applied to quantised links), with a reliable update every 50
iterations.  When the recomputed residual is much larger than the recursed
one, lambda/delta makes the next direction repeat the last one and the
solve stalls; the Hestenes-Stiefel beta keeps the directions conjugate."""
import numpy as np

from openstaple_gb300 import fields as F

DIMS = (8, 8, 8, 8)
MASS = 0.01


def quantise_q16(u):
    """Rows 0-1 rounded to FP32, then to multiples of 2^-15, row 2 rebuilt."""
    re = np.clip(np.rint(u.real.astype(np.float32).astype(np.float64) * 32768.0), -32767, 32767)
    im = np.clip(np.rint(u.imag.astype(np.float32).astype(np.float64) * 32768.0), -32767, 32767)
    q = (re + 1j * im) / 32768.0
    a, c = q[:, 0], q[:, 1]
    q[:, 2] = np.conj(np.stack([a[:, 1] * c[:, 2] - a[:, 2] * c[:, 1],
                                a[:, 2] * c[:, 0] - a[:, 0] * c[:, 2],
                                a[:, 0] * c[:, 1] - a[:, 1] * c[:, 0]], axis=1))
    return np.ascontiguousarray(q)


def mixed_cg_model(o, u, ph, b, every, hestenes_stiefel, max_iter):
    """FP32 CG on the sloppy operator with FP64 reliable updates every
    `every` iterations; returns (iterations, FP64 true relative residual)."""
    m2 = MASS * MASS
    uq = quantise_q16(u)
    a32 = lambda v: o.mdagm(uq, np.ascontiguousarray(v.astype(np.complex128)), ph, m2).astype(np.complex64)
    a64 = lambda v: o.mdagm(u, np.ascontiguousarray(v), ph, m2)
    dot = lambda x, y: float(np.sum(x.real.astype(np.float64) * y.real + x.imag.astype(np.float64) * y.imag))
    bn = dot(b, b)
    x = np.zeros_like(b)
    r = b.astype(np.complex64)
    p = r.copy()
    xf = np.zeros_like(r)
    delta = dot(r, r)
    it = 0
    while it < max_iter:
        s = a32(p)
        pap = dot(p, s)
        alpha = delta / pap
        it += 1
        xf = (xf + np.float32(alpha) * p).astype(np.complex64)
        if it % every == 0:
            x = x + xf.astype(np.complex128)
            xf[:] = 0
            r64 = b - a64(x)
            true = np.sqrt(dot(r64, r64) / bn)
            if true < 1e-10:
                return it, true
            r = r64.astype(np.complex64)
            lam = dot(r64, r64)
            beta = -dot(r, s) / pap if hestenes_stiefel else lam / delta
            delta = lam
            p = (r + np.float32(beta) * p).astype(np.complex64)
            continue
        r = (r - np.float32(alpha) * s).astype(np.complex64)
        lam = dot(r, r)
        beta = lam / delta
        delta = lam
        p = (r + np.float32(beta) * p).astype(np.complex64)
    x = x + xf.astype(np.complex128)
    r64 = b - a64(x)
    return it, np.sqrt(dot(r64, r64) / bn)


def test_hestenes_stiefel_beta_keeps_the_fixed_interval_solve_converging():
    from oracle import Oracle
    o = Oracle(DIMS)
    u = F.random_su3_links(DIMS, 81)
    ph = F.staggered_phases(DIMS)
    b = F.gaussian_vec3(DIMS, 82)
    it_hs, res_hs = mixed_cg_model(o, u, ph, b, 50, True, 400)
    assert res_hs < 1e-10 and it_hs <= 200, (it_hs, res_hs)
    it_ref, res_ref = mixed_cg_model(o, u, ph, b, 50, False, 400)
    assert res_ref > 1e-6, (it_ref, res_ref)   # stalls far above the target
