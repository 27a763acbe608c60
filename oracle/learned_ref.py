"""CPU restatement of the gauge-covariant network used as the learned
preconditioner (checker only: tests and nothing else use it).

Conventions (same as the CUDA kernels): fields on one parity of the half
lattice, complex128 arrays (channels, 3, sizeh); links su3_soa[8] complex
(8, 3, 3, sizeh), third row rebuilt from the first two; staggered signs
from the phase angles (pi -> -1).  Layer l maps parity 1-p_out(l) to
p_out(l) = 1, 0, 1, 0 for l = 0..3:

    h[d, c](x) = s U_mu(x) in_c(x+mu)          d = mu
    h[d, c](x) = s U_mu(x-mu)^+ in_c(x-mu)     d = 4 + mu
    out_n(x)   = sum_{d,c} W[l][8 d + c][n] h[d, c](x)

`bf16=True` rounds weights, transported vectors and hidden activations to
bfloat16 as the tensor-core path does; the gradient is the exact FP64
gradient of the unrounded network.
"""
from __future__ import annotations

import numpy as np

C = 8
LAYERS = 4


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round float values to the nearest bfloat16 (ties to even), keep float64."""
    if np.iscomplexobj(a):
        return bf16_round(a.real) + 1j * bf16_round(a.imag)
    f = np.asarray(a, dtype=np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    lsb = (b >> 16) & 1
    b = ((b + 0x7FFF + lsb) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


class Geometry:
    def __init__(self, dims):
        self.dims = tuple(dims)
        n0, n1, n2, n3 = dims
        self.sizeh = n0 * n1 * n2 * n3 // 2
        self._nb = {}
        for p in (0, 1):
            idx = np.arange(self.sizeh)
            nh0 = n0 // 2
            hd0 = idx % nh0
            r = idx // nh0
            d1 = r % n1
            r //= n1
            d2 = r % n2
            d3 = r // n2
            d0 = 2 * hd0 + ((d1 + d2 + d3 + p) & 1)
            coords = [d0, d1, d2, d3]
            fwd, bwd = [], []
            for mu in range(4):
                for step, lst in ((1, fwd), (-1, bwd)):
                    c = [x.copy() for x in coords]
                    c[mu] = (c[mu] + step) % dims[mu]
                    lst.append((c[0] + n0 * (c[1] + n1 * (c[2] + n2 * c[3]))) // 2)
            self._nb[p] = (fwd, bwd)

    def neighbours(self, p):
        return self._nb[p]


def full_links(u: np.ndarray, fp32: bool = True) -> np.ndarray:
    """(8, sizeh, 3, 3) matrices with the third row rebuilt (optionally from FP32-rounded rows)."""
    r = u[:, :2].astype(np.complex64).astype(np.complex128) if fp32 else u[:, :2]
    m = np.zeros((8, 3, 3, u.shape[-1]), np.complex128)
    m[:, :2] = r
    m[:, 2] = np.conj(np.cross(r[:, 0], r[:, 1], axis=1))
    return np.transpose(m, (0, 3, 1, 2))


def signs_of(phases: np.ndarray) -> np.ndarray:
    return np.where(phases == np.float64(0.5 * (2 * 3.14159265358979323846)), -1.0, 1.0)


def transport(geo: Geometry, U: np.ndarray, sg: np.ndarray, act: np.ndarray, p_out: int, bf16: bool):
    """h[d, c, 3, sizeh] for output parity p_out from act[c, 3, sizeh] on the other parity."""
    fwd, bwd = geo.neighbours(p_out)
    h = np.zeros((8, act.shape[0], 3, geo.sizeh), np.complex128)
    for d in range(8):
        mu = d & 3
        if d < 4:
            dr, li, j = 2 * mu + p_out, np.arange(geo.sizeh), fwd[mu]
            M = U[dr, li]
        else:
            dr, li, j = 2 * mu + (1 - p_out), bwd[mu], bwd[mu]
            M = np.conj(np.transpose(U[dr, li], (0, 2, 1)))
        s = sg[dr, li]
        v = act[:, :, j]                                      # (c, 3, sites)
        h[d] = s[None, None, :] * np.einsum("sab,cbs->cas", M, v)
    return bf16_round(h) if bf16 else h


def forward(geo: Geometry, U, sg, W: np.ndarray, r: np.ndarray, bf16: bool = True, keep: bool = False):
    """z = N(r); r, z: (3, sizeh) complex on the even sub-lattice."""
    Wl = bf16_round(W) if bf16 else W
    act = np.zeros((C, 3, geo.sizeh), np.complex128)
    act[0] = bf16_round(r) if bf16 else r
    acts = [act]
    for layer in range(LAYERS):
        p_out = 1 if layer % 2 == 0 else 0
        h = transport(geo, U, sg, act, p_out, bf16)
        out = np.einsum("kn,kas->nas", Wl[layer], h.reshape(8 * C, 3, geo.sizeh))
        if layer < LAYERS - 1:
            act = bf16_round(out) if bf16 else out
            acts.append(act)
        else:
            z = out[0]
    return (z, acts) if keep else z


def adjoint_transport(geo: Geometry, U, sg, dh: np.ndarray, p_out: int) -> np.ndarray:
    """Adjoint of transport(): gradient on the input parity from dh[d, c, 3, sites]."""
    fwd, bwd = geo.neighbours(p_out)
    g = np.zeros((dh.shape[1], 3, geo.sizeh), np.complex128)
    for d in range(8):
        mu = d & 3
        if d < 4:
            dr, li, j = 2 * mu + p_out, np.arange(geo.sizeh), fwd[mu]
            MH = np.conj(np.transpose(U[dr, li], (0, 2, 1)))
        else:
            dr, li, j = 2 * mu + (1 - p_out), bwd[mu], bwd[mu]
            MH = U[dr, li]
        s = sg[dr, li]
        contrib = s[None, None, :] * np.einsum("sab,cbs->cas", MH, dh[d])
        np.add.at(g, (slice(None), slice(None), j), contrib)
    return g


def loss_and_grad(geo: Geometry, U, sg, W, b, x, apply_a):
    """FP64 residual loss |A (N(b) - x)|^2 / |b|^2 of the unrounded network and
    dloss/dW.  apply_a is the Hermitian operator A (M^+M + shift on even
    sites); dloss/dz = 2 A A (z - x) / |b|^2."""
    z, acts = forward(geo, U, sg, W, b, bf16=False, keep=True)
    bn = np.sum(np.abs(b) ** 2)
    w = apply_a(np.ascontiguousarray(z - x))
    loss = np.sum(np.abs(w) ** 2) / bn
    gz = np.zeros((C, 3, geo.sizeh), np.complex128)
    gz[0] = 2.0 * apply_a(np.ascontiguousarray(w)) / bn
    dW = np.zeros_like(W)
    g = gz
    for layer in range(LAYERS - 1, -1, -1):
        p_out = 1 if layer % 2 == 0 else 0
        h = transport(geo, U, sg, acts[layer], p_out, bf16=False).reshape(8 * C, 3, geo.sizeh)
        dW[layer] = np.einsum("kas,nas->kn", h.real, g.real) + np.einsum("kas,nas->kn", h.imag, g.imag)
        dh = np.einsum("kn,nas->kas", W[layer], g).reshape(8, C, 3, geo.sizeh)
        g = adjoint_transport(geo, U, sg, dh, p_out)
    return loss, dW
