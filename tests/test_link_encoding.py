"""The link encoders of the FP32 iteration, run on the host from the same
source the kernels use, against numpy bit for bit: the 16-bit fixed-point
words of the sloppy links and the hi/lo split of the double-float links."""
import ctypes as C

import numpy as np

from openstaple_gb300.native import lib


def q16_reference(h):
    """rint(32768 h) of FP32 h (half to even), clamped to +-32767, + 32768."""
    q = np.clip(np.rint(h.astype(np.float64) * 32768.0), -32767, 32767)
    return (q + 32768).astype(np.uint32)


def test_q16_encoder_matches_numpy(built):
    rng = np.random.default_rng(5)
    h = np.concatenate([
        rng.uniform(-1.0, 1.0, 200000),
        np.array([0.0, -0.0, 1.0, -1.0, 0.99999, -0.99999, 2.0, -3.0]),
        (np.arange(-64, 65) + 0.5) / 32768.0,          # exact halves round to even
        np.array([1e-30, -1e-30, 2.0 ** -16, -(2.0 ** -16), 3 * 2.0 ** -17]),
    ]).astype(np.float32)
    q = np.zeros(h.size, np.uint32)
    lib().ostaple_q16_encode_host(h.ctypes.data, h.size, q.ctypes.data)
    assert np.array_equal(q, q16_reference(h))
    # decoding as the kernels do it: (2^23 + u) * 2^-15 - 257, exact
    dec = ((2.0 ** 23 + q.astype(np.float64)) * 2.0 ** -15 - 257.0).astype(np.float32)
    inside = np.abs(h) <= 32767 / 32768
    assert np.abs(dec[inside].astype(np.float64) - h[inside]).max() <= 2.0 ** -16


def test_double_float_split_matches_fp64_expression(built):
    rng = np.random.default_rng(6)
    x = np.concatenate([
        rng.standard_normal(200000) * rng.choice([1e-3, 0.1, 1.0, 10.0], 200000),
        np.array([0.0, -0.0, 1.0, -1.0, 0.5, 2.0 ** -40, -(2.0 ** -50), 1e-300, 3e30, -7e35]),
        # ties and near-ties of the FP32 rounding
        (1.0 + (np.arange(1, 200) * 2.0 ** -24)) * rng.choice([1.0, -1.0], 199),
        (1.0 + 2.0 ** -24 + np.array([-1, 0, 1]) * 2.0 ** -52),
        np.array([np.float64(np.nextafter(np.float32(1.0), np.float32(2.0))) - 2.0 ** -30]),
    ])
    hi = np.zeros(x.size, np.float32)
    lo = np.zeros(x.size, np.float32)
    lib().ostaple_df_split_host(x.ctypes.data, x.size, hi.ctypes.data, lo.ctypes.data)
    hi_ref = x.astype(np.float32)
    lo_ref = (x - hi_ref.astype(np.float64)).astype(np.float32)
    assert np.array_equal(hi.view(np.uint32), hi_ref.view(np.uint32))
    assert np.array_equal(lo.view(np.uint32), lo_ref.view(np.uint32))
