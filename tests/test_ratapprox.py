"""Rational approximations (rationalapprox.c): the library's host functions
read and write the .REMEZ format, rescale and evaluate exactly as the
reference does (bitwise against the reference compiled from source where it
is available), and the rescaled approximation tracks x^(num/den) within the
approximation's stated error over its range.  CPU only."""
import ctypes as C
import json
import math

import numpy as np
import pytest

from conftest import GOLDEN
from openstaple_gb300.native import RationalApprox, lib


def mother(name):
    ap = json.loads((GOLDEN / "ratapprox.json").read_text())[name]
    ra = RationalApprox()
    ra.exponent_num, ra.exponent_den = ap["exponent_num"], ap["exponent_den"]
    ra.approx_order = ap["order"]
    ra.lambda_min, ra.lambda_max = ap["lambda_min"], ap["lambda_max"]
    ra.gmp_remez_precision = 100
    ra.error = ap["error"]
    ra.RA_a0 = ap["a0"]
    for k in range(ap["order"]):
        ra.RA_a[k], ra.RA_b[k] = ap["a"][k], ap["b"][k]
    return ra


def fields(ra):
    return (ra.exponent_num, ra.exponent_den, ra.approx_order, ra.lambda_min, ra.lambda_max,
            ra.gmp_remez_precision, ra.error, ra.RA_a0, tuple(ra.RA_a[:ra.approx_order]),
            tuple(ra.RA_b[:ra.approx_order]))


@pytest.mark.parametrize("name", ["order8", "order19"])
def test_remez_file_round_trip(tmp_path, name):
    L = lib()
    ra = mother(name)
    path = str(tmp_path / "a.REMEZ").encode()
    L.rationalapprox_save(path, C.byref(ra))
    back = RationalApprox()
    assert L.rationalapprox_read_custom_nomefile(C.byref(back), path) == 0
    assert fields(back) == fields(ra)
    assert L.rationalapprox_read_custom_nomefile(C.byref(back), str(tmp_path / "missing").encode()) == 1


def test_file_names_follow_the_reference_pattern():
    L = lib()
    libc = C.CDLL(None)
    p = L.rational_approx_filename(10 ** -3.8, -1, 4, 10 ** -6.2)
    assert C.string_at(p).decode() == "approx_-1_over_4_mlogerr_3.8_mloglm_6.2.REMEZ"
    libc.free(C.c_void_p(p))
    p = L.rational_approx_filename_old(19, -1, 4, 10 ** -6.4)
    assert C.string_at(p).decode() == "approx_-1_over_4_order_19_mloglm_6.4.REMEZ"
    libc.free(C.c_void_p(p))


@pytest.mark.parametrize("name", ["order8", "order19"])
def test_rescaled_approximation_tracks_the_power(name):
    L = lib()
    ra, out = mother(name), RationalApprox()
    minmax = np.array([1e-4, 4.6])
    L.rescale_rational_approximation(C.byref(ra), C.byref(out), minmax.ctypes.data)
    p = ra.exponent_num / ra.exponent_den
    assert math.isclose(out.lambda_max, 4.6 * 1.05, rel_tol=1e-15)
    xs = np.geomspace(out.lambda_min, out.lambda_max, 200)
    worst = max(abs(L.rational_approx_evaluate(C.byref(out), x) / x ** p - 1.0) for x in xs)
    assert worst <= 2 * ra.error
    back = RationalApprox()
    L.renormalize_rational_approximation(C.byref(out), C.byref(back))
    assert math.isclose(back.RA_a0, ra.RA_a0, rel_tol=1e-13)
    assert np.allclose(back.RA_b[:ra.approx_order], ra.RA_b[:ra.approx_order], rtol=1e-13, atol=0)


@pytest.mark.parametrize("name", ["order8", "order19"])
def test_matches_compiled_reference(tmp_path, built, name):
    from oracle import Reference, ref_available
    dims = (4, 4, 4, 4)
    if not ref_available(dims):
        pytest.skip("reference not compiled here (no reference source tree)")
    R = Reference(dims)
    L = lib()
    ra = mother(name)
    path = str(tmp_path / "r.REMEZ").encode()
    R.L.ref_ra_save(path, C.addressof(ra))
    ours, theirs = RationalApprox(), RationalApprox()
    assert L.rationalapprox_read_custom_nomefile(C.byref(ours), path) == 0
    assert R.L.ref_ra_read(path, C.addressof(theirs)) == 0
    assert fields(ours) == fields(theirs)
    minmax = np.array([2.5e-3 ** 2, 4.56])
    o1, o2 = RationalApprox(), RationalApprox()
    L.rescale_rational_approximation(C.byref(ours), C.byref(o1), minmax.ctypes.data)
    R.L.ref_ra_rescale(C.addressof(theirs), C.addressof(o2), minmax.ctypes.data)
    assert fields(o1) == fields(o2)
    for x in (o1.lambda_min, 0.01, 1.0, o1.lambda_max):
        assert L.rational_approx_evaluate(C.byref(o1), x) == R.L.ref_ra_evaluate(C.addressof(o2), x)
    n1, n2 = RationalApprox(), RationalApprox()
    L.renormalize_rational_approximation(C.byref(o1), C.byref(n1))
    R.L.ref_ra_renormalize(C.addressof(o2), C.addressof(n2))
    assert fields(n1) == fields(n2)
    buf = C.create_string_buffer(64)
    R.L.ref_ra_filename(ra.error, ra.exponent_num, ra.exponent_den, ra.lambda_min, C.addressof(buf))
    p = L.rational_approx_filename(ra.error, ra.exponent_num, ra.exponent_den, ra.lambda_min)
    assert C.string_at(p) == buf.value
