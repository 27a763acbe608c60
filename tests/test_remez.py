"""The library's own rational-approximation generator (host code, no GPU)
against the outputs of the reference's multiprecision Remez program: every
.REMEZ file the reference ships in its current format
(tests/golden/remez_reference.json, copied by tests/golden/make_golden.py).

The best relative-error approximation of a given order is unique, so the
generator must reproduce the reference's numbers: a0, every residue and
every shift within 1e-9 relative (the measured agreement is 3e-11 or
better), the error within 1e-6.  Also: Chebyshev equioscillation of the
error for other exponents and orders, the reference driver's order loop, a
.REMEZ round trip through the library's own writer and reader, the error
bound on a dense set of points, the command line and the rejected
arguments."""
import ctypes as C
import json

import numpy as np
import pytest

from conftest import GOLDEN

FIXTURES = json.loads((GOLDEN / "remez_reference.json").read_text())


@pytest.fixture
def L(built):
    from openstaple_gb300.native import lib
    return lib()


@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_generator_reproduces_the_reference_remez_files(L, name):
    from openstaple_gb300 import api
    ref = FIXTURES[name]
    ra = api.remez(ref["exponent_num"], ref["exponent_den"], ref["lambda_min"], order=ref["order"])
    n = ref["order"]
    assert ra.approx_order == n and ra.lambda_max == 1.0
    assert abs(ra.RA_a0 / ref["a0"] - 1) <= 1e-9
    assert np.max(np.abs(np.array(ra.RA_b[:n]) / np.array(ref["b"]) - 1)) <= 1e-9
    assert np.max(np.abs(np.array(ra.RA_a[:n]) / np.array(ref["a"]) - 1)) <= 1e-9
    assert abs(ra.error / ref["error"] - 1) <= 1e-6
    assert all(v == 0.0 for v in ra.RA_a[n:]) and all(v == 0.0 for v in ra.RA_b[n:])


def test_error_bound_holds_on_dense_points(L):
    from openstaple_gb300 import api
    for num, den in ((-1, 4), (1, 8)):
        ra = api.remez(num, den, 1e-5, order=10)
        xs = np.geomspace(1e-5, 1.0, 20001)
        r = np.array([L.rational_approx_evaluate(C.byref(ra), float(x)) for x in xs])
        rel = np.abs(r / xs ** (num / den) - 1)
        # the error is levelled for x^|num/den|; for a negative exponent the
        # inverse carries |1/(1+e) - 1| <= E/(1-E)
        assert rel.max() <= ra.error / (1 - ra.error) * (1 + 1e-6)
        assert rel.max() >= 0.99 * ra.error


def test_order_loop_of_the_reference_driver(L):
    from openstaple_gb300 import api
    ref = FIXTURES["tools/test/ratapproxes/approx_-1_over_4_mlogerr_3.8_mloglm_6.2.REMEZ"]
    # goal just above the order-8 error: the driver's guess, int(ln(goal) ln(lmin)/19 + 2) = 8, is kept
    ra = api.remez(-1, 4, ref["lambda_min"], goal_error=1.6e-4)
    assert ra.approx_order == 8 and abs(ra.RA_a0 / ref["a0"] - 1) <= 1e-9
    # a tighter goal raises the order until the error is below it
    ra = api.remez(-1, 4, ref["lambda_min"], goal_error=1e-6)
    lower = api.remez(-1, 4, ref["lambda_min"], order=ra.approx_order - 1)
    assert ra.error <= 1e-6 < lower.error


def test_remez_file_round_trip(L, tmp_path):
    from openstaple_gb300 import api
    from openstaple_gb300.native import RationalApprox
    ra = api.remez(1, 8, 5.890909e-07, order=12)
    path = tmp_path / "r.REMEZ"
    L.rationalapprox_save(str(path).encode(), C.byref(ra))
    back = RationalApprox()
    assert L.rationalapprox_read_custom_nomefile(C.byref(back), str(path).encode()) == 0
    assert back.approx_order == 12 and back.exponent_num == 1 and back.exponent_den == 8
    assert back.RA_a0 == ra.RA_a0 and list(back.RA_a[:12]) == list(ra.RA_a[:12])
    assert list(back.RA_b[:12]) == list(ra.RA_b[:12]) and back.error == ra.error


@pytest.mark.parametrize("num,den,order,lmin", [(1, 1, 8, 1e-4), (3, 2, 8, 1e-4), (0, 4, 8, 1e-4), (1, 4, 0, 1e-4),
                                                (1, 4, 26, 1e-4), (1, 4, 8, 0.0), (1, 4, 8, 2.0)])
def test_rejected_arguments(L, num, den, order, lmin):
    from openstaple_gb300.native import RationalApprox
    ra = RationalApprox()
    ra.exponent_num, ra.exponent_den, ra.approx_order, ra.lambda_min = num, den, order, lmin
    assert L.ostaple_remez_approximation(C.byref(ra)) == -3
    L.ostaple_clear_error()


def test_command_line_writes_the_reference_file_name(L, tmp_path, monkeypatch):
    from openstaple_gb300 import remez as cli
    from openstaple_gb300.native import RationalApprox
    monkeypatch.chdir(tmp_path)
    assert cli.main(["1e-4", "-1", "4", "5.890909e-07"]) == 0
    files = list(tmp_path.glob("*.REMEZ"))
    assert [f.name for f in files] == ["approx_-1_over_4_mlogerr_4.0_mloglm_6.2.REMEZ"]
    back = RationalApprox()
    assert L.rationalapprox_read_custom_nomefile(C.byref(back), str(files[0]).encode()) == 0
    assert back.error <= 1e-4 and back.approx_order == 9


@pytest.mark.parametrize("num,den,order,lmin", [(-1, 4, 12, 1e-5), (1, 8, 9, 1e-4), (-1, 2, 10, 1e-6)])
def test_error_equioscillates(L, num, den, order, lmin):
    """The defining property of the best approximation (Chebyshev's
    alternation theorem): the relative error of the approximation of
    x^|num/den| (1/r for a negative exponent) takes its extreme value E with
    alternating signs at 2n+2 points of [lambda_min, 1]."""
    from openstaple_gb300 import api
    ra = api.remez(num, den, lmin, order=order)
    xs = np.geomspace(lmin, 1.0, 200001)
    r = np.array([L.rational_approx_evaluate(C.byref(ra), float(x)) for x in xs])
    b = abs(num / den)
    e = (r ** (-1.0 if num < 0 else 1.0)) / xs ** b - 1.0
    runs, start = [], 0
    for i in range(1, len(e) + 1):
        if i == len(e) or np.sign(e[i]) != np.sign(e[start]):
            runs.append(np.abs(e[start:i]).max())
            start = i
    assert len(runs) == 2 * order + 2
    assert np.max(np.abs(np.array(runs) / ra.error - 1)) <= 1e-4
