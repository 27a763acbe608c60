"""Host-side fault injection that needs no GPU: corrupted, truncated and
foreign network weight files are rejected (checksum, shape, magic), and a
corrupted .REMEZ file ends the program with the reference's message and exit
status (rationalapprox.c:8-11, 96-104) instead of producing an approximation."""
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT
from openstaple_gb300 import api


def _weights(seed=5):
    return np.random.default_rng(seed).uniform(-0.2, 0.2, api.NET_SHAPE).astype(np.float32)


def test_weight_file_round_trip(tmp_path):
    w = _weights()
    path = tmp_path / "net.bin"
    api.net_weights_save(path, w)
    assert np.array_equal(api.net_weights_load(path), w)


def test_weight_file_faults_are_detected(tmp_path):
    w = _weights()
    path = tmp_path / "net.bin"
    api.net_weights_save(path, w)
    raw = bytearray(path.read_bytes())
    flipped = bytearray(raw)
    flipped[100] ^= 0x01                        # one bit of one weight
    (tmp_path / "flip.bin").write_bytes(bytes(flipped))
    with pytest.raises(RuntimeError, match="checksum mismatch"):
        api.net_weights_load(tmp_path / "flip.bin")
    (tmp_path / "short.bin").write_bytes(bytes(raw[: len(raw) // 2]))
    with pytest.raises(RuntimeError, match="truncated"):
        api.net_weights_load(tmp_path / "short.bin")
    foreign = bytearray(raw)
    foreign[0:8] = b"NOTANET!"
    (tmp_path / "foreign.bin").write_bytes(bytes(foreign))
    with pytest.raises(RuntimeError, match="not a version-1 weight file"):
        api.net_weights_load(tmp_path / "foreign.bin")
    with pytest.raises(RuntimeError, match="cannot open"):
        api.net_weights_load(tmp_path / "missing.bin")
    # the library's error state is clear again after each reported failure
    assert np.array_equal(api.net_weights_load(path), w)


def test_corrupted_remez_file_ends_the_program(tmp_path):
    bad = tmp_path / "bad.REMEZ"
    bad.write_text("\nApproximation to f(x) = (x)^(-1/4)\nOrder: 8\nLambda Min: 1e-7\nLambda Max: 1\n"
                   "GMP Remez Precision: 100\nError: 1e-4\nRA_a0 = 0.5\nRA_a[0] = garbage\n")
    code = ("import ctypes as C, sys; sys.path.insert(0, %r)\n"
            "from openstaple_gb300.native import lib, RationalApprox\n"
            "ra = RationalApprox()\n"
            "print(lib().rationalapprox_read_custom_nomefile(C.byref(ra), %r.encode()))\n") % (str(ROOT), str(bad))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    assert "Error, not read expected number of entries" in r.stdout
