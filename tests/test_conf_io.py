"""Configuration files (host code, no GPU): the library's ASCII and ILDG
writers produce byte-identical files to the reference's own io.c (compiled
from source where the reference tree is present), each reads the other's
files back to the same links (bitwise for ILDG; to the 18 printed decimals
for ASCII), and the staggered-sign convention of the ASCII format round
trips.  The lattice is given by ostaple_init, which on a machine without a
GPU returns an error but still records the lattice for these functions."""
import ctypes as C

import numpy as np
import pytest

from openstaple_gb300 import fields as F

DIMS = (4, 6, 8, 10)


@pytest.fixture
def L(built):
    from openstaple_gb300.native import act_params, lib
    lib_ = lib()
    lib_.ostaple_init(*DIMS)      # -7 without a device; the lattice is recorded either way
    lib_.ostaple_clear_error()
    act_params().beta = 3.75
    C.c_char.in_dll(lib_, "input_file_str")
    buf = (C.c_char * (300 * 500)).in_dll(lib_, "input_file_str")
    buf.value = b"Beta 3.75\nStoutSteps 2\n"
    yield lib_
    buf.value = b""


def _links():
    u = F.random_su3_links(DIMS, 1201, eps=0.7)
    # the writers rebuild row 2 from rows 0-1: compare on exactly unitary rows
    a, c = u[:, 0], u[:, 1]
    u[:, 2] = np.conj(np.stack([a[:, 1] * c[:, 2] - a[:, 2] * c[:, 1], a[:, 2] * c[:, 0] - a[:, 0] * c[:, 2],
                                a[:, 0] * c[:, 1] - a[:, 1] * c[:, 0]], axis=1))
    return np.ascontiguousarray(u)


def test_ildg_round_trip_and_reference_bytes(L, tmp_path):
    from oracle import Reference, ref_available
    u = _links()
    ours = tmp_path / "ours.ildg"
    assert L.print_su3_soa_ildg_binary(u.ctypes.data, str(ours).encode(), 42) == 0
    back = np.zeros_like(u)
    traj = C.c_int(0)
    assert L.read_su3_soa_ildg_binary(back.ctypes.data, str(ours).encode(), C.byref(traj)) == 0
    assert traj.value == 42
    assert np.array_equal(back[:, :2], u[:, :2])
    assert np.abs(back - u).max() <= 1e-15
    # 144-byte LIME headers, big-endian magic number
    raw = ours.read_bytes()
    assert raw[:4] == bytes.fromhex("456789ab") and raw[16:27] == b"ildg-format"
    if not ref_available(DIMS):
        pytest.skip("reference not compiled here (no reference source tree)")
    r = Reference(DIMS)
    theirs = tmp_path / "theirs.ildg"
    assert r.write_ildg(u, theirs, 42, "Beta 3.75\nStoutSteps 2\n") == 0
    assert theirs.read_bytes() == raw
    t, ur = r.read_ildg(ours)
    assert t == 42 and np.array_equal(ur[:, :2], u[:, :2])


def test_ascii_round_trip_and_reference_bytes(L, tmp_path):
    from oracle import Reference, ref_available
    u = _links()
    ours = tmp_path / "ours.txt"
    assert L.print_su3_soa_ASCII(u.ctypes.data, str(ours).encode(), 7, None) == 0
    back = np.zeros_like(u)
    traj = C.c_int(0)
    assert L.read_su3_soa_ASCII(back.ctypes.data, str(ours).encode(), C.byref(traj)) == 0
    assert traj.value == 7
    assert np.abs(back - u).max() <= 1e-15   # row 2 is rebuilt by the writer
    # the staggered sign: written negated where the phase angle is nonzero,
    # read back with the determinant -1 undone
    ph = F.staggered_phases(DIMS)
    signed = tmp_path / "signed.txt"
    assert L.print_su3_soa_ASCII(u.ctypes.data, str(signed).encode(), 7, ph.ctypes.data) == 0
    back2 = np.zeros_like(u)
    assert L.read_su3_soa_ASCII(back2.ctypes.data, str(signed).encode(), C.byref(traj)) == 0
    assert np.abs(back2 - u).max() <= 1e-15
    if not ref_available(DIMS):
        pytest.skip("reference not compiled here (no reference source tree)")
    r = Reference(DIMS)
    theirs = tmp_path / "theirs.txt"
    assert r.write_ascii(u, theirs, 7, beta=3.75) == 0
    assert theirs.read_bytes() == ours.read_bytes()
    theirs_signed = tmp_path / "theirs_signed.txt"
    assert r.write_ascii(u, theirs_signed, 7, beta=3.75, phases=ph) == 0
    assert theirs_signed.read_bytes() == signed.read_bytes()
    t, ur = r.read_ascii(ours)
    assert t == 7 and np.array_equal(ur, back)


def test_reading_a_missing_file_or_a_wrong_lattice(L, tmp_path):
    u = np.zeros((8, 3, 3, F.sizeh(DIMS)), np.complex128)
    traj = C.c_int(0)
    assert L.read_su3_soa_ildg_binary(u.ctypes.data, str(tmp_path / "none").encode(), C.byref(traj)) == 1
    assert traj.value == -1
    bad = tmp_path / "bad.txt"
    bad.write_text("4 4 4 4 3.75 0.0 0 1\n")
    assert L.read_su3_soa_ASCII(u.ctypes.data, str(bad).encode(), C.byref(traj)) == 2
