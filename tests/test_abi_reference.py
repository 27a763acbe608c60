"""The C ABI against the reference's own headers (CPU, gcc): the plain
structs that cross the boundary have the reference's size and field
offsets, the SoA types have the element sizes the kernels assume, and every
prototype in include/ostaple_gb300.h compiles beside the reference's
declaration of the same function (a conflicting type is a compile error).
Skipped where the reference source tree is absent."""
import os
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT


def reference_src():
    from openstaple_gb300.build import reference_root
    ref = reference_root()
    return None if ref is None else ref / "src"


def _build_and_run(tmp_path, with_ref: bool, src: Path | None) -> str:
    exe = tmp_path / ("abi_ref" if with_ref else "abi_lib")
    cmd = [os.environ.get("CC", "gcc"), "-std=gnu99", "-O0", "-w", "-I", str(ROOT / "include")]
    if with_ref:
        cmd += ["-DWITH_REFERENCE_HEADERS", "-DLOC_N0=4", "-DLOC_N1=4", "-DLOC_N2=4", "-DLOC_N3=4",
                "-DNRANKS_D3=1", "-DACTION_TYPE=TLSM", "-DNREPLICAS=1",
                "-I", str(ROOT / "oracle" / "ref_shim" / "OpenAcc"), "-I", str(src / "OpenAcc")]
    cmd += [str(ROOT / "tests" / "abi" / "abi_layout.c"), "-o", str(exe)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout


def test_structs_and_prototypes_match_the_reference_headers(tmp_path):
    src = reference_src()
    if src is None:
        pytest.skip("reference source tree not available")
    ours = _build_and_run(tmp_path, False, None)
    theirs = _build_and_run(tmp_path, True, src)
    assert ours == theirs
