"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on
a CPU-only machine (oracle, host logic, C-ABI symbol checks)."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    from openstaple_gb300 import build
    build.build_library()
    build.build_oracle()
    return True


@pytest.fixture(scope="session")
def gpu(built):
    """The library initialised on the GPU; skips nothing -- a GPU test that
    cannot reach the device fails loudly."""
    import ctypes
    from openstaple_gb300.native import lib
    L = lib()
    return L


def relerr(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def load_golden(tag: str):
    return dict(np.load(GOLDEN / f"dirac_{tag}.npz"))
