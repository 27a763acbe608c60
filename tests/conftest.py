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
    build.build_reference_oracles()   # no-op where the reference tree is absent
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


def rebuild_row2(q):
    """Row 2 of su3_soa links as conj(row0 x row1), the kernels' rebuild."""
    a, c = q[:, 0], q[:, 1]
    q[:, 2] = np.conj(np.stack([a[:, 1] * c[:, 2] - a[:, 2] * c[:, 1],
                                a[:, 2] * c[:, 0] - a[:, 0] * c[:, 2],
                                a[:, 0] * c[:, 1] - a[:, 1] * c[:, 0]], axis=1))
    return np.ascontiguousarray(q)


def quantise_links(u, fmt):
    """The sloppy links as the FP32 kernels see them.  "q16": rows 0-1
    rounded to FP32, then to multiples of 2^-15 (half to even, clamped to
    +-32767/32768); "f32" / "f16": rows 0-1 rounded to that type; row 2
    rebuilt in every case."""
    if fmt == "q16":
        re = np.clip(np.rint(u.real.astype(np.float32).astype(np.float64) * 32768.0), -32767, 32767)
        im = np.clip(np.rint(u.imag.astype(np.float32).astype(np.float64) * 32768.0), -32767, 32767)
        return rebuild_row2((re + 1j * im) / 32768.0)
    dt = {"f32": np.float32, "f16": np.float16}[fmt]
    return rebuild_row2(u.real.astype(dt).astype(np.float64) + 1j * u.imag.astype(dt).astype(np.float64))


def load_golden(tag: str):
    return dict(np.load(GOLDEN / f"dirac_{tag}.npz"))


def load_gauge_fixture(tag: str):
    """(fixture, dims, links, Sigma', shift solutions X_k, pseudofermions)
    of tests/golden/gauge_<tag>.npz, the inputs regenerated from their seeds
    and checked against the stored checksums."""
    sys.path.insert(0, str(GOLDEN))
    import make_golden as mg
    g = dict(np.load(GOLDEN / f"gauge_{tag}.npz"))
    dims = tuple(int(d) for d in g["dims"])
    u, sig, xs, phis = mg.gauge_inputs(dims, int(g["link_seed"]), float(g["eps"]))
    for name, arr in (("u", u), ("sig", sig), ("xs", xs), ("phi", phis)):
        assert np.isclose(np.sum(np.abs(arr) ** 2), float(g[f"{name}_checksum"]), rtol=1e-14), name
    return g, dims, u, sig, xs, phis


def sample_sites(f, g):
    """su3/vec3 field at the fixture's sampled half-lattice sites."""
    return np.asarray(f)[..., g["sites"]]


def sample_alg(f, g):
    """tamat/thmat field (8, 8*sizeh) at the fixture's sampled sites."""
    return np.asarray(f)[:, g["alg_idx"]]
