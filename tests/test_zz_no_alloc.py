"""The allocation-free reduction entry point.

Callers that cannot allocate device memory at the point of call -- a host
thread while another thread holds a global-mode stream capture, a loop that
must not take cudaMalloc's implicit device synchronisation, a process under a
fixed device-memory budget -- use ostaple_real_scal_prod_global_noalloc, whose
scratch is a fixed static device array.  This file runs last so that a
failure here leaves every other test already run; it passes alone in a fresh
process and after the other tests."""
import numpy as np
import pytest

from openstaple_gb300 import api, fields as F

pytestmark = pytest.mark.gpu


@pytest.fixture
def lat(gpu):
    lat = api.Lattice((8, 8, 8, 16))
    yield lat
    lat.close()


def test_noalloc_matches_allocating_entry_point_twice(lat):
    from openstaple_gb300.native import lib
    L = lib()
    dims = lat.dims
    pairs = [(F.gaussian_vec3(dims, 901), F.gaussian_vec3(dims, 902)),
             (F.gaussian_vec3(dims, 903), F.gaussian_vec3(dims, 904))]
    for a, b in pairs:
        lat.present(a)
        lat.present(b)
    # two calls in a row: the second must not see the first call's scratch
    for a, b in pairs:
        ref = api.real_scal_prod_global(a, b)
        got = L.ostaple_real_scal_prod_global_noalloc(a.ctypes.data, b.ctypes.data)
        assert L.ostaple_get_error() == 0
        # same tolerance as the other reduction tests: 1e-12 relative
        assert abs(got - ref) <= 1e-12 * abs(ref)
        exact = float(np.sum(a.real * b.real + a.imag * b.imag))
        assert abs(got - exact) <= 1e-12 * abs(exact)
