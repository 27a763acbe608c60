"""The allocation-free reduction entry point.

Callers that cannot allocate device memory at the point of call -- a loop
that must not take cudaMalloc's implicit device synchronisation, a process
under a fixed device-memory budget -- use ostaple_real_scal_prod_global_noalloc,
whose scratch is a fixed static device array.  This file runs last so that a
failure here leaves every other test already run; it passes alone in a fresh
process and after the other tests."""
import math

import numpy as np
import pytest

from openstaple_gb300 import api, fields as F

pytestmark = pytest.mark.gpu


def _lat(gpu, dims):
    return api.Lattice(dims)


# 8x8x8x16: 6 blocks (one group); 16^3x32: 96 blocks (two groups of the
# two-level reduction)
@pytest.mark.parametrize("dims", [(8, 8, 8, 16), (16, 16, 16, 32)])
def test_noalloc_matches_allocating_entry_point_twice(gpu, dims):
    from openstaple_gb300.native import lib
    L = lib()
    lat = _lat(gpu, dims)
    try:
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
    finally:
        lat.close()


def test_noalloc_result_does_not_depend_on_an_earlier_error(gpu):
    """An unrelated failure recorded earlier (the error word keeps the first
    one) must not turn a successful reduction into NAN."""
    from openstaple_gb300.native import lib
    L = lib()
    dims = (8, 8, 8, 8)
    lat = _lat(gpu, dims)
    try:
        a, b = F.gaussian_vec3(dims, 911), F.gaussian_vec3(dims, 912)
        lat.present(a)
        lat.present(b)
        ref = api.real_scal_prod_global(a, b)
        unregistered = np.zeros_like(a)   # neither registered nor device memory
        L.ostaple_real_scal_prod_global_noalloc(unregistered.ctypes.data, b.ctypes.data)
        assert L.ostaple_get_error() == -4
        got = L.ostaple_real_scal_prod_global_noalloc(a.ctypes.data, b.ctypes.data)
        assert abs(got - ref) <= 1e-12 * abs(ref)
        L.ostaple_clear_error()
    finally:
        lat.close()


def test_noalloc_rejects_lattices_beyond_its_scratch(gpu):
    """sizeh > 2,796,202 does not fit the fixed scratch: error -14 and NAN,
    before any pointer is looked at or any kernel launched."""
    from openstaple_gb300.native import lib
    L = lib()
    lat = _lat(gpu, (48, 48, 48, 52))      # sizeh = 2,875,392
    try:
        assert lat.sizeh > 2_796_202
        n0 = L.ostaple_kernel_launches()
        got = L.ostaple_real_scal_prod_global_noalloc(None, None)
        assert math.isnan(got)
        assert L.ostaple_get_error() == -14
        assert b"fixed scratch" in L.ostaple_last_error()
        assert L.ostaple_kernel_launches() == n0
        L.ostaple_clear_error()
    finally:
        lat.close()
