"""plbm_velocity_l2_error_noalloc against plbm_velocity_l2_error.

The no-allocation entry point serves callers that cannot allocate device
memory at the moment they want the diagnostic (HBM filled by a large run,
memory owned by another allocator, a loop that must not allocate).  It must
give the same number as the allocating entry point, call after call, through
the C ABI.  This file is collected last so that a stop at the first failure
has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, the binary64 tolerance of the other parity tests


def _fields(nx, ny, seed):
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) + 0.5)[:, None] * 2 * np.pi / nx
    y = (np.arange(ny) + 0.5)[None, :] * 2 * np.pi / ny
    ux = 0.03 * np.cos(x) * np.sin(y) + 1e-4 * rng.standard_normal((nx, ny))
    uy = -0.03 * np.sin(x) * np.cos(y) + 1e-4 * rng.standard_normal((nx, ny))
    return np.ascontiguousarray(ux), np.ascontiguousarray(uy)


@pytest.mark.parametrize("nx,ny", [(300, 200), (1024, 1024)])  # 1024^2 = the capacity, 2^20 cells
@pytest.mark.parametrize("storage", ["f64", "f32dev", "f16dev"])
def test_noalloc_matches_allocating_entry_point_twice(gpu_lib, storage, nx, ny):
    from plbm import LatticeGrid, _lib
    lib = _lib.load()
    ux, uy = _fields(nx, ny, 1)
    g = LatticeGrid(nx, ny, storage=storage)
    g.set_relaxation(1.6, 0.25)
    g.set_pdf_to_equilibrium(np.ones((nx, ny)), ux, uy)
    g.perform_lbm_step(7)
    g.synchronize()
    fdev = g.device_ptr(g.iold)
    for seed in (2, 3):  # two calls in a row, different reference fields
        uxa, uya = _fields(nx, ny, seed)
        want = g.velocity_l2_error(uxa, uya, g.iold)
        got = C.c_double(-1.0)
        rc = lib.plbm_velocity_l2_error_noalloc(_lib.STORAGES[storage], nx, ny, g.ld, C.c_void_p(fdev),
                                                uxa.ctypes.data, uya.ctypes.data, C.byref(got), None)
        assert rc == 0, _lib.last_error()
        assert abs(got.value - want) <= TOL * want
    g.close()


def test_noalloc_rejects_sizes_beyond_its_capacity(gpu_lib):
    from plbm import _lib
    lib = _lib.load()
    err = C.c_double()
    dummy = np.zeros(4)
    rc = lib.plbm_velocity_l2_error_noalloc(0, 2048, 1024, 1024, C.c_void_p(dummy.ctypes.data),
                                            dummy.ctypes.data, dummy.ctypes.data, C.byref(err), None)
    assert rc == _lib.PLBM_E_INVALID
    assert "exceeds the fixed staging capacity" in _lib.last_error()
    big = (1 << 30) + 1
    for nx, ny, ld in ((big, 1, 16), (1, 8, big)):
        rc = lib.plbm_velocity_l2_error_noalloc(0, nx, ny, ld, C.c_void_p(dummy.ctypes.data),
                                                dummy.ctypes.data, dummy.ctypes.data, C.byref(err), None)
        assert rc == _lib.PLBM_E_INVALID and "bad sizes" in _lib.last_error()
