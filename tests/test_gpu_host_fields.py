"""set_pdf_to_equilibrium / update_macros with page-locked host fields.

The kernels then read (write) the host arrays in place over the host link
instead of staging them through device memory with copy-engine transfers.
The results must be those of the staged path for pageable arrays, bit for bit,
in every arithmetic mode, on one-launch grids and on grids of 2^22 cells or
more (where pageable fields go through the slab pipeline); mixed pinned and
pageable outputs, and NULL outputs, take the staged path.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def pinned(shape):
    import torch
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


def fields(nx, ny, seed):
    rng = np.random.default_rng(seed)
    rho = 1.0 + 1e-3 * rng.standard_normal((nx, ny))
    ux, uy = 0.04 * rng.standard_normal((2, nx, ny))
    return rho, ux, uy


@pytest.mark.parametrize("math_mode", ["fma", "strict", "hybrid"])
@pytest.mark.parametrize("nx,ny", [(40, 24), (2048, 2048)])
def test_pinned_fields_equal_the_staged_path(gpu_lib, math_mode, nx, ny):
    from plbm import LatticeGrid, _lib
    lib = _lib.load()
    rho, ux, uy = fields(nx, ny, 7)
    pin_in = [pinned((nx, ny)) for _ in range(3)]
    for d, s in zip(pin_in, (rho, ux, uy)):
        d[...] = s
    out = {}
    for label, src in (("pageable", (rho, ux, uy)), ("pinned", pin_in)):
        g = LatticeGrid(nx, ny, collision="bgk", math=math_mode)
        g.set_relaxation(1.7, 0.25)
        g.set_pdf_to_equilibrium(*src)
        f0 = g.download(g.iold)
        g.perform_lbm_step(3)
        if label == "pinned":
            m = [pinned((nx, ny)) for _ in range(3)]
            _lib.check(lib.plbm_update_macros(g.handle, *[a.ctypes.data for a in m]))
            m = [a.copy() for a in m]
        else:
            m = list(g.update_macros())
        out[label] = (f0, m)
        g.close()
    assert np.array_equal(out["pinned"][0], out["pageable"][0])
    for a, b in zip(out["pinned"][1], out["pageable"][1]):
        assert np.array_equal(a, b)


def test_mixed_and_null_outputs(gpu_lib):
    from plbm import LatticeGrid, _lib
    lib = _lib.load()
    nx, ny = 33, 20
    g = LatticeGrid(nx, ny, collision="trt", math="hybrid")
    g.set_pdf_to_equilibrium(*fields(nx, ny, 8))
    g.perform_lbm_step(2)
    want = g.update_macros()
    pr, pageable_uy = pinned((nx, ny)), np.zeros((nx, ny))
    _lib.check(lib.plbm_update_macros(g.handle, pr.ctypes.data, None, pageable_uy.ctypes.data))
    assert np.array_equal(pr, want[0]) and np.array_equal(pageable_uy, want[2])
    pu = pinned((nx, ny))
    _lib.check(lib.plbm_update_macros(g.handle, None, pu.ctypes.data, None))
    assert np.array_equal(pu, want[1])
    g.close()


@pytest.mark.parametrize("storage", ["f64", "f32dev", "f16dev"])
def test_pinned_lattice_upload_and_download(gpu_lib, storage):
    """plbm_upload / plbm_download with a page-locked lattice: copied (and for
    deviation storage converted) by kernels reading or writing it in place;
    the same lattices as through the staged path."""
    from plbm import LatticeGrid, _lib
    from oracle import oracle as O
    lib = _lib.load()
    nx, ny = 48, 30
    f = O.set_pdf_to_equilibrium(*fields(nx, ny, 9))
    g = LatticeGrid(nx, ny, collision="bgk", storage=storage)
    fp = pinned(f.shape)
    fp[...] = f
    _lib.check(lib.plbm_upload(g.handle, fp.ctypes.data, 1))
    g.upload(f, 2)
    a = g.download(1)
    b = g.download(2)
    assert np.array_equal(a, b)
    dp = pinned(f.shape)
    dp[...] = np.nan
    _lib.check(lib.plbm_download(g.handle, dp.ctypes.data, 1))
    assert np.array_equal(dp, a)  # deviation storage downloads stay staged
    g.close()
