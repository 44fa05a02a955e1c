"""The integer moments and equilibria of hybrid-mode grids on the GPU
(csrc/exact_fields.cuh through k_macros / k_equilibrium).

* The device results are bit-identical to the host build of the same header
  (tests/exact_fields_host.cpp), whose rounding the CPU tests pin against
  exact rational arithmetic; sampled cells are checked against the exact
  values here too.
* Against the oracle's restatement of the reference (set_pdf_to_equilibrium,
  update_macros, sim/sim.F90 eqinit and macros): within a few ulps.
* The slab-pipelined path (grids of 2^22 cells or more) gives the same fields
  as the host build over the whole grid.
* Cells outside the integer forms' range take the reference's expressions:
  bit-identical to the oracle there.
"""
import math
from fractions import Fraction as Fr

import numpy as np
import pytest

from oracle import oracle as O
import test_exact_fields_host as H

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def X(tmp_path_factory):
    return H.load_host_build(tmp_path_factory.mktemp("xfg"))


def host_equilibrium(X, rho, ux, uy, shifted=False, from_pressure=False):
    """(9, nx, ny) equilibrium of (nx, ny) fields by the host build; NaN where out of range."""
    r, u, v = (np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (rho, ux, uy))
    out = np.empty((9, r.size))
    X.xf_equilibrium_field(r.size, r.ctypes.data, u.ctypes.data, v.ctypes.data, int(shifted), int(from_pressure),
                           out.ctypes.data)
    return out.reshape((9,) + np.shape(rho))


def host_macros(X, f, shifted=False):
    """rho, ux, uy of a (9, nx, ny) lattice by the host build."""
    g = np.ascontiguousarray(f.reshape(9, -1))
    out = np.empty((3, g.shape[1]))
    X.xf_macros_field(g.shape[1], g.ctypes.data, int(shifted), out.ctypes.data)
    return out.reshape((3,) + f.shape[1:])


def fields(nx, ny, seed, u0=0.05):
    rng = np.random.default_rng(seed)
    x = (np.arange(nx)[:, None] + 0.5) * 2 * math.pi / nx
    y = (np.arange(ny)[None, :] + 0.5) * 2 * math.pi / ny
    ux = u0 * np.cos(x) * np.sin(y) + 1e-3 * rng.standard_normal((nx, ny))
    uy = -u0 * np.sin(x) * np.cos(y) + 1e-3 * rng.standard_normal((nx, ny))
    rho = 1.0 - 0.75 * u0 ** 2 * (np.cos(2 * x) + np.cos(2 * y)) + 1e-4 * rng.standard_normal((nx, ny))
    return rho, ux, uy


def ulps(a, b):
    return np.max(np.abs(a - b) / np.spacing(np.abs(b)))


@pytest.mark.parametrize("nx,ny", [(24, 20), (100, 37)])
def test_grid_equilibrium_and_moments(gpu_lib, X, nx, ny):
    from plbm import LatticeGrid
    rho, ux, uy = fields(nx, ny, 1)
    g = LatticeGrid(nx, ny, collision="bgk", math="hybrid")
    g.set_pdf_to_equilibrium(rho, ux, uy)
    full = g.download(g.iold)
    f = full[:, :, :ny]
    want = host_equilibrium(X, rho, ux, uy)
    assert np.array_equal(f, want)
    ref = O.set_pdf_to_equilibrium(rho, ux, uy)[:, :, :ny]
    assert ulps(f, ref) <= 8
    rs = np.random.default_rng(2)
    for x, y in zip(rs.integers(0, nx, 40), rs.integers(0, ny, 40)):
        for q in range(9):
            e = H.exact_equilibrium(rho[x, y], ux[x, y], uy[x, y], q)
            assert abs(Fr(f[q, x, y]) - e) <= Fr(H.ulp(e)) / 2 + Fr(H.W[q]) / (1 << 58)
    # the moments of the same lattice (update_macros reads inew: upload it there)
    g.upload(full, g.inew)
    r2, u2, v2 = g.update_macros()
    g.close()
    hr, hu, hv = host_macros(X, f)
    assert np.array_equal(r2, hr) and np.array_equal(u2, hu) and np.array_equal(v2, hv)
    for a, b in zip((r2, u2, v2), O.update_macros(full, ny)):
        assert np.max(np.abs(a - b)) <= 4 * np.spacing(np.max(np.abs(b)))
    for x, y in zip(rs.integers(0, nx, 40), rs.integers(0, ny, 40)):
        F = [Fr(v) for v in f[:, x, y]]
        R = sum(F)
        assert r2[x, y] == float(R)
        assert u2[x, y] == float(sum(c * v for c, v in zip(H.CX, F)) / R)
        assert v2[x, y] == float(sum(c * v for c, v in zip(H.CY, F)) / R)


def test_grid_out_of_range_cells_take_the_reference_expressions(gpu_lib, X):
    from plbm import LatticeGrid
    nx, ny = 16, 12
    rho, ux, uy = fields(nx, ny, 3)
    rho[2, 3], ux[5, 5], uy[7, 1], rho[9, 9] = 2.5, 0.3, -0.26, -0.1
    g = LatticeGrid(nx, ny, collision="bgk", math="hybrid")
    g.set_pdf_to_equilibrium(rho, ux, uy)
    full = g.download(g.iold)
    f = full[:, :, :ny]
    want = host_equilibrium(X, rho, ux, uy)
    ref = O.set_pdf_to_equilibrium(rho, ux, uy)[:, :, :ny]
    out = np.isnan(want[0])
    assert out.sum() == 4
    assert np.array_equal(f[:, out], ref[:, out])
    assert np.array_equal(f[:, ~out], want[:, ~out])
    # moments: populations >= 1 (rho = 5 at rest) or negative leave the integer
    # range; so do the cells set above to rho = 2.5 (f_0 > 1) and rho = -0.1
    f[0, 4, 4], f[:, 6, 2] = 1.5, 5.0 * np.array(H.W)
    f[3, 8, 8] = -0.01
    g.upload(full, g.inew)
    m = g.update_macros()
    g.close()
    hm = host_macros(X, f)
    bad = np.isnan(hm[0])
    assert bad.sum() == 5 and bad[2, 3] and bad[9, 9]
    for a, b, c in zip(m, O.update_macros(full, ny), hm):
        assert np.array_equal(a[bad], b[bad])
        assert np.array_equal(a[~bad], c[~bad])


def test_fma_and_strict_grids_keep_the_reference_sequence(gpu_lib):
    from plbm import LatticeGrid
    nx, ny = 24, 20
    rho, ux, uy = fields(nx, ny, 4)
    ref = O.set_pdf_to_equilibrium(rho, ux, uy)[:, :, :ny]
    for m in ("fma", "strict"):
        g = LatticeGrid(nx, ny, collision="bgk", math=m)
        g.set_pdf_to_equilibrium(rho, ux, uy)
        full = g.download(g.iold)
        assert np.array_equal(full[:, :, :ny], ref)
        g.upload(full, g.inew)
        for a, b in zip(g.update_macros(), O.update_macros(full, ny)):
            assert np.array_equal(a, b)
        g.close()


def test_slab_pipelined_fields_match_the_host_build(gpu_lib, X):
    """4096^2 cells (several x-column slabs on the transfer stream): the
    equilibrium and the moments of the whole grid equal the host build."""
    from plbm import LatticeGrid
    n = 4096
    rho, ux, uy = fields(n, n, 5)
    g = LatticeGrid(n, n, collision="bgk", math="hybrid")
    g.set_pdf_to_equilibrium(rho, ux, uy)
    full = g.download(g.iold)  # ld = n: no padding
    want = host_equilibrium(X, rho, ux, uy)
    assert np.array_equal(full, want)
    del want
    g.upload(full, g.inew)
    m = g.update_macros()
    g.close()
    hm = host_macros(X, full)
    for a, b in zip(m, hm):
        assert np.array_equal(a, b)


def test_plugin_hybrid_init_and_vars(gpu_lib, X):
    """c_plbmgpu_init (sim/sim.F90:181-199, rho = 1 + p / cs^2 and the shifted
    equilibrium) then c_plbmgpu_vars (sim/sim.F90:160-173) with no step in
    between: the host build's shifted equilibrium and moments, bit for bit,
    and the oracle's plugin restatement within a few ulps."""
    from plbm.plugin import SimPlugin, make_params
    import test_gpu_plugin as TP
    nx, ny = 40, 24
    p, u = TP.tgv_fields(nx, ny, umax=0.05)
    sim = SimPlugin()
    sim.init((nx, ny), 1.0, p, u, params=make_params(math="hybrid"))
    rho, uu = sim.vars()
    sim.free()
    h = host_equilibrium(X, p, u[:, :, 0], u[:, :, 1], shifted=True, from_pressure=True)
    assert not np.isnan(h).any()
    hr, hu, hv = host_macros(X, h, shifted=True)
    assert np.array_equal(rho, hr) and np.array_equal(uu[:, :, 0], hu) and np.array_equal(uu[:, :, 1], hv)
    orr, oux, ouy = TP.oracle_run(p, u, 1.0, 0)
    assert np.max(np.abs(rho - orr)) <= 4 * np.spacing(1.0)
    for a, b in ((uu[:, :, 0], oux), (uu[:, :, 1], ouy)):
        assert np.max(np.abs(a - b)) <= 1e-15 * np.max(np.abs(b))
