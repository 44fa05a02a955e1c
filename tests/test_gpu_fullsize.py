"""Parity at full sizes: the bench's 8192^2 binary64 state against the oracle,
conservation over its time loop, and a lattice past 2^32 elements (the 64-bit
index path of the fused kernels) checked on windows.

The oracle runs the whole 8192^2 lattice (a step takes well under a second on
the host cores).  The large lattice is checked through locality instead: K
steps of the periodic grid and of a window of it with a halo of K cells (run as
its own periodic grid) agree on the window's interior, so the oracle only sees
windows at the corners (periodic wrap) and at the top of the index range.

Both tests skip when the host or the device lacks the memory they need.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

KIND = {"bgk": 0, "trt": 1, "rr": 2}


def host_available_bytes() -> int:
    try:
        with open("/proc/meminfo") as fh:
            for line in fh:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def need_memory(host_gb: float, device_gb: float) -> None:
    import torch
    if host_available_bytes() < host_gb * 2**30:
        pytest.skip(f"needs {host_gb:.0f} GiB of free host memory")
    free, _ = torch.cuda.mem_get_info()
    if free < device_gb * 2**30:
        pytest.skip(f"needs {device_gb:.0f} GiB of free device memory")


def relinf(a, b) -> float:
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def bench_state():
    """The bench workload at its full size: 8192^2 TGV u0 = 0.05 + N(0, 1e-4^2)
    velocity noise (seed 1234), tau = 0.6."""
    need_memory(40, 24)
    from plbm import cases
    n, tau = 8192, 0.6
    rho, ux, uy = cases.tgv_with_noise(n, u0=0.05, sigma=1e-4, seed=1234, nu=(tau - 0.5) / 3.0)
    return {"n": n, "omega": 1.0 / tau, "fields": (rho, ux, uy)}


@pytest.mark.parametrize("math_mode", ["strict", "hybrid"])
@pytest.mark.parametrize("kind", ["bgk", "trt", "rr"])
def test_bench_size_against_oracle(gpu_lib, bench_state, kind, math_mode):
    """3 steps of the 8192^2 bench state: the strict build bit-identical to the
    oracle over the whole lattice, the hybrid arithmetic within 1e-12 in f and
    in rho, u."""
    from plbm import LatticeGrid
    s = bench_state
    n, steps = s["n"], 3
    f2 = np.empty((2, 9, n, O.pad16(n)))
    f2[1] = O.set_pdf_to_equilibrium(*s["fields"])
    iold, _ = O.perform_lbm_step(f2, n, 2, 1, KIND[kind], s["omega"], 0.25, steps)
    ref = f2[iold - 1]
    g = LatticeGrid(n, n, collision=kind, math=math_mode)
    g.set_relaxation(s["omega"], 0.25)
    g.set_pdf_to_equilibrium(*s["fields"])
    g.perform_lbm_step(steps)
    got = g.download(g.iold)
    g.close()
    if math_mode == "strict":
        assert np.array_equal(got, ref)
    else:
        assert relinf(got, ref) <= 1e-12
        for a, b in zip(O.update_macros(got, n), O.update_macros(ref, n)):
            assert relinf(a, b) <= 1e-12


def test_bench_size_conservation(gpu_lib, bench_state):
    """100 hybrid steps of the 8192^2 bench state on the periodic grid: total
    mass and momentum are invariants of the operator; the change stays at the
    rounding level (mass drifts ~1e-16 per cell-step in binary64, as in the
    reference's own arithmetic)."""
    from plbm import LatticeGrid
    s = bench_state
    n = s["n"]
    g = LatticeGrid(n, n, collision="bgk", math="hybrid")
    g.set_relaxation(s["omega"], 0.25)
    g.set_pdf_to_equilibrium(*s["fields"])
    g.perform_lbm_step(1)  # update_macros reads f(:,:,:,inew)
    rho0, ux0, uy0 = g.update_macros()
    m0 = math.fsum(rho0.ravel())
    jx0, jy0 = math.fsum((rho0 * ux0).ravel()), math.fsum((rho0 * uy0).ravel())
    del rho0, ux0, uy0
    g.perform_lbm_step(100)
    rho, ux, uy = g.update_macros()
    g.close()
    m = math.fsum(rho.ravel())
    jx, jy = math.fsum((rho * ux).ravel()), math.fsum((rho * uy).ravel())
    assert abs(m - m0) / m0 <= 1e-13
    assert abs(jx - jx0) / m0 <= 1e-14 and abs(jy - jy0) / m0 <= 1e-14


def windows(nx, ny, half):
    """Window centres: the four corners (periodic wrap in x and y), the top of
    the index range (largest x) and the middle."""
    return [(0, 0), (nx - 1, ny - 1), (nx - 1 - half, 0), (nx - 2, ny // 2), (nx // 2, ny - 3)]


@pytest.mark.parametrize("math_mode", ["strict", "hybrid"])
def test_lattice_past_2_32_elements(gpu_lib, math_mode):
    """16384 x 29128 (ld 29136): 9 ld nx = 4,296,278,016 elements per lattice,
    past 2^32, so the fused kernels take their 64-bit offsets.  Two steps of a
    smooth flow; rho, u on 16x16 windows (corners with periodic wrap, the
    largest offsets) against the oracle on the window plus a 2-cell halo."""
    need_memory(56, 96)
    from plbm import LatticeGrid
    nx, ny, steps, omega = 16384, 29128, 2, 1.0 / 0.6
    assert 9 * O.pad16(ny) * nx > 2**32
    x = np.arange(nx) * (2 * math.pi / nx)
    y = np.arange(ny) * (2 * math.pi / ny)
    sx, cx, sy, cy = np.sin(x), np.cos(x), np.sin(y), np.cos(y)
    c5 = np.cos(5 * y)

    def fields(ix, iy):
        """rho, ux, uy at the cells ix (x indices) x iy (y indices)."""
        rho = 1.0 + 1e-3 * np.outer(sx[ix], cy[iy])
        ux = 0.02 * np.outer(sx[ix], cy[iy]) + 0.01 * c5[iy][None, :]
        uy = -0.02 * np.outer(cx[ix], sy[iy])
        return rho, ux, uy

    g = LatticeGrid(nx, ny, collision="bgk", math=math_mode)
    g.set_relaxation(omega, 0.25)
    g.set_pdf_to_equilibrium(*fields(np.arange(nx), np.arange(ny)))
    g.perform_lbm_step(steps + 1)
    got = g.update_macros()  # reads f(:,:,:,inew): the lattice after `steps` steps
    g.close()
    # tolerance relative to each field's largest magnitude over the grid, as
    # relinf does for whole fields (a window near a zero of uy has |uy| ~ 1e-5)
    scale = [float(np.max(np.abs(a))) for a in got]
    w, h = 16, steps
    for (x0, y0) in windows(nx, ny, w // 2):
        ix = (x0 - w // 2 - h + np.arange(w + 2 * h)) % nx
        iy = (y0 - w // 2 - h + np.arange(w + 2 * h)) % ny
        f2 = np.empty((2, 9, w + 2 * h, O.pad16(w + 2 * h)))
        f2[1] = O.set_pdf_to_equilibrium(*fields(ix, iy))
        iold, _ = O.perform_lbm_step(f2, w + 2 * h, 2, 1, KIND["bgk"], omega, 0.25, steps)
        ref = O.update_macros(f2[iold - 1], w + 2 * h)
        inner = slice(h, h + w)
        for a, b, sc in zip(got, ref, scale):
            sub = a[np.ix_(ix[inner], iy[inner])]
            if math_mode == "strict":
                assert np.array_equal(sub, b[inner, inner]), (x0, y0)
            else:
                assert np.max(np.abs(sub - b[inner, inner])) <= 1e-12 * sc, (x0, y0)


@pytest.mark.parametrize("math_mode,threads,persistent", [("hybrid", 128, 0), ("fma", 128, 0), ("hybrid", 256, 1)])
def test_batched_512_grids_against_oracle(gpu_lib, math_mode, threads, persistent):
    """The bench's batched workload at its full size: 512 Taylor-Green grids of
    uneven sizes (32..1024 per side, 39.1 M cells) and relaxation times, BGK and
    TRT, 5 steps; every grid's rho, u against the oracle within 1e-12.  The
    per-step 128-thread launch (one kernel per collision kind) and the
    persistent kernel."""
    from plbm import batched
    from plbm.batched import Schedule
    specs, flds = batched.random_tgv_batch(512, 2024)
    b = batched.BatchedGrids(specs, "f64", math=math_mode)
    fields = [batched.tgv_fields(*fl) for fl in flds]
    for i, f in enumerate(fields):
        b.set_equilibrium(i, *f)
    b.schedule = Schedule.from_dict({"threads": threads, "ctas_per_sm": 0, "persistent": persistent,
                                     "ty": [32, 32, 64, 64, 64]})
    steps = 5
    b.run(steps)
    b.synchronize()
    kinds = {"bgk": KIND["bgk"], "trt": KIND["trt"]}
    for i, sp in enumerate(specs):
        f2 = np.empty((2, 9, sp.nx, O.pad16(sp.ny)))
        f2[1] = O.set_pdf_to_equilibrium(*fields[i])
        iold, _ = O.perform_lbm_step(f2, sp.ny, 2, 1, kinds[sp.kind], sp.omega, sp.trt_magic, steps)
        got = b.download(i)
        for a, c in zip(O.update_macros(got, sp.ny), O.update_macros(f2[iold - 1], sp.ny)):
            assert relinf(a, c) <= 1e-12, (i, sp)
    b.close()


@pytest.mark.parametrize("math_mode", ["strict", "hybrid"])
def test_plugin_bench_size_against_oracle(gpu_lib, math_mode):
    """The sim/ plugin ABI (shifted binary64 BGK, collide then push) on an
    8192^2 Taylor-Green state, 3 steps, against the oracle's restatement of
    sim/sim_slbm.F90: strict bit-identical, hybrid within 1e-12."""
    need_memory(48, 24)
    from plbm.plugin import SimPlugin, make_params
    n, omega, steps = 8192, 1.0 / 0.6, 3
    k = 2 * math.pi / n
    x = (np.arange(n) + 0.5) * k
    u = np.empty((n, n, 2), order="F")
    u[:, :, 0] = -0.05 * np.outer(np.cos(x), np.sin(x))
    u[:, :, 1] = 0.05 * np.outer(np.sin(x), np.cos(x))
    p = np.asfortranarray(-0.25 * 0.05 ** 2 * (np.cos(2 * x)[:, None] + np.cos(2 * x)[None, :]))
    sim = SimPlugin()
    sim.init((n, n), 1.0, p, u, params=make_params(math=math_mode))
    sim.steps(omega, steps)
    rho, uu = sim.vars()
    sim.free()
    f = O.sim_eqinit(p.T, u[:, :, 0].T, u[:, :, 1].T)
    f = O.sim_slbm_steps(f, omega, steps)
    r, ux, uy = (a.T for a in O.sim_macros(f))
    del f
    if math_mode == "strict":
        assert np.array_equal(rho, r)
        assert np.array_equal(uu[:, :, 0], ux) and np.array_equal(uu[:, :, 1], uy)
    else:
        assert relinf(rho, r) <= 1e-12
        assert relinf(uu[:, :, 0], ux) <= 1e-12 and relinf(uu[:, :, 1], uy) <= 1e-12


@pytest.mark.parametrize("nx,ny", [(4099, 2047), (2053, 4103)])
def test_slab_pipelined_equilibrium_and_macros_bit_identical(gpu_lib, nx, ny):
    """Grids of 2^22 cells and more move rho/ux/uy in x-column slabs on a
    second stream, overlapped with the equilibrium and moments kernels of the
    neighbouring slabs.  Uneven slab bounds: the equilibrium lattice and the
    update_macros fields equal the oracle's bit for bit (strict build)."""
    from plbm import LatticeGrid
    rng = np.random.default_rng(21)
    rho = 1.0 + 1e-3 * rng.standard_normal((nx, ny))
    ux, uy = 0.04 * rng.standard_normal((2, nx, ny))
    g = LatticeGrid(nx, ny, collision="bgk", math="strict")
    g.set_pdf_to_equilibrium(rho, ux, uy)
    f0 = O.set_pdf_to_equilibrium(rho, ux, uy)
    got = g.download(g.iold)
    assert np.array_equal(got[:, :, :ny], f0[:, :, :ny])
    g.set_relaxation(1.6, 0.25)
    g.perform_lbm_step(1)  # update_macros then reads inew: the initial state
    r, u, v = g.update_macros()
    g.close()
    ro, uo, vo = O.update_macros(f0, ny)
    assert np.array_equal(r, ro) and np.array_equal(u, uo) and np.array_equal(v, vo)
