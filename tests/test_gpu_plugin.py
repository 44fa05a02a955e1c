"""GPU tests of the plugin C ABI (sim/lbm.h semantics) against the oracle's
restatement of sim/sim_slbm.F90 + sim/sim.F90, through SimPlugin."""
import math

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def tgv_fields(nx, ny, umax=0.02, seed=0):
    """TGV p, u (Fortran (nx,ny) order) as sim/cases.py:TGVStudy.solution builds them."""
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) + 0.5)[:, None]
    y = (np.arange(ny) + 0.5)[None, :]
    kx, ky = 2 * math.pi / nx, 2 * math.pi / ny
    u = np.empty((nx, ny, 2), order="F")
    u[:, :, 0] = -umax * math.sqrt(ky / kx) * np.cos(kx * x) * np.sin(ky * y) + 1e-5 * rng.standard_normal((nx, ny))
    u[:, :, 1] = umax * math.sqrt(kx / ky) * np.sin(kx * x) * np.cos(ky * y)
    p = np.asfortranarray(-0.25 * umax ** 2 * ((ky / kx) * np.cos(2 * kx * x) + (kx / ky) * np.cos(2 * ky * y)))
    return p, u


def oracle_run(p, u, omega, nsteps):
    # oracle plugin arrays are (ny, nx) C-order == (nx, ny) Fortran order
    f = O.sim_eqinit(p.T, u[:, :, 0].T, u[:, :, 1].T)
    f = O.sim_slbm_steps(f, omega, nsteps)
    rho, ux, uy = O.sim_macros(f)
    return rho.T, ux.T, uy.T


@pytest.mark.parametrize("nx,ny", [(13, 11), (64, 64), (100, 37)])
def test_plugin_strict_bit_identical(gpu_lib, nx, ny):
    from plbm.plugin import SimPlugin, make_params
    p, u = tgv_fields(nx, ny)
    sim = SimPlugin()
    sim.init((nx, ny), 1.0, p, u, params=make_params(math="strict"))
    for _ in range(25):
        sim.step(1.6)
    rho, uu = sim.vars()
    sim.free()
    r, ux, uy = oracle_run(p, u, 1.6, 25)
    assert np.array_equal(rho, r)
    assert np.array_equal(uu[:, :, 0], ux) and np.array_equal(uu[:, :, 1], uy)


def test_plugin_default_fma_within_1e12(gpu_lib):
    from plbm.plugin import SimPlugin
    nx, ny = 96, 80
    p, u = tgv_fields(nx, ny)
    sim = SimPlugin()
    sim.init((nx, ny), 1.0, p, u)  # params = NULL, as sim/cases.py passes it
    sim.steps(1.3, 200)
    rho, uu = sim.vars()
    sim.free()
    r, ux, uy = oracle_run(p, u, 1.3, 200)
    rel = lambda a, b: np.max(np.abs(a - b)) / np.max(np.abs(b))  # noqa: E731
    assert rel(rho, r) <= 1e-12
    assert rel(uu[:, :, 0], ux) <= 1e-12 and rel(uu[:, :, 1], uy) <= 1e-12


def test_plugin_steps_equals_repeated_step(gpu_lib):
    from plbm.plugin import SimPlugin
    p, u = tgv_fields(20, 30)
    a, b = SimPlugin(), SimPlugin()
    a.init((20, 30), 1.0, p, u)
    b.init((20, 30), 1.0, p, u)
    for _ in range(9):
        a.step(1.5)
    b.steps(1.5, 9)
    ra, ua = a.vars()
    rb, ub = b.vars()
    assert np.array_equal(ra, rb) and np.array_equal(ua, ub)
    a.free()
    b.free()


@pytest.mark.parametrize("math,storage", [("strict", "f64"), ("hybrid", "f64"), ("fma", "f32dev")])
def test_plugin_graph_replay_equals_repeated_step(gpu_lib, math, storage):
    """c_plbmgpu_steps on a small grid replays a captured loop of steps: the
    state equals single c_plbmgpu_step calls across odd counts and a change of
    omega (recapture)."""
    from plbm.plugin import SimPlugin, make_params
    p, u = tgv_fields(40, 24)
    a, b = SimPlugin(), SimPlugin()
    for s in (a, b):
        s.init((40, 24), 1.0, p, u, params=make_params(math=math, storage=storage))
    for n, omega in ((37, 1.5), (50, 1.5), (33, 1.8), (64, 1.8)):
        for _ in range(n):
            a.step(omega)
        b.steps(omega, n)
        ra, ua = a.vars()
        rb, ub = b.vars()
        assert np.array_equal(ra, rb) and np.array_equal(ua, ub)
    a.free()
    b.free()


def test_tgv_study_convergence_through_plugin(gpu_lib):
    """The reference's TGV study (sim/cases.py:236-330) on this plugin: second-order
    convergence of the L2 velocity error under grid refinement at fixed Re."""
    from plbm.plugin import SimPlugin
    cs = math.sqrt(1.0 / 3.0)
    errs = []
    for n in (16, 32, 64):
        umax = 0.01 / (n / 16)
        nu = umax * n / 10.0
        tau = nu / cs ** 2
        dt = 1.0
        omega = dt / (tau + 0.5 * dt)
        k = 2 * math.pi / n
        td = 1.0 / (nu * 2 * k * k)
        nsteps = round(-math.log(0.5) * td / dt)
        x = (np.arange(n) + 0.5)[:, None]
        y = (np.arange(n) + 0.5)[None, :]
        u = np.empty((n, n, 2), order="F")
        u[:, :, 0] = -umax * np.cos(k * x) * np.sin(k * y)
        u[:, :, 1] = umax * np.sin(k * x) * np.cos(k * y)
        p = np.asfortranarray(-0.25 * umax ** 2 * (np.cos(2 * k * x) + np.cos(2 * k * y)))
        sim = SimPlugin()
        sim.init((n, n), dt, p, u)
        sim.steps(omega, nsteps)
        _, uu = sim.vars()
        sim.free()
        decay = math.exp(-nsteps * dt / td)
        ua = u * decay
        mag = np.hypot(uu[:, :, 0], uu[:, :, 1])
        mref = np.hypot(ua[:, :, 0], ua[:, :, 1])
        errs.append(np.linalg.norm(mref - mag) / np.linalg.norm(mref))
    assert errs[0] / errs[1] > 3.0 and errs[1] / errs[2] > 3.0, errs


@pytest.mark.parametrize("kind", ["trt", "rr"])
def test_plugin_other_collisions_conserve(gpu_lib, kind):
    from plbm.plugin import SimPlugin, make_params
    nx, ny = 40, 24
    p, u = tgv_fields(nx, ny)
    sim = SimPlugin()
    sim.init((nx, ny), 1.0, p, u, params=make_params(kind=kind))
    r0, u0 = sim.vars()
    sim.steps(1.7, 50)
    r1, u1 = sim.vars()
    sim.free()
    assert abs(r1.sum() - r0.sum()) < 1e-10 * r0.sum()
    jx0, jx1 = (r0 * u0[:, :, 0]).sum(), (r1 * u1[:, :, 0]).sum()
    assert abs(jx1 - jx0) < 1e-12


def test_studies_convergence_on_gpu_plugin(gpu_lib):
    """plbm.studies.convergence (sim/cases.py:main) through libplbmgpu.so: the
    same errors as the oracle's plugin restatement, second order, and the L2
    errors listed beside the reference study (sim/cases.py:357-365) to 1.5 %."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).parent))
    from test_studies import OraclePlugin
    from plbm import studies
    from plbm.plugin import SimPlugin
    gpu = studies.convergence(SimPlugin(), None, base=10, nref=4)
    cpu = studies.convergence(OraclePlugin(), None, base=10, nref=4)
    for a, b in zip(gpu["levels"], cpu["levels"]):
        assert abs(a["l2"] - b["l2"]) <= 1e-9 * b["l2"]
        assert abs(a["l2"] / studies.REFERENCE_FERR[a["n"]] - 1.0) < 0.015
    for r in gpu["ratios"]:
        assert 3.9 < r["l2"] < 4.1


def test_studies_perfsweep_on_gpu_plugin(gpu_lib):
    from plbm import studies
    from plbm.plugin import SimPlugin
    out = studies.perfsweep(SimPlugin(), 256, 1024, step=256, tsteps=50, dt=1.0)
    assert out["grids"] == [256, 512, 768] and min(out["mlups"]) > 0


def test_plugin_hybrid_bgk_within_1e12(gpu_lib):
    """PLBM_MATH_HYBRID on the plugin's shifted binary64 populations against
    the oracle's restatement of sim/sim_slbm.F90 + sim/sim.F90."""
    from plbm.plugin import SimPlugin, make_params
    nx, ny = 96, 80
    p, u = tgv_fields(nx, ny)
    sim = SimPlugin()
    sim.init((nx, ny), 1.0, p, u, params=make_params(math="hybrid"))
    sim.steps(1.3, 300)
    rho, uu = sim.vars()
    sim.free()
    r, ux, uy = oracle_run(p, u, 1.3, 300)
    rel = lambda a, b: np.max(np.abs(a - b)) / np.max(np.abs(b))  # noqa: E731
    assert rel(rho, r) <= 1e-12
    assert rel(uu[:, :, 0], ux) <= 1e-12 and rel(uu[:, :, 1], uy) <= 1e-12


@pytest.mark.parametrize("tau", [0.6, 0.55])
def test_plugin_hybrid_bgk_long_horizon(gpu_lib, tau):
    """10,000 plugin steps (sim/ BGK, shifted binary64, hybrid arithmetic) of a
    256 x 192 TGV (amplitude decays by ~e^-1.1) against the oracle: the rounded
    constants' mass and momentum factors are corrected on DH = sum h and J as in
    the unshifted form."""
    from plbm.plugin import SimPlugin, make_params
    nx, ny, steps = 256, 192, 10000
    p, u = tgv_fields(nx, ny, umax=0.05)
    sim = SimPlugin()
    sim.init((nx, ny), 1.0, p, u, params=make_params(math="hybrid"))
    sim.steps(1.0 / tau, steps)
    rho, uu = sim.vars()
    sim.free()
    r, ux, uy = oracle_run(p, u, 1.0 / tau, steps)
    rel = lambda a, b: np.max(np.abs(a - b)) / np.max(np.abs(b))  # noqa: E731
    assert rel(rho, r) <= 1e-12
    assert rel(uu[:, :, 0], ux) <= 1e-12 and rel(uu[:, :, 1], uy) <= 1e-12


@pytest.mark.parametrize("kind", ["trt", "rr"])
def test_plugin_hybrid_other_collisions_match_fma(gpu_lib, kind):
    from plbm.plugin import SimPlugin, make_params
    nx, ny = 64, 48
    p, u = tgv_fields(nx, ny)
    out = []
    for m in ("fma", "hybrid"):
        sim = SimPlugin()
        sim.init((nx, ny), 1.0, p, u, params=make_params(kind=kind, math=m))
        sim.steps(1.6, 200)
        out.append(sim.vars())
        sim.free()
    (r0, u0), (r1, u1) = out
    assert np.max(np.abs(r1 - r0)) <= 1e-12 * np.max(np.abs(r0))
    assert np.max(np.abs(u1 - u0)) <= 1e-12 * np.max(np.abs(u0))


def test_plugin_hybrid_needs_f64(gpu_lib):
    from plbm import PlbmError
    from plbm.plugin import SimPlugin, make_params
    p, u = tgv_fields(16, 16)
    sim = SimPlugin()
    with pytest.raises(PlbmError):
        sim.init((16, 16), 1.0, p, u, params=make_params(storage="f32dev", math="hybrid"))


REFERENCE_FIXTURE = __import__("pathlib").Path(__file__).resolve().parent / "golden" / "reference_plugin.npz"


@pytest.mark.parametrize("case", ["n10", "n20", "n40", "rect48x32"])
@pytest.mark.parametrize("math_mode,tol", [("strict", 0.0), ("fma", 1e-12), ("hybrid", 1e-12)])
def test_reference_study_fixture(gpu_lib, case, math_mode, tol):
    """libplbmgpu.so, started from the fields the reference's TGVStudy built
    and run the reference study's step count, against the state the
    reference's own SimPlugin and run produced over the oracle plugin
    (tests/golden/reference_plugin.npz, made by make_reference_fixtures.py):
    strict bit-identical, FMA and hybrid within 1e-12; the study's error norms
    recomputed here (plbm.studies.TGVStudy, the plugin's norm) equal the
    reference's to 1e-9 (the analytic solution is re-evaluated on this
    machine, whose numpy sin/cos/exp may differ from the fixture machine's in
    the last ulp)."""
    from plbm.plugin import SimPlugin, make_params
    from plbm.studies import TGVStudy, run
    z = np.load(REFERENCE_FIXTURE)
    umax, kx, ky, nu, omega, nsteps, tend = z[case + "_params"]
    p0, u0 = z[case + "_p0"], z[case + "_u0"]
    grid_size = p0.shape
    sim = SimPlugin()
    sim.init(grid_size, 1.0, p0, u0, params=make_params(math=math_mode))
    tm, _ = run(sim, omega, int(nsteps))
    rho, u = sim.vars()
    study = TGVStudy(grid_size, umax=umax, k=(kx, ky), nu=nu)
    _, uref = study.solution(t=tm)
    norms = np.array([study.norm1(tm, u), study.norm2(tm, u), sim.my_norm(u[:, :, 0], uref[:, :, 0]),
                      study.norm2x(tm, u[:, :, 0]), study.norm2y(tm, u[:, :, 1])])
    sim.free()
    assert tm == tend
    r_ref, u_ref = z[case + "_rho"], z[case + "_u"]
    rel = lambda a, b: float(np.max(np.abs(a - b)) / np.max(np.abs(b)))  # noqa: E731
    errs = (rel(rho, r_ref), rel(u[:, :, 0], u_ref[:, :, 0]), rel(u[:, :, 1], u_ref[:, :, 1]))
    if tol == 0.0:
        assert np.array_equal(rho, r_ref) and np.array_equal(u, u_ref), errs
    else:
        assert max(errs) <= tol, errs
    np.testing.assert_allclose(norms, z[case + "_norms"], rtol=1e-9)
