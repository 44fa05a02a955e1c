"""The reference's own Python study code (sim/cases.py) against this package.

CPU tests; skipped where the reference checkout is absent.  They pin:
* plbm.studies.TGVStudy (analytic solution, grid, stress tensor, the four
  error norms) to the reference's TGVStudy, bit for bit;
* plbm.plugin.SimPlugin and plbm.studies.run to the reference's SimPlugin and
  run: both drive the oracle's plugin library (liboracleplugin.so, the
  restatement of sim/sim_slbm.F90 over sim/sim.F90) to identical states;
* libplbmgpu.so to the reference's loader: SimPlugin binds its five
  c_plbmgpu_* entry points with the reference's own argument types;
* the committed fixture tests/golden/reference_plugin.npz (made by
  tests/golden/make_reference_fixtures.py with the reference's classes) to a
  rerun through the reference's classes.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np
import pytest

import reference_python as RP
from oracle import oracle as O

pytestmark = pytest.mark.skipif(not RP.available(), reason="reference checkout not present")

ROOT = Path(__file__).resolve().parents[1]
ORACLE_PLUGIN = ROOT / "oracle" / "liboracleplugin.so"
FIXTURE = ROOT / "tests" / "golden" / "reference_plugin.npz"

STUDIES = [((10, 10), 0.01, (2 * math.pi / 10, 2 * math.pi / 10), 0.1),
           ((32, 24), 0.05, (2 * math.pi / 32, 2 * math.pi / 24), 0.02),
           ((64, 64), 0.0025, (4 * math.pi / 64, 2 * math.pi / 64), 0.1)]


@pytest.fixture(scope="module")
def R():
    return RP.load_cases()


@pytest.fixture(scope="module")
def oracle_plugin():
    O.build()
    assert ORACLE_PLUGIN.exists()
    return str(ORACLE_PLUGIN)


@pytest.mark.parametrize("grid_size,umax,k,nu", STUDIES)
def test_tgv_study_is_the_reference_bit_for_bit(R, grid_size, umax, k, nu):
    from plbm.studies import TGVStudy
    ref = R.TGVStudy(grid_size, umax=umax, k=k, nu=nu)
    ours = TGVStudy(grid_size, umax=umax, k=k, nu=nu)
    assert ours.decay_time == ref.decay_time
    for a, b in zip(ours.grid, ref.grid):
        assert np.array_equal(a, b)
    rng = np.random.default_rng(3)
    for t in (0.0, 0.37 * ref.decay_time, 2.0 * ref.decay_time):
        p0, u0 = ref.solution(t)
        p1, u1 = ours.solution(t)
        assert np.array_equal(p0, p1) and np.array_equal(u0, u1)
        _, _, s0 = ref.solution(t, ret_stress_tensor=True)
        _, _, s1 = ours.solution(t, ret_stress_tensor=True)
        assert np.array_equal(s0, s1)
        u = u0 * (1.0 + 1e-3 * rng.standard_normal(u0.shape))
        assert ours.norm1(t, u) == ref.norm1(t, u)
        assert ours.norm2(t, u) == ref.norm2(t, u)
        assert ours.norm2x(t, u[:, :, 0]) == ref.norm2x(t, u[:, :, 0])
        assert ours.norm2y(t, u[:, :, 1]) == ref.norm2y(t, u[:, :, 1])


def test_tgv_study_and_the_oracle_initial_condition(R):
    """The reference has two statements of the TGV: sim/cases.py (Python, the
    plugin studies) and src/benchmarks/taylor_green.f90 (the src/ drivers),
    restated by the oracle.  Same formulas in another association: equal to
    within a few ulps."""
    n = 48
    k = 2 * math.pi / n
    ref = R.TGVStudy((n, n), umax=0.05, k=(k, k), nu=0.02)
    t = 0.25 * ref.decay_time
    p, u = ref.solution(t)
    po, uxo, uyo = O.taylor_green(n, n, k, k, 0.05, 0.02, t)
    for a, b in ((p, po), (u[:, :, 0], uxo), (u[:, :, 1], uyo)):
        assert np.max(np.abs(a - b)) <= 8 * np.finfo(float).eps * np.max(np.abs(b))


def test_reference_loader_and_run_drive_the_oracle_plugin(R, oracle_plugin):
    """The reference's SimPlugin + run and this package's SimPlugin + run
    give identical states and times on the same plugin library, equal to the
    oracle's own plugin restatement (O.sim_slbm_steps)."""
    from plbm import plugin as P
    from plbm import studies as S
    grid_size, umax, k, nu, omega, nsteps = RP.study_level(20)
    case = R.TGVStudy(grid_size, umax=umax, k=k, nu=nu)
    p0, u0 = case.solution(t=0.0)
    ref = R.SimPlugin(oracle_plugin)
    ref.init(grid_size, 1.0, p0, u0)
    tm_ref, _ = R.run(ref, omega, nsteps)
    rho_ref, u_ref = ref.vars()
    ref.free()
    ours = P.SimPlugin(oracle_plugin)
    ours.init(grid_size, 1.0, p0, u0)
    tm, _ = S.run(ours, omega, nsteps, batched=False)
    rho, u = ours.vars()
    ours.free()
    assert tm == tm_ref
    assert np.array_equal(rho, rho_ref) and np.array_equal(u, u_ref)
    f = O.sim_eqinit(p0.T, u0[:, :, 0].T, u0[:, :, 1].T)
    f = O.sim_slbm_steps(f, omega, nsteps)
    r2, ux2, uy2 = O.sim_macros(f)
    assert np.array_equal(rho, r2.T) and np.array_equal(u[:, :, 0], ux2.T) and np.array_equal(u[:, :, 1], uy2.T)


def test_reference_loader_binds_libplbmgpu(R):
    """The reference's loader resolves c_plbmgpu_{init,step,vars,free,norm}
    from the library's file stem and binds them with its own argument types;
    the host-side norm runs without a device."""
    from plbm import _lib
    lib = _lib.load()
    sim = R.SimPlugin(str(_lib.LIB_PATH))
    assert sim.lib._name == lib._name
    rng = np.random.default_rng(1)
    u, ua = rng.standard_normal((2, 12, 9))
    want = np.linalg.norm(u - ua) / np.linalg.norm(ua)
    assert sim.my_norm(u, ua) == pytest.approx(want, rel=1e-15)
    assert sim.my_norm(u, ua) == O.lib().oref_sim_norm(12, 9, np.asfortranarray(u).ctypes.data,
                                                       np.asfortranarray(ua).ctypes.data)


def test_fixture_reproduces_through_the_reference(R, oracle_plugin):
    """tests/golden/reference_plugin.npz is what the reference's classes give
    (rerun here) -- the expected states and norms of the GPU plugin tests."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_reference_fixtures",
                                                  ROOT / "tests" / "golden" / "make_reference_fixtures.py")
    M = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(M)
    z = np.load(FIXTURE)
    again = M.make(R, oracle_plugin)
    assert sorted(z.files) == sorted(again)
    for key in z.files:
        assert np.array_equal(z[key], again[key]), key
