"""The plugin-driven studies (plbm.studies, after sim/cases.py) on the CPU:
the analytic TGV, and the drivers run against a stand-in plugin built on the
oracle's restatement of the plugin path (sim/sim_slbm.F90 + sim/sim.F90)."""
import math

import numpy as np
import pytest

from oracle import oracle as O


class OraclePlugin:
    """SimPlugin interface over the oracle's plugin-path restatement."""

    def init(self, grid_size, dt, rho, u, sigma=None, params=None):
        assert dt == 1.0 and sigma is None
        self.grid_size = tuple(grid_size)
        self._dt = dt
        p = np.asarray(rho)
        self.f = O.sim_eqinit(p.T, np.asarray(u)[:, :, 0].T, np.asarray(u)[:, :, 1].T)

    @property
    def dt(self):
        return self._dt

    def step(self, omega):
        self.f = O.sim_slbm_steps(self.f, omega, 1)

    def steps(self, omega, n):
        self.f = O.sim_slbm_steps(self.f, omega, n)

    def vars(self):
        rho, ux, uy = O.sim_macros(self.f)
        u = np.empty(self.grid_size + (2,), order="F")
        u[:, :, 0], u[:, :, 1] = ux.T, uy.T
        return np.asfortranarray(rho.T), u

    def my_norm(self, u, ua):
        return float(np.linalg.norm(u - ua) / np.linalg.norm(ua))

    def free(self):
        self.f = None


def test_tgv_solution_decays_and_is_divergence_free():
    from plbm.studies import TGVStudy
    n = 32
    k = 2 * math.pi / n
    case = TGVStudy((n, n), umax=0.02, k=(k, k), nu=0.05)
    p0, u0 = case.solution(0.0)
    p1, u1 = case.solution(37.0)
    assert np.allclose(u1, u0 * math.exp(-37.0 / case.decay_time), rtol=0, atol=1e-15)
    assert np.allclose(p1, p0 * math.exp(-2 * 37.0 / case.decay_time), rtol=0, atol=1e-15)
    # spectral divergence of the sampled field vanishes
    kk = 2 * np.pi * np.fft.fftfreq(n)
    div = np.fft.ifft2(1j * kk[:, None] * np.fft.fft2(u0[:, :, 0]) + 1j * kk[None, :] * np.fft.fft2(u0[:, :, 1]))
    assert np.max(np.abs(div)) < 1e-14
    assert case.norm2(37.0, u1) < 1e-13 and case.norm1(37.0, u1) < 1e-16
    _, _, S = case.solution(0.0, ret_stress_tensor=True)
    assert S.shape == (n, n, 3) and np.array_equal(S[:, :, 2], -S[:, :, 0])


def test_convergence_driver_second_order():
    from plbm import studies
    out = studies.convergence(OraclePlugin(), None, base=10, nref=3)
    lv = out["levels"]
    assert [x["n"] for x in lv] == [10, 20, 40]
    assert all(x["dt"] == 1.0 and x["nsteps"] > 0 for x in lv)
    for r in out["ratios"]:
        assert 3.5 < r["l2"] < 4.6, out["ratios"]
    assert abs(lv[0]["l2x"] - lv[0]["l2x_plugin"]) < 1e-15


def test_perfsweep_driver_reports_every_grid():
    from plbm import studies
    out = studies.perfsweep(OraclePlugin(), 16, 48, step=16, tsteps=5, dt=1.0)
    assert out["grids"] == [16, 32] and len(out["mlups"]) == 2 and min(out["mlups"]) > 0
    assert studies.mem9(10, 10) == pytest.approx(12 * 12 * 2 * 9 * 8 / 1024 ** 2)
