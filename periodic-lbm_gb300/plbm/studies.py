"""Plugin-driven studies of the reference's sim/cases.py, without plotting.

``TGVStudy`` (sim/cases.py:128-213), ``run`` (:221-233), the grid-refinement
study of ``main`` (:236-383) as ``convergence`` and ``perfsweep`` (:388-426)
with the same formulas, parameters and printed quantities; they return the
numbers instead of drawing them (matplotlib is not a dependency).  They drive
any object with the ``SimPlugin`` interface -- ``plbm.plugin.SimPlugin`` over
libplbmgpu.so, or the reference's own loader over another plugin.

Command line (the reference's ``python cases.py <dt/tau>``)::

    python -m plbm.studies convergence lattice [--nref 4] [--base 10]
    python -m plbm.studies perfsweep 256 1024 --step 256 --tsteps 200
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

CS = math.sqrt(1.0 / 3.0)

# L2 errors for N = 10, 20, ..., 320 listed beside the study in
# sim/cases.py:357-365 (method and parameters unstated there; kept for
# comparison only, not a golden).
REFERENCE_FERR = {10: 7.006e-02, 20: 1.741e-02, 40: 4.339e-03, 80: 1.084e-03, 160: 2.709e-04, 320: 6.772e-05}


def _vnorm(v) -> float:
    return float(np.linalg.norm(v))


class TGVStudy:
    """Taylor-Green vortex on a regular periodic grid of cell centres
    (sim/cases.py:128-213); arrays are (nx, ny), Fortran order."""

    def __init__(self, grid_size, umax: float, k, nu: float):
        self.umax = umax
        self.nu = nu
        self.k = tuple(k)
        nx, ny = grid_size
        x = np.arange(nx, dtype=float) + 0.5
        y = np.arange(ny, dtype=float) + 0.5
        self._xv, self._yv = np.meshgrid(x, y, indexing="ij")

    @property
    def decay_time(self) -> float:
        """The vortex decay constant 1 / (nu |k|^2)."""
        kx, ky = self.k
        return 1.0 / (self.nu * (kx ** 2 + ky ** 2))

    @property
    def grid(self):
        return self._xv, self._yv

    def solution(self, t: float, ret_stress_tensor: bool = False):
        """Pressure p (nx, ny) and velocity u (nx, ny, 2) at time t [and the
        stress tensor components S (nx, ny, 3)]."""
        td = self.decay_time
        kx, ky = self.k
        a = self.umax
        x, y = self._xv, self._yv
        e1 = math.exp(-t / td)
        u = np.empty(x.shape + (2,), order="F")
        p = np.empty(x.shape, order="F")
        u[:, :, 0] = -a * math.sqrt(ky / kx) * np.cos(kx * x) * np.sin(ky * y) * e1
        u[:, :, 1] = a * math.sqrt(kx / ky) * np.sin(kx * x) * np.cos(ky * y) * e1
        p[:, :] = -0.25 * a ** 2 * ((ky / kx) * np.cos(2.0 * kx * x) + (kx / ky) * np.cos(2.0 * ky * y)) \
            * math.exp(-2.0 * t / td)
        if ret_stress_tensor:
            S = np.empty(x.shape + (3,), order="F")
            S[:, :, 0] = a * math.sqrt(kx * ky) * np.sin(kx * x) * np.sin(ky * y) * e1
            S[:, :, 1] = 0.5 * a * (math.sqrt(kx ** 3 / ky) - math.sqrt(ky ** 3 / kx)) * np.cos(kx * x) \
                * np.cos(ky * y) * e1
            S[:, :, 2] = -S[:, :, 0]
            return p, u, S
        return p, u

    def norm1(self, t: float, u) -> float:
        """Maximum pointwise velocity error magnitude at time t."""
        _, uref = self.solution(t)
        uerr = u - uref
        return float(np.max(np.hypot(uerr[:, :, 0], uerr[:, :, 1])))

    def norm2(self, t: float, u) -> float:
        """Relative L2 error of the velocity magnitude at time t."""
        _, uref = self.solution(t)
        mag = np.hypot(u[:, :, 0], u[:, :, 1])
        magref = np.hypot(uref[:, :, 0], uref[:, :, 1])
        return _vnorm(magref - mag) / _vnorm(magref)

    def norm2x(self, t: float, ux) -> float:
        _, uref = self.solution(t)
        return _vnorm(ux - uref[:, :, 0]) / _vnorm(uref[:, :, 0])

    def norm2y(self, t: float, uy) -> float:
        _, uref = self.solution(t)
        return _vnorm(uy - uref[:, :, 1]) / _vnorm(uref[:, :, 1])


def _finish(sim) -> None:
    sync = getattr(sim, "synchronize", None)
    if sync is not None:
        sync()


def run(sim, omega: float, nsteps: int, batched: bool = True):
    """Advance nsteps steps; returns (simulated time, elapsed seconds).

    As sim/cases.py:221-233, with the elapsed time taken after the plugin's
    queued work has finished.  batched=True issues the steps in one call when
    the plugin offers it (``steps``), which gives the same state."""
    start = time.perf_counter()
    tm = 0.0
    if batched and hasattr(sim, "steps"):
        sim.steps(omega, nsteps)
        tm = nsteps * sim.dt
    else:
        for _ in range(nsteps):
            sim.step(omega)
            tm += sim.dt
    _finish(sim)
    return tm, time.perf_counter() - start


def tgv_case(n: int, base: int, dt_over_tau: float | None, re: float = 1.0):
    """Parameters of one refinement level of sim/cases.py:main (:252-282).

    dt_over_tau=None takes dt = 1 (lattice units), which the lattice Boltzmann
    plugins require (sim/sim_slbm.F90:48-51); the reference's study sets
    dt = (dt/tau) tau for its finite-difference plugins."""
    umax = 0.01 / (n / base)
    k = (2 * math.pi / n, 2 * math.pi / n)
    nu = umax * n / re
    tau = nu / CS ** 2
    dt = 1.0 if dt_over_tau is None else dt_over_tau * tau
    omega = dt / (tau + 0.5 * dt)
    case = TGVStudy((n, n), umax=umax, k=k, nu=nu)
    tend = -math.log(0.1) * case.decay_time
    nsteps = round(tend / dt)
    return case, {"n": n, "umax": umax, "nu": nu, "tau": tau, "dt": dt, "omega": omega, "nsteps": nsteps,
                  "cfl": math.sqrt(2) * dt, "mach": umax / CS, "Re": umax * n / nu, "taulb": 1.0 / omega}


def convergence(sim, dt_over_tau: float | None = None, base: int = 10, nref: int = 2, re: float = 1.0,
                params=None, verbose: bool = False) -> dict:
    """The grid-refinement study of sim/cases.py:main: for n = base * 2^i, run
    the TGV until it decays to 0.1 of its amplitude and record the errors.
    Returns per-level parameters, L1/L2/L2x/L2y errors, MLUPS and the ratios
    of successive errors (4 for second order)."""
    levels = []
    for i in range(nref):
        n = base * 2 ** i
        case, prm = tgv_case(n, base, dt_over_tau, re)
        p0, u0 = case.solution(t=0.0)
        sim.init((n, n), prm["dt"], p0, u0, params=params) if params is not None else \
            sim.init((n, n), prm["dt"], p0, u0)
        tend, elapsed = run(sim, prm["omega"], prm["nsteps"])
        _, u = sim.vars()
        _, uref = case.solution(t=tend)
        lvl = dict(prm, tend=tend, elapsed=elapsed,
                   mlups=n * n * prm["nsteps"] / max(elapsed, 1e-12) * 1e-6,
                   l1=case.norm1(tend, u), l2=case.norm2(tend, u),
                   l2x_plugin=float(sim.my_norm(u[:, :, 0], uref[:, :, 0])),
                   l2x=case.norm2x(tend, u[:, :, 0]), l2y=case.norm2y(tend, u[:, :, 1]))
        sim.free()
        levels.append(lvl)
        if verbose:
            print((n, n), lvl["l1"], lvl["l2"], lvl["elapsed"], lvl["mlups"], flush=True)
    ratios = [{"l2": levels[i]["l2"] / levels[i + 1]["l2"], "l1": levels[i]["l1"] / levels[i + 1]["l1"]}
              for i in range(len(levels) - 1)]
    return {"dt_over_tau": dt_over_tau, "levels": levels, "ratios": ratios}


def mem9(nx: int, ny: int, nhalo: int = 1) -> float:
    """MiB of a two-lattice D2Q9 binary64 halo grid (sim/cases.py:385-386)."""
    return (nx + 2 * nhalo) * (ny + 2 * nhalo) * 2 * 9 * 8 / (1024 ** 2)


def perfsweep(sim, lo: int, hi: int, step: int = 20, tsteps: int = 1000, dt: float | None = None,
              params=None, verbose: bool = False) -> dict:
    """MLUPS over square grids range(lo, hi, step) (sim/cases.py:388-426):
    TGV with umax = 0.01/(n/lo), Re = 100, dt = tau unless given."""
    grids = list(range(lo, hi, step))
    mlups, elapsed = [], []
    for n in grids:
        umax = 0.01 / (n / lo)
        k = (2 * math.pi / n, 2 * math.pi / n)
        nu = umax * n / 100
        tau = nu / CS ** 2
        dt_n = tau if dt is None else dt
        omega = dt_n / (tau + 0.5 * dt_n)
        case = TGVStudy((n, n), umax=umax, k=k, nu=nu)
        p0, u0 = case.solution(t=0.0)
        if verbose:
            print(f"Running grid size {(n, n)}; est. memory = {mem9(n, n)} MiB", flush=True)
        sim.init((n, n), dt_n, p0, u0, params=params) if params is not None else sim.init((n, n), dt_n, p0, u0)
        _, el = run(sim, omega, tsteps)
        elapsed.append(el)
        mlups.append(n * n / 1e6 * tsteps / el)
        sim.free()
    return {"grids": grids, "mlups": mlups, "elapsed": elapsed, "tsteps": tsteps}


def _main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    c = sub.add_parser("convergence")
    c.add_argument("dt_over_tau", help="dt/tau, or 'lattice' for dt = 1 (lattice Boltzmann plugins)")
    c.add_argument("--base", type=int, default=10)
    c.add_argument("--nref", type=int, default=2)
    p = sub.add_parser("perfsweep")
    p.add_argument("lo", type=int)
    p.add_argument("hi", type=int)
    p.add_argument("--step", type=int, default=20)
    p.add_argument("--tsteps", type=int, default=1000)
    for q in (c, p):
        q.add_argument("--plugin", default=None, help="plugin .so (default: libplbmgpu.so)")
    args = ap.parse_args(argv)
    from .plugin import SimPlugin
    sim = SimPlugin(args.plugin)
    if args.cmd == "convergence":
        dto = None if args.dt_over_tau == "lattice" else float(args.dt_over_tau)
        out = convergence(sim, dto, args.base, args.nref, verbose=True)
    else:
        out = perfsweep(sim, args.lo, args.hi, args.step, args.tsteps, verbose=True)
    print(json.dumps(out))


if __name__ == "__main__":
    _main()
