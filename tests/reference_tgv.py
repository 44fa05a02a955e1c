"""The reference's own Taylor-Green temporal-error record, for the tests.

The reference ships, beside its sources, the output of its Taylor-Green
driver on a 64 x 64 grid with the finite-difference Bardow streaming
(stream_fdm_bardow, src/fvm_bardow.F90:475-598) and BGK collision
(src/collision_bgk.F90): graphs/fvm_bardow_64.txt, the velocity L2 error at
the end of the run for 21 values of dt/tau from 0.5 to 50, eight
significant digits (plotted by graphs/graph1.plt as "Temporal error for
Taylor-Green vortex on a 64x64 grid").  It is the one record of numbers
that the reference's compiled code produced, so it pins the whole chain --
initial condition, set_properties, set_pdf_to_equilibrium, the streaming
scheme, the collision, update_macros and the error norm -- to the
reference binary rather than to a restatement.

tests/golden/make_reference_fixtures.py copies the 21 pairs into
tests/golden/reference_bardow64.npz (read where the reference checkout is
present; the GPU tests read only the fixture).

This module restates the driver that made them, app/main_taylor_green.f90:

* set-up (:43-90) with nx = ny = 64 and dt read as dt/tau (the commented
  lines :62-63, ``dt = dt_over_tau*tau``): umax = 0.01/sqrt(3),
  nu = umax nx / 100, tau = 3 nu, set_properties(nu, dt, magic = 1/4),
  kx = ky = 2 pi / 64, t_d = 1/(nu (kx^2 + ky^2)), tmax = ln 2 t_d,
  nsteps = int(1.1 tmax / dt);
* initial condition (:142-157): the TGV pressure and velocity at t = 0
  (src/benchmarks/taylor_green.f90:55-80), rho = p / csqr + 1, f at
  equilibrium;
* the time loop (:98-119): t = t + dt after each perform_lbm_step, stop at
  the first step with t >= tmax, then update_macros -- which reads
  f(:,:,:,inew), the state one step behind (src/fvm_bardow.F90:351);
* calc_L2_norm (:174-212): norm2(hypot(ux - uxa, uy - uya)) /
  norm2(hypot(uxa, uya)) against the analytic field at the final t.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
FIXTURE = HERE / "golden" / "reference_bardow64.npz"
REFERENCE_FILE = Path("graphs") / "fvm_bardow_64.txt"

NX = NY = 64


def read_reference_file(reference_dir: Path) -> np.ndarray:
    """The (dt/tau, L2 error) pairs of graphs/fvm_bardow_64.txt, shape (21, 2)."""
    return np.loadtxt(Path(reference_dir) / REFERENCE_FILE, dtype=np.float64, ndmin=2)


def points() -> np.ndarray:
    """The committed copy of the reference's pairs, shape (21, 2)."""
    with np.load(FIXTURE) as z:
        return np.array(z["dt_over_tau_l2"])


def case(dt_over_tau: float) -> dict:
    """Parameters of one point as app/main_taylor_green.f90:43-90 forms them
    (binary64, the same operations in the same order)."""
    umax = 0.01 / math.sqrt(3.0)
    nu = (umax * float(NX)) / 100.0
    tau = 3.0 * nu
    dt = dt_over_tau * tau
    pi = 4.0 * math.atan(1.0)
    kx = 2 * pi / float(NX)
    ky = 2 * pi / float(NY)
    td = 1.0 / (nu * (kx * kx + ky * ky))
    tmax = math.log(2.0) * td
    nsteps = int(1.1 * tmax / dt)
    # the time loop's clock: the steps actually taken and the final t
    t, taken = 0.0, 0
    for step in range(1, nsteps + 1):
        t = t + dt
        taken = step
        if t >= tmax:
            break
    return dict(umax=umax, nu=nu, tau=tau, dt=dt, kx=kx, ky=ky, td=td, tmax=tmax, nsteps=taken, t=t)


def taylor_green(c: dict, t: float):
    """TGV pressure and velocity at time t as (nx, ny) arrays indexed [x, y]
    (src/benchmarks/taylor_green.f90:55-80, cell centres at (i - 1) + 0.5),
    element by element with the C library's cos, sin and exp as the Fortran
    calls them, in the Fortran's left-to-right order."""
    kx, ky, umax, td = c["kx"], c["ky"], c["umax"], c["td"]
    p, ux, uy = (np.empty((NX, NY)) for _ in range(3))
    e1, e2 = math.exp(-t / td), math.exp(-2.0 * t / td)
    ax, ay = -umax * math.sqrt(ky / kx), umax * math.sqrt(kx / ky)
    ap = -0.25 * (umax * umax)
    for x in range(NX):
        xx = x + 0.5
        for y in range(NY):
            yy = y + 0.5
            ux[x, y] = ax * math.cos(kx * xx) * math.sin(ky * yy) * e1
            uy[x, y] = ay * math.sin(kx * xx) * math.cos(ky * yy) * e1
            p[x, y] = ap * ((ky / kx) * math.cos(2.0 * kx * xx) + (kx / ky) * math.cos(2.0 * ky * yy)) * e2
    return p, ux, uy


def initial_fields(c: dict):
    """rho, ux, uy of apply_initial_condition (app/main_taylor_green.f90:142-157)."""
    p, ux, uy = taylor_green(c, 0.0)
    rho = p / (1.0 / 3.0) + 1.0
    return rho, ux, uy


def l2_norm(c: dict, ux: np.ndarray, uy: np.ndarray) -> float:
    """calc_L2_norm (app/main_taylor_green.f90:174-212) at the final t."""
    _, uxa, uya = taylor_green(c, c["t"])
    above = np.sqrt(np.sum(np.hypot(ux - uxa, uy - uya) ** 2))
    below = np.sqrt(np.sum(np.hypot(uxa, uya) ** 2))
    return float(above / below)


def print_unit(printed: float) -> float:
    """One unit of the last printed digit (eight significant digits)."""
    return 10.0 ** (math.floor(math.log10(abs(printed))) - 7)


# Allowed |computed - printed| of a norm, beyond half a printed unit.  The
# reference binary's rounding is not known: the same restatement compiled
# without and with FMA contraction (gcc -ffp-contract=off against -O3
# -march=haswell -ffp-contract=fast) differs by up to 2.0e-10 in these norms
# after 10^4 - 10^6 steps, and the printed values lie within 2.2e-10 of the
# first and 9.3e-11 of the second beyond half a unit.  A viscosity 1e-6 off
# moves the norm at dt/tau = 50 by about 7e-7.
NOISE = 3e-10


def within(got: float, printed: float) -> bool:
    return abs(got - printed) <= 0.5 * print_unit(printed) + NOISE
