"""The oracle against the reference's own recorded output (CPU).

graphs/fvm_bardow_64.txt holds what the reference's Taylor-Green driver
(app/main_taylor_green.f90) printed with the finite-difference Bardow
streaming and BGK collision on a 64 x 64 grid: the velocity L2 error for 21
values of dt/tau, eight significant digits.  tests/reference_tgv.py restates
the driver; here the oracle runs it at the three largest dt/tau (fewest
steps) and must print the same digits, within the rounding of the
reference's own build.  tests/test_gpu_reference_bardow64.py runs all 21
points on the GPU.
"""
from __future__ import annotations

import numpy as np
import pytest

import reference_python as RP
import reference_tgv as RT
from oracle import oracle as O

def run_oracle(dt_over_tau: float) -> tuple[float, dict]:
    c = RT.case(dt_over_tau)
    _, omega, magic = O.set_properties(c["nu"], c["dt"], 0.25)
    rho, ux, uy = RT.initial_fields(c)
    f2 = np.zeros((2, 9, RT.NX, O.pad16(RT.NY)))
    # alloc_grid: inew = 1, iold = 2; set_pdf_to_equilibrium fills iold
    f2[1] = O.set_pdf_to_equilibrium(rho, ux, uy)
    iold, inew = O.perform_step_scheme(f2, RT.NY, 2, 1, "fdm_bardow", c["dt"], O.BGK, omega, magic,
                                       c["nsteps"])
    _, u, v = O.update_macros(f2[inew - 1], RT.NY)
    return RT.l2_norm(c, u, v), c


def test_fixture_is_the_reference_file():
    if not RP.available():
        pytest.skip("reference checkout not present")
    assert np.array_equal(RT.points(), RT.read_reference_file(RP.reference_dir()))


def test_fixture_shape():
    pts = RT.points()
    assert pts.shape == (21, 2)
    assert pts[0, 0] == 0.5 and pts[-1, 0] == 50.0
    assert np.all(np.diff(pts[:, 0]) > 0) and np.all(pts[:, 1] > 0)


def test_case_parameters():
    """The driver's parameters: omega = dt/(tau + dt/2) with tau = 3 nu and
    the step count of its time loop."""
    c = RT.case(50.0)
    assert c["nsteps"] == 17558
    assert c["t"] >= c["tmax"] > c["t"] - c["dt"]
    tau, omega, magic = O.set_properties(c["nu"], c["dt"], 0.25)
    assert tau == c["tau"] and magic == 0.25
    assert omega == c["dt"] / (c["tau"] + 0.5 * c["dt"])


def test_initial_condition_equals_the_oracle():
    c = RT.case(1.0)
    for t in (0.0, c["t"]):
        p, ux, uy = RT.taylor_green(c, t)
        po, uxo, uyo = O.taylor_green(RT.NX, RT.NY, c["kx"], c["ky"], c["umax"], c["nu"], t)
        assert np.array_equal(p, po) and np.array_equal(ux, uxo) and np.array_equal(uy, uyo)


@pytest.mark.parametrize("dt_over_tau", [50.0, 40.0, 30.0])
def test_oracle_reproduces_the_reference_output(dt_over_tau):
    printed = dict(RT.points().tolist())[dt_over_tau]
    got, _ = run_oracle(dt_over_tau)
    assert RT.within(got, printed), (got, printed)


def test_a_planted_mistake_in_the_oracle_is_seen():
    """The comparison separates: the same run with tau 1e-6 off (the
    driver's viscosity, as a wrong set_properties would give) misses the
    printed value by far more than the tolerance."""
    c = RT.case(50.0)
    _, omega, magic = O.set_properties(c["nu"] * (1 + 1e-6), c["dt"], 0.25)
    rho, ux, uy = RT.initial_fields(c)
    f2 = np.zeros((2, 9, RT.NX, O.pad16(RT.NY)))
    f2[1] = O.set_pdf_to_equilibrium(rho, ux, uy)
    _, inew = O.perform_step_scheme(f2, RT.NY, 2, 1, "fdm_bardow", c["dt"], O.BGK, omega, magic, c["nsteps"])
    _, u, v = O.update_macros(f2[inew - 1], RT.NY)
    printed = dict(RT.points().tolist())[50.0]
    assert abs(RT.l2_norm(c, u, v) - printed) > 100 * (0.5 * RT.print_unit(printed) + RT.NOISE)
