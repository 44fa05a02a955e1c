"""The GPU path against the reference's own recorded output.

The reference's Taylor-Green driver (app/main_taylor_green.f90), run with
the finite-difference Bardow streaming and BGK collision on a 64 x 64 grid,
printed the velocity L2 errors of graphs/fvm_bardow_64.txt (21 values of
dt/tau from 0.5 to 50, eight significant digits; committed as
tests/golden/reference_bardow64.npz).  The same driver runs here through
libplbmgpu.so -- plbm_set_properties, plbm_set_streaming(fdm_bardow),
plbm_set_pdf_to_equilibrium, plbm_perform_lbm_step, plbm_update_macros --
and must print the same digits: the fused stencil form with FMA arithmetic
and the fused hybrid collision at every point (17,558 to 1,755,763 steps),
the strict build (the reference's operations in order, two passes per step;
bit-identical to the oracle) at the points with dt/tau >= 1.5.  A point
takes 0.1 - 12 s on a GB300 (the 56 cases about 2.5 minutes).  "The same
digits" allows half a printed unit plus 3e-10 (reference_tgv.NOISE): the
spread between builds of the same arithmetic with and without FMA
contraction.
"""
from __future__ import annotations

import numpy as np
import pytest

import reference_tgv as RT

pytestmark = pytest.mark.gpu

POINTS = [float(d) for d in RT.points()[:, 0]]


def run_gpu(dt_over_tau: float, math: str) -> float:
    from plbm import LatticeGrid
    c = RT.case(dt_over_tau)
    rho, ux, uy = RT.initial_fields(c)
    with LatticeGrid(RT.NX, RT.NY, collision="bgk", math=math, streaming="fdm_bardow") as g:
        g.set_properties(c["nu"], c["dt"], 0.25)
        g.set_pdf_to_equilibrium(rho, ux, uy)
        g.perform_lbm_step(c["nsteps"])
        _, u, v = g.update_macros()
    return RT.l2_norm(c, u, v)


CASES = [(d, m) for m in ("fma", "hybrid") for d in POINTS] + [(d, "strict") for d in POINTS if d >= 1.5]


@pytest.mark.parametrize("dt_over_tau,math", CASES)
def test_gpu_reproduces_the_reference_output(gpu_lib, dt_over_tau, math):
    printed = dict(RT.points().tolist())[dt_over_tau]
    got = run_gpu(dt_over_tau, math)
    assert RT.within(got, printed), (got, printed)
