"""Fixture of the reference's own plugin study, for the GPU plugin tests.

Run where the reference checkout is present (it is read in place, see
tests/reference_python.py):

    python tests/golden/make_reference_fixtures.py

With the reference's TGVStudy, SimPlugin and run (sim/cases.py:13-233) it
drives the oracle's plugin library (oracle/liboracleplugin.so: the
restatement of sim/sim_slbm.F90 over sim/sim.F90) through three refinement
levels of the reference's TGV study (sim/cases.py:236-330 at dt = 1, the
lattice Boltzmann setting) and one rectangular grid, and stores per case the
initial fields, the state after the run, the simulated time and the error
norms the reference's study computes (norm1, norm2, the plugin's my_norm of
u_x, norm2x, norm2y) in tests/golden/reference_plugin.npz.  The GPU plugin
tests start libplbmgpu.so from the same fields and compare with these.

It also copies the reference's recorded Taylor-Green temporal-error curve
(graphs/fvm_bardow_64.txt: dt/tau and the velocity L2 error of its driver
with the finite-difference Bardow streaming and BGK on a 64 x 64 grid, 21
points) into tests/golden/reference_bardow64.npz as the expected values of
tests/test_reference_bardow64.py and tests/test_gpu_reference_bardow64.py.
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
OUT = HERE / "reference_plugin.npz"
OUT_BARDOW = HERE / "reference_bardow64.npz"


def cases():
    """(name, grid_size, umax, k, nu, omega, nsteps) of each fixture case."""
    import reference_python as RP
    out = []
    for n in (10, 20, 40):
        grid_size, umax, k, nu, omega, nsteps = RP.study_level(n)
        out.append((f"n{n}", grid_size, umax, k, nu, omega, nsteps))
    nu = 0.05
    out.append(("rect48x32", (48, 32), 0.04, (2 * math.pi / 48, 2 * math.pi / 32), nu, 1.0 / (3 * nu + 0.5), 200))
    return out


def make(R, plugin_path: str) -> dict:
    """The fixture arrays, computed with the reference module R (sim/cases.py)."""
    out = {}
    for name, grid_size, umax, k, nu, omega, nsteps in cases():
        case = R.TGVStudy(grid_size, umax=umax, k=k, nu=nu)
        p0, u0 = case.solution(t=0.0)
        sim = R.SimPlugin(plugin_path)
        sim.init(grid_size, 1.0, p0, u0)
        tend, _ = R.run(sim, omega, nsteps)
        rho, u = sim.vars()
        _, uref = case.solution(t=tend)
        norms = [case.norm1(tend, u), case.norm2(tend, u), sim.my_norm(u[:, :, 0], uref[:, :, 0]),
                 case.norm2x(tend, u[:, :, 0]), case.norm2y(tend, u[:, :, 1])]
        sim.free()
        out[name + "_params"] = np.array([umax, k[0], k[1], nu, omega, nsteps, tend])
        out[name + "_p0"] = p0
        out[name + "_u0"] = u0
        out[name + "_rho"] = rho
        out[name + "_u"] = u
        out[name + "_norms"] = np.array(norms)
    return out


def main() -> None:
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import reference_python as RP
    from oracle import oracle as O
    if not RP.available():
        raise SystemExit("the reference checkout is not present (set PLBM_REFERENCE_DIR)")
    O.build()
    z = make(RP.load_cases(), str(ROOT / "oracle" / "liboracleplugin.so"))
    np.savez_compressed(OUT, **z)
    print(f"wrote {OUT} ({len(z)} arrays)")
    import reference_tgv as RT
    pts = RT.read_reference_file(RP.reference_dir())
    np.savez_compressed(OUT_BARDOW, dt_over_tau_l2=pts)
    print(f"wrote {OUT_BARDOW} ({pts.shape[0]} points)")


if __name__ == "__main__":
    main()
