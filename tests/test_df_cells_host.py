"""The compensated binary32 cell operators of csrc/coll_df64.cuh, built for
the host with g++ from the same header and checked against binary64
evaluations of the formulas they restate:

* bgk_dev_comp (binary32 deviation storage, PLBM_MATH_HYBRID): the BGK
  collision of src/collision_bgk.F90:58-71 with the equilibrium of
  src/fvm_bardow.F90:99-126 on h = f - w, to about one rounding of the
  stored value;
* adj_step_comp (the adjoint's compensated reverse step): mu_q = (1 - omega)
  lambda_q + omega (A + c_q.(B - 3 S0 u)) and the dL/domega term
  sum_q lambda_q (feq_q - g_q), to about one rounding of lambda, and both
  several times closer than the same formulas in plain binary32.
"""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "periodic-lbm_gb300" / "csrc"
CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1.0])
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1.0])
W = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)


@pytest.fixture(scope="module")
def L(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    so = tmp_path_factory.mktemp("dc") / "libdc.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", str(CSRC),
                    str(ROOT / "tests" / "df_cells_host.cpp"), "-o", str(so)], check=True)
    lib = C.CDLL(str(so))
    lib.dc_bgk_comp.argtypes = [C.c_void_p, C.c_double]
    lib.dc_adj_comp.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
    lib.dc_adj_comp.restype = C.c_float
    return lib


def equilibrium(rho, ux, uy):
    cu = CX * ux + CY * uy
    return W * rho * (1 + 3 * cu + 4.5 * cu ** 2 - 1.5 * (ux * ux + uy * uy))


def moments(g):
    drho = g.sum()
    rho = 1 + drho
    return drho, rho, (CX @ g) / rho, (CY @ g) / rho


def near_equilibrium_cell(rng, neq=1e-5):
    rho = 1 + 1e-3 * rng.standard_normal()
    ux, uy = 0.03 * rng.standard_normal(2)
    return (equilibrium(rho, ux, uy) - W + neq * W * rng.standard_normal(9)).astype(np.float32)


def test_bgk_comp_is_one_rounding_from_binary64(L):
    """Error in units of the binary32 spacing of the cell's largest stored
    value: the storage rounding the compensated form is limited by (a
    population near zero is not resolved beyond its cell's scale)."""
    rng = np.random.default_rng(11)
    errs = []
    for _ in range(2000):
        h = near_equilibrium_cell(rng)
        omega = rng.uniform(0.7, 1.95)
        g = h.astype(np.float64)
        drho, rho, ux, uy = moments(g)
        ref = g + omega * ((equilibrium(rho, ux, uy) - W) - g)
        out = h.copy()
        L.dc_bgk_comp(out.ctypes.data, omega)
        unit = float(np.spacing(np.float32(np.abs(h).max())))
        errs.append(float(np.max(np.abs(out - ref))) / unit)
    assert max(errs) <= 1.0 and np.mean(errs) <= 0.5, (max(errs), np.mean(errs))


def adjoint_reference(g, l, omega):
    g, l = g.astype(np.float64), l.astype(np.float64)
    drho, rho, ux, uy = moments(g)
    cu = CX * ux + CY * uy
    usq = ux * ux + uy * uy
    neq = (equilibrium(rho, ux, uy) - W) - g
    wl = W * l
    s0 = wl.sum()
    a = (wl * (1 - 4.5 * cu ** 2 + 1.5 * usq)).sum()
    bx, by = (wl * (3 + 9 * cu) * CX).sum(), (wl * (3 + 9 * cu) * CY).sum()
    ex, ey = bx - 3 * s0 * ux, by - 3 * s0 * uy
    return (1 - omega) * l + omega * (a + CX * ex + CY * ey), (l * neq).sum(), np.abs(l * neq).sum()


def adjoint_plain32(g, l, omega):
    """The same formulas in binary32, in the order of k_adj_step."""
    f = np.float32
    g, l, om = g.astype(f), l.astype(f), f(omega)
    s, jx, jy = f(0), f(0), f(0)
    for q in range(9):
        s, jx, jy = f(s + g[q]), f(jx + f(CX[q]) * g[q]), f(jy + f(CY[q]) * g[q])
    rho = f(s + 1)
    ux, uy = f(jx / rho), f(jy / rho)
    u2 = f(ux * ux + uy * uy)
    d = s0 = a = bx = by = f(0)
    for q in range(9):
        cu = f(f(CX[q]) * ux + f(CY[q]) * uy)
        w = f(W[q])
        heq = f(w * f(s + rho * f(f(3) * cu + f(4.5) * cu * cu - f(1.5) * u2)))
        d = f(d + l[q] * f(heq - g[q]))
        wl = f(w * l[q])
        s0, a = f(s0 + wl), f(a + wl * f(f(1) - f(4.5) * cu * cu + f(1.5) * u2))
        b = f(wl * f(f(3) + f(9) * cu))
        bx, by = f(bx + b * f(CX[q])), f(by + b * f(CY[q]))
    ex, ey = f(bx - f(3) * s0 * ux), f(by - f(3) * s0 * uy)
    mu = np.array([f(f(f(1) - om) * l[p] + om * f(a + f(CX[p]) * ex + f(CY[p]) * ey)) for p in range(9)])
    return mu, d


def test_adjoint_comp_against_binary64(L):
    rng = np.random.default_rng(5)
    e_comp, e_plain, d_comp, d_plain = [], [], [], []
    for _ in range(2000):
        g = near_equilibrium_cell(rng)
        c0, cx, cy = rng.standard_normal(3)
        l = (c0 + 3 * (CX * cx + CY * cy) + 0.01 * rng.standard_normal(9)).astype(np.float32)
        omega = rng.uniform(0.7, 1.95)
        mu_ref, d_ref, d_scale = adjoint_reference(g, l, omega)
        mu = np.zeros(9, np.float32)
        d = L.dc_adj_comp(g.ctypes.data, l.ctypes.data, mu.ctypes.data, omega)
        mp, dp = adjoint_plain32(g, l, omega)
        sc = np.abs(l).max()
        e_comp.append(np.abs(mu - mu_ref).max() / sc)
        e_plain.append(np.abs(mp - mu_ref).max() / sc)
        d_comp.append(abs(d - d_ref) / d_scale)
        d_plain.append(abs(dp - d_ref) / d_scale)
    # mu: one binary32 rounding of lambda (spacing 2^-23 relative, 6e-8 half)
    assert max(e_comp) <= 1.2e-7 and np.mean(e_comp) <= 4e-8
    assert np.mean(e_comp) * 2.5 < np.mean(e_plain)
    # dL/domega term: relative to sum |lambda (feq - g)|
    assert np.mean(d_comp) * 10 < np.mean(d_plain)
