"""The integer forms of the moments and equilibria (csrc/exact_fields.cuh),
the arithmetic of hybrid-mode grids around the step, built for the host with
g++ from the same header and checked against exact rational arithmetic:

* the integer division, fixed-point and weight conversions are correctly
  rounded (round to nearest even) on random and edge-case operands;
* the moments of a cell whose populations are at least 2^-7 are the correctly
  rounded rho = sum f and u = j / rho of the exact sums (update_macros,
  src/fvm_bardow.F90:368-382, evaluated without its roundings);
* the equilibrium is within 0.5 ulp + w_q 2^-58 of the exact
  w_q rho (1 + 3 c.u + 4.5 (c.u)^2 - 1.5 u^2) (src/fvm_bardow.F90:99-126),
  and within a few ulps of the reference's binary64 sequence;
* cells outside the stated ranges report `bad` (the kernels then use the
  reference's expressions).
"""
import ctypes as C
import random
import shutil
import subprocess
from fractions import Fraction as Fr
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "periodic-lbm_gb300" / "csrc"
W = [4 / 9] + [1 / 9] * 4 + [1 / 36] * 4
CX = [0, 1, 0, -1, 0, 1, -1, -1, 1]
CY = [0, 0, 1, 0, -1, 1, 1, -1, -1]


def load_host_build(tmpdir):
    """g++ build of tests/exact_fields_host.cpp in tmpdir, with its argument types."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    so = Path(tmpdir) / "libxf.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", str(CSRC),
                    str(ROOT / "tests" / "exact_fields_host.cpp"), "-o", str(so)], check=True)
    L = C.CDLL(str(so))
    L.xf_equilibrium_field.argtypes = [C.c_long] + [C.c_void_p] * 3 + [C.c_int, C.c_int, C.c_void_p]
    L.xf_equilibrium_field.restype = C.c_long
    L.xf_macros_field.argtypes = [C.c_long, C.c_void_p, C.c_int, C.c_void_p]
    L.xf_macros_field.restype = C.c_long
    L.xf_macros.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    L.xf_equilibrium.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_void_p]
    L.xf_rho_fixed_from_pressure.argtypes = [C.c_double]
    L.xf_rho_fixed_from_pressure.restype = C.c_int64
    L.xf_div.argtypes = [C.c_int64, C.c_uint64, C.POINTER(C.c_double)]
    L.xf_recip.argtypes = [C.c_uint64, C.POINTER(C.c_uint64)]
    L.xf_recip.restype = C.c_uint64
    L.xf_fixed_to_double.argtypes = [C.c_int64, C.c_int]
    L.xf_fixed_to_double.restype = C.c_double
    L.xf_weighted.argtypes = [C.c_double, C.c_int64, C.c_int]
    L.xf_weighted.restype = C.c_double
    return L


@pytest.fixture(scope="module")
def X(tmp_path_factory):
    return load_host_build(tmp_path_factory.mktemp("xf"))


def ulp(x):
    return float(np.spacing(abs(float(x))))


def ref_equilibrium(rho, ux, uy):
    """equilibrium() of src/fvm_bardow.F90:99-126 in the reference's order."""
    uxx, uyy = ux * ux, uy * uy
    indp = 1.0 - 1.5 * (uxx + uyy)
    p, m = ux + uy, ux - uy
    return [W[0] * rho * indp,
            W[1] * rho * (indp + 3.0 * ux + 4.5 * uxx), W[2] * rho * (indp + 3.0 * uy + 4.5 * uyy),
            W[3] * rho * (indp - 3.0 * ux + 4.5 * uxx), W[4] * rho * (indp - 3.0 * uy + 4.5 * uyy),
            W[5] * rho * (indp + 3.0 * p + 4.5 * p * p), W[6] * rho * (indp - 3.0 * m + 4.5 * m * m),
            W[7] * rho * (indp - 3.0 * p + 4.5 * p * p), W[8] * rho * (indp + 3.0 * m + 4.5 * m * m)]


def exact_equilibrium(rho, ux, uy, q, shifted=False):
    U, V = Fr(ux), Fr(uy)
    cu = CX[q] * U + CY[q] * V
    e = Fr(W[q]) * Fr(rho) * (1 + 3 * cu + Fr(9, 2) * cu * cu - Fr(3, 2) * (U * U + V * V))
    return e - Fr(W[q]) if shifted else e


def test_division_is_correctly_rounded(X):
    rnd = random.Random(11)
    out = C.c_double()
    cases = []
    for i in range(20000):
        b = rnd.randrange(1 << 57, 1 << 61) if i % 2 else rnd.randrange(1 << 32, 1 << 62)
        a = rnd.randrange(-(1 << rnd.randrange(1, 63)), 1 << rnd.randrange(1, 63))
        cases.append((a, b))
    cases += [(b * k, b) for b in (1 << 32, 1 << 59, (1 << 62) - 1, 3 << 58) for k in (-1, 1)]
    cases += [((1 << 63) - 1, 1 << 32), (-(1 << 63) + 1, (1 << 62) - 1), (1, (1 << 62) - 1)]
    for a, b in cases:
        assert X.xf_div(a, b, C.byref(out)) == 0
        assert out.value == float(Fr(a, b)), (a, b)


def test_reciprocal_within_one_unit(X):
    rnd = random.Random(12)
    bn = C.c_uint64()
    bs = [rnd.randrange(1, 1 << 62) for _ in range(20000)] + [1 << k for k in range(62)] + [(1 << 62) - 1]
    for b in bs:
        v = X.xf_recip(b, C.byref(bn))
        assert abs(v - (1 << 127) // bn.value) <= 1, b


def test_fixed_and_weight_conversions_round_to_nearest_even(X):
    rnd = random.Random(13)
    for _ in range(20000):
        t = rnd.randrange(-(1 << 63) + 1, 1 << 63) >> rnd.randrange(0, 63)
        assert X.xf_fixed_to_double(t, 59) == float(Fr(t, 1 << 59))
        w = W[rnd.randrange(9)]
        assert X.xf_weighted(w, t, 60) == float(Fr(w) * Fr(t, 1 << 60))
    # exact ties: the even neighbour
    for t in ((1 << 53) + 1, (1 << 53) + 3, -((1 << 54) + 2)):
        assert X.xf_fixed_to_double(t, 0) == float(t)


def test_moments_are_the_rounded_exact_moments(X):
    rs = np.random.default_rng(14)
    out = np.zeros(3)
    for i in range(3000):
        rho = 1 + 0.05 * rs.standard_normal()
        ux, uy = 0.08 * rs.standard_normal(2)
        if i % 4 == 0:
            ux *= 1e-7  # u far below the populations: no cancellation error
        f = np.array(ref_equilibrium(rho, ux, uy)) * (1 + 1e-3 * rs.standard_normal(9))
        assert X.xf_macros(f.ctypes.data, 0, out.ctypes.data) == 0
        F = [Fr(x) for x in f]
        R = sum(F)
        JX = sum(c * x for c, x in zip(CX, F))
        JY = sum(c * x for c, x in zip(CY, F))
        assert tuple(out) == (float(R), float(JX / R), float(JY / R))


def test_shifted_moments_within_half_ulp(X):
    """sim/sim.F90:160-173 on h = f - w: rho = 1 + sum h, u = j / rho."""
    rs = np.random.default_rng(15)
    out = np.zeros(3)
    for _ in range(2000):
        rho = 1 + 0.05 * rs.standard_normal()
        ux, uy = 0.08 * rs.standard_normal(2)
        h = np.array(ref_equilibrium(rho, ux, uy)) * (1 + 1e-3 * rs.standard_normal(9)) - np.array(W)
        assert X.xf_macros(h.ctypes.data, 1, out.ctypes.data) == 0
        H = [Fr(x) for x in h]
        R = 1 + sum(H)
        for got, want in ((out[0], R), (out[1], sum(c * x for c, x in zip(CX, H)) / R),
                          (out[2], sum(c * x for c, x in zip(CY, H)) / R)):
            assert abs(Fr(got) - want) <= Fr(ulp(want)) * Fr(1, 2) + Fr(1, 1 << 58)


def test_moments_out_of_range_report_bad(X):
    out = np.zeros(3)
    f = np.array(ref_equilibrium(1.0, 0.02, 0.01))
    for q, v in ((0, -1e-3), (0, 1.0), (5, np.nan), (1, np.inf)):
        g = f.copy()
        g[q] = v
        assert X.xf_macros(g.ctypes.data, 0, out.ctypes.data) == 1
    g = np.full(9, 0.95)  # rho = 8.55 >= 8
    assert X.xf_macros(g.ctypes.data, 0, out.ctypes.data) == 1
    h = f - np.array(W)
    h[0] = 0.5
    assert X.xf_macros(h.ctypes.data, 1, out.ctypes.data) == 1


def test_equilibrium_within_half_ulp_of_exact(X):
    rs = np.random.default_rng(16)
    o = np.zeros(9)
    for i in range(3000):
        rho = 1 + 0.05 * rs.standard_normal()
        ux, uy = np.clip(0.08 * rs.standard_normal(2), -0.2499, 0.2499)
        if i % 3 == 0:
            rho = rs.uniform(0.01, 1.99)
        if i % 5 == 0:
            uy *= 1e-9
        assert X.xf_equilibrium(rho, ux, uy, 0, 0, o.ctypes.data) == 0
        ref = ref_equilibrium(rho, ux, uy)
        for q in range(9):
            e = exact_equilibrium(rho, ux, uy, q)
            assert abs(Fr(o[q]) - e) <= Fr(ulp(e)) / 2 + Fr(W[q]) / (1 << 58)
            assert abs(o[q] - ref[q]) <= 8 * ulp(ref[q])


def test_shifted_equilibrium_from_pressure(X):
    """sim/sim.F90:181-199 and :357-384: rho = 1 + p / cs^2 with the binary64
    cs^2 = RN(1/3), h_q = feq_q - w_q, to 0.5 ulp + w_q 2^-58 absolute."""
    rs = np.random.default_rng(17)
    o = np.zeros(9)
    csqr = 1.0 / 3.0
    for _ in range(2000):
        p = 0.01 * rs.standard_normal()
        ux, uy = np.clip(0.08 * rs.standard_normal(2), -0.24, 0.24)
        assert X.xf_equilibrium(p, ux, uy, 1, 1, o.ctypes.data) == 0
        rho = 1 + Fr(p) / Fr(csqr)
        assert abs(Fr(X.xf_rho_fixed_from_pressure(p), 1 << 60) - rho) <= Fr(1, 1 << 60)
        U, V = Fr(ux), Fr(uy)
        for q in range(9):
            cu = CX[q] * U + CY[q] * V
            e = Fr(W[q]) * rho * (1 + 3 * cu + Fr(9, 2) * cu * cu - Fr(3, 2) * (U * U + V * V)) - Fr(W[q])
            assert abs(Fr(o[q]) - e) <= Fr(ulp(e)) / 2 + Fr(W[q]) * Fr(9, 1 << 61)


def test_equilibrium_out_of_range_reports_bad(X):
    o = np.zeros(9)
    for rho, ux, uy in ((2.0, 0.0, 0.0), (-0.5, 0.0, 0.0), (0.0, 0.0, 0.0), (1.0, 0.25, 0.0),
                        (1.0, 0.0, -0.3), (np.nan, 0.0, 0.0), (1.0, np.inf, 0.0)):
        assert X.xf_equilibrium(rho, ux, uy, 0, 0, o.ctypes.data) == 1
    assert X.xf_equilibrium(1.0, 0.2499, -0.2499, 0, 0, o.ctypes.data) == 0
