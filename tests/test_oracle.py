"""CPU tests of the oracle (the C restatement of the reference's Fortran).

The reference has no golden vectors of its own, so the oracle is pinned by
(1) a second, independent numpy restatement (tests/golden/make_golden.py)
that must agree bit for bit, (2) integer checks of the periodic wrap maps,
(3) conservation laws and the equilibrium fixed point, and (4) the analytic
Taylor-Green decay.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O

CASES = [(17, 13), (12, 32)]


def _lat2(f0):
    return np.stack([np.zeros_like(f0), f0])  # buffer 1 = inew, buffer 2 = iold


@pytest.mark.parametrize("nx,ny", CASES)
def test_stream_matches_golden(golden, nx, ny):
    tag = f"{nx}x{ny}"
    f0 = golden[f"{tag}_f0"]
    out = O.lbm_stream(f0, ny)
    assert np.array_equal(out[:, :, :ny], golden[f"{tag}_stream"][:, :, :ny])


@pytest.mark.parametrize("nx,ny", CASES)
@pytest.mark.parametrize("kind,omega", [(O.BGK, 1.25), (O.TRT, 1.6), (O.RR, 1.9)])
def test_ten_steps_match_golden(golden, nx, ny, kind, omega):
    tag = f"{nx}x{ny}"
    f2 = _lat2(golden[f"{tag}_f0"])
    iold, inew = O.perform_lbm_step(f2, ny, 2, 1, kind, omega, 0.25, 10)
    name = {O.BGK: "bgk", O.TRT: "trt", O.RR: "rr"}[kind]
    assert (iold, inew) == (2, 1)  # ten swaps
    assert np.array_equal(f2[iold - 1][:, :, :ny], golden[f"{tag}_{name}_10"][:, :, :ny])


@pytest.mark.parametrize("nx,ny", CASES)
def test_bgk_improved_sequence_association(golden, nx, ny):
    tag = f"{nx}x{ny}"
    f = golden[f"{tag}_f0"].copy()
    O.collide(f, ny, O.BGKI, 1.3)
    assert np.array_equal(f, golden[f"{tag}_bgki_collide"])


@pytest.mark.parametrize("nx,ny", CASES)
def test_macros_equilibrium_vorticity_match_golden(golden, nx, ny):
    tag = f"{nx}x{ny}"
    f0 = golden[f"{tag}_f0"]
    assert np.array_equal(np.stack(O.update_macros(f0, ny)), golden[f"{tag}_macros"])
    fe = O.set_pdf_to_equilibrium(golden[f"{tag}_eq_rho"], golden[f"{tag}_eq_ux"], golden[f"{tag}_eq_uy"])
    assert np.array_equal(fe[:, :, :ny], golden[f"{tag}_equilibrium"][:, :, :ny])
    ux, uy = golden[f"{tag}_eq_ux"], golden[f"{tag}_eq_uy"]
    assert np.array_equal(O.vorticity(ux, uy, 2), golden[f"{tag}_vort2"])
    assert np.array_equal(O.vorticity(ux, uy, 4), golden[f"{tag}_vort4"])


def test_plugin_semantics_match_golden(golden):
    p, u, v = golden["sim_p"], golden["sim_u"], golden["sim_v"]
    f = O.sim_eqinit(p, u, v)
    assert np.array_equal(f[:, 1:-1, 1:-1], golden["sim_h0"])
    f10 = O.sim_slbm_steps(f, 1.7, 10)
    assert np.array_equal(f10[:, 1:-1, 1:-1], golden["sim_h10"])
    assert np.array_equal(np.stack(O.sim_macros(f10)), golden["sim_macros10"])


def test_properties_match_golden(golden):
    tau, omega, magic = O.set_properties(0.1 / 3.0, 1.0)
    ref = golden["props"]
    assert (tau, omega, magic) == (ref[0], ref[1], ref[2])
    assert O.lambda_d(1.25, 0.25) == ref[3]
    # explicit magic
    assert O.set_properties(0.1, 1.0, 0.25)[2] == 0.25


@pytest.mark.parametrize("nx,ny", [(1, 1), (1, 5), (2, 3), (3, 2), (5, 17), (16, 16), (17, 31)])
def test_wrap_maps_exhaustive(nx, ny):
    """Each destination of lbm_stream holds the source the 1-based Fortran maps name
    (src/periodic_lbm.f90:63-64,79-80): xp1 = mod(x,nx)+1, xm1 = mod(nx+x-2,nx)+1."""
    ld = O.pad16(ny)
    src = np.arange(9 * nx * ld, dtype=np.float64).reshape(9, nx, ld)
    dst = O.lbm_stream(src, ny)
    cx = [0, 1, 0, -1, 0, 1, -1, -1, 1]
    cy = [0, 0, 1, 0, -1, 1, 1, -1, -1]
    for q in range(9):
        for x1 in range(1, nx + 1):
            xp1, xm1 = (x1 % nx) + 1, ((nx + x1 - 2) % nx) + 1
            sx = {1: xm1, -1: xp1, 0: x1}[cx[q]]
            for y1 in range(1, ny + 1):
                yp1, ym1 = (y1 % ny) + 1, ((ny + y1 - 2) % ny) + 1
                sy = {1: ym1, -1: yp1, 0: y1}[cy[q]]
                assert int(dst[q, x1 - 1, y1 - 1]) == int(src[q, sx - 1, sy - 1])


def _moments(f, ny):
    rho, ux, uy = O.update_macros(f, ny)
    return rho, rho * ux, rho * uy


@pytest.mark.parametrize("kind", [O.BGK, O.TRT, O.RR])
def test_collision_conserves_mass_and_momentum(golden, kind):
    f = golden["17x13_f0"].copy()
    r0, jx0, jy0 = _moments(f, 13)
    O.collide(f, 13, kind, 1.7, 0.25)
    r1, jx1, jy1 = _moments(f, 13)
    assert np.max(np.abs(r1 - r0)) < 1e-14
    assert np.max(np.abs(jx1 - jx0)) < 1e-15
    assert np.max(np.abs(jy1 - jy0)) < 1e-15


def test_equilibrium_is_a_fixed_point_of_bgk_and_rr():
    rng = np.random.default_rng(3)
    nx, ny = 9, 7
    rho = 1 + 1e-3 * rng.standard_normal((nx, ny))
    ux, uy = 0.03 * rng.standard_normal((2, nx, ny))
    fe = O.set_pdf_to_equilibrium(rho, ux, uy)
    f = fe.copy()
    O.collide(f, ny, O.BGK, 1.3)
    assert np.max(np.abs(f[:, :, :ny] - fe[:, :, :ny])) < 1e-15  # a few ulps of 4/9
    # RR adds 3rd/4th order Hermite terms to the same equilibrium: at rest they vanish
    fz = O.set_pdf_to_equilibrium(np.ones((nx, ny)), np.zeros((nx, ny)), np.zeros((nx, ny)))
    g = fz.copy()
    O.collide(g, ny, O.RR, 1.3)
    assert np.max(np.abs(g[:, :, :ny] - fz[:, :, :ny])) < 1e-15


def test_split_variants_agree_with_naive():
    """bgk_kernel_cache / trt_split (-DSPLIT builds) give the same states to rounding."""
    rng = np.random.default_rng(5)
    nx, ny = 11, 9
    rho = 1 + 1e-3 * rng.standard_normal((nx, ny))
    ux, uy = 0.02 * rng.standard_normal((2, nx, ny))
    f = O.set_pdf_to_equilibrium(rho, ux, uy) * (1 + 1e-4 * rng.standard_normal((9, nx, O.pad16(ny))))
    for kind in (O.BGK, O.TRT):
        a, b = f.copy(), f.copy()
        O.collide(a, ny, kind, 1.4, 0.25, split=False)
        O.collide(b, ny, kind, 1.4, 0.25, split=True)
        assert np.max(np.abs(a[:, :, :ny] - b[:, :, :ny])) < 1e-15


def test_taylor_green_decay_64():
    """Config: TGV 64^2, BGK, tau = 0.8, u0 = 0.01, 1000 steps: the velocity
    amplitude decays as exp(-2 nu k^2 t) with nu = (tau - 1/2)/3."""
    n, tau, u0 = 64, 0.8, 0.01
    nu = (tau - 0.5) / 3.0
    k = 2 * math.pi / n
    p, ux, uy = O.taylor_green(n, n, k, k, u0, nu)
    rho = p / (1.0 / 3.0) + 1.0
    f2 = _lat2(O.set_pdf_to_equilibrium(rho, ux, uy))
    _, omega, _ = O.set_properties(nu, 1.0)
    assert abs(omega - 1.25) < 1e-15
    e0 = O.kinetic_energy(rho, ux, uy)
    iold, inew = O.perform_lbm_step(f2, n, 2, 1, O.BGK, omega, 0.25, 1000)
    r, u, v = O.update_macros(f2[iold - 1], n)
    e1 = O.kinetic_energy(r, u, v)
    ratio = math.sqrt(e1 / e0)
    expect = math.exp(-2 * nu * k * k * 1000)
    assert abs(ratio / expect - 1) < 5e-3
    # L2 error against the analytic field (app/main_taylor_green.f90:174-212)
    _, uxa, uya = O.taylor_green(n, n, k, k, u0, nu, t=1000.0)
    assert O.tgv_l2_norm(u, v, uxa, uya) < 5e-3


def test_cpu_adjoint_matches_central_differences():
    """The FP64 CPU adjoint (the check for the GPU adjoint) against central
    finite differences of the same forward model, loss 0.5 |u_T - u*|^2."""
    nx, ny, steps, omega = 12, 10, 25, 1.3
    rng = np.random.default_rng(9)
    ux0, uy0 = 0.02 * rng.standard_normal((2, nx, ny))
    tx, ty = 0.01 * rng.standard_normal((2, nx, ny))

    def loss(u, v, om):
        a, b = O.forward_bgk(u, v, om, steps)
        return 0.5 * np.sum((a - tx) ** 2 + (b - ty) ** 2)

    (uT, vT) = O.forward_bgk(ux0, uy0, omega, steps)
    _, (gx, gy), gom = O.adjoint_bgk(ux0, uy0, omega, steps, uT - tx, vT - ty)
    h = 1e-6
    for (i, j, comp) in [(0, 0, 0), (3, 7, 1), (11, 9, 0), (5, 2, 1), (7, 4, 0)]:
        up, vp_ = ux0.copy(), uy0.copy()
        um, vm = ux0.copy(), uy0.copy()
        (up if comp == 0 else vp_)[i, j] += h
        (um if comp == 0 else vm)[i, j] -= h
        fd = (loss(up, vp_, omega) - loss(um, vm, omega)) / (2 * h)
        ad = (gx if comp == 0 else gy)[i, j]
        assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-3 * np.max(np.abs(gx)))
    fd_om = (loss(ux0, uy0, omega + h) - loss(ux0, uy0, omega - h)) / (2 * h)
    assert abs(fd_om - gom) <= 1e-6 * abs(gom)


def test_taylor_green_reference_loop_quirk():
    """The reference TGV loop runs y = 1..nx; on nx == ny both loops agree."""
    a = O.taylor_green(8, 8, 0.7, 0.7, 0.01, 0.1, ref_loop=True)
    b = O.taylor_green(8, 8, 0.7, 0.7, 0.01, 0.1, ref_loop=False)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    c = O.taylor_green(4, 8, 0.7, 0.7, 0.01, 0.1, ref_loop=True)
    assert np.all(c[1][:, 4:] == 0.0) and np.any(c[1][:, :4] != 0.0)


SCHEME_NAMES = ["fvm_bardow", "fdm_bardow", "fdm_bardow_iso", "fdm_bardow_wls", "fdm_bardow_wls_gauss_v1",
                "fdm_bardow_wls_gauss_v2", "fdm_sofonea"]


@pytest.mark.parametrize("nx,ny", [(17, 13), (16, 16)])
@pytest.mark.parametrize("scheme", SCHEME_NAMES)
def test_streaming_schemes_match_golden(golden, nx, ny, scheme):
    """stream_fvm_bardow / stream_fdm_bardow (5 variants) / stream_fdm_sofonea
    (src/fvm_bardow.F90:393-886): the C oracle against the independent numpy
    restatement, one application and 5 steps with BGK, bit for bit."""
    tag = f"schemes_{nx}x{ny}"
    f0 = golden[f"{tag}_f0"]
    out = O.stream_scheme(f0, ny, scheme, 0.7)
    assert np.array_equal(out[:, :, :ny], golden[f"{tag}_{scheme}"][:, :, :ny])
    f2 = _lat2(f0)
    iold, _ = O.perform_step_scheme(f2, ny, 2, 1, scheme, 0.7, O.BGK, 1.1, 0.25, 5)
    assert np.array_equal(f2[iold - 1][:, :, :ny], golden[f"{tag}_{scheme}_bgk5"][:, :, :ny])


@pytest.mark.parametrize("scheme", SCHEME_NAMES)
def test_streaming_schemes_conserve_each_population(scheme):
    rng = np.random.default_rng(8)
    nx, ny = 20, 11
    f = rng.random((9, nx, O.pad16(ny)))
    g = O.stream_scheme(f, ny, scheme, 0.6)
    for q in range(9):
        assert abs(g[q, :, :ny].sum() - f[q, :, :ny].sum()) < 1e-12 * f[q, :, :ny].sum()
    # dt = 0 leaves every population unchanged (no transport)
    h = O.stream_scheme(f, ny, scheme, 0.0)
    assert np.allclose(h[:, :, :ny], f[:, :, :ny], rtol=0, atol=1e-15)
