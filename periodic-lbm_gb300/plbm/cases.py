"""Initial conditions of the benchmark cases (host, binary64, numpy).

Fields are returned as (nx, ny) C-order arrays, which is the memory order of
the Fortran (ny,nx) arrays of the reference (``a[x, y]`` = ``a(y+1, x+1)``).
"""
from __future__ import annotations

import math

import numpy as np

CSQR = 1.0 / 3.0


def cell_centres(n: int) -> np.ndarray:
    """(i - 1) + 0.5 for i = 1..n (src/benchmarks/taylor_green.f90:65,67)."""
    return np.arange(n, dtype=np.float64) + 0.5


def taylor_green(nx: int, ny: int, kx: float, ky: float, umax: float, nu: float, t: float = 0.0,
                 ref_loop: bool = False):
    """taylor_green_eval, src/benchmarks/taylor_green.f90:51-84: (p, ux, uy).

    The reference loops ``y = 1, self%nx`` (:68), which is only right for
    nx == ny; ``ref_loop=False`` (default) loops y over 1..ny so rectangular
    grids are filled completely.  With ref_loop=True rows y > nx are left 0
    (and for ny < nx the reference writes out of bounds; here rows stop at ny).
    """
    td = 1.0 / (nu * (kx ** 2 + ky ** 2))
    xx = cell_centres(nx)[:, None]
    yy = cell_centres(ny)[None, :]
    ux = -umax * math.sqrt(ky / kx) * np.cos(kx * xx) * np.sin(ky * yy) * math.exp(-t / td)
    uy = umax * math.sqrt(kx / ky) * np.sin(kx * xx) * np.cos(ky * yy) * math.exp(-t / td)
    p = (-0.25 * (umax ** 2) * ((ky / kx) * np.cos(2.0 * kx * xx) + (kx / ky) * np.cos(2.0 * ky * yy))
         * math.exp(-2.0 * t / td))
    ux = np.ascontiguousarray(np.broadcast_to(ux, (nx, ny)))
    uy = np.ascontiguousarray(np.broadcast_to(uy, (nx, ny)))
    p = np.ascontiguousarray(np.broadcast_to(p, (nx, ny)))
    if ref_loop and ny > nx:
        for a in (ux, uy, p):
            a[:, nx:] = 0.0
    return p, ux, uy


def tgv_density(p: np.ndarray, rho0: float = 1.0) -> np.ndarray:
    """Lattice density from TGV pressure, app/main_taylor_green.f90:145."""
    return p / CSQR + rho0


def shear_layer(nx: int, ny: int, length: float, u0: float, k: float, delta: float, rho0: float = 1.0):
    """eval_shear_layer_grid, src/benchmarks/shear_layer.f90:31-50: (rho, ux, uy)."""
    xd = (np.arange(nx, dtype=np.float64) + 0.5)[:, None] / length
    yd = (np.arange(ny, dtype=np.float64) + 0.5)[None, :] / length
    uy = u0 * delta * np.sin(2 * math.pi * (xd + 0.25))
    ux = np.where(yd <= 0.5, u0 * np.tanh(k * (yd - 0.25)), u0 * np.tanh(k * (0.75 - yd)))
    rho = np.full((nx, ny), rho0)
    return rho, np.ascontiguousarray(np.broadcast_to(ux, (nx, ny))), \
        np.ascontiguousarray(np.broadcast_to(uy, (nx, ny)))


def tgv_with_noise(n: int, u0: float = 0.05, sigma: float = 1e-4, seed: int = 1234, nu: float = 0.1 / 3):
    """Bandwidth-bench state: TGV (k = 2 pi / n) plus i.i.d. N(0, sigma^2) velocity noise.

    Returns (rho, ux, uy) with rho = 1 + p/cs^2.
    """
    k = 2.0 * math.pi / n
    p, ux, uy = taylor_green(n, n, k, k, u0, nu)
    rng = np.random.default_rng(seed)
    ux = ux + rng.normal(0.0, sigma, ux.shape)
    uy = uy + rng.normal(0.0, sigma, uy.shape)
    return tgv_density(p), ux, uy


def divergence_free_modes(n: int, nmodes: int = 16, kmax: int = 8, amp: float = 0.01, seed: int = 1):
    """Velocity u = curl(psi) of a streamfunction with `nmodes` integer wave vectors |k| <= kmax.

    psi = sum_m a_m/|k_m| * sin(k_m . x + phi_m) with a_m ~ N(0, amp^2), phases
    ~ U[0, 2 pi); u = d psi/dy, v = -d psi/dx, so div u = 0 exactly in the
    continuum.  Returns (ux, uy) as (n, n) arrays.
    """
    rng = np.random.default_rng(seed)
    ks = []
    while len(ks) < nmodes:
        kx, ky = rng.integers(-kmax, kmax + 1, size=2)
        if (kx, ky) != (0, 0) and kx * kx + ky * ky <= kmax * kmax and (kx, ky) not in ks and (-kx, -ky) not in ks:
            ks.append((int(kx), int(ky)))
    a = rng.normal(0.0, amp, nmodes)
    phi = rng.uniform(0.0, 2 * math.pi, nmodes)
    x = cell_centres(n)[:, None] * (2 * math.pi / n)
    y = cell_centres(n)[None, :] * (2 * math.pi / n)
    ux = np.zeros((n, n))
    uy = np.zeros((n, n))
    for (kx, ky), am, ph in zip(ks, a, phi):
        kk = math.hypot(kx, ky)
        c = np.cos(kx * x + ky * y + ph) * (am / kk)
        ux += ky * c
        uy -= kx * c
    return ux, uy
