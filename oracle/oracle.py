"""ctypes wrapper of the CPU restatement (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, as the checker.  The product never imports it.

Parity status: pinned to the reference binary's printed Taylor-Green errors
for the finite-difference Bardow streaming with BGK; unpinned for TRT, RR,
the improved BGK and lbm_stream (see plbm_oracle.h).

Array conventions follow the Fortran memory order:
  lattice f(ld,nx,0:8)        -> C-order numpy array (9, nx, ld)
  both buffers f(ld,nx,0:8,2) -> (2, 9, nx, ld)
  field (ny,nx)               -> (nx, ny)
  plugin lattice f(0:nx+1,0:ny+1,0:8) -> (9, ny+2, nx+2)
  plugin field (nx,ny)        -> (ny, nx)
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BGK, TRT, RR, BGKI = 0, 1, 2, 3

_libs: dict = {}


def build() -> None:
    """Compile liboracle.so and liboracle_fast.so with make (gcc + OpenMP)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


def lib(fast: bool = False) -> C.CDLL:
    name = "liboracle_fast.so" if fast else "liboracle.so"
    if name not in _libs:
        path = HERE / name
        if not path.exists():
            build()
        L = C.CDLL(str(path))
        d, i, vp = C.c_double, C.c_int, C.c_void_p
        sig = {
            "oref_pad16": (i, [i]),
            "oref_lbm_stream": (None, [i, i, i, vp, vp]),
            "oref_collide_bgk": (None, [i, i, i, vp, d, i]),
            "oref_magic_number": (d, [d, d]),
            "oref_lambda_d": (d, [d, d]),
            "oref_collide_trt": (None, [i, i, i, vp, d, d, i]),
            "oref_collide_rr": (None, [i, i, i, vp, d]),
            "oref_collide_bgk_improved": (None, [i, i, vp, d]),
            "oref_update_macros": (None, [i, i, i, vp, vp, vp, vp]),
            "oref_vorticity_2nd": (None, [i, i, vp, vp, vp]),
            "oref_vorticity_4th": (None, [i, i, vp, vp, vp]),
            "oref_set_properties": (None, [d, d, vp, vp, vp, vp]),
            "oref_equilibrium": (None, [d, d, d, vp]),
            "oref_set_pdf_to_equilibrium": (None, [i, i, i, vp, vp, vp, vp]),
            "oref_perform_lbm_step": (None, [i, i, i, vp, vp, vp, i, d, d, i]),
            "oref_stream_fvm_bardow": (None, [i, i, i, vp, vp, d]),
            "oref_stream_fdm_bardow": (None, [i, i, i, vp, vp, d, i]),
            "oref_stream_fdm_sofonea": (None, [i, i, i, vp, vp, d]),
            "oref_perform_step_scheme": (None, [i, i, i, vp, vp, vp, i, d, i, d, d, i]),
            "oref_taylor_green_eval": (None, [i, i, d, d, d, d, d, vp, vp, vp, i]),
            "oref_shear_layer_eval": (None, [i, i, d, d, d, d, d, vp, vp, vp]),
            "oref_tgv_l2_norm": (d, [i, i, vp, vp, vp, vp]),
            "oref_kinetic_energy": (d, [i, i, vp, vp, vp]),
            "oref_sim_eqinit_fields": (None, [i, i, i, vp, vp, vp, vp]),
            "oref_sim_macros": (None, [i, i, i, vp, vp, vp, vp]),
            "oref_sim_collide_stream_fused": (None, [i, i, vp, vp, d]),
            "oref_sim_bc_push": (None, [i, i, vp]),
            "oref_sim_slbm_steps": (None, [i, i, vp, vp, d, i]),
            "oref_sim_norm": (d, [i, i, vp, vp]),
            "oref_num_threads": (i, []),
            "oref_adjoint_bgk": (None, [i, i, vp, vp, d, i, vp, vp, vp, vp, vp, vp, vp]),
            "oref_forward_bgk": (None, [i, i, vp, vp, d, i, vp, vp]),
        }
        for n, (r, a) in sig.items():
            fn = getattr(L, n)
            fn.restype = r
            fn.argtypes = a
        _libs[name] = L
    return _libs[name]


def _p(a: np.ndarray) -> int:
    assert a.flags.c_contiguous and a.dtype == np.float64
    return a.ctypes.data


def pad16(n: int) -> int:
    return lib().oref_pad16(int(n))


def _nx_ld(f: np.ndarray) -> tuple[int, int]:
    return f.shape[-2], f.shape[-1]


# ---- src/ path ------------------------------------------------------------
def lbm_stream(fsrc: np.ndarray, ny: int, fast: bool = False) -> np.ndarray:
    nx, ld = _nx_ld(fsrc)
    fdst = np.zeros_like(fsrc)
    lib(fast).oref_lbm_stream(nx, ny, ld, _p(fsrc), _p(fdst))
    return fdst


def collide(f: np.ndarray, ny: int, kind: int, omega: float, trt_magic: float = 0.25,
            split: bool = False, fast: bool = False) -> None:
    """Collision in place on f (9, nx, ld)."""
    nx, ld = _nx_ld(f)
    L = lib(fast)
    if kind == BGK:
        L.oref_collide_bgk(nx, ny, ld, _p(f), omega, int(split))
    elif kind == TRT:
        L.oref_collide_trt(nx, ny, ld, _p(f), omega, L.oref_lambda_d(omega, trt_magic), int(split))
    elif kind == RR:
        L.oref_collide_rr(nx, ny, ld, _p(f), omega)
    elif kind == BGKI:
        L.oref_collide_bgk_improved(nx, ny, _p(f), omega)
    else:
        raise ValueError(kind)


def update_macros(f: np.ndarray, ny: int):
    nx, ld = _nx_ld(f)
    rho, ux, uy = (np.empty((nx, ny)) for _ in range(3))
    lib().oref_update_macros(nx, ny, ld, _p(f), _p(rho), _p(ux), _p(uy))
    return rho, ux, uy


def set_pdf_to_equilibrium(rho, ux, uy, ld: int | None = None) -> np.ndarray:
    rho, ux, uy = (np.ascontiguousarray(a, dtype=np.float64) for a in (rho, ux, uy))
    nx, ny = rho.shape
    ld = ld or pad16(ny)
    f = np.zeros((9, nx, ld))
    lib().oref_set_pdf_to_equilibrium(nx, ny, ld, _p(rho), _p(ux), _p(uy), _p(f))
    return f


def perform_lbm_step(f2: np.ndarray, ny: int, iold: int, inew: int, kind: int, omega: float,
                     trt_magic: float, nsteps: int, fast: bool = False):
    """perform_lbm_step x nsteps on both buffers f2 (2, 9, nx, ld); returns (iold, inew)."""
    nx, ld = _nx_ld(f2)
    a, b = C.c_int(iold), C.c_int(inew)
    lib(fast).oref_perform_lbm_step(nx, ny, ld, _p(f2), C.addressof(a), C.addressof(b), kind, omega,
                                    trt_magic, nsteps)
    return a.value, b.value


# streaming schemes of src/fvm_bardow.F90 (grid%streaming)
SCHEMES = {"lbm": 0, "fvm_bardow": 1, "fdm_bardow": 2, "fdm_bardow_iso": 3, "fdm_bardow_wls": 4,
           "fdm_sofonea": 5, "fdm_bardow_wls_gauss_v1": 6, "fdm_bardow_wls_gauss_v2": 7}


def stream_scheme(fold: np.ndarray, ny: int, scheme: str, dt: float, fnew: np.ndarray | None = None,
                  fast: bool = False) -> np.ndarray:
    """grid%streaming of the named scheme from fold (9, nx, ld) into fnew
    (src/fvm_bardow.F90:393-886; lbm_stream for "lbm")."""
    nx, ld = _nx_ld(fold)
    fnew = np.zeros_like(fold) if fnew is None else fnew
    L = lib(fast)
    s = SCHEMES[scheme]
    if s == 0:
        L.oref_lbm_stream(nx, ny, ld, _p(fold), _p(fnew))
    elif s == 1:
        L.oref_stream_fvm_bardow(nx, ny, ld, _p(fold), _p(fnew), dt)
    elif s in (2, 3, 4):
        L.oref_stream_fdm_bardow(nx, ny, ld, _p(fold), _p(fnew), dt, s - 2)
    elif s in (6, 7):
        L.oref_stream_fdm_bardow(nx, ny, ld, _p(fold), _p(fnew), dt, s - 3)
    else:
        L.oref_stream_fdm_sofonea(nx, ny, ld, _p(fold), _p(fnew), dt)
    return fnew


def perform_step_scheme(f2: np.ndarray, ny: int, iold: int, inew: int, scheme: str, dt: float, kind: int,
                        omega: float, trt_magic: float, nsteps: int, fast: bool = False):
    """perform_lbm_step x nsteps with grid%streaming => the named scheme."""
    nx, ld = _nx_ld(f2)
    a, b = C.c_int(iold), C.c_int(inew)
    lib(fast).oref_perform_step_scheme(nx, ny, ld, _p(f2), C.addressof(a), C.addressof(b), SCHEMES[scheme],
                                       dt, kind, omega, trt_magic, nsteps)
    return a.value, b.value


def perform_triple_step(f: np.ndarray, ny: int, iold: int, inew: int, imid: int, kind: int, omega: float,
                        trt_magic: float, nsteps: int):
    """perform_triple_step x nsteps (src/fvm_bardow.F90:322-340) with lbm_stream as
    grid%streaming, on f (nf, 9, nx, ld): stream iold -> inew (rows 1:ny,
    src/periodic_lbm.f90:45-127), f(iold) = f(inew), collide inew in place,
    then iold <- inew, inew <- imid, imid <- iold.  Returns (iold, inew, imid)."""
    for _ in range(nsteps):
        streamed = lbm_stream(f[iold - 1], ny)
        f[inew - 1][:, :, :ny] = streamed[:, :, :ny]
        f[iold - 1][...] = f[inew - 1]
        collide(f[inew - 1], ny, kind, omega, trt_magic)
        iold, inew, imid = inew, imid, iold
    return iold, inew, imid


def set_properties(nu: float, dt: float, magic: float | None = None):
    t, o, m = C.c_double(), C.c_double(), C.c_double()
    mp = None
    if magic is not None:
        mv = C.c_double(magic)
        mp = C.addressof(mv)
    lib().oref_set_properties(nu, dt, mp, C.addressof(t), C.addressof(o), C.addressof(m))
    return t.value, o.value, m.value


def lambda_d(omega: float, x: float) -> float:
    return lib().oref_lambda_d(omega, x)


def equilibrium(rho: float, ux: float, uy: float) -> np.ndarray:
    out = np.empty(9)
    lib().oref_equilibrium(rho, ux, uy, _p(out))
    return out


def vorticity(ux, uy, order: int = 2) -> np.ndarray:
    ux, uy = (np.ascontiguousarray(a, dtype=np.float64) for a in (ux, uy))
    nx, ny = ux.shape
    w = np.empty_like(ux)
    fn = lib().oref_vorticity_2nd if order == 2 else lib().oref_vorticity_4th
    fn(nx, ny, _p(ux), _p(uy), _p(w))
    return w


def taylor_green(nx, ny, kx, ky, umax, nu, t=0.0, ref_loop=False):
    p, ux, uy = (np.zeros((nx, ny)) for _ in range(3))
    lib().oref_taylor_green_eval(nx, ny, kx, ky, umax, nu, t, _p(p), _p(ux), _p(uy), int(ref_loop))
    return p, ux, uy


def shear_layer(nx, ny, length, u0, k, delta, rho0=1.0):
    rho, ux, uy = (np.zeros((nx, ny)) for _ in range(3))
    lib().oref_shear_layer_eval(nx, ny, length, u0, k, delta, rho0, _p(rho), _p(ux), _p(uy))
    return rho, ux, uy


def tgv_l2_norm(ux, uy, uxa, uya) -> float:
    nx, ny = ux.shape
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (ux, uy, uxa, uya)]
    return lib().oref_tgv_l2_norm(nx, ny, *[_p(a) for a in arrs])


def kinetic_energy(rho, ux, uy) -> float:
    nx, ny = rho.shape
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (rho, ux, uy)]
    return lib().oref_kinetic_energy(nx, ny, *[_p(a) for a in arrs])


# ---- sim/ plugin path -------------------------------------------------------
def sim_eqinit(p, u, v) -> np.ndarray:
    """lbm_eqinit_fields on (nx,ny) Fortran fields given as (ny, nx) arrays -> halo lattice."""
    p, u, v = (np.ascontiguousarray(a, dtype=np.float64) for a in (p, u, v))
    ny, nx = p.shape
    f = np.zeros((9, ny + 2, nx + 2))
    lib().oref_sim_eqinit_fields(nx, ny, 1, _p(f), _p(p), _p(u), _p(v))
    return f


def sim_macros(f: np.ndarray):
    ny, nx = f.shape[1] - 2, f.shape[2] - 2
    rho, u, v = (np.empty((ny, nx)) for _ in range(3))
    lib().oref_sim_macros(nx, ny, 1, _p(f), _p(rho), _p(u), _p(v))
    return rho, u, v


def sim_slbm_steps(f1: np.ndarray, omega: float, nsteps: int) -> np.ndarray:
    """nsteps plugin steps starting from f1 (f2 = f1 initially, sim/sim_slbm.F90:76)."""
    ny, nx = f1.shape[1] - 2, f1.shape[2] - 2
    a = f1.copy()
    b = f1.copy()
    lib().oref_sim_slbm_steps(nx, ny, _p(a), _p(b), omega, nsteps)
    return a


def forward_bgk(ux0, uy0, omega: float, nsteps: int):
    """u_T of f_0 = feq(1, u0) advanced nsteps BGK steps; fields (nx, ny)."""
    ux0, uy0 = (np.ascontiguousarray(a, dtype=np.float64) for a in (ux0, uy0))
    nx, ny = ux0.shape
    ux, uy = np.empty((nx, ny)), np.empty((nx, ny))
    lib().oref_forward_bgk(nx, ny, _p(ux0), _p(uy0), omega, nsteps, _p(ux), _p(uy))
    return ux, uy


def adjoint_bgk(ux0, uy0, omega: float, nsteps: int, gux, guy):
    """(u_T, dL/du0, dL/domega) for a loss with dL/du_T = (gux, guy)."""
    ux0, uy0, gux, guy = (np.ascontiguousarray(a, dtype=np.float64) for a in (ux0, uy0, gux, guy))
    nx, ny = ux0.shape
    out = [np.empty((nx, ny)) for _ in range(4)]
    dom = C.c_double()
    lib().oref_adjoint_bgk(nx, ny, _p(ux0), _p(uy0), omega, nsteps, _p(gux), _p(guy),
                           *[_p(a) for a in out], C.addressof(dom))
    return (out[0], out[1]), (out[2], out[3]), dom.value


def num_threads(fast: bool = False) -> int:
    return lib(fast).oref_num_threads()
