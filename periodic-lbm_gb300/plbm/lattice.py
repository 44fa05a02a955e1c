"""Device-resident ``lattice_grid`` over the plbm_* C ABI.

Mirrors the reference's Fortran interface (src/fvm_bardow.F90,
src/periodic_lbm.f90) one routine for one routine:

=====================================  ====================================
reference                               here
=====================================  ====================================
``alloc_grid(grid,nx,ny,nf)``           ``LatticeGrid(nx, ny, nf)``
``set_properties(grid,nu,dt,magic)``    ``grid.set_properties(nu, dt, magic)``
``grid%collision => collide_rr``        ``grid.collision = "rr"``
``grid%streaming => stream_fvm_bardow`` ``grid.streaming = "fvm_bardow"``
``set_pdf_to_equilibrium(grid)``        ``grid.set_pdf_to_equilibrium(rho, ux, uy)``
``perform_lbm_step(grid)``              ``grid.perform_lbm_step(nsteps=1)``
``grid%streaming()`` / ``collision()``  ``grid.stream()`` / ``grid.collide()``
``update_macros(grid)``                 ``rho, ux, uy = grid.update_macros()``
``dealloc_grid(grid)``                  ``grid.close()``
=====================================  ====================================

Arrays follow the Fortran layout: macroscopic fields are (ny, nx) with y
fastest, i.e. numpy arrays of shape (nx, ny) in C order (``a[x, y]``), and a
lattice f(ld,nx,0:8) is a C-order numpy array of shape (9, nx, ld).
Buffer indices are 1-based as in the Fortran.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, ptr


def pad16(n: int) -> int:
    """ld of alloc_grid: n rounded up to a multiple of 16 (src/fvm_bardow.F90:144-147)."""
    r = n % 16
    return n + (16 - r) if r else n


def _f64(a, shape) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


class LatticeGrid:
    """A D2Q9 periodic lattice on the GPU with the reference's semantics."""

    def __init__(self, nx: int, ny: int, nf: int = 2, storage: str | int = "f64",
                 collision: str | int = "bgk", math: str | int = "fma", streaming: str | int = "lbm"):
        self._lib = _lib.load()
        st = _lib.STORAGES[storage] if isinstance(storage, str) else int(storage)
        h = C.c_void_p()
        check(self._lib.plbm_grid_create(int(nx), int(ny), int(nf), st, C.byref(h)))
        self._h = h
        self.nx, self.ny, self.nf, self.storage = int(nx), int(ny), int(nf), st
        self.ld = pad16(self.ny)
        self.collision = collision
        self.math = math
        self.streaming = streaming

    # -- lifecycle ------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.plbm_grid_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise RuntimeError("grid is closed")
        return self._h

    # -- settings ---------------------------------------------------------------
    @property
    def collision(self) -> int:
        return self._kind

    @collision.setter
    def collision(self, kind) -> None:
        k = _lib.KINDS[kind] if isinstance(kind, str) else int(kind)
        check(self._lib.plbm_set_collision(self.handle, k))
        self._kind = k

    @property
    def math(self) -> int:
        return self._math

    @math.setter
    def math(self, m) -> None:
        v = _lib.MATHS[m] if isinstance(m, str) else int(m)
        check(self._lib.plbm_set_math(self.handle, v))
        self._math = v

    @property
    def streaming(self) -> int:
        return self._streaming

    @streaming.setter
    def streaming(self, scheme) -> None:
        """grid%streaming => lbm_stream | stream_fvm_bardow |
        stream_fdm_bardow[_iso|_wls|_wls_gauss_v1|_wls_gauss_v2] | stream_fdm_sofonea
        ("lbm", "fvm_bardow", "fdm_bardow", "fdm_bardow_iso", "fdm_bardow_wls",
        "fdm_bardow_wls_gauss_v1", "fdm_bardow_wls_gauss_v2", "fdm_sofonea")."""
        v = _lib.SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
        check(self._lib.plbm_set_streaming(self.handle, v))
        self._streaming = v

    def set_properties(self, nu: float, dt: float, magic: float | None = None) -> None:
        """set_properties, src/fvm_bardow.F90:242-269."""
        mp = C.byref(C.c_double(magic)) if magic is not None else None
        check(self._lib.plbm_set_properties(self.handle, float(nu), float(dt), mp))

    def set_time_step(self, dt: float) -> None:
        """grid%dt alone (the finite-volume / finite-difference schemes' time step)."""
        check(self._lib.plbm_set_time_step(self.handle, float(dt)))

    def set_relaxation(self, omega: float, trt_magic: float = 0.25) -> None:
        check(self._lib.plbm_set_relaxation(self.handle, float(omega), float(trt_magic)))

    def properties(self) -> dict:
        v = [C.c_double() for _ in range(5)]
        check(self._lib.plbm_get_properties(self.handle, *[C.byref(x) for x in v]))
        return dict(zip(("nu", "dt", "tau", "omega", "trt_magic"), (x.value for x in v)))

    @property
    def omega(self) -> float:
        return self.properties()["omega"]

    @property
    def indices(self) -> tuple[int, int]:
        """(iold, inew), 1-based."""
        a, b = C.c_int(), C.c_int()
        check(self._lib.plbm_grid_indices(self.handle, C.byref(a), C.byref(b)))
        return a.value, b.value

    @indices.setter
    def indices(self, v) -> None:
        check(self._lib.plbm_grid_set_indices(self.handle, int(v[0]), int(v[1])))

    @property
    def iold(self) -> int:
        return self.indices[0]

    @property
    def inew(self) -> int:
        return self.indices[1]

    @property
    def indices3(self) -> tuple[int, int, int]:
        """(iold, inew, imid), 1-based; imid = -1 for a two-lattice grid."""
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        check(self._lib.plbm_grid_indices3(self.handle, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    @indices3.setter
    def indices3(self, v) -> None:
        check(self._lib.plbm_grid_set_indices3(self.handle, int(v[0]), int(v[1]), int(v[2])))

    @property
    def imid(self) -> int:
        return self.indices3[2]

    def set_stream(self, stream) -> None:
        """Queue the handle's work on a torch stream or raw cudaStream_t; None = own stream.

        torch's legacy default stream (handle 0) maps to cudaStreamLegacy."""
        s = _lib.stream_handle(stream)
        check(self._lib.plbm_grid_set_stream(self.handle, C.c_void_p(s) if s else None))

    def device_ptr(self, ibuf: int) -> int:
        p = C.c_void_p()
        check(self._lib.plbm_grid_device_ptr(self.handle, int(ibuf), C.byref(p)))
        return p.value

    # -- transfers ----------------------------------------------------------------
    def lattice_shape(self) -> tuple[int, int, int]:
        return (9, self.nx, self.ld)

    def upload(self, f: np.ndarray, ibuf: int) -> None:
        """Host f(:,:,:,ibuf), shape (9, nx, ld) float64, to the device."""
        a = _f64(f, self.lattice_shape())
        check(self._lib.plbm_upload(self.handle, ptr(a), int(ibuf)))

    def download(self, ibuf: int) -> np.ndarray:
        out = np.zeros(self.lattice_shape(), dtype=np.float64)
        check(self._lib.plbm_download(self.handle, ptr(out), int(ibuf)))
        return out

    # -- the hot path -------------------------------------------------------------
    def set_pdf_to_equilibrium(self, rho, ux, uy) -> None:
        """set_pdf_to_equilibrium: (nx, ny) arrays -> f(:,:,:,iold)."""
        shp = (self.nx, self.ny)
        r, u, v = _f64(rho, shp), _f64(ux, shp), _f64(uy, shp)
        check(self._lib.plbm_set_pdf_to_equilibrium(self.handle, ptr(r), ptr(u), ptr(v)))

    def stream(self) -> None:
        """lbm_stream: f(:,:,:,iold) -> f(:,:,:,inew)."""
        check(self._lib.plbm_stream(self.handle))

    def collide(self) -> None:
        """grid%collision(): in place on f(:,:,:,inew)."""
        check(self._lib.plbm_collide(self.handle))

    def swap(self) -> None:
        o, n = self.indices
        self.indices = (n, o)

    def perform_lbm_step(self, nsteps: int = 1) -> None:
        """perform_lbm_step, nsteps times (fused stream+collide, then swap)."""
        check(self._lib.plbm_perform_lbm_step(self.handle, int(nsteps)))

    def perform_triple_step(self, nsteps: int = 1) -> None:
        """perform_triple_step (src/fvm_bardow.F90:322-340), nsteps times; nf >= 3."""
        check(self._lib.plbm_perform_triple_step(self.handle, int(nsteps)))

    # -- files ----------------------------------------------------------------------
    def output_npy(self, path) -> None:
        """output_npy: mf(ny,nx,3) of f(:,:,:,inew) as a Fortran-order .npy of shape (ny, nx, 3)."""
        check(self._lib.plbm_output_npy(self.handle, str(path).encode()))

    def output_npy_step(self, folder, filename: str, step: int = -1) -> str:
        """The reference's file name: folder/filename + %09d step + .npy (folder created)."""
        check(self._lib.plbm_output_npy_step(self.handle, str(folder).encode() if folder else None,
                                             filename.encode(), int(step)))
        name = filename + (f"{step:09d}" if step >= 0 else "") + ".npy"
        return f"{folder}/{name}" if folder else name

    def save_state(self, path) -> None:
        """All nf lattices as a Fortran-order binary64 .npy of shape (ld, nx, 9, nf)."""
        check(self._lib.plbm_save_state(self.handle, str(path).encode()))

    def load_state(self, path) -> None:
        check(self._lib.plbm_load_state(self.handle, str(path).encode()))

    def update_macros(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """update_macros: moments of f(:,:,:,inew) as (nx, ny) arrays."""
        shp = (self.nx, self.ny)
        rho, ux, uy = (np.empty(shp) for _ in range(3))
        check(self._lib.plbm_update_macros(self.handle, ptr(rho), ptr(ux), ptr(uy)))
        return rho, ux, uy

    def kinetic_energy(self, ibuf: int | None = None) -> float:
        e = C.c_double()
        check(self._lib.plbm_kinetic_energy(self.handle, int(ibuf or self.iold), C.byref(e)))
        return e.value

    def velocity_l2_error(self, uxa, uya, ibuf: int | None = None) -> float:
        shp = (self.nx, self.ny)
        a, b = _f64(uxa, shp), _f64(uya, shp)
        e = C.c_double()
        check(self._lib.plbm_velocity_l2_error(self.handle, int(ibuf or self.iold), ptr(a), ptr(b), C.byref(e)))
        return e.value

    def synchronize(self) -> None:
        check(self._lib.plbm_synchronize(self.handle))


def vorticity(ux, uy, order: int = 2) -> np.ndarray:
    """vorticity_2nd (order=2) / vorticity_4th (order=4) of src/vorticity.f90 on the GPU.

    ux, uy are (nx, ny) arrays (Fortran (ny,nx)); order=44 selects standard
    fourth-order weights.
    """
    lib = _lib.load()
    ux = np.ascontiguousarray(ux, dtype=np.float64)
    uy = np.ascontiguousarray(uy, dtype=np.float64)
    if ux.shape != uy.shape or ux.ndim != 2:
        raise ValueError("ux and uy must be 2-D arrays of one shape")
    nx, ny = ux.shape
    w = np.empty_like(ux)
    check(lib.plbm_vorticity(int(order), nx, ny, ptr(ux), ptr(uy), ptr(w)))
    return w


def write_npy(path, a: np.ndarray, fortran_order: bool = True) -> None:
    """Write a float64 array with the library's .npy writer (host only).

    fortran_order=True writes a's Fortran-order data (numpy reads back ``a``)."""
    arr = np.asarray(a, dtype=np.float64)
    data = np.asfortranarray(arr) if fortran_order else np.ascontiguousarray(arr)
    shape = (C.c_longlong * max(arr.ndim, 1))(*arr.shape)
    buf = data.ravel(order="F" if fortran_order else "C")
    check(_lib.load().plbm_write_npy(str(path).encode(), ptr(buf), arr.ndim, C.cast(shape, C.c_void_p),
                                     int(bool(fortran_order))))


def read_npy_header(path) -> dict:
    """Header of a .npy file as the library parses it."""
    nd, fo, off = C.c_int(), C.c_int(), C.c_longlong()
    shape = (C.c_longlong * 8)()
    check(_lib.load().plbm_read_npy_header(str(path).encode(), C.byref(nd), C.cast(shape, C.c_void_p),
                                           C.byref(fo), C.byref(off)))
    return {"shape": tuple(shape[i] for i in range(nd.value)), "fortran_order": bool(fo.value),
            "data_offset": off.value}

