"""The C side of the Fortran drop-in module (periodic-lbm_gb300/fortran/plbm_gpu.f90).

No Fortran compiler exists on the build machines, so the module itself is not
compiled here.  This test issues, through ctypes, exactly the sequence of C
calls the module makes when a reference driver runs
(app/main_taylor_green.f90: grid%streaming => lbm_stream_gpu,
grid%collision => collide_*_gpu, perform_lbm_step of src/periodic_lbm.f90:15-29,
update_macros):

* plbm_gpu_attach: plbm_grid_create(nx, ny, nf = 2, PLBM_F64), plbm_set_math,
  plbm_upload of every buffer b = 1..nf of the host grid%f;
* per step, lbm_stream_gpu then collide_*_gpu, each first calling
  sync_state (plbm_grid_set_indices with the Fortran's iold/inew,
  plbm_set_relaxation, plbm_set_collision for the collision), then
  plbm_stream / plbm_collide; the driver then swaps iold and inew on the
  Fortran side;
* update_macros_gpu: sync_state, plbm_update_macros into grid%mf(ny,nx,3);
* plbm_gpu_detach: plbm_grid_destroy.

The resulting moments and lattices are compared with the fused
plbm_perform_lbm_step path and with the oracle.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

KIND = {"bgk": O.BGK, "trt": O.TRT, "rr": O.RR}


class FortranGrid:
    """Host state of a lattice_grid (iold, inew, omega, trt_magic, f, mf) as the
    Fortran driver holds it, and the module's calls on it."""

    def __init__(self, lib, nx, ny, f_host, omega, magic, math):
        from plbm import _lib
        self.L, self._lib = lib, _lib
        self.nx, self.ny = nx, ny
        self.iold, self.inew = 2, 1  # alloc_grid, src/fvm_bardow.F90:172-177
        self.omega, self.magic = omega, magic
        self.f = f_host  # (2, 9, nx, ld): f(ld,nx,0:8,2) in Fortran order
        self.mf = np.zeros((3, nx, ny))  # mf(ny,nx,3)
        h = C.c_void_p()
        self.check(lib.plbm_grid_create(nx, ny, 2, _lib.STORAGES["f64"], C.byref(h)))
        self.h = h
        self.check(lib.plbm_set_math(h, _lib.MATHS[math]))
        for b in (1, 2):
            self.check(lib.plbm_upload(h, self.f[b - 1].ctypes.data, b))

    def check(self, rc):
        assert rc == 0, self._lib.last_error()

    def sync_state(self, kind):
        self.check(self.L.plbm_grid_set_indices(self.h, self.iold, self.inew))
        self.check(self.L.plbm_set_relaxation(self.h, self.omega, self.magic))
        if kind is not None:
            self.check(self.L.plbm_set_collision(self.h, self._lib.KINDS[kind]))

    def perform_lbm_step(self, kind):
        self.sync_state(None)  # lbm_stream_gpu
        self.check(self.L.plbm_stream(self.h))
        self.sync_state(kind)  # collide_<kind>_gpu
        self.check(self.L.plbm_collide(self.h))
        self.iold, self.inew = self.inew, self.iold  # src/periodic_lbm.f90:24-26

    def update_macros(self):
        self.sync_state(None)
        self.check(self.L.plbm_update_macros(self.h, self.mf[0].ctypes.data, self.mf[1].ctypes.data,
                                             self.mf[2].ctypes.data))
        return self.mf

    def download(self, b):
        out = np.empty_like(self.f[0])
        self.check(self.L.plbm_download(self.h, out.ctypes.data, b))
        return out

    def detach(self):
        self.check(self.L.plbm_grid_destroy(self.h))


@pytest.mark.parametrize("kind", ["bgk", "trt", "rr"])
@pytest.mark.parametrize("math_mode,tol", [("strict", 0.0), ("hybrid", 1e-12)])
def test_fortran_module_call_sequence(gpu_lib, kind, math_mode, tol):
    from plbm import LatticeGrid
    nx, ny, steps, omega = 40, 28, 30, 1.6
    rng = np.random.default_rng(4)
    rho = 1.0 + 1e-3 * rng.standard_normal((nx, ny))
    ux, uy = 0.03 * rng.standard_normal((2, nx, ny))
    f2 = np.stack([np.zeros((9, nx, O.pad16(ny))), O.set_pdf_to_equilibrium(rho, ux, uy)])
    fg = FortranGrid(gpu_lib, nx, ny, f2.copy(), omega, 0.25, math_mode)
    for _ in range(steps):
        fg.perform_lbm_step(kind)
    mf = fg.update_macros().copy()
    last = fg.download(fg.iold)
    fg.detach()
    # the oracle: the reference's perform_lbm_step with lbm_stream + collide_<kind>
    ref = f2.copy()
    iold, inew = O.perform_lbm_step(ref, ny, 2, 1, KIND[kind], omega, 0.25, steps)
    assert (fg.iold, fg.inew) == (iold, inew)
    want = O.update_macros(ref[inew - 1], ny)  # update_macros reads inew
    # the fused path of the same library
    g = LatticeGrid(nx, ny, collision=kind, math=math_mode)
    g.set_relaxation(omega, 0.25)
    g.upload(f2[1], 2)
    g.perform_lbm_step(steps)
    fused = g.update_macros()
    g.close()
    for a, b, c in zip(mf, want, fused):
        if tol == 0.0:
            assert np.array_equal(a, b) and np.array_equal(a, c)
        else:
            assert np.max(np.abs(a - b)) <= tol * np.max(np.abs(b))
            assert np.max(np.abs(a - c)) <= tol * np.max(np.abs(c))
    if tol == 0.0:
        assert np.array_equal(last[:, :, :ny], ref[iold - 1][:, :, :ny])
