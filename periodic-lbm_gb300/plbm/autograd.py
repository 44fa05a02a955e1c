"""Differentiable LBM time stepper for PyTorch.

``lbm_final_velocity(u0, tau, nsteps)`` runs the D2Q9 BGK model
f_0 = feq(1, u0), f_{n+1} = collide(stream(f_n)) for nsteps steps on the GPU and
returns the final velocity field u_T; its backward pass is the hand-written
discrete adjoint of libplbmgpu.so (plbm_adjoint_*), returning gradients with
respect to the initial velocity field and tau.

Shapes: u0 is a CUDA float64 tensor (2, nx, ny) -- component, x, y with y
fastest, i.e. the two (ny,nx) Fortran fields of the reference -- and tau a
0-d float64 tensor (omega = 1/tau).  storage "f64" differentiates the binary64
model, "f32dev" the binary32 deviation-storage model (gradients still
accumulated in binary64; ``Adjoint(..., math="hybrid")`` runs its reverse step
in compensated binary32).  Memory is bounded by checkpointing every
``checkpoint_every`` steps (default ~sqrt(nsteps)) and recomputing.
"""
from __future__ import annotations

import ctypes as C
from math import sqrt as _sqrt

import torch

from . import _lib
from ._lib import check


class Adjoint:
    """Owner of one plbm_adjoint handle (checkpoints of one forward run)."""

    def __init__(self, nx: int, ny: int, nsteps: int, checkpoint_every: int | None = None,
                 storage: str = "f64", math: str = "fma"):
        self._lib = _lib.load()
        k = checkpoint_every or max(1, int(round(_sqrt(nsteps))))
        h = C.c_void_p()
        check(self._lib.plbm_adjoint_create(int(nx), int(ny), _lib.STORAGES[storage], int(nsteps), int(k),
                                            C.byref(h)))
        self._h = h
        if math != "fma":
            try:
                check(self._lib.plbm_adjoint_set_math(h, _lib.MATHS[math]))
            except Exception:
                self.close()
                raise
        self.nx, self.ny, self.nsteps, self.checkpoint_every, self.storage = nx, ny, nsteps, k, storage

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.plbm_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def memory_bytes(self) -> int:
        v = C.c_size_t()
        check(self._lib.plbm_adjoint_memory(self._h, C.byref(v)))
        return v.value

    def _stream(self):
        s = _lib.stream_handle(torch.cuda.current_stream())
        check(self._lib.plbm_adjoint_set_stream(self._h, C.c_void_p(s)))

    def forward(self, u0: torch.Tensor, omega: float) -> torch.Tensor:
        u0 = u0.detach().contiguous()
        uT = torch.empty_like(u0)
        self._stream()
        check(self._lib.plbm_adjoint_forward(self._h, u0.data_ptr(), float(omega), uT.data_ptr()))
        return uT

    def backward(self, grad_uT: torch.Tensor) -> tuple[torch.Tensor, float]:
        g = grad_uT.detach().contiguous().to(torch.float64)
        out = torch.empty_like(g)
        dom = C.c_double()
        self._stream()
        check(self._lib.plbm_adjoint_backward(self._h, g.data_ptr(), out.data_ptr(), C.byref(dom)))
        return out, dom.value


class LBMFinalVelocity(torch.autograd.Function):
    """u_T = LBM_BGK^nsteps(u0, tau); backward = discrete adjoint."""

    @staticmethod
    def forward(ctx, u0, tau, nsteps, checkpoint_every, storage):
        if not (u0.is_cuda and u0.dtype == torch.float64 and u0.dim() == 3 and u0.shape[0] == 2):
            raise ValueError("u0 must be a CUDA float64 tensor of shape (2, nx, ny)")
        tau_v = float(tau)
        adj = Adjoint(u0.shape[1], u0.shape[2], int(nsteps), checkpoint_every, storage)
        uT = adj.forward(u0, 1.0 / tau_v)
        ctx.adj = adj
        ctx.tau = tau_v
        ctx.tau_is_tensor = torch.is_tensor(tau)
        return uT

    @staticmethod
    def backward(ctx, grad_uT):
        grad_u0, dom = ctx.adj.backward(grad_uT)
        ctx.adj.close()
        grad_tau = None
        if ctx.tau_is_tensor:
            # omega = 1/tau  =>  dL/dtau = -dL/domega / tau^2
            grad_tau = torch.tensor(-dom / (ctx.tau * ctx.tau), dtype=torch.float64, device=grad_u0.device)
        return grad_u0, grad_tau, None, None, None


def lbm_final_velocity(u0: torch.Tensor, tau, nsteps: int, checkpoint_every: int | None = None,
                       storage: str = "f64") -> torch.Tensor:
    return LBMFinalVelocity.apply(u0, tau, nsteps, checkpoint_every, storage)


def velocity_misfit(u0: torch.Tensor, tau, target: torch.Tensor, nsteps: int,
                    checkpoint_every: int | None = None, storage: str = "f64") -> torch.Tensor:
    """L = 1/2 |u_T - target|^2 (sum over cells and components)."""
    uT = lbm_final_velocity(u0, tau, nsteps, checkpoint_every, storage)
    return 0.5 * torch.sum((uT - target) ** 2)
