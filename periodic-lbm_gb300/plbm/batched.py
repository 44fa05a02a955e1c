"""Batched periodic grids: many D2Q9 lattices of uneven sizes and relaxation
times stepped together on the GPU (plbm_batch_* of include/plbm_gpu.h).

``BatchedGrids`` owns a device batch; ``random_tgv_batch`` builds the 512-grid
Taylor-Green workload (sizes log-uniform in [32, 1024], tau in [0.51, 1.5],
BGK/TRT 50/50, integer wavenumbers 1..4, u0 in [0.005, 0.05]).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _lib, cases
from ._lib import check, ptr

BUCKETS = 5


class Schedule(C.Structure):
    """plbm_batch_schedule."""

    _fields_ = [("threads", C.c_int), ("ctas_per_sm", C.c_int), ("persistent", C.c_int),
                ("ty", C.c_int * BUCKETS)]

    def as_dict(self) -> dict:
        return {"threads": self.threads, "ctas_per_sm": self.ctas_per_sm, "persistent": self.persistent,
                "ty": list(self.ty)}

    @classmethod
    def from_dict(cls, d: dict) -> "Schedule":
        s = cls()
        s.threads, s.ctas_per_sm, s.persistent = int(d["threads"]), int(d["ctas_per_sm"]), int(d["persistent"])
        for i, v in enumerate(d["ty"]):
            s.ty[i] = int(v)
        return s


def _bind():
    return _lib.load()


def default_schedule() -> Schedule:
    s = Schedule()
    check(_bind().plbm_batch_default_schedule(C.addressof(s)))
    return s


@dataclass
class GridSpec:
    nx: int
    ny: int
    kind: str      # "bgk" | "trt"
    omega: float
    trt_magic: float = 0.25


class BatchedGrids:
    """A device batch of periodic grids; state lives on the GPU."""

    def __init__(self, specs: list[GridSpec], storage: str = "f64", math: str = "fma"):
        self._lib = _bind()
        self.specs = list(specs)
        n = len(specs)
        nx = np.array([s.nx for s in specs], dtype=np.int32)
        ny = np.array([s.ny for s in specs], dtype=np.int32)
        kind = np.array([_lib.KINDS[s.kind] for s in specs], dtype=np.int32)
        om = np.array([s.omega for s in specs], dtype=np.float64)
        mg = np.array([s.trt_magic for s in specs], dtype=np.float64)
        h = C.c_void_p()
        check(self._lib.plbm_batch_create(n, ptr(nx), ptr(ny), ptr(kind), ptr(om), ptr(mg),
                                          _lib.STORAGES[storage], C.byref(h)))
        self._h = h
        self.storage = storage
        self.math = "fma"
        if math != "fma":
            self.set_math(math)

    def set_math(self, math: str) -> None:
        """"fma" or, for binary64 storage, "hybrid" (BGK and TRT grids)."""
        check(self._lib.plbm_batch_set_math(self._h, _lib.MATHS[math]))
        self.math = math

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.plbm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- info / schedule --------------------------------------------------------
    def info(self) -> dict:
        a, c, t, k = C.c_int(), C.c_longlong(), C.c_int(), C.c_int()
        check(self._lib.plbm_batch_info(self._h, C.byref(a), C.byref(c), C.byref(t), C.byref(k)))
        return {"ngrids": a.value, "cells": c.value, "ntiles": t.value, "ctas": k.value}

    @property
    def cells(self) -> int:
        return self.info()["cells"]

    @property
    def schedule(self) -> Schedule:
        s = Schedule()
        check(self._lib.plbm_batch_get_schedule(self._h, C.addressof(s)))
        return s

    @schedule.setter
    def schedule(self, s: Schedule) -> None:
        check(self._lib.plbm_batch_set_schedule(self._h, C.addressof(s)))

    def set_stream(self, stream) -> None:
        """torch stream or raw cudaStream_t; None = the batch's own stream."""
        s = _lib.stream_handle(stream)
        check(self._lib.plbm_batch_set_stream(self._h, C.c_void_p(s) if s else None))

    # -- state ------------------------------------------------------------------
    def set_equilibrium(self, i: int, rho, ux, uy) -> None:
        sp = self.specs[i]
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(sp.nx, sp.ny) for a in (rho, ux, uy)]
        check(self._lib.plbm_batch_set_equilibrium(self._h, i, *[ptr(a) for a in arrs]))

    def run(self, nsteps: int) -> None:
        check(self._lib.plbm_batch_run(self._h, int(nsteps)))

    def capture(self, nsteps: int) -> None:
        check(self._lib.plbm_batch_capture(self._h, int(nsteps)))

    def launch_graph(self) -> None:
        check(self._lib.plbm_batch_launch_graph(self._h))

    def inject_stall(self) -> None:
        """Test hook: the next persistent run's barrier wait runs out (PLBM_E_TIMEOUT)."""
        check(self._lib.plbm_batch_inject_stall(self._h))

    def synchronize(self) -> None:
        check(self._lib.plbm_batch_synchronize(self._h))

    @property
    def steps(self) -> int:
        v = C.c_longlong()
        check(self._lib.plbm_batch_steps(self._h, C.byref(v)))
        return v.value

    def macros(self, i: int):
        sp = self.specs[i]
        out = [np.empty((sp.nx, sp.ny)) for _ in range(3)]
        check(self._lib.plbm_batch_macros(self._h, i, *[ptr(a) for a in out]))
        return tuple(out)

    def download(self, i: int) -> np.ndarray:
        sp = self.specs[i]
        ld = sp.ny + (16 - sp.ny % 16) % 16
        f = np.zeros((9, sp.nx, ld))
        check(self._lib.plbm_batch_download(self._h, i, ptr(f)))
        return f


def random_tgv_batch(n: int = 512, seed: int = 2024, lo: int = 32, hi: int = 1024):
    """Specs and initial fields of the uneven-batch Taylor-Green workload."""
    rng = np.random.default_rng(seed)
    specs, fields = [], []
    for _ in range(n):
        nx = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        ny = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        tau = rng.uniform(0.51, 1.5)
        kind = "bgk" if rng.uniform() < 0.5 else "trt"
        kx, ky = int(rng.integers(1, 5)), int(rng.integers(1, 5))
        u0 = rng.uniform(0.005, 0.05)
        specs.append(GridSpec(nx, ny, kind, 1.0 / tau, 0.25))
        fields.append((nx, ny, kx, ky, u0, (tau - 0.5) / 3.0))
    return specs, fields


def tgv_fields(nx: int, ny: int, kx: int, ky: int, u0: float, nu: float):
    p, ux, uy = cases.taylor_green(nx, ny, 2 * math.pi * kx / nx, 2 * math.pi * ky / ny, u0, nu)
    return cases.tgv_density(p), ux, uy


def build_tgv_batch(n: int = 512, seed: int = 2024, storage: str = "f64") -> BatchedGrids:
    specs, fields = random_tgv_batch(n, seed)
    b = BatchedGrids(specs, storage)
    for i, fl in enumerate(fields):
        b.set_equilibrium(i, *tgv_fields(*fl))
    return b
