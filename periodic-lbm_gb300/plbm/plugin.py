"""Loader for simulation plugins with the reference's C ABI (sim/lbm.h).

``SimPlugin`` keeps the interface of the reference loader (sim/cases.py:13-122:
``init(grid_size, dt, rho, u, sigma=None, params=None)``, ``step(omega)``,
``vars()``, ``free()``, ``my_norm(u, ua)``, ``dt``) without its matplotlib
import, so the reference's studies can drive ``libplbmgpu.so`` unchanged.
Symbols are ``c_<stem>_{init,step,vars,free,norm}`` with <stem> the file
name without ``lib`` (sim/cases.py:21-32); for this library the stem is
``plbmgpu``.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import _lib


class PluginParams(ctypes.Structure):
    """plbm_plugin_params of include/plbm_plugin.h (version 2)."""

    _fields_ = [("version", ctypes.c_int), ("kind", ctypes.c_int), ("storage", ctypes.c_int),
                ("trt_magic", ctypes.c_double), ("math", ctypes.c_int)]


def make_params(kind="bgk", storage="f64", trt_magic=0.25, math="fma") -> PluginParams:
    k = _lib.KINDS[kind] if isinstance(kind, str) else int(kind)
    s = _lib.STORAGES[storage] if isinstance(storage, str) else int(storage)
    m = _lib.MATHS[math] if isinstance(math, str) else int(math)
    return PluginParams(2, k, s, float(trt_magic), m)


class SimPlugin:
    """ctypes plugin wrapper with the call signatures of sim/cases.py:SimPlugin."""

    def __init__(self, path=None):
        self.ptr = None
        path = str(path or _lib.LIB_PATH)
        name = Path(path).stem.removeprefix("lib")
        self.lib = ctypes.CDLL(path)
        self.c_init = self.lib["c_" + name + "_init"]
        self.c_vars = self.lib["c_" + name + "_vars"]
        self.c_step = self.lib["c_" + name + "_step"]
        self.c_free = self.lib["c_" + name + "_free"]
        self.c_norm = self.lib["c_" + name + "_norm"]
        _type = float
        self.c_norm.restype = ctypes.c_double
        self.c_norm.argtypes = (ctypes.c_int, ctypes.c_int,
                                np.ctypeslib.ndpointer(_type, ndim=2, flags="f_contiguous"),
                                np.ctypeslib.ndpointer(_type, ndim=2, flags="f_contiguous"))
        self.c_init.restype = ctypes.c_void_p
        self.c_init.argtypes = (ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                np.ctypeslib.ndpointer(_type, ndim=2, flags="f_contiguous"),
                                np.ctypeslib.ndpointer(_type, ndim=3, flags="f_contiguous"),
                                ctypes.POINTER(ctypes.c_double), ctypes.c_void_p)
        self.c_step.restype = None
        self.c_step.argtypes = (ctypes.c_void_p, ctypes.c_double)
        self.c_vars.restype = None
        self.c_vars.argtypes = (ctypes.c_void_p,
                                np.ctypeslib.ndpointer(_type, ndim=2, flags="f_contiguous,writeable"),
                                np.ctypeslib.ndpointer(_type, ndim=3, flags="f_contiguous,writeable"))
        self.c_free.restype = None
        self.c_free.argtypes = (ctypes.c_void_p,)
        self._status = getattr(self.lib, "c_" + name + "_status", None)
        if self._status is not None:
            self._status.restype = ctypes.c_int
            self._status.argtypes = (ctypes.c_void_p,)
        self._sync = getattr(self.lib, "c_" + name + "_synchronize", None)
        if self._sync is not None:
            self._sync.restype = ctypes.c_int
            self._sync.argtypes = (ctypes.c_void_p,)
        self._steps = getattr(self.lib, "c_" + name + "_steps", None)
        if self._steps is not None:
            self._steps.restype = ctypes.c_int
            self._steps.argtypes = (ctypes.c_void_p, ctypes.c_double, ctypes.c_int)
        self._params = None

    def my_norm(self, u, ua):
        nx, ny = u.shape
        u = np.require(u, np.float64, ["F_CONTIGUOUS"])
        ua = np.require(ua, np.float64, ["F_CONTIGUOUS"])
        return self.c_norm(nx, ny, u, ua)

    def init(self, grid_size, dt, rho, u, sigma=None, params=None):
        self.grid_size = tuple(grid_size)
        self._dt = dt
        nx, ny = grid_size
        rho = np.require(rho, float, ["F_CONTIGUOUS"])
        u = np.require(u, float, ["F_CONTIGUOUS"])
        if isinstance(params, PluginParams):
            self._params = params
            pp = ctypes.cast(ctypes.byref(params), ctypes.c_void_p)
        else:
            pp = params
        sp = None
        if sigma is not None:
            sigma = np.require(sigma, float, ["F_CONTIGUOUS"])
            sp = sigma.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self.ptr = self.c_init(nx, ny, ctypes.c_double(dt), rho, u, sp, pp)
        if not self.ptr:
            self.ptr = None
            raise _lib.PlbmError(_lib.PLBM_E_INVALID, _lib.last_error())

    @property
    def dt(self):
        return self._dt

    def vars(self):
        rho = np.empty(self.grid_size, dtype=float, order="F")
        u = np.empty(self.grid_size + (2,), dtype=float, order="F")
        if self.ptr is None:
            raise Warning("The plugin has not been initalized. Call .init() first")
        self.c_vars(self.ptr, rho, u)
        self._check()
        return rho, u

    def step(self, omega):
        if self.ptr is not None:
            self.c_step(self.ptr, ctypes.c_double(omega))

    def steps(self, omega, nsteps):
        """nsteps steps in one call (same result as nsteps step() calls)."""
        if self._steps is None:
            for _ in range(nsteps):
                self.step(omega)
        else:
            _lib.check(self._steps(self.ptr, ctypes.c_double(omega), int(nsteps)))

    def synchronize(self):
        """Wait for queued steps (a no-op for plugins without the entry point,
        whose steps are synchronous)."""
        if self._sync is not None and self.ptr is not None:
            _lib.check(self._sync(self.ptr))

    def _check(self):
        if self._status is not None and self.ptr is not None:
            _lib.check(self._status(self.ptr))

    def free(self):
        if self.ptr is not None:
            self.c_free(self.ptr)
            self.ptr = None
