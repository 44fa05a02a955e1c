"""Import of the reference's own Python module sim/cases.py, for the tests.

The reference checkout is read in place (``PLBM_REFERENCE_DIR``, default
/root/reference); nothing of it is copied.  sim/cases.py imports matplotlib
at module top for its plots (sim/cases.py:2-3); matplotlib is not installed,
so empty stand-in modules are registered under those names first.  The
classes and functions this package restates -- SimPlugin (:13-122), TGVStudy
(:128-213), run (:221-233) -- do not touch them.
"""
from __future__ import annotations

import importlib.util
import os
import sys
import types
from pathlib import Path

DEFAULT_DIR = "/root/reference"


def reference_dir() -> Path:
    return Path(os.environ.get("PLBM_REFERENCE_DIR", DEFAULT_DIR))


def available() -> bool:
    return (reference_dir() / "sim" / "cases.py").is_file()


def load_cases():
    """The reference's sim/cases.py as a module (cached)."""
    name = "reference_sim_cases"
    if name in sys.modules:
        return sys.modules[name]
    for stub in ("matplotlib", "matplotlib.pyplot"):
        if stub not in sys.modules:
            sys.modules[stub] = types.ModuleType(stub)
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    spec = importlib.util.spec_from_file_location(name, reference_dir() / "sim" / "cases.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def study_level(n: int, base: int = 10, re: float = 1.0):
    """Parameters of one refinement level of the reference's study
    (sim/cases.py:252-282) for a lattice Boltzmann plugin, which takes
    dt = 1 exactly.  Returns (grid_size, umax, k, nu, omega, nsteps)."""
    import numpy as np
    cs = np.sqrt(1.0 / 3.0)
    umax = 0.01 / (n / base)
    k = (2 * np.pi / n, 2 * np.pi / n)
    nu = umax * n / re
    tau = nu / cs ** 2
    dt = 1.0
    omega = dt / (tau + 0.5 * dt)
    decay = 1.0 / (nu * (k[0] ** 2 + k[1] ** 2))
    nsteps = round(-np.log(0.1) * decay / dt)
    return (n, n), umax, k, nu, omega, nsteps
