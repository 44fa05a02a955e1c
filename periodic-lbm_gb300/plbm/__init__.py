"""plbm -- GB300 (sm_103a) D2Q9 periodic stream-collide library, Python side.

The compute path is libplbmgpu.so (CUDA kernels behind a C ABI); this package
binds it with ctypes and mirrors the reference's interfaces:

* :mod:`plbm.lattice` -- the ``lattice_grid`` routines of src/ (alloc_grid,
  set_properties, set_pdf_to_equilibrium, perform_lbm_step, update_macros, ...);
* :mod:`plbm.plugin`  -- the sim/ plugin loader (``SimPlugin``);
* :mod:`plbm.cases`   -- initial conditions of the benchmark cases.
"""
from ._lib import (BGK, BGKI, F16DEV, F32DEV, F64, MATH_HYBRID, MATH_FMA, MATH_STRICT, RR, TRT,
                   PlbmError, load)
from .lattice import LatticeGrid, pad16, vorticity

__all__ = ["LatticeGrid", "pad16", "vorticity", "load", "PlbmError", "BGK", "TRT", "RR", "BGKI",
           "F64", "F32DEV", "F16DEV", "MATH_FMA", "MATH_STRICT", "MATH_HYBRID"]
