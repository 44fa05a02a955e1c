"""ctypes binding of libplbmgpu.so (the C ABI declared in include/plbm_gpu.h
and include/plbm_plugin.h).

The library is the only compute path: when it is missing or cannot be loaded
every entry point raises, there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_ROOT / "libplbmgpu.so"

# status codes, include/plbm_gpu.h
PLBM_OK = 0
PLBM_E_INVALID = -1
PLBM_E_NOMEM = -2
PLBM_E_CUDA = -3
PLBM_E_UNSUPPORTED = -4
PLBM_E_TIMEOUT = -5
PLBM_E_NODEVICE = -6

# collision kinds
BGK, TRT, RR, BGKI = 0, 1, 2, 3
KINDS = {"bgk": BGK, "trt": TRT, "rr": RR, "bgki": BGKI}
# storage
F64, F32DEV, F16DEV = 0, 1, 2
STORAGES = {"f64": F64, "f32dev": F32DEV, "f16dev": F16DEV}
# math
MATH_FMA, MATH_STRICT, MATH_HYBRID, MATH_DF64 = 0, 1, 2, 3
MATHS = {"fma": MATH_FMA, "strict": MATH_STRICT, "hybrid": MATH_HYBRID, "df64": MATH_DF64}

# streaming schemes (grid%streaming)
SCHEMES = {"lbm": 0, "fvm_bardow": 1, "fdm_bardow": 2, "fdm_bardow_iso": 3, "fdm_bardow_wls": 4,
           "fdm_sofonea": 5, "fdm_bardow_wls_gauss_v1": 6, "fdm_bardow_wls_gauss_v2": 7}

F16_SCALE_LOG2 = 15

_ERRNAMES = {
    PLBM_E_INVALID: "PLBM_E_INVALID",
    PLBM_E_NOMEM: "PLBM_E_NOMEM",
    PLBM_E_CUDA: "PLBM_E_CUDA",
    PLBM_E_UNSUPPORTED: "PLBM_E_UNSUPPORTED",
    PLBM_E_TIMEOUT: "PLBM_E_TIMEOUT",
    PLBM_E_NODEVICE: "PLBM_E_NODEVICE",
}


class PlbmError(RuntimeError):
    """A plbm_* call returned a negative status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


_dp = C.POINTER(C.c_double)
_vp = C.c_void_p
_ip = C.POINTER(C.c_int)

# name -> (restype, argtypes)
SIGNATURES = {
    "plbm_last_error": (C.c_char_p, []),
    "plbm_version": (C.c_int, []),
    "plbm_grid_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(_vp)]),
    "plbm_grid_destroy": (C.c_int, [_vp]),
    "plbm_grid_info": (C.c_int, [_vp, _ip, _ip, _ip, _ip, _ip]),
    "plbm_grid_indices": (C.c_int, [_vp, _ip, _ip]),
    "plbm_grid_set_indices": (C.c_int, [_vp, C.c_int, C.c_int]),
    "plbm_grid_indices3": (C.c_int, [_vp, _ip, _ip, _ip]),
    "plbm_grid_set_indices3": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int]),
    "plbm_perform_triple_step": (C.c_int, [_vp, C.c_int]),
    "plbm_output_npy": (C.c_int, [_vp, C.c_char_p]),
    "plbm_output_npy_step": (C.c_int, [_vp, C.c_char_p, C.c_char_p, C.c_int]),
    "plbm_save_state": (C.c_int, [_vp, C.c_char_p]),
    "plbm_load_state": (C.c_int, [_vp, C.c_char_p]),
    "plbm_write_npy": (C.c_int, [C.c_char_p, _vp, C.c_int, _vp, C.c_int]),
    "plbm_read_npy_header": (C.c_int, [C.c_char_p, _ip, _vp, _ip, C.POINTER(C.c_longlong)]),
    "plbm_grid_set_stream": (C.c_int, [_vp, _vp]),
    "plbm_grid_device_ptr": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "plbm_set_properties": (C.c_int, [_vp, C.c_double, C.c_double, _dp]),
    "plbm_get_properties": (C.c_int, [_vp, _dp, _dp, _dp, _dp, _dp]),
    "plbm_set_relaxation": (C.c_int, [_vp, C.c_double, C.c_double]),
    "plbm_set_collision": (C.c_int, [_vp, C.c_int]),
    "plbm_set_math": (C.c_int, [_vp, C.c_int]),
    "plbm_set_streaming": (C.c_int, [_vp, C.c_int]),
    "plbm_set_time_step": (C.c_int, [_vp, C.c_double]),
    "plbm_upload": (C.c_int, [_vp, _vp, C.c_int]),
    "plbm_download": (C.c_int, [_vp, _vp, C.c_int]),
    "plbm_set_pdf_to_equilibrium": (C.c_int, [_vp, _vp, _vp, _vp]),
    "plbm_stream": (C.c_int, [_vp]),
    "plbm_collide": (C.c_int, [_vp]),
    "plbm_perform_lbm_step": (C.c_int, [_vp, C.c_int]),
    "plbm_update_macros": (C.c_int, [_vp, _vp, _vp, _vp]),
    "plbm_macros_device": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    "plbm_equilibrium_device": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    "plbm_vorticity": (C.c_int, [C.c_int, C.c_int, C.c_int, _vp, _vp, _vp]),
    "plbm_vorticity_device": (C.c_int, [C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp]),
    "plbm_kinetic_energy": (C.c_int, [_vp, C.c_int, _dp]),
    "plbm_velocity_l2_error": (C.c_int, [_vp, C.c_int, _vp, _vp, _dp]),
    "plbm_synchronize": (C.c_int, [_vp]),
    "plbm_hybrid_range_flag": (C.c_int, [_ip, C.c_int]),
    "plbm_velocity_l2_error_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _dp, _vp]),
    "plbm_launch_step": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp,
                                   C.c_double, C.c_double, _vp]),
    # batched grids
    "plbm_batch_default_schedule": (C.c_int, [_vp]),
    "plbm_batch_create": (C.c_int, [C.c_int, _vp, _vp, _vp, _vp, _vp, C.c_int, C.POINTER(_vp)]),
    "plbm_batch_destroy": (C.c_int, [_vp]),
    "plbm_batch_info": (C.c_int, [_vp, _ip, C.POINTER(C.c_longlong), _ip, _ip]),
    "plbm_batch_set_schedule": (C.c_int, [_vp, _vp]),
    "plbm_batch_get_schedule": (C.c_int, [_vp, _vp]),
    "plbm_batch_set_stream": (C.c_int, [_vp, _vp]),
    "plbm_batch_set_math": (C.c_int, [_vp, C.c_int]),
    "plbm_batch_set_equilibrium": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    "plbm_batch_run": (C.c_int, [_vp, C.c_int]),
    "plbm_batch_capture": (C.c_int, [_vp, C.c_int]),
    "plbm_batch_launch_graph": (C.c_int, [_vp]),
    "plbm_batch_synchronize": (C.c_int, [_vp]),
    "plbm_batch_inject_stall": (C.c_int, [_vp]),
    "plbm_batch_steps": (C.c_int, [_vp, C.POINTER(C.c_longlong)]),
    "plbm_batch_macros": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    "plbm_batch_download": (C.c_int, [_vp, C.c_int, _vp]),
    # adjoint
    "plbm_adjoint_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(_vp)]),
    "plbm_adjoint_destroy": (C.c_int, [_vp]),
    "plbm_adjoint_set_stream": (C.c_int, [_vp, _vp]),
    "plbm_adjoint_set_math": (C.c_int, [_vp, C.c_int]),
    "plbm_adjoint_memory": (C.c_int, [_vp, C.POINTER(C.c_size_t)]),
    "plbm_adjoint_forward": (C.c_int, [_vp, _vp, C.c_double, _vp]),
    "plbm_adjoint_backward": (C.c_int, [_vp, _vp, _vp, _dp]),
    # plugin ABI (include/plbm_plugin.h)
    "c_plbmgpu_init": (_vp, [C.c_int, C.c_int, C.c_double, _vp, _vp, _vp, _vp]),
    "c_plbmgpu_step": (None, [_vp, C.c_double]),
    "c_plbmgpu_vars": (None, [_vp, _vp, _vp]),
    "c_plbmgpu_free": (None, [_vp]),
    "c_plbmgpu_norm": (C.c_double, [C.c_int, C.c_int, _vp, _vp]),
    "c_plbmgpu_status": (C.c_int, [_vp]),
    "c_plbmgpu_steps": (C.c_int, [_vp, C.c_double, C.c_int]),
    "c_plbmgpu_synchronize": (C.c_int, [_vp]),
}

# Entry points added after the first release; bound when the library has them.
OPTIONAL_SIGNATURES: dict = {}

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load (once) and bind libplbmgpu.so; raises when it is absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()' "
            "or python periodic-lbm_gb300/build.py).  There is no CPU fallback.")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    for name, (res, args) in OPTIONAL_SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is not None:
            fn.restype = res
            fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def last_error() -> str:
    msg = load().plbm_last_error()
    return msg.decode() if msg else ""


def check(code: int) -> int:
    if code < 0:
        raise PlbmError(code, last_error())
    return code


CUDA_STREAM_LEGACY = 0x1  # cudaStreamLegacy


def stream_handle(stream) -> int | None:
    """cudaStream_t value for a torch stream / raw handle.

    torch reports the legacy default stream as 0, which the plbm_* entry points
    read as "the handle's own stream"; it is passed as cudaStreamLegacy so the
    library's work is ordered with torch's default-stream work.  None keeps the
    handle's own stream.
    """
    if stream is None:
        return None
    s = getattr(stream, "cuda_stream", stream)
    return int(s) if s else CUDA_STREAM_LEGACY


def ptr(a) -> int | None:
    """Address of a numpy array's data or of a torch tensor (None for None)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data
