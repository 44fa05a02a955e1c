"""CPU tests of the C ABI library: it builds, loads, exports every declared
entry point, and rejects bad arguments before touching a device."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as ge
    ge.build()
    from plbm import _lib
    return _lib.load()


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b((?:plbm|c_plbmgpu)_\w+)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_headers_declare_the_abi():
    names = declared_functions()
    for must in ("plbm_grid_create", "plbm_perform_lbm_step", "plbm_update_macros", "plbm_vorticity",
                 "c_plbmgpu_init", "c_plbmgpu_step", "c_plbmgpu_vars", "c_plbmgpu_free", "c_plbmgpu_norm"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "periodic-lbm_gb300" / "libplbmgpu.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(\w+)$", out, flags=re.M))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for n in declared_functions():
        assert getattr(lib, n) is not None


def test_python_binding_covers_every_symbol(lib):
    from plbm import _lib
    bound = set(_lib.SIGNATURES) | set(_lib.OPTIONAL_SIGNATURES)
    assert set(declared_functions()) <= bound


def test_invalid_arguments_are_rejected_without_a_device(lib):
    from plbm import _lib
    h = C.c_void_p()
    assert lib.plbm_grid_create(0, 8, 2, 0, C.byref(h)) == _lib.PLBM_E_INVALID
    assert "nx and ny" in _lib.last_error()
    assert lib.plbm_grid_create(8, 8, 1, 0, C.byref(h)) == _lib.PLBM_E_INVALID
    assert lib.plbm_grid_create(8, 8, 2, 7, C.byref(h)) == _lib.PLBM_E_INVALID
    assert lib.plbm_grid_create(8, 8, 2, 0, None) == _lib.PLBM_E_INVALID
    assert lib.plbm_grid_destroy(None) == _lib.PLBM_OK
    assert lib.plbm_perform_lbm_step(None, 1) == _lib.PLBM_E_INVALID
    assert lib.plbm_vorticity(3, 4, 4, None, None, None) == _lib.PLBM_E_INVALID
    assert lib.plbm_launch_step(0, 0, 0, 8, 8, 4, None, None, 1.0, 0.25, None) == _lib.PLBM_E_INVALID
    assert lib.plbm_adjoint_set_math(None, 0) == _lib.PLBM_E_INVALID
    assert lib.plbm_adjoint_set_stream(None, None) == _lib.PLBM_E_INVALID


def test_extents_above_the_32_bit_cell_limit_are_rejected(lib):
    """PLBM_MAX_EXTENT (2^30) bounds nx, ny and ld at every entry point that
    takes grid sizes, before any device work: the kernels' 32-bit cell
    coordinates, rounded up to whole tiles, must not overflow."""
    from plbm import _lib
    big = (1 << 30) + 1
    h = C.c_void_p()
    for nx, ny in ((big, 8), (8, big)):
        assert lib.plbm_grid_create(nx, ny, 2, 2, C.byref(h)) == _lib.PLBM_E_INVALID
        assert "<= 1073741824" in _lib.last_error()
        assert lib.plbm_vorticity(2, nx, ny, None, None, None) == _lib.PLBM_E_INVALID
        assert "grid size" in _lib.last_error()
        assert lib.plbm_adjoint_create(nx, ny, 0, 10, 3, C.byref(h)) == _lib.PLBM_E_INVALID
        p = np.zeros(1)
        assert not lib.c_plbmgpu_init(nx, ny, 1.0, p.ctypes.data, p.ctypes.data, None, None)
        assert "grid size" in _lib.last_error()
        nxa, nya = (C.c_int * 1)(nx), (C.c_int * 1)(ny)
        kind, om = (C.c_int * 1)(0), (C.c_double * 1)(1.0)
        assert lib.plbm_batch_create(1, nxa, nya, kind, om, None, 0, C.byref(h)) == _lib.PLBM_E_INVALID
    assert lib.plbm_launch_step(0, 0, 0, 8, 8, big, C.c_void_p(16), C.c_void_p(32), 1.0, 0.25,
                                None) == _lib.PLBM_E_INVALID
    assert "bad sizes" in _lib.last_error()
    d, err = np.zeros(4), C.c_double()
    for nx, ny, ld in ((big, 1, 16), (1, 8, big)):
        assert lib.plbm_velocity_l2_error_noalloc(0, nx, ny, ld, C.c_void_p(16), d.ctypes.data, d.ctypes.data,
                                                  C.byref(err), None) == _lib.PLBM_E_INVALID
        assert "bad sizes" in _lib.last_error()
    assert "#define PLBM_MAX_EXTENT (1 << 30)" in (ROOT / "include" / "plbm_gpu.h").read_text()


def test_create_without_device_reports_nodevice_or_succeeds(lib):
    from plbm import _lib
    h = C.c_void_p()
    rc = lib.plbm_grid_create(8, 8, 2, 0, C.byref(h))
    if rc == _lib.PLBM_OK:
        assert lib.plbm_grid_destroy(h) == _lib.PLBM_OK
    else:
        assert rc == _lib.PLBM_E_NODEVICE, _lib.last_error()


def test_plugin_init_rejects_reference_error_cases(lib):
    from plbm import _lib
    nx, ny = 4, 3
    p = np.zeros((nx, ny), order="F")
    u = np.zeros((nx, ny, 2), order="F")
    # dt /= 1 (sim/sim_slbm.F90:48-51)
    assert not lib.c_plbmgpu_init(nx, ny, 0.5, p.ctypes.data, u.ctypes.data, None, None)
    assert "dt = 1.0" in _lib.last_error()
    # sigma present (sim/sim_slbm.F90:64-70)
    s = np.zeros((nx, ny, 3), order="F")
    assert not lib.c_plbmgpu_init(nx, ny, 1.0, p.ctypes.data, u.ctypes.data, s.ctypes.data, None)
    assert "sigma" in _lib.last_error()
    assert lib.c_plbmgpu_status(None) == _lib.PLBM_E_INVALID


def test_plugin_norm_is_host_arithmetic(lib):
    rng = np.random.default_rng(0)
    u = np.asfortranarray(rng.standard_normal((5, 7)))
    ua = np.asfortranarray(rng.standard_normal((5, 7)))
    got = lib.c_plbmgpu_norm(5, 7, u.ctypes.data, ua.ctypes.data)
    ref = np.linalg.norm(u - ua) / np.linalg.norm(ua)
    assert abs(got - ref) < 1e-14 * ref


def test_simplugin_symbol_names_follow_file_stem(lib):
    from plbm.plugin import SimPlugin
    sp = SimPlugin()
    assert sp.c_init.__name__ == "c_plbmgpu_init"
    with pytest.raises(Exception):
        sp.init((4, 3), 0.5, np.zeros((4, 3)), np.zeros((4, 3, 2)))


def test_cases_match_oracle_initial_conditions():
    from oracle import oracle as O
    from plbm import cases
    p, ux, uy = cases.taylor_green(12, 12, 0.5, 0.5, 0.01, 0.1, t=3.0)
    q = O.taylor_green(12, 12, 0.5, 0.5, 0.01, 0.1, t=3.0)
    for a, b in zip((p, ux, uy), q):
        assert np.max(np.abs(a - b)) <= 1e-17 + 1e-15 * np.max(np.abs(b))
    r, u, v = cases.shear_layer(10, 14, 14.0, 0.04, 80.0, 0.05)
    s = O.shear_layer(10, 14, 14.0, 0.04, 80.0, 0.05)
    for a, b in zip((r, u, v), s):
        assert np.max(np.abs(a - b)) <= 1e-15 * max(1.0, np.max(np.abs(b)))


def test_batch_default_schedule_and_workload(lib):
    from plbm import batched
    s = batched.default_schedule()
    assert s.threads == 256 and s.persistent == 1 and list(s.ty) == [32, 64, 128, 256, 256]
    specs, fields = batched.random_tgv_batch(512, seed=2024)
    cells = sum(sp.nx * sp.ny for sp in specs)
    assert 25e6 < cells < 70e6  # expected ~42 M for log-uniform sizes in [32, 1024]
    assert all(32 <= sp.nx <= 1024 and 32 <= sp.ny <= 1024 for sp in specs)
    assert all(0.51 <= 1 / sp.omega <= 1.5 for sp in specs)
    kinds = [sp.kind for sp in specs]
    assert 0.4 < kinds.count("bgk") / len(kinds) < 0.6
    assert all(1 <= f[2] <= 4 and 1 <= f[3] <= 4 and 0.005 <= f[4] <= 0.05 for f in fields)


def test_batch_bucket_edges_match_library():
    from plbm import autotune
    assert [autotune.bucket_of(n) for n in (1, 48, 49, 96, 97, 192, 193, 384, 385, 5000)] == \
        [0, 0, 1, 1, 2, 2, 3, 3, 4, 4]


def test_pad16():
    from plbm import pad16
    assert [pad16(n) for n in (1, 15, 16, 17, 32, 33)] == [16, 16, 16, 32, 32, 48]
