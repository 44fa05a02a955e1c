"""GPU tests of the file side of the path: output_npy snapshots (the
reference's output_npy, src/fvm_bardow.F90:930-961) and binary64 state
save / load for restarts."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def stepped_grid(nx=40, ny=24, storage="f64", steps=7, kind="bgk", nf=2):
    from plbm import LatticeGrid, cases
    rho, ux, uy = cases.tgv_with_noise(nx, u0=0.03, sigma=1e-4, seed=7, nu=0.05)
    rho, ux, uy = (a[:, :ny].copy() for a in (rho, ux, uy))
    g = LatticeGrid(nx, ny, nf=nf, storage=storage, collision=kind)
    g.set_relaxation(1.3, 0.25)
    g.set_pdf_to_equilibrium(rho, ux, uy)
    g.perform_lbm_step(steps)
    return g


@pytest.mark.parametrize("storage", ["f64", "f32dev"])
def test_output_npy_is_mf_of_update_macros(gpu_lib, tmp_path, storage):
    g = stepped_grid(storage=storage)
    p = tmp_path / "snap.npy"
    g.output_npy(p)
    mf = np.load(p)
    assert mf.shape == (g.ny, g.nx, 3) and mf.flags.f_contiguous
    rho, ux, uy = g.update_macros()  # (nx, ny) arrays, y fastest
    for k, a in enumerate((rho, ux, uy)):
        assert np.array_equal(mf[:, :, k], a.T)
    g.close()


def test_output_npy_step_file_name(gpu_lib, tmp_path):
    g = stepped_grid()
    folder = tmp_path / "out" / "run1"
    name = g.output_npy_step(str(folder), "tgv_", 1200)
    assert name.endswith("out/run1/tgv_000001200.npy")
    assert (folder / "tgv_000001200.npy").exists()
    g.output_npy_step(str(folder), "final")
    assert (folder / "final.npy").exists()
    ref = O.update_macros(g.download(g.inew), g.ny)
    mf = np.load(folder / "final.npy")
    for k in range(3):
        assert np.array_equal(mf[:, :, k], ref[k].T)
    g.close()


@pytest.mark.parametrize("storage", ["f64", "f32dev", "f16dev"])
def test_save_load_state_resumes_bit_exactly(gpu_lib, tmp_path, storage):
    a = stepped_grid(storage=storage, steps=5)
    p = tmp_path / "state.npy"
    a.save_state(p)
    idx = a.indices
    a.perform_lbm_step(9)
    want = a.download(a.iold)
    h = np.load(p)
    assert h.shape == (a.ld, a.nx, 9, a.nf)
    from plbm import LatticeGrid
    b = LatticeGrid(a.nx, a.ny, storage=storage, collision="bgk")
    b.set_relaxation(1.3, 0.25)
    b.load_state(p)
    b.indices = idx
    b.perform_lbm_step(9)
    assert np.array_equal(b.download(b.iold), want)
    a.close()
    b.close()


def test_load_state_rejects_wrong_shape(gpu_lib, tmp_path):
    from plbm import LatticeGrid, PlbmError
    a = stepped_grid(nx=16, ny=16, steps=1)
    p = tmp_path / "s.npy"
    a.save_state(p)
    b = LatticeGrid(16, 32)
    with pytest.raises(PlbmError):
        b.load_state(p)
    a.close()
    b.close()


def test_triple_step_state_roundtrip(gpu_lib, tmp_path):
    """save/load follows buffer indices, also after triple steps permuted the lattices."""
    a = stepped_grid(nf=3, steps=2)
    a.perform_triple_step(3)
    p = tmp_path / "t.npy"
    a.save_state(p)
    saved = np.load(p)
    for b in range(3):
        assert np.array_equal(saved[:, :, :, b].T, a.download(b + 1))
    a.close()


def test_output_npy_step_without_folder_writes_to_the_working_directory(gpu_lib, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    g = stepped_grid(nx=16, ny=16, steps=1)
    name = g.output_npy_step(None, "snap", 7)
    assert name == "snap000000007.npy" and (tmp_path / name).exists()
    g.close()
