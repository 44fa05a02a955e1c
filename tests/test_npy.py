"""The library's .npy writer and header reader (host code, no GPU): files it
writes load in NumPy unchanged, and it parses NumPy's own files."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def lattice():
    import __graft_entry__ as ge
    ge.build()
    from plbm import _lib, lattice
    _lib.load()
    return lattice


@pytest.mark.parametrize("shape", [(7,), (5, 3), (4, 6, 3), (16, 5, 9, 2)])
@pytest.mark.parametrize("fortran", [True, False])
def test_written_npy_loads_in_numpy(lattice, tmp_path, shape, fortran):
    a = np.random.default_rng(1).standard_normal(shape)
    p = tmp_path / "a.npy"
    lattice.write_npy(p, a, fortran_order=fortran)
    b = np.load(p)
    assert b.shape == a.shape and np.array_equal(a, b)
    assert b.flags.f_contiguous == fortran or b.ndim == 1
    raw = p.read_bytes()
    assert raw[:8] == b"\x93NUMPY\x01\x00"
    hlen = raw[8] | (raw[9] << 8)
    assert (10 + hlen) % 64 == 0 and raw[10 + hlen - 1:10 + hlen] == b"\n"


@pytest.mark.parametrize("order", ["F", "C"])
def test_reads_numpy_headers(lattice, tmp_path, order):
    a = np.zeros((3, 4, 5), order=order)
    p = tmp_path / "n.npy"
    np.save(p, a)
    h = lattice.read_npy_header(p)
    assert h["shape"] == (3, 4, 5) and h["fortran_order"] == (order == "F")
    assert h["data_offset"] == p.stat().st_size - a.nbytes


def test_rejects_other_dtypes_and_garbage(lattice, tmp_path):
    from plbm import PlbmError
    p = tmp_path / "i.npy"
    np.save(p, np.zeros(4, dtype=np.int32))
    with pytest.raises(PlbmError):
        lattice.read_npy_header(p)
    q = tmp_path / "g.npy"
    q.write_bytes(b"not an npy file at all")
    with pytest.raises(PlbmError):
        lattice.read_npy_header(q)
    with pytest.raises(PlbmError):
        lattice.read_npy_header(tmp_path / "missing.npy")
