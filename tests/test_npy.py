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


def _raw_npy(path, header: str, version=(1, 0), data=b""):
    h = header.encode()
    pad = 64 - (len(h) + 11) % 64
    h = h + b" " * pad + b"\n"
    pre = b"\x93NUMPY" + bytes(version)
    pre += len(h).to_bytes(2 if version[0] == 1 else 4, "little")
    path.write_bytes(pre + h + data)


@pytest.mark.parametrize("header", [
    "{'descr': '<f8', 'fortran_order': False, 'shape': (99999999999999999999999, 2), }",
    "{'descr': '<f8', 'fortran_order': False, 'shape': (1, 2, 3, 4, 5, 6, 7, 8, 9), }",
    "{'descr': '<f8', 'fortran_order': False, 'shape': (3, -4), }",
    "{'descr': '<f8', 'fortran_order': Maybe, 'shape': (3,), }",
    "{'descr': '<f8', 'fortran_order': False, 'shape': 3, }",
    "{'descr': '<f8', 'fortran_order': False, }",
    "{'descr': '>f8', 'fortran_order': False, 'shape': (3,), }",
])
def test_rejects_malformed_headers(lattice, tmp_path, header):
    from plbm import PlbmError
    p = tmp_path / "m.npy"
    _raw_npy(p, header)
    with pytest.raises(PlbmError):
        lattice.read_npy_header(p)


def test_truncated_header_and_other_versions(lattice, tmp_path):
    from plbm import PlbmError
    p = tmp_path / "t.npy"
    _raw_npy(p, "{'descr': '<f8', 'fortran_order': True, 'shape': (3, 4), }")
    p.write_bytes(p.read_bytes()[:30])
    with pytest.raises(PlbmError):
        lattice.read_npy_header(p)
    q = tmp_path / "v2.npy"
    _raw_npy(q, "{'descr': '<f8', 'fortran_order': True, 'shape': (3, 4), }", version=(2, 0))
    h = lattice.read_npy_header(q)
    assert h["shape"] == (3, 4) and h["fortran_order"] and h["data_offset"] == q.stat().st_size
    r = tmp_path / "v9.npy"
    _raw_npy(r, "{'descr': '<f8', 'fortran_order': True, 'shape': (3, 4), }", version=(9, 0))
    with pytest.raises(PlbmError):
        lattice.read_npy_header(r)


def test_reads_numpy_version2_and_scalar_headers(lattice, tmp_path):
    p = tmp_path / "v2np.npy"
    a = np.arange(6.0).reshape(2, 3)
    with open(p, "wb") as fh:
        np.lib.format.write_array(fh, a, version=(2, 0))
    h = lattice.read_npy_header(p)
    assert h["shape"] == (2, 3) and not h["fortran_order"] and h["data_offset"] == p.stat().st_size - a.nbytes
    s = tmp_path / "s.npy"
    np.save(s, np.float64(2.5))
    assert lattice.read_npy_header(s)["shape"] == ()
