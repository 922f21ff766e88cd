"""Table files (nt2_gb300/tableio.py; the C++ side is nt2cuda::save / nt2cuda::load, exercised on the
GPU by tests/test_demos_gpu.py::test_io_demo).  NT2 serializes a table as its extent and its elements
(modules/core/container/table/include/nt2/core/container/io/serialization.hpp:48-83)."""
import struct

import numpy as np
import pytest

from nt2_gb300 import tableio


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.uint8, np.int32, np.int64])
def test_round_trip(tmp_path, dtype):
    rng = np.random.default_rng(1)
    a = (rng.standard_normal(37 * 11) * 100).astype(dtype)
    p = tmp_path / "t.tbl"
    tableio.save(p, a, 37, 11)
    b, ext = tableio.load(p)
    assert ext == (37, 11) and b.dtype == np.dtype(dtype) and np.array_equal(a, b)


def test_layout(tmp_path):
    p = tmp_path / "t.tbl"
    tableio.save(p, np.array([1.5, -2.0, 3.25], np.float32), 3, 1)
    raw = p.read_bytes()
    assert raw[:8] == b"NT2TABLE"
    assert struct.unpack("<IIQQ", raw[8:32]) == (4, ord("f"), 3, 1)
    assert np.array_equal(np.frombuffer(raw[32:], "<f4"), [1.5, -2.0, 3.25])


def test_empty_and_torch(tmp_path):
    torch = pytest.importorskip("torch")
    p = tmp_path / "e.tbl"
    tableio.save(p, np.zeros(0, np.float64), 0, 5)
    b, ext = tableio.load(p)
    assert ext == (0, 5) and b.size == 0
    tableio.save(p, torch.arange(6, dtype=torch.float32), 2, 3)
    b, ext = tableio.load(p)
    assert ext == (2, 3) and b.tolist() == [0, 1, 2, 3, 4, 5]


def test_errors(tmp_path):
    p = tmp_path / "bad.tbl"
    with pytest.raises(ValueError):
        tableio.save(p, np.zeros(5), 2, 2)
    p.write_bytes(b"NOTTABLE" + bytes(24))
    with pytest.raises(ValueError):
        tableio.load(p)
    tableio.save(p, np.arange(10, dtype=np.float64), 10, 1)
    p.write_bytes(p.read_bytes()[:-8])
    with pytest.raises(ValueError):
        tableio.load(p)
    with pytest.raises(TypeError):
        tableio.save(p, np.array([1 + 2j]), 1, 1)
