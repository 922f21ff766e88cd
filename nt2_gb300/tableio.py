"""Table files: the layout that nt2cuda::save / nt2cuda::load (include/nt2cuda/table.hpp) read and
write, for golden-data dumps shared between Python and the C++ front end.

NT2 serializes a table as its extent followed by its elements
(modules/core/container/table/include/nt2/core/container/io/serialization.hpp:48-83, through
Boost.Serialization).  The same two fields, little-endian:
    8 bytes  b"NT2TABLE"
    4 bytes  element size          4 bytes  element kind: ord('f'), ord('i') or ord('u')
    8 bytes  rows                  8 bytes  columns
    rows * columns elements, column-major
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"NT2TABLE"
_HEAD = struct.Struct("<8sIIQQ")


def _kind(dt: np.dtype) -> int:
    if dt.kind == "f":
        return ord("f")
    if dt.kind == "i":
        return ord("i")
    if dt.kind == "u":
        return ord("u")
    raise TypeError(f"tables hold numbers, not {dt}")


def save(path, data, rows: int | None = None, cols: int = 1) -> None:
    """Write `data` (a numpy array or a torch tensor, read in memory order) as a rows x cols table."""
    if hasattr(data, "detach"):
        data = data.detach().cpu().numpy()
    a = np.ascontiguousarray(data).reshape(-1)
    if rows is None:
        rows = a.size // cols if cols else 0
    if rows * cols != a.size:
        raise ValueError(f"{a.size} elements do not make a {rows} x {cols} table")
    dt = a.dtype.newbyteorder("<")
    with open(path, "wb") as f:
        f.write(_HEAD.pack(MAGIC, a.dtype.itemsize, _kind(a.dtype), rows, cols))
        f.write(a.astype(dt, copy=False).tobytes())


def load(path) -> tuple[np.ndarray, tuple[int, int]]:
    """Read a table file: (flat column-major elements, (rows, cols))."""
    with open(path, "rb") as f:
        head = f.read(_HEAD.size)
        if len(head) != _HEAD.size:
            raise ValueError("not a table file: short header")
        magic, size, kind, rows, cols = _HEAD.unpack(head)
        if magic != MAGIC:
            raise ValueError("not a table file")
        code = {ord("f"): "f", ord("i"): "i", ord("u"): "u"}.get(kind)
        if code is None:
            raise ValueError(f"unknown element kind {kind}")
        dt = np.dtype(f"<{code}{size}")
        n = rows * cols
        a = np.frombuffer(f.read(n * size), dtype=dt)
        if a.size != n:
            raise ValueError("table file ends early")
    return a.astype(dt.newbyteorder("="), copy=True), (rows, cols)
