"""Reader of the VTK XML rectilinear-grid files the engine's time-domain dumps write
(``<name>_<numTS>.vtr``: raw appended binary, UInt64 block headers, Float64 coordinates and one
Float32 vector field).  Returns the arrays in the dump's index order."""
from __future__ import annotations

import re

import numpy as np


def read_vtr(path):
    """(field name, coords [x, y, z] in metres, field float32 [3][nx][ny][nz])."""
    raw = open(path, "rb").read()
    cut = raw.index(b"<AppendedData")
    head = raw[:cut].decode()
    start = raw.index(b"_", cut) + 1
    ext = [int(v) for v in re.search(r'WholeExtent="([^"]+)"', head).group(1).split()]
    nx, ny, nz = ext[1] - ext[0] + 1, ext[3] - ext[2] + 1, ext[5] - ext[4] + 1
    arrays = re.findall(r'<DataArray type="(\w+)" Name="([^"]+)"[^>]*offset="(\d+)"', head)

    def block(off, dtype):
        n = int(np.frombuffer(raw, np.uint64, 1, start + off)[0])
        return np.frombuffer(raw, dtype, n // np.dtype(dtype).itemsize, start + off + 8)
    field_name, field, coords = None, None, {}
    for typ, name, off in arrays:
        dt = np.float32 if typ == "Float32" else np.float64
        a = block(int(off), dt)
        if name in ("x", "y", "z"):
            coords[name] = a.copy()
        else:
            field_name = name
            # VTK points run x fastest with 3 components each
            field = a.reshape(nz, ny, nx, 3).transpose(3, 2, 1, 0).copy()
    return field_name, [coords["x"], coords["y"], coords["z"]], field
