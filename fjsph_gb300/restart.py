"""Reader of the restart container written by fjsph_restart_write (fjsph_gb300/csrc/restart.cpp):
the reference's restart groups, datasets and attributes (src/H5IO.cpp) by their names."""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

_TYPES = {0: np.float64, 1: np.int64, 2: np.int32, 3: None}


def read_restart(path: str | Path) -> dict:
    """{name: value}: attributes as Python scalars or str, datasets as numpy arrays; names are
    "Simulation current time", "Fluid 0/Position coordinate x", ..."""
    data = Path(path).read_bytes()
    if data[:8] != b"FJSPHRST":
        raise ValueError(f"{path}: not a restart container")
    version, nrec = struct.unpack_from("<II", data, 8)
    if version != 1:
        raise ValueError(f"{path}: container version {version}")
    off, out = 16, {}
    for _ in range(nrec):
        (ln,) = struct.unpack_from("<H", data, off)
        off += 2
        name = data[off: off + ln].decode()
        off += ln
        kind, typ, count = struct.unpack_from("<BBQ", data, off)
        off += 10
        if typ == 3:
            val = data[off: off + count].decode()
            off += count
        else:
            dt = np.dtype(_TYPES[typ]).newbyteorder("<")
            arr = np.frombuffer(data, dtype=dt, count=count, offset=off).copy()
            off += dt.itemsize * count
            val = arr[0].item() if (kind == 0 and count == 1) else arr
        out[name] = val
    return out
