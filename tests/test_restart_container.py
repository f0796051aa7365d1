"""The restart container reader against a container built by hand (CPU only): magic, version,
attribute and dataset records of every type."""
import struct

import numpy as np
import pytest

from fjsph_gb300.restart import read_restart


def _rec(name, kind, typ, payload, count):
    nb = name.encode()
    return struct.pack("<H", len(nb)) + nb + struct.pack("<BBQ", kind, typ, count) + payload


def test_reader_parses_records(tmp_path):
    x = np.array([1.5, -2.0, 3.25])
    ids = np.array([4, 5, 6], dtype=np.int64)
    b = np.array([0, 5, 5], dtype=np.int32)
    recs = [_rec("Simulation current time", 0, 0, struct.pack("<d", 0.125), 1),
            _rec("Current frame", 0, 1, struct.pack("<q", 3), 1),
            _rec("Variable list", 0, 3, b"", 0),
            _rec("Fluid 0/Position coordinate x", 1, 0, x.tobytes(), 3),
            _rec("Fluid 0/Particle ID", 1, 1, ids.tobytes(), 3),
            _rec("Fluid 0/Boundary condition", 1, 2, b.tobytes(), 3)]
    p = tmp_path / "c.fjrst"
    p.write_bytes(b"FJSPHRST" + struct.pack("<II", 1, len(recs)) + b"".join(recs))
    r = read_restart(p)
    assert r["Simulation current time"] == 0.125 and r["Current frame"] == 3 and r["Variable list"] == ""
    np.testing.assert_array_equal(r["Fluid 0/Position coordinate x"], x)
    np.testing.assert_array_equal(r["Fluid 0/Particle ID"], ids)
    np.testing.assert_array_equal(r["Fluid 0/Boundary condition"], b)


def test_reader_rejects_other_files(tmp_path):
    p = tmp_path / "bad"
    p.write_bytes(b"NOTAFILE" + bytes(8))
    with pytest.raises(ValueError):
        read_restart(p)
