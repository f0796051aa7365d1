"""The TAU readers on files written here: a NetCDF-classic writer (the layout the parser reads)
stores a tetrahedral box as a TAU 3D face mesh with a per-vertex solution; `read_tau_3d` gives
back its faces, each cell's faces and the vertex averages, and the oracle's FindCell locates the
cell centres in their own cells."""
import struct

import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d


def _name(s: str) -> bytes:
    b = s.encode()
    return struct.pack(">I", len(b)) + b + b"\0" * ((4 - len(b) % 4) % 4)


def write_netcdf(path, dims: dict, variables: dict) -> None:
    """variables: name -> (dim names, array); int32 and float64 arrays, fixed size."""
    dnames = list(dims)
    types = {np.dtype(np.int32): (4, ">i4"), np.dtype(np.float64): (6, ">f8")}
    header_wo_offsets = [b"CDF\x01", struct.pack(">I", 0), struct.pack(">II", 10, len(dims))]
    for k in dnames:
        header_wo_offsets.append(_name(k) + struct.pack(">I", dims[k]))
    header_wo_offsets.append(struct.pack(">II", 0, 0))  # no global attributes
    var_heads, blobs = [], []
    for name, (vd, arr) in variables.items():
        t, be = types[arr.dtype]
        data = np.ascontiguousarray(arr).astype(be).tobytes()
        data += b"\0" * ((4 - len(data) % 4) % 4)
        var_heads.append((name, vd, t, len(data)))
        blobs.append(data)
    fixed = b"".join(header_wo_offsets) + struct.pack(">II", 11, len(variables))
    head_len = len(fixed) + sum(len(_name(n)) + 4 + 4 * len(vd) + 8 + 4 + 4 + 4 for n, vd, _, _ in var_heads)
    out, off = [fixed], head_len
    for (name, vd, t, size), blob in zip(var_heads, blobs):
        out.append(_name(name) + struct.pack(">I", len(vd)) + b"".join(struct.pack(">I", dnames.index(x)) for x in vd)
                   + struct.pack(">II", 0, 0) + struct.pack(">III", t, size, off))
        off += size
    path.write_bytes(b"".join(out) + b"".join(blobs))


@pytest.fixture(scope="module", autouse=True)
def _libs(oracle_lib):
    return oracle_lib


def test_tau_3d_round_trip(tmp_path):
    from fjsph_gb300.mesh import tet_mesh_3d
    from fjsph_gb300.tau import read_netcdf, read_tau_3d
    m = tet_mesh_3d(n=(4, 3, 3))
    nf = len(m.face_right)
    tri = m.face_verts.reshape(nf, 3).astype(np.int32)
    # left element: the first cell listing the face; right: the other one or -2
    left = np.full(nf, -1, dtype=np.int32)
    for c in range(m.n_cells):
        for f in m.cell_faces[m.cell_face_offsets[c]:m.cell_face_offsets[c + 1]]:
            if left[f] < 0:
                left[f] = c
    right = m.face_right.astype(np.int32).copy()
    right[right == left] = -2  # defensive: the builder records the second owner as right
    rng = np.random.Generator(np.random.PCG64(9))
    nv = len(m.verts)
    vel = rng.normal(size=(nv, 3))
    p, rho = rng.uniform(9e4, 1.1e5, nv), rng.uniform(1.1, 1.3, nv)
    write_netcdf(tmp_path / "mesh.grid", {"no_of_elements": m.n_cells, "no_of_faces": nf, "no_of_points": nv,
                                          "no_of_triangles": nf, "points_per_triangle": 3,
                                          "no_of_surfaceelements": int((right < 0).sum())},
                 {"points_of_triangles": (["no_of_triangles", "points_per_triangle"], tri),
                  "left_element_of_faces": (["no_of_faces"], left), "right_element_of_faces": (["no_of_faces"], right),
                  "points_xc": (["no_of_points"], m.verts[:, 0]), "points_yc": (["no_of_points"], m.verts[:, 1]),
                  "points_zc": (["no_of_points"], m.verts[:, 2])})
    write_netcdf(tmp_path / "sol.pval", {"no_of_points": nv},
                 {"x_velocity": (["no_of_points"], vel[:, 0]), "y_velocity": (["no_of_points"], vel[:, 1]),
                  "z_velocity": (["no_of_points"], vel[:, 2]), "pressure": (["no_of_points"], p),
                  "density": (["no_of_points"], rho)})
    assert read_netcdf(tmp_path / "mesh.grid")["dims"]["no_of_faces"] == nf
    r = read_tau_3d(tmp_path / "mesh.grid", tmp_path / "sol.pval")
    np.testing.assert_array_equal(r.face_verts, m.face_verts)
    np.testing.assert_array_equal(r.face_right, right)
    for c in range(m.n_cells):
        got = set(r.cell_faces[r.cell_face_offsets[c]:r.cell_face_offsets[c + 1]])
        assert got == set(m.cell_faces[m.cell_face_offsets[c]:m.cell_face_offsets[c + 1]])
        vs = sorted({int(v) for f in got for v in m.face_verts[3 * f:3 * f + 3]})
        np.testing.assert_allclose(r.centres[c], m.verts[vs].mean(axis=0), rtol=1e-14, atol=1e-15)
        np.testing.assert_allclose(r.vel[c], vel[vs].mean(axis=0), rtol=1e-13, atol=1e-14)
        np.testing.assert_allclose(r.p[c], p[vs].mean(), rtol=1e-14)
    # the oracle locates every centre in its own cell
    from fjsph_gb300.settings import defaults, derive
    from fjsph_gb300.state import BlockSpec, SPHState
    from oracle.pyoracle import Oracle
    s = defaults(3)
    s.asource = d.MESH_INFL
    s.particle_step = 1e-2
    derive(s)
    st = SPHState(r.n_cells, 3)
    st.xi[:] = r.centres
    st.b[:] = d.FREE
    st.rho[:] = 1000.0
    st.m[:] = 1e-3
    st.cellID[:] = -3
    o = Oracle(s, [BlockSpec(0, st.n, True, name="fluid")])
    o.mesh_set(r)
    o.set_states(st, st)
    o.get_aero_velocity()
    np.testing.assert_array_equal(o.download().cellID, np.arange(r.n_cells))
