"""TAU (DLR) mesh and solution files for the mesh-cell air source (2D edge meshes, 3D face meshes).

`read_netcdf` parses the NetCDF classic format (CDF-1 / CDF-2: the header's dimension, attribute
and variable lists, then each fixed-size variable at its offset, big-endian); there is no NetCDF
library on this system.  `read_tau_2d` restates what the reference's readers build from a TAU
edge mesh and its solution (src/CDFIO.cpp:992-1091 Read_tau_mesh_EDGE, :831-990 Place_Edges,
:655-819 Read_SOLUTION, :16-158 the vertex-to-cell averages):

  - faces are the mesh's edges ("points_of_element_edges"), each cell lists the edges whose left
    or right element it is, in edge order; an edge's right element is its right-hand cell or,
    when negative, the boundary kind the reference's FindCell reads (-1 inner, -2 outer);
  - vertices are scaled by the grid scale;
  - the solution holds twice the used vertices (the 2D mesh is one layer of a 3D one); the
    values of the used vertices ("vertices_in_use") are kept, the velocity from the two in-plane
    components the offset axis leaves (1: y, z; 2: x, z; 3: x, y);
  - a cell's centre, velocity, pressure and density are the averages over its distinct vertices.
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

from .mesh import CellMesh

_NC_TYPES = {1: ("b", 1), 2: ("S1", 1), 3: (">i2", 2), 4: (">i4", 4), 5: (">f4", 4), 6: (">f8", 8)}


class _Reader:
    def __init__(self, buf: bytes):
        self.b = buf
        self.o = 0

    def u32(self) -> int:
        v = struct.unpack_from(">I", self.b, self.o)[0]
        self.o += 4
        return v

    def u64(self) -> int:
        v = struct.unpack_from(">Q", self.b, self.o)[0]
        self.o += 8
        return v

    def name(self) -> str:
        n = self.u32()
        s = self.b[self.o:self.o + n].decode("latin-1")
        self.o += (n + 3) & ~3
        return s

    def values(self, t: int, n: int):
        dt, size = _NC_TYPES[t]
        raw = self.b[self.o:self.o + n * size]
        self.o += (n * size + 3) & ~3
        return raw.decode("latin-1") if t == 2 else np.frombuffer(raw, dtype=dt)

    def attrs(self) -> dict:
        tag, n = self.u32(), self.u32()
        out = {}
        if tag == 0 and n == 0:
            return out
        for _ in range(n):
            k = self.name()
            t, m = self.u32(), self.u32()
            out[k] = self.values(t, m)
        return out


def read_netcdf(path) -> dict:
    """{"dims": {name: length}, "vars": {name: array}} of a classic-format NetCDF file (fixed-size
    variables; record variables are not used by the TAU files)."""
    buf = Path(path).read_bytes()
    if buf[:3] != b"CDF" or buf[3] not in (1, 2):
        raise ValueError(f"{path}: not a classic NetCDF file")
    r = _Reader(buf)
    r.o = 4
    offset64 = buf[3] == 2
    r.u32()  # numrecs
    dims = []
    tag, n = r.u32(), r.u32()
    for _ in range(n if tag else 0):
        dims.append((r.name(), r.u32()))
    r.attrs()  # global attributes
    tag, n = r.u32(), r.u32()
    out = {}
    for _ in range(n if tag else 0):
        name = r.name()
        nd = r.u32()
        dimids = [r.u32() for _ in range(nd)]
        r.attrs()
        t = r.u32()
        r.u32()  # vsize
        begin = r.u64() if offset64 else r.u32()
        shape = tuple(dims[k][1] for k in dimids)
        if any(s == 0 for s in shape):
            continue  # a record variable
        dt, size = _NC_TYPES[t]
        count = int(np.prod(shape)) if shape else 1
        arr = np.frombuffer(buf, dtype=dt, count=count, offset=begin)
        out[name] = arr.reshape(shape) if shape else arr[0]
    return {"dims": dict(dims), "vars": out}


def _cell_lists(n_cells: int, left: np.ndarray, right: np.ndarray):
    """each cell's faces in face order: a face belongs to its left element and, when the right
    element is a cell (>= 0), to that one too (Place_Edges / Place_Faces)"""
    owner = np.concatenate([left, right[right >= 0]])
    fid = np.concatenate([np.arange(len(left)), np.nonzero(right >= 0)[0]])
    order = np.lexsort((fid, owner))
    owner, fid = owner[order], fid[order]
    off = np.zeros(n_cells + 1, dtype=np.int64)
    np.add.at(off, owner + 1, 1)
    return np.cumsum(off), fid


def _vertex_averages(n_cells, cell_off, cell_faces, face_off, face_verts, arrays):
    """Average_Point_Data_to_Cell (src/CDFIO.cpp:112-155): Kahan sums over each cell's distinct
    vertices in index order, divided by their count"""
    cv_cell, cv_vert = [], []
    counts = np.diff(cell_off)
    cell_of_face_entry = np.repeat(np.arange(n_cells), counts)
    nv = np.diff(face_off)
    for e in range(int(nv.max())):  # the e-th vertex of every listed face that has one
        has = nv[cell_faces] > e
        cv_cell.append(cell_of_face_entry[has])
        cv_vert.append(face_verts[face_off[cell_faces[has]] + e])
    pairs = np.unique(np.stack([np.concatenate(cv_cell), np.concatenate(cv_vert)], axis=1), axis=0)
    cnt = np.bincount(pairs[:, 0], minlength=n_cells)
    first = np.concatenate([[0], np.cumsum(cnt)])
    rank = np.arange(len(pairs)) - first[pairs[:, 0]]

    def avg(a):
        tot = np.zeros((n_cells,) + a.shape[1:])
        comp = np.zeros_like(tot)
        for k in range(int(cnt.max())):
            sel = rank == k
            c = pairs[sel, 0]
            y = a[pairs[sel, 1]] - comp[c]
            t = tot[c] + y
            comp[c] = (t - tot[c]) - y
            tot[c] = t
        den = cnt.astype(np.float64)
        return tot / (den[:, None] if tot.ndim == 2 else den)

    return [avg(a) for a in arrays]


def read_tau_2d(mesh_path, sol_path, offset_axis: int = 2, scale: float = 1.0) -> CellMesh:
    """The reference's MESH from a TAU 2D edge mesh and its solution (see the module docstring)."""
    m = read_netcdf(mesh_path)
    v = m["vars"]
    n_elem = int(m["dims"]["no_of_elements"])
    edges = np.asarray(v["points_of_element_edges"], dtype=np.int64)
    left = np.asarray(v["left_element_of_edges"], dtype=np.int64)
    right = np.asarray(v["right_element_of_edges"], dtype=np.int64)
    used = np.asarray(v["vertices_in_use"], dtype=np.int64)
    # the in-plane coordinates: the two axes the offset axis leaves (x and z for the usual y)
    names = {1: ("points_yc", "points_zc"), 2: ("points_xc", "points_zc"), 3: ("points_xc", "points_yc")}
    verts = np.stack([np.asarray(v[k], dtype=np.float64) for k in names[offset_axis]], axis=1) * scale
    cell_off, cell_faces = _cell_lists(n_elem, left, right)
    face_off = np.arange(len(edges) + 1, dtype=np.int64) * 2
    face_verts = edges.ravel()
    # solution: the used vertices' values
    s = read_netcdf(sol_path)["vars"]
    comp = {1: ("y_velocity", "z_velocity"), 2: ("x_velocity", "z_velocity"), 3: ("x_velocity", "y_velocity")}
    vx, vy = (np.asarray(s[k], dtype=np.float64) for k in comp[offset_axis])
    p = np.asarray(s["pressure"], dtype=np.float64)
    rho = np.asarray(s["density"], dtype=np.float64)
    if len(vx) != len(verts):
        vx, vy, p, rho = vx[used], vy[used], p[used], rho[used]
    vel = np.stack([vx, vy], axis=1)
    centres, cvel, cp, crho = _vertex_averages(n_elem, cell_off, cell_faces, face_off, face_verts,
                                               [verts, vel, p, rho])
    return CellMesh(2, verts, face_off, face_verts, right.astype(np.int32), cell_off, cell_faces, centres, cvel, cp,
                    crho)


def read_tau_3d(mesh_path, sol_path, scale: float = 1.0) -> CellMesh:
    """The reference's MESH from a TAU 3D face mesh and its solution (src/CDFIO.cpp:1093-1357
    Place_Faces / Read_tau_mesh_FACE, :655-819 Read_SOLUTION): triangle faces, then
    quadrilaterals, each with its left / right element (-1 wall, -2 far field), vertex values
    averaged to the cells.  The solution must hold one value per mesh vertex."""
    m = read_netcdf(mesh_path)
    v, dims = m["vars"], m["dims"]
    n_elem = int(dims["no_of_elements"])
    faces = []
    if "points_of_triangles" in v:
        faces += [list(r) for r in np.asarray(v["points_of_triangles"], dtype=np.int64)]
    if "points_of_quadrilaterals" in v:
        faces += [list(r) for r in np.asarray(v["points_of_quadrilaterals"], dtype=np.int64)]
    nvf = np.array([len(f) for f in faces], dtype=np.int64)
    face_off = np.concatenate([[0], np.cumsum(nvf)]).astype(np.int64)
    face_verts = np.concatenate([np.asarray(f, dtype=np.int64) for f in faces])
    verts = np.stack([np.asarray(v[k], dtype=np.float64) for k in ("points_xc", "points_yc", "points_zc")],
                     axis=1) * scale
    left = np.asarray(v["left_element_of_faces"], dtype=np.int64)
    right = np.asarray(v["right_element_of_faces"], dtype=np.int64)
    cell_off, cell_faces = _cell_lists(n_elem, left, right)
    s = read_netcdf(sol_path)["vars"]
    if len(s["x_velocity"]) != len(verts):
        raise ValueError("the solution does not hold one value per mesh vertex")
    vel = np.stack([np.asarray(s[k], dtype=np.float64) for k in ("x_velocity", "y_velocity", "z_velocity")], axis=1)
    p = np.asarray(s["pressure"], dtype=np.float64)
    rho = np.asarray(s["density"], dtype=np.float64)
    centres, cvel, cp, crho = _vertex_averages(n_elem, cell_off, cell_faces, face_off, face_verts,
                                               [verts, vel, p, rho])
    return CellMesh(3, verts, face_off, face_verts, right.astype(np.int32), cell_off, cell_faces, centres, cvel, cp,
                    crho)
