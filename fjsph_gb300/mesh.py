"""Meshes for the mesh-cell air source (the MESH of src/Var.h:396-451) in numpy form.

`CellMesh` holds what the reference's TAU / OpenFOAM readers produce -- vertices, faces as vertex
lists with their right-hand cell (-1 inner boundary, -2 outer boundary), each cell's faces,
centre and solution -- and converts to the C ABI's fjsph_mesh.  `quad_mesh_2d` and `tet_mesh_3d`
build structured test meshes (a rectangle with an optional rectangular hole; a box of cubes each
split into six tetrahedra) with a seeded analytic solution.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _cdefs as d


@dataclass
class CellMesh:
    dim: int
    verts: np.ndarray         # (n_verts, dim)
    face_offsets: np.ndarray  # (n_faces + 1,)
    face_verts: np.ndarray
    face_right: np.ndarray    # (n_faces,) int32
    cell_face_offsets: np.ndarray
    cell_faces: np.ndarray
    centres: np.ndarray       # (n_cells, dim)
    vel: np.ndarray           # (n_cells, dim)
    p: np.ndarray
    rho: np.ndarray

    @property
    def n_cells(self) -> int:
        return len(self.centres)

    def to_c(self) -> d.Mesh:
        """fjsph_mesh over this mesh's arrays (valid while the mesh is alive)."""
        self._keep = [np.ascontiguousarray(a, dtype=t) for a, t in (
            (self.verts, np.float64), (self.face_offsets, np.int64), (self.face_verts, np.int64),
            (self.face_right, np.int32), (self.cell_face_offsets, np.int64), (self.cell_faces, np.int64),
            (self.centres, np.float64), (self.vel, np.float64), (self.p, np.float64), (self.rho, np.float64))]
        v, fo, fv, fr, co, cf, ce, ve, p, r = self._keep
        m = d.Mesh()
        m.dim = self.dim
        m.n_verts, m.n_faces, m.n_cells = len(self.verts), len(self.face_right), len(self.centres)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))
        m.verts, m.face_offsets, m.face_verts = dp(v), ip(fo), ip(fv)
        m.face_right = fr.ctypes.data_as(C.POINTER(C.c_int32))
        m.cell_face_offsets, m.cell_faces = ip(co), ip(cf)
        m.cell_centres, m.cell_vel, m.cell_p, m.cell_rho = dp(ce), dp(ve), dp(p), dp(r)
        return m


def _solution(centres: np.ndarray, u0: float, seed: int):
    """A smooth seeded field: velocity u0 (1 + 0.1 y) along x plus small waves, p and rho around
    the reference state."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = rng.uniform(0.5, 1.5, size=3)
    x = centres
    vel = np.zeros_like(x)
    vel[:, 0] = u0 * (1.0 + 0.1 * x[:, 1]) + 0.05 * u0 * np.sin(a[0] * x[:, 0])
    vel[:, 1] = 0.05 * u0 * np.cos(a[1] * x[:, 0] + a[2] * x[:, 1])
    if x.shape[1] == 3:
        vel[:, 2] = 0.02 * u0 * np.sin(x[:, 2])
    p = 101325.0 * (1.0 + 0.01 * np.sin(x[:, 0]))
    rho = 1.225 * (1.0 + 0.01 * np.cos(x[:, 1]))
    return vel, p, rho


def quad_mesh_2d(lo=(-1.0, -1.0), hi=(3.0, 2.0), n=(40, 30), hole=None, u0=20.0, seed=0) -> CellMesh:
    """Structured quads on [lo, hi] with n cells per axis; `hole` = ((x0, y0), (x1, y1)) removes
    the cells inside that box, whose edges become an inner boundary (-1).  Edges on the outer
    rectangle are the outer boundary (-2)."""
    nx, ny = n
    xs = np.linspace(lo[0], hi[0], nx + 1)
    ys = np.linspace(lo[1], hi[1], ny + 1)
    vid = lambda i, j: j * (nx + 1) + i
    verts = np.array([(x, y) for y in ys for x in xs])
    cid = -np.ones((nx, ny), dtype=np.int64)
    cells = []
    for j in range(ny):
        for i in range(nx):
            cx, cy = 0.5 * (xs[i] + xs[i + 1]), 0.5 * (ys[j] + ys[j + 1])
            if hole and hole[0][0] < cx < hole[1][0] and hole[0][1] < cy < hole[1][1]:
                continue
            cid[i, j] = len(cells)
            cells.append((i, j, cx, cy))
    faces, right, owner = [], [], {}
    cell_faces = [[] for _ in cells]

    def edge(a, b, c_left, c_right, outer):
        key = (min(a, b), max(a, b))
        if key in owner:
            f = owner[key]
            if c_left >= 0:
                cell_faces[c_left].append(f)
            return
        f = len(faces)
        owner[key] = f
        faces.append((a, b))
        right.append(c_right if c_right >= 0 else (-2 if outer else -1))
        if c_left >= 0:
            cell_faces[c_left].append(f)

    for c, (i, j, _, _) in enumerate(cells):
        nb = {"s": (i, j - 1), "e": (i + 1, j), "n": (i, j + 1), "w": (i - 1, j)}
        # clockwise around the cell, so the cell lies to the right of each edge: the boundary
        # crossing test (get_line_intersection) counts a segment entering across an edge only in
        # that orientation
        ends = {"s": (vid(i + 1, j), vid(i, j)), "e": (vid(i + 1, j + 1), vid(i + 1, j)),
                "n": (vid(i, j + 1), vid(i + 1, j + 1)), "w": (vid(i, j), vid(i, j + 1))}
        for side in ("s", "e", "n", "w"):
            ii, jj = nb[side]
            outer = not (0 <= ii < nx and 0 <= jj < ny)
            other = -1 if outer else int(cid[ii, jj])
            edge(*ends[side], c, other, outer)
    centres = np.array([(cx, cy) for (_, _, cx, cy) in cells])
    vel, p, rho = _solution(centres, u0, seed)
    fo = np.arange(len(faces) + 1, dtype=np.int64) * 2
    co = np.concatenate([[0], np.cumsum([len(f) for f in cell_faces])]).astype(np.int64)
    return CellMesh(2, verts, fo, np.array(faces, dtype=np.int64).ravel(), np.array(right, dtype=np.int32), co,
                    np.concatenate(cell_faces).astype(np.int64), centres, vel, p, rho)


def tet_mesh_3d(lo=(-1.0, -1.0, -1.0), hi=(1.0, 1.0, 1.0), n=(8, 8, 8), u0=20.0, seed=0) -> CellMesh:
    """A box of n cubes, each split into six tetrahedra around its main diagonal; triangular
    faces, outer boundary (-2) on the box."""
    nx, ny, nz = n
    xs, ys, zs = (np.linspace(lo[k], hi[k], n[k] + 1) for k in range(3))
    vid = lambda i, j, k: (k * (ny + 1) + j) * (nx + 1) + i
    verts = np.array([(x, y, z) for z in zs for y in ys for x in xs])
    # the six tets of a cube with corners c0 (0,0,0) and c7 (1,1,1) along paths through the edges
    paths = [(1, 3), (1, 5), (2, 3), (2, 6), (4, 5), (4, 6)]  # corner bits: x=1, y=2, z=4
    tets = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                corner = lambda b: vid(i + (b & 1), j + ((b >> 1) & 1), k + ((b >> 2) & 1))
                for a, b in paths:
                    tets.append((corner(0), corner(a), corner(b), corner(7)))
    face_of, faces, right, cell_faces = {}, [], [], []
    for t, tv in enumerate(tets):
        cf = []
        for drop in range(4):
            tri = tuple(v for q, v in enumerate(tv) if q != drop)
            key = tuple(sorted(tri))
            if key in face_of:
                f = face_of[key]
                right[f] = t
            else:
                f = len(faces)
                face_of[key] = f
                faces.append(tri)
                right.append(-2)
            cf.append(f)
        cell_faces.append(cf)
    centres = verts[np.array(tets)].mean(axis=1)
    vel, p, rho = _solution(centres, u0, seed)
    fo = np.arange(len(faces) + 1, dtype=np.int64) * 3
    co = np.arange(len(tets) + 1, dtype=np.int64) * 4
    return CellMesh(3, verts, fo, np.array(faces, dtype=np.int64).ravel(), np.array(right, dtype=np.int32), co,
                    np.array(cell_faces, dtype=np.int64).ravel(), centres, vel, p, rho)
