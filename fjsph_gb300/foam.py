"""OpenFOAM (ASCII) polyMesh and solution for the mesh-cell air source.

Restates FOAM::Read_FOAM (src/FOAMIO.cpp:346-955) for ASCII files: constant/polyMesh/boundary
(each patch's face range; a patch whose type line names "wall" is an inner boundary, -1, every
other patch the outer one, -2), points, faces, owner and neighbour, then the solution's p (p_rgh
for a buoyant run) and U at the cells of the given time directory.  As upstream:

  - faces with more than three points are split into the fan (f0, f[j+1], f[j+2]);
  - a cell's centre averages the sorted list of its faces' vertices after std::unique without the
    erase: the unique vertices, then the sorted list's own tail, over the full list length;
  - the reader sets no cell density upstream; here it is read from <time>/rho when that file
    exists and is the given constant otherwise.

Binary polyMesh files are not read (the C ABI takes any mesh as arrays).
"""
from __future__ import annotations

import re
from pathlib import Path

import numpy as np

from .mesh import CellMesh

_NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"


def _body(text: str) -> str:
    """the text after the FoamFile header dictionary"""
    i = text.find("FoamFile")
    if i < 0:
        return text
    depth, j = 0, text.index("{", i)
    for k in range(j, len(text)):
        depth += text[k] == "{"
        depth -= text[k] == "}"
        if depth == 0:
            return text[k + 1:]
    raise ValueError("unterminated FoamFile header")


def _list(text: str):
    """(count, the text inside the outer parentheses) of the first "N ( ... )" list"""
    m = re.search(r"(\d+)\s*\(", text)
    if not m:
        raise ValueError("no list found")
    start, depth = m.end(), 1
    for k in range(start, len(text)):
        depth += text[k] == "("
        depth -= text[k] == ")"
        if depth == 0:
            return int(m.group(1)), text[start:k]
    raise ValueError("unterminated list")


def _scalars(path) -> np.ndarray:
    body = _body(Path(path).read_text())
    i = body.find("internalField")
    if i >= 0:
        body = body[i:]
    n, inner = _list(body)
    vals = np.array([float(x) for x in re.findall(_NUM, inner)])
    if len(vals) != n:
        raise ValueError(f"{path}: {len(vals)} values for a list of {n}")
    return vals


def _vectors(path) -> np.ndarray:
    body = _body(Path(path).read_text())
    i = body.find("internalField")
    if i >= 0:
        body = body[i:]
    n, inner = _list(body)
    rows = re.findall(r"\(([^()]*)\)", inner)
    out = np.array([[float(x) for x in re.findall(_NUM, r)] for r in rows])
    if out.shape != (n, 3):
        raise ValueError(f"{path}: expected {n} vectors")
    return out


def _labels(path) -> np.ndarray:
    n, inner = _list(_body(Path(path).read_text()))
    vals = np.array([int(x) for x in re.findall(r"-?\d+", inner)], dtype=np.int64)
    if len(vals) != n:
        raise ValueError(f"{path}: {len(vals)} labels for a list of {n}")
    return vals


def _faces(path) -> list:
    n, inner = _list(_body(Path(path).read_text()))
    faces = [[int(x) for x in f.split()] for f in re.findall(r"\d+\s*\(([^()]*)\)", inner)]
    if len(faces) != n:
        raise ValueError(f"{path}: expected {n} faces")
    return faces


def _boundary(path) -> list:
    """[(nFaces, startFace, is_wall)] in file order (Read_Patch)"""
    n, inner = _list(_body(Path(path).read_text()))
    out = []
    for m in re.finditer(r"(\w+)\s*\{([^{}]*)\}", inner):
        block = m.group(2)
        wall = 0
        for line in block.splitlines():
            if "type" in line:
                wall = 1 if "wall" in line else 0
        nf = int(re.search(r"nFaces\s+(\d+)", block).group(1))
        sf = int(re.search(r"startFace\s+(\d+)", block).group(1))
        out.append((nf, sf, wall))
    if len(out) != n:
        raise ValueError(f"{path}: expected {n} patches")
    return out


def read_foam(case_dir, time_dir: str, buoyant: bool = False, rho: float = 1.225, scale: float = 1.0) -> CellMesh:
    case_dir = Path(case_dir)
    poly = case_dir / "constant" / "polyMesh"
    patches = _boundary(poly / "boundary")
    pts = _vectors(poly / "points") * scale
    faces_in = _faces(poly / "faces")
    owner = _labels(poly / "owner")
    neigh = _labels(poly / "neighbour")
    right = list(neigh)
    for nf, _, wall in patches:
        right += [-1 if wall else -2] * nf
    right = np.array(right, dtype=np.int64)
    n_cells = int(max(owner.max(), neigh.max() if len(neigh) else 0)) + 1
    # fan triangulation (Post_Process)
    tri, lr = [], []
    for k, f in enumerate(faces_in):
        if len(f) > 3:
            for j in range(len(f) - 2):
                tri.append((f[0], f[j + 1], f[j + 2]))
                lr.append(k)
        else:
            tri.append(tuple(f))
            lr.append(k)
    lr = np.array(lr)
    left_t, right_t = owner[lr], right[lr]
    cfaces = [[] for _ in range(n_cells)]
    for t in range(len(tri)):
        cfaces[left_t[t]].append(t)
        if right_t[t] >= 0:
            cfaces[right_t[t]].append(t)
    centres = np.zeros((n_cells, 3))
    for c in range(n_cells):
        v = sorted(x for t in cfaces[c] for x in tri[t])
        uniq = sorted(set(v))
        seq = uniq + v[len(uniq):]  # std::unique leaves the list's own tail in place
        centres[c] = pts[seq].sum(axis=0) / len(v)
    tdir = case_dir / time_dir
    p = _scalars(tdir / ("p_rgh" if buoyant else "p"))
    vel = _vectors(tdir / "U")
    crho = _scalars(tdir / "rho") if (tdir / "rho").exists() else np.full(n_cells, rho)
    if len(p) != n_cells or len(vel) != n_cells:
        raise ValueError("the solution and the mesh have different cell counts")
    face_off = np.arange(len(tri) + 1, dtype=np.int64) * 3
    cell_off = np.concatenate([[0], np.cumsum([len(f) for f in cfaces])]).astype(np.int64)
    return CellMesh(3, pts, face_off, np.array(tri, dtype=np.int64).ravel(), right_t.astype(np.int32), cell_off,
                    np.concatenate(cfaces).astype(np.int64), centres, vel, p, crho)
