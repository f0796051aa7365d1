"""The OpenFOAM (ASCII) reader on a polyMesh written here: a 3 x 2 x 2 box of hexahedra with one
wall patch and one far-field patch, cell-centred p and U.  Quadrilateral faces come back as
triangle fans, boundary faces as -1 (wall) / -2, and the oracle's FindCell locates every cell
centre in its own cell."""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d

HDR = 'FoamFile\n{{\n    version 2.0;\n    format ascii;\n    class {cls};\n    object {obj};\n}}\n\n'


@pytest.fixture(scope="module", autouse=True)
def _libs(oracle_lib):
    return oracle_lib


def _write_case(root, n=(3, 2, 2)):
    nx, ny, nz = n
    vid = lambda i, j, k: (k * (ny + 1) + j) * (nx + 1) + i
    cid = lambda i, j, k: (k * ny + j) * nx + i
    pts = [(i * 0.5, j * 0.4, k * 0.3) for k in range(nz + 1) for j in range(ny + 1) for i in range(nx + 1)]
    internal, bwall, bfar = [], [], []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                c = cid(i, j, k)
                if i + 1 < nx:
                    internal.append(((vid(i + 1, j, k), vid(i + 1, j + 1, k), vid(i + 1, j + 1, k + 1), vid(i + 1, j, k + 1)), c, cid(i + 1, j, k)))
                if j + 1 < ny:
                    internal.append(((vid(i, j + 1, k), vid(i, j + 1, k + 1), vid(i + 1, j + 1, k + 1), vid(i + 1, j + 1, k)), c, cid(i, j + 1, k)))
                if k + 1 < nz:
                    internal.append(((vid(i, j, k + 1), vid(i + 1, j, k + 1), vid(i + 1, j + 1, k + 1), vid(i, j + 1, k + 1)), c, cid(i, j, k + 1)))
                if i == 0:
                    bwall.append(((vid(0, j, k), vid(0, j, k + 1), vid(0, j + 1, k + 1), vid(0, j + 1, k)), c))
                if i == nx - 1:
                    bfar.append(((vid(nx, j, k), vid(nx, j + 1, k), vid(nx, j + 1, k + 1), vid(nx, j, k + 1)), c))
                if j == 0:
                    bfar.append(((vid(i, 0, k), vid(i + 1, 0, k), vid(i + 1, 0, k + 1), vid(i, 0, k + 1)), c))
                if j == ny - 1:
                    bfar.append(((vid(i, ny, k), vid(i, ny, k + 1), vid(i + 1, ny, k + 1), vid(i + 1, ny, k)), c))
                if k == 0:
                    bfar.append(((vid(i, j, 0), vid(i, j + 1, 0), vid(i + 1, j + 1, 0), vid(i + 1, j, 0)), c))
                if k == nz - 1:
                    bfar.append(((vid(i, j, nz), vid(i + 1, j, nz), vid(i + 1, j + 1, nz), vid(i, j + 1, nz)), c))
    faces = [f for f, _, _ in internal] + [f for f, _ in bwall] + [f for f, _ in bfar]
    owner = [o for _, o, _ in internal] + [o for _, o in bwall] + [o for _, o in bfar]
    neigh = [nb for _, _, nb in internal]
    poly = root / "constant" / "polyMesh"
    poly.mkdir(parents=True)
    (poly / "points").write_text(HDR.format(cls="vectorField", obj="points") + f"{len(pts)}\n(\n"
                                 + "\n".join(f"({x} {y} {z})" for x, y, z in pts) + "\n)\n")
    (poly / "faces").write_text(HDR.format(cls="faceList", obj="faces") + f"{len(faces)}\n(\n"
                                + "\n".join("4(" + " ".join(map(str, f)) + ")" for f in faces) + "\n)\n")
    (poly / "owner").write_text(HDR.format(cls="labelList", obj="owner") + f"{len(owner)}\n(\n"
                                + "\n".join(map(str, owner)) + "\n)\n")
    (poly / "neighbour").write_text(HDR.format(cls="labelList", obj="neighbour") + f"{len(neigh)}\n(\n"
                                    + "\n".join(map(str, neigh)) + "\n)\n")
    ni = len(internal)
    (poly / "boundary").write_text(HDR.format(cls="polyBoundaryMesh", obj="boundary") + "2\n(\n"
                                   f"    inlet_wall\n    {{\n        type wall;\n        inGroups 1(wall);\n"
                                   f"        nFaces {len(bwall)};\n        startFace {ni};\n    }}\n"
                                   f"    far\n    {{\n        type patch;\n        nFaces {len(bfar)};\n"
                                   f"        startFace {ni + len(bwall)};\n    }}\n)\n")
    ncell = nx * ny * nz
    rng = np.random.Generator(np.random.PCG64(2))
    p, u = rng.uniform(1e5, 1.01e5, ncell), rng.normal(size=(ncell, 3))
    t = root / "100"
    t.mkdir()
    (t / "p").write_text(HDR.format(cls="volScalarField", obj="p") + "dimensions [1 -1 -2 0 0 0 0];\n\n"
                         f"internalField   nonuniform List<scalar>\n{ncell}\n(\n" + "\n".join(repr(float(x)) for x in p) + "\n)\n;\n")
    (t / "U").write_text(HDR.format(cls="volVectorField", obj="U") + "dimensions [0 1 -1 0 0 0 0];\n\n"
                         f"internalField   nonuniform List<vector>\n{ncell}\n(\n"
                         + "\n".join(f"({float(a)!r} {float(b)!r} {float(c)!r})" for a, b, c in u) + "\n)\n;\n")
    return np.array(pts), faces, owner, neigh, len(bwall), len(bfar), p, u


def test_foam_round_trip(tmp_path):
    from fjsph_gb300.foam import read_foam
    pts, faces, owner, neigh, nwall, nfar, p, u = _write_case(tmp_path)
    m = read_foam(tmp_path, "100", rho=1.2)
    assert len(m.face_right) == 2 * len(faces)  # every quad is a fan of two triangles
    ni = len(neigh)
    right = np.asarray(m.face_right).reshape(-1, 2)[:, 0]
    np.testing.assert_array_equal(right[:ni], neigh)
    assert np.all(right[ni:ni + nwall] == -1) and np.all(right[ni + nwall:] == -2)
    np.testing.assert_array_equal(m.p, p)
    np.testing.assert_array_equal(m.vel, u)
    assert np.all(m.rho == 1.2)
    # centres: the sorted vertex list with std::unique's tail left in place, over its length
    for c in range(m.n_cells):
        fs = m.cell_faces[m.cell_face_offsets[c]:m.cell_face_offsets[c + 1]]
        v = sorted(int(x) for f in fs for x in m.face_verts[3 * f:3 * f + 3])
        uq = sorted(set(v))
        np.testing.assert_allclose(m.centres[c], pts[uq + v[len(uq):]].sum(axis=0) / len(v), rtol=1e-15)
    from fjsph_gb300.settings import defaults, derive
    from fjsph_gb300.state import BlockSpec, SPHState
    from oracle.pyoracle import Oracle
    s = defaults(3)
    s.asource = d.MESH_INFL
    s.particle_step = 1e-2
    derive(s)
    st = SPHState(m.n_cells, 3)
    st.xi[:] = m.centres
    st.b[:] = d.FREE
    st.rho[:] = 1000.0
    st.m[:] = 1e-3
    st.cellID[:] = -3
    o = Oracle(s, [BlockSpec(0, st.n, True, name="fluid")])
    o.mesh_set(m)
    o.set_states(st, st)
    o.get_aero_velocity()
    np.testing.assert_array_equal(o.download().cellID, np.arange(m.n_cells))
