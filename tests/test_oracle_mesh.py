"""The oracle's mesh-cell air source (CheckCell / FindCell, src/Containment.cpp:385-821) against
known answers on structured meshes: random points are located in the quad or tetrahedron that
contains them, points in the hole keep no cell, points beyond the outer boundary are marked lost
and deleted at the end of the step."""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases
from fjsph_gb300.state import SPHState

KNOCELL, KLOST = -3, -4


@pytest.fixture(scope="module", autouse=True)
def _libs(oracle_lib):
    return oracle_lib


def _points_state(c, pts):
    st = SPHState(len(pts), c.settings.dim)
    st.xi[:] = pts
    st.b[:] = d.FREE
    st.rho[:] = c.settings.rho_rest
    st.m[:] = c.settings.sim_mass
    st.lam_nb[:] = 0.0  # below the cutoff: every particle asks for its cell
    st.cellID[:] = KNOCELL
    return st


def _locate(c, mesh, pts):
    from oracle.pyoracle import Oracle
    from fjsph_gb300.state import BlockSpec
    st = _points_state(c, pts)
    o = Oracle(c.settings, [BlockSpec(0, st.n, True, name="fluid")])
    o.mesh_set(mesh)
    o.set_states(st, st)
    o.get_aero_velocity()
    return o.download()


def test_quads_contain_their_points():
    c, mesh = cases.droplet_in_mesh(2)
    rng = np.random.Generator(np.random.PCG64(3))
    lo, hi, n = np.array([-2e-3, -2e-3]), np.array([6e-3, 3e-3]), np.array([56, 35])
    pts = rng.uniform(lo + 1e-9, hi - 1e-9, size=(4000, 2))
    h = (hi - lo) / n
    ij = np.floor((pts - lo) / h).astype(int)
    centre = lo + (ij + 0.5) * h
    in_hole = (centre[:, 0] > 3.5e-3) & (centre[:, 0] < 4.6e-3) & (centre[:, 1] > -0.6e-3) & (centre[:, 1] < 0.6e-3)
    out = _locate(c, mesh, pts)
    # the expected cell: the one whose centre is the quad's centre
    want = np.array([np.argmin(np.sum((mesh.centres - q) ** 2, axis=1)) for q in centre])
    np.testing.assert_array_equal(out.cellID[~in_hole], want[~in_hole])
    assert np.all(out.cellID[in_hole] == KNOCELL)
    np.testing.assert_array_equal(out.cellV[~in_hole], mesh.vel[want[~in_hole]])
    np.testing.assert_array_equal(out.cellP[~in_hole], mesh.p[want[~in_hole]])
    np.testing.assert_array_equal(out.cellRho[~in_hole], mesh.rho[want[~in_hole]])


def _in_tet(p, a, b, cc, dd):
    m = np.stack([b - a, cc - a, dd - a], axis=1)
    lam = np.linalg.solve(m, p - a)
    return np.all(lam > 1e-12) and lam.sum() < 1 - 1e-12


def test_tets_contain_their_points():
    c, mesh = cases.droplet_in_mesh(3)
    rng = np.random.Generator(np.random.PCG64(4))
    pts = rng.uniform((-1.5e-3, -1.5e-3, -1.5e-3), (2.5e-3, 1.5e-3, 1.5e-3), size=(600, 3))
    out = _locate(c, mesh, pts)
    fo, fv, co, cf = mesh.face_offsets, mesh.face_verts, mesh.cell_face_offsets, mesh.cell_faces
    for q, cid in zip(pts, out.cellID):
        assert cid >= 0
        vs = sorted({int(v) for f in cf[co[cid]:co[cid + 1]] for v in fv[fo[f]:fo[f + 1]]})
        assert len(vs) == 4
        assert _in_tet(q, *mesh.verts[vs])


def test_outer_boundary_crossing_is_lost_and_deleted():
    c, mesh = cases.droplet_in_mesh(2)
    pts = np.array([[6e-3 + 2e-5, 0.0], [0.0, 3e-3 + 2e-5], [0.0, 0.0]])
    out = _locate(c, mesh, pts)
    assert list(out.cellID[:2]) == [KLOST, KLOST] and out.cellID[2] >= 0
