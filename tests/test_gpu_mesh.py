"""The mesh-cell air source on the device (FindCell in place of the uniform aero velocity pass)
against the oracle: cells and cell values of scattered points, bit for bit (containment is a
sequence of sign tests on the same products, built without fused multiply-adds on both sides);
whole Runge-Kutta steps of a droplet in a 2D quad mesh with a hole and in a 3D tetrahedral mesh;
particles leaving through the outer boundary deleted at the end of the step."""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases
from fjsph_gb300.state import BlockSpec, SPHState
from tests._util import assert_fields

pytestmark = pytest.mark.gpu

RTOL_STEP = 1e-7


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib, oracle_lib):
    return built_lib, oracle_lib


def _pair(c, mesh, st, blocks):
    from fjsph_gb300.api import Context
    from oracle.pyoracle import Oracle
    ctx = Context(c.settings, st.n + 64, blocks)
    orc = Oracle(c.settings, blocks)
    for h in (ctx, orc):
        h.mesh_set(mesh)
        h.set_states(st, st)
    return ctx, orc


def _points(c, pts):
    st = SPHState(len(pts), c.settings.dim)
    st.xi[:] = pts
    st.b[:] = d.FREE
    st.rho[:] = c.settings.rho_rest
    st.m[:] = c.settings.sim_mass
    st.cellID[:] = -3
    return st


@pytest.mark.parametrize("dim", [2, 3])
def test_find_cell_matches_oracle(dim):
    c, mesh = cases.droplet_in_mesh(dim)
    rng = np.random.Generator(np.random.PCG64(20 + dim))
    if dim == 2:
        pts = rng.uniform((-2.1e-3, -2.1e-3), (6.1e-3, 3.1e-3), size=(5000, 2))  # some outside
    else:
        pts = rng.uniform((-1.6e-3, -1.6e-3, -1.6e-3), (2.6e-3, 1.6e-3, 1.6e-3), size=(3000, 3))
    st = _points(c, pts)
    st.lam_nb[:] = np.where(rng.uniform(size=st.n) < 0.9, 0.0, 1.0)  # a tenth above the cutoff
    ctx, orc = _pair(c, mesh, st, [BlockSpec(0, st.n, True, name="fluid")])
    for h in (ctx, orc):
        h.update_neighbours()
        h.get_aero_velocity()
    g, o = ctx.download(), orc.download()
    np.testing.assert_array_equal(g.cellID, o.cellID)
    np.testing.assert_array_equal(g.cellV, o.cellV)
    np.testing.assert_array_equal(g.cellP, o.cellP)
    np.testing.assert_array_equal(g.cellRho, o.cellRho)
    assert (g.cellID >= 0).sum() > 0.7 * st.n
    if dim == 2:
        assert (g.cellID == -4).sum() > 0  # beyond the outer boundary


@pytest.mark.parametrize("dim", [2, 3])
def test_droplet_steps_match_oracle(dim):
    c, mesh = cases.droplet_in_mesh(dim)
    ctx, orc = _pair(c, mesh, c.state, c.blocks)
    for h in (ctx, orc):
        for _ in range(3):
            h.integrate()
    g, o = ctx.download(), orc.download()
    assert g.n == o.n
    np.testing.assert_array_equal(g.cellID, o.cellID)
    assert (g.cellID >= 0).sum() > 0  # the surface particles found their cells
    assert_fields(g, o, ["xi", "v", "rho", "p", "Af"], RTOL_STEP, slice(0, None), label=f"mesh {dim}d")


def test_fill_value_cells_contain_nothing():
    """Cells with a vertex at a fill value (NetCDF's 9.97e36, as in the RAE2822 example's far field)
    are never candidates, on the device as in the oracle."""
    c, mesh = cases.droplet_in_mesh(2)
    m = mesh
    m.verts = m.verts.copy()
    top = m.verts[:, 1] > 2.9e-3
    m.verts[top, 1] = 9.969209968386869e36
    fo, fv, co, cf = m.face_offsets, m.face_verts, m.cell_face_offsets, m.cell_faces
    for cc in range(m.n_cells):  # centres as the reader makes them: vertex averages
        vs = np.unique([fv[q] for f in cf[co[cc]:co[cc + 1]] for q in range(fo[f], fo[f + 1])])
        m.centres[cc] = m.verts[vs].mean(axis=0)
    rng = np.random.Generator(np.random.PCG64(31))
    st = _points(c, rng.uniform((-2e-3, -2e-3), (6e-3, 3e-3), size=(3000, 2)))
    ctx, orc = _pair(c, m, st, [BlockSpec(0, st.n, True, name="fluid")])
    for h in (ctx, orc):
        h.update_neighbours()
        h.get_aero_velocity()
    g, o = ctx.download(), orc.download()
    np.testing.assert_array_equal(g.cellID, o.cellID)
    np.testing.assert_array_equal(g.cellV, o.cellV)
    near_top = st.xi[:, 1] > 3e-3 - 5e-3 / 35 + 1e-9  # the top row of cells, now fill cells
    assert np.all(g.cellID[near_top] < 0) and (g.cellID[~near_top] >= 0).mean() > 0.9


def test_leaving_particles_are_deleted():
    c, mesh = cases.droplet_in_mesh(2)
    st = c.state.copy()
    st.xi[:, 0] += 6e-3 - 0.3e-3  # the drop's downstream third past the outer boundary
    ctx, orc = _pair(c, mesh, st, c.blocks)
    for h in (ctx, orc):
        h.integrate()
    g, o = ctx.download(), orc.download()
    assert g.n == o.n < st.n
    np.testing.assert_array_equal(np.sort(g.part_id), np.sort(o.part_id))


def test_split_precision_runs():
    c, mesh = cases.droplet_in_mesh(3)
    s = c.settings.copy()
    s.precision = d.PREC_MIXED
    from fjsph_gb300.api import Context
    ctx = Context(s, c.state.n + 64, c.blocks)
    ctx.mesh_set(mesh)
    ctx.set_states(c.state, c.state)
    for _ in range(10):
        ctx.integrate()
    st = ctx.download()
    assert np.all(np.isfinite(st.xi)) and (st.cellID >= 0).sum() > 0
