"""The TAU 2D reader (fjsph_gb300.tau: NetCDF classic parser + the reference's edge-mesh MESH) on
the reference's Examples/RAE2822 mesh and solution, and the mesh-cell air source of the oracle on
it: every cell's centre lies in that cell, and points across the far field are lost."""
from pathlib import Path

import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d

from tests._util import reference_examples

_EXAMPLES = reference_examples()
EX = _EXAMPLES / "RAE2822" if _EXAMPLES else Path("RAE2822")
pytestmark = pytest.mark.skipif(_EXAMPLES is None or not EX.exists(), reason="FJSPH_REFERENCE_EXAMPLES is not set")


@pytest.fixture(scope="module", autouse=True)
def _libs(oracle_lib):
    return oracle_lib


@pytest.fixture(scope="module")
def mesh():
    from fjsph_gb300.tau import read_tau_2d
    return read_tau_2d(EX / "mesh.grid.conf.edges", EX / "sol.pval.10000", offset_axis=2)


def test_rae2822_mesh_shape(mesh):
    assert mesh.n_cells == 23552
    assert len(mesh.face_right) == 47504
    assert (mesh.face_right == -1).sum() == 304 and (mesh.face_right == -2).sum() == 496
    nf = np.diff(mesh.cell_face_offsets)
    assert nf.min() >= 3 and nf.max() <= 4  # triangles and quads
    assert np.all(np.isfinite(mesh.vel)) and np.all(mesh.rho > 0) and np.all(mesh.p > 0)
    # far from the aerofoil the flow is the free stream: one speed, small spread
    far = np.linalg.norm(mesh.centres - np.array([0.5, 0.0]), axis=1) > 10.0
    speed = np.linalg.norm(mesh.vel[far], axis=1)
    assert speed.std() < 0.05 * speed.mean()


def test_cell_centres_are_inside_their_cells(mesh):
    from fjsph_gb300.settings import defaults, derive
    from fjsph_gb300.state import BlockSpec, SPHState
    from oracle.pyoracle import Oracle
    s = defaults(2)
    s.asource = d.MESH_INFL
    s.particle_step = 1e-3
    derive(s)
    rng = np.random.Generator(np.random.PCG64(0))
    # 1351 far-field cells have a vertex at the NetCDF fill value (9.97e36) in this file: their
    # centres are not points of the domain and such cells contain nothing
    real = np.nonzero(np.abs(mesh.centres).max(axis=1) < 1e30)[0]
    assert len(real) == mesh.n_cells - 1351
    idx = rng.choice(real, 3000, replace=False)
    pts = np.concatenate([mesh.centres[idx], [[40.0, 0.0], [0.5, 30.0]]])
    st = SPHState(len(pts), 2)
    st.xi[:] = pts
    st.b[:] = d.FREE
    st.rho[:] = 1000.0
    st.m[:] = 1e-3
    st.cellID[:] = -3
    o = Oracle(s, [BlockSpec(0, st.n, True, name="fluid")])
    o.mesh_set(mesh)
    o.set_states(st, st)
    o.get_aero_velocity()
    out = o.download()
    np.testing.assert_array_equal(out.cellID[:-2], idx)
    np.testing.assert_array_equal(out.cellV[:-2], mesh.vel[idx])


def test_rae2822_case_steps_on_the_oracle():
    """Examples/RAE2822 as shipped (para, block files, TAU mesh; the solution file named here
    because the para names none): the liquid jet near the aerofoil takes its air from the mesh
    cells and steps."""
    from fjsph_gb300.geometry import load_case
    from oracle.pyoracle import Oracle
    c = load_case(EX / "para", 2, tau_solution="sol.pval.10000")
    assert c.settings.asource == d.MESH_INFL and c.mesh is not None and c.mesh.n_cells == 23552
    o = Oracle(c.settings, c.blocks, c.inlets)
    o.mesh_set(c.mesh)
    o.set_states(c.state, c.state)
    for _ in range(5):
        o.integrate()
    st = o.download()
    assert np.all(np.isfinite(st.xi))
    fl = st.b == d.FREE
    assert (st.cellID[fl] >= 0).sum() > 0 or fl.sum() == 0
