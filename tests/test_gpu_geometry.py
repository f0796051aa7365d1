"""Cases built from block files (fjsph_gb300.geometry, the Init_Particles restatement) run on the
device and on the oracle from the same starting state: a 2D tank with all three boundary solvers
and an inlet jet, and a 3D jet leaving a hollow-cylinder pipe into a crossflow (Gissler aero).
The block files and para files are under tests/golden/cases."""
from pathlib import Path

import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from tests._util import assert_fields, n_bound

pytestmark = pytest.mark.gpu

CASES = Path(__file__).resolve().parent / "golden" / "cases"
RTOL_STEP = 1e-7


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib, oracle_lib):
    return built_lib, oracle_lib


@pytest.mark.parametrize("name,dim,steps", [("tank2d", 2, 10), ("jet3d", 3, 4)])
def test_block_file_case_matches_oracle(name, dim, steps):
    from fjsph_gb300.api import Context
    from fjsph_gb300.geometry import load_case
    from oracle.pyoracle import Oracle
    c = load_case(CASES / name / "para", dim)
    cap = c.state.n + 4096
    ctx = Context(c.settings, cap, c.blocks, c.inlets)
    orc = Oracle(c.settings, c.blocks, c.inlets)
    for h in (ctx, orc):
        h.set_states(c.state, c.state)
        for _ in range(steps):
            h.integrate()
    g, o = ctx.download(), orc.download()
    assert g.n == o.n
    assert ctx.settings.current_time == pytest.approx(orc.settings.current_time, rel=1e-9)
    nb = n_bound(c.blocks)
    assert_fields(g, o, ["xi", "v", "rho", "p"], RTOL_STEP, slice(nb, None), label=name)
    np.testing.assert_array_equal(g.b, o.b)


@pytest.mark.parametrize("name,dim", [("tank2d", 2), ("jet3d", 3)])
def test_block_file_case_split_precision(name, dim):
    from fjsph_gb300.api import Context
    from fjsph_gb300.geometry import load_case
    c = load_case(CASES / name / "para", dim)
    s = c.settings.copy()
    s.precision = d.PREC_MIXED
    ctx = Context(s, c.state.n + 4096, c.blocks, c.inlets)
    ctx.set_states(c.state, c.state)
    for _ in range(20):
        ctx.integrate()
    st = ctx.download()
    assert np.all(np.isfinite(st.xi)) and np.all(np.isfinite(st.v))
    assert ctx.settings.current_time > 0
