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


@pytest.mark.parametrize("name,dim,steps", [("tank2d", 2, 10), ("jet3d", 3, 6)])
def test_block_file_case_split_precision(name, dim, steps):
    """The FP32 form along the oracle's trajectory: every step starts from the oracle's state
    (both time levels) and is compared with the oracle's own step -- displacement and density
    change within 1e-4 relative RMS, the same particle set and types after inlet updates."""
    from fjsph_gb300.api import Context
    from fjsph_gb300.geometry import load_case
    from oracle.pyoracle import Oracle
    from tests._util import rel_rms
    c = load_case(CASES / name / "para", dim)
    orc = Oracle(c.settings, c.blocks, c.inlets)
    orc.set_states(c.state, c.state)
    nb = n_bound(c.blocks)
    worst = 0.0
    for k in range(steps):
        pn, pnp1 = orc.download(d.PN), orc.download(d.PNP1)
        sk = orc.settings  # time, time step, CFL state of the oracle's integrator
        sk.precision = d.PREC_MIXED
        ctx = Context(sk, pnp1.n + 4096, _blocks_now(orc, c), _inlets_now(orc, c))
        ctx.set_states(pn, pnp1)
        ctx.integrate()
        orc.integrate()
        g, o = ctx.download(), orc.download()
        assert g.n == o.n, f"step {k}: {g.n} particles, oracle {o.n}"
        np.testing.assert_array_equal(g.b, o.b)
        m = min(pnp1.n, o.n)
        e_x = rel_rms(g.xi[nb:m] - pnp1.xi[nb:m], o.xi[nb:m] - pnp1.xi[nb:m])
        e_rho = rel_rms(g.rho[nb:m] - pnp1.rho[nb:m], o.rho[nb:m] - pnp1.rho[nb:m])
        worst = max(worst, e_x, e_rho)
        assert e_x <= 1e-4 and e_rho <= 1e-4, f"{name} step {k}: displacement {e_x:.2e}, density {e_rho:.2e}"
        ctx.close()
    assert worst > 0.0


def _blocks_now(orc, c):
    """The case's blocks with the ranges update_data has left them in."""
    import dataclasses
    return [dataclasses.replace(b, first=f, second=t) for b, (f, t) in zip(c.blocks, orc.limits())]


def _inlets_now(orc, c):
    """The oracle's current inlet tables (reference indices) in InletSpec form."""
    from fjsph_gb300.state import InletSpec
    out = []
    for inl in c.inlets:
        back, buf = orc.get_inlet(inl.block, len(inl.back), inl.buffer.shape[1])
        out.append(InletSpec(inl.block, back, buf))
    return out
