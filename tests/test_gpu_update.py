"""Particle insertion and deletion on the device (update_data) against the oracle on the
live-inlet jet: after whole integrate() steps the particle count, the LIMITS ranges, the inlet
tables and every particle's id and type agree exactly, and the states agree to the whole-step
tolerance of each form (FP64: 1e-7 of the field's max; split precision: displacement and density
change within 1e-3 relative RMS)."""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases
from tests._util import rel_err, rel_rms

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib, oracle_lib):
    return built_lib, oracle_lib


def _run(c, prec, steps):
    from fjsph_gb300.api import Context
    from oracle.pyoracle import Oracle
    s = c.settings.copy()
    s.precision = prec
    ctx = Context(s, int(s.max_points) + 64, c.blocks, c.inlets)
    o = Oracle(c.settings, c.blocks, c.inlets)
    for h in (ctx, o):
        h.set_states(c.state, c.state)
    for _ in range(steps):
        ctx.integrate()
        o.integrate()
    return ctx, o


def _check_bookkeeping(c, ctx, o):
    g, r = ctx.download(), o.download()
    assert g.n == r.n
    assert ctx.limits() == o.limits()
    inl = c.inlets[0]
    nd, depth = len(inl.back), inl.buffer.shape[1]
    gb, gf = ctx.get_inlet(inl.block, nd, depth)
    rb, rf = o.get_inlet(inl.block, nd, depth)
    np.testing.assert_array_equal(gb, rb)
    np.testing.assert_array_equal(gf, rf)
    np.testing.assert_array_equal(g.part_id, r.part_id)
    np.testing.assert_array_equal(g.b, r.b)
    assert ctx.update_counts()[1] == o.deleted()
    return g, r


@pytest.mark.parametrize("steps", [1, 3])
def test_update_data_fp64(steps):
    c = cases.jet_inlet()
    ctx, o = _run(c, d.PREC_FP64, steps)
    g, r = _check_bookkeeping(c, ctx, o)
    ins, dele = ctx.update_counts()
    assert ins == len(c.inlets[0].back) and dele > 0
    for f in ("xi", "v", "rho", "p"):
        assert rel_err(getattr(g, f), getattr(r, f)) < 1e-7, f
    ctx.close()


def test_update_data_split_precision():
    c = cases.jet_inlet()
    ctx, o = _run(c, d.PREC_MIXED, 2)
    g, r = _check_bookkeeping(c, ctx, o)
    by_id = {pid: i for i, pid in enumerate(c.state.part_id)}
    old = np.array([by_id.get(pid, -1) for pid in r.part_id])
    m = old >= 0
    nb = c.blocks[0].second
    m[:nb] = False
    assert rel_rms(g.xi[m] - c.state.xi[old[m]], r.xi[m] - c.state.xi[old[m]]) < 1e-3
    assert rel_rms(g.rho[m] - c.state.rho[old[m]], r.rho[m] - c.state.rho[old[m]]) < 1e-3
    ctx.close()


def test_max_points_caps_insertion():
    c0 = cases.jet_inlet()
    c = cases.jet_inlet(max_points=c0.state.n + 10)
    ctx, o = _run(c, d.PREC_FP64, 1)
    _check_bookkeeping(c, ctx, o)
    assert ctx.update_counts()[0] == 10
    ctx.close()
