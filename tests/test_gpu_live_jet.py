"""Config 2's live-inlet jet in crossflow (fjsph_gb300.cases.jet_crossflow_live) on a small pipe:
insertion at the inlet plane, deletion at the domain exit, the 1/7-power-law air field.

The device (FP64 form) and the oracle step the same start: particle counts, block ranges and
inlet tables exactly equal, fields within 1e-7 after the steps; the air velocity of the
aero-active particles within 1e-12.  The FP32 form runs along the oracle's trajectory, each step
from the oracle's state: displacement and density change within 1e-4 relative RMS.
"""
import dataclasses

import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases
from tests._util import assert_fields, n_bound, rel_rms

pytestmark = pytest.mark.gpu

STEPS = 18  # the inlet inserts a layer every ~14 steps at this spacing


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib, oracle_lib):
    return built_lib, oracle_lib


@pytest.fixture(scope="module")
def live():
    return cases.jet_crossflow_live(n_target=30000, D=0.5e-3, cap=30000, headroom=3000, pipe_layers=20)


def _pair(c, settings=None):
    from fjsph_gb300.api import Context
    from oracle.pyoracle import Oracle
    s = settings if settings is not None else c.settings
    ctx = Context(s, c.settings.max_points + 1024, c.blocks, c.inlets)
    orc = Oracle(c.settings, c.blocks, c.inlets)
    for h in (ctx, orc):
        h.air_power_law(*c.power_law_params)
        h.set_states(c.state, c.state)
    return ctx, orc


def test_live_jet_fp64_matches_oracle(live):
    c = live
    ctx, orc = _pair(c)
    n0 = c.state.n
    for k in range(STEPS):
        ctx.integrate()
        orc.integrate()
        assert ctx.particle_count() == orc.download().n, f"step {k}"
    g, o = ctx.download(), orc.download()
    assert g.n > n0, "no insertion happened"
    assert ctx.limits() == orc.limits()
    inl = c.inlets[0]
    gb, gf = ctx.get_inlet(inl.block, len(inl.back), inl.buffer.shape[1])
    ob, of = orc.get_inlet(inl.block, len(inl.back), inl.buffer.shape[1])
    np.testing.assert_array_equal(gb, ob)
    np.testing.assert_array_equal(gf, of)
    np.testing.assert_array_equal(g.b, o.b)
    nb = n_bound(c.blocks)
    assert_fields(g, o, ["xi", "v", "rho", "p"], 1e-7, slice(nb, None), label="live jet")
    active = (o.b == d.FREE) & (o.cellID == 1)
    assert active.sum() > 0
    assert np.max(np.abs(g.cellV[active] - o.cellV[active])) <= 1e-12 * 50.0


def test_live_jet_deletes_at_the_exit():
    """Particles past x = 20.5 D leave at the next update, on both sides alike."""
    c = cases.jet_crossflow_live(n_target=30000, D=0.5e-3, cap=30000, headroom=3000, pipe_layers=20)
    st = c.state.copy()
    nb = n_bound(c.blocks)
    free = np.flatnonzero(st.b == d.FREE)
    far = free[np.argsort(-st.xi[free, 0])[:40]]
    st.xi[far, 0] = 20.5 * 0.5e-3 + 1e-5  # beyond the plane
    c2 = dataclasses.replace(c, state=st)
    ctx, orc = _pair(c2)
    ctx.integrate()
    orc.integrate()
    assert ctx.particle_count() == orc.download().n
    _, deleted = ctx.update_counts()
    assert deleted == orc.deleted() and deleted >= 40
    g, o = ctx.download(), orc.download()
    assert_fields(g, o, ["xi", "v", "rho"], 1e-7, slice(nb, None), label="after deletion")


def test_live_jet_split_precision_along_oracle(live):
    from fjsph_gb300.api import Context
    from oracle.pyoracle import Oracle
    c = live
    orc = Oracle(c.settings, c.blocks, c.inlets)
    orc.air_power_law(*c.power_law_params)
    orc.set_states(c.state, c.state)
    nb = n_bound(c.blocks)
    for k in range(STEPS):
        pn, pnp1 = orc.download(d.PN), orc.download(d.PNP1)
        sk = orc.settings
        sk.precision = d.PREC_MIXED
        blocks = [dataclasses.replace(b, first=f, second=t) for b, (f, t) in zip(c.blocks, orc.limits())]
        inlets = []
        for inl in c.inlets:
            back, buf = orc.get_inlet(inl.block, len(inl.back), inl.buffer.shape[1])
            inlets.append(dataclasses.replace(inl, back=back, buffer=buf))
        ctx = Context(sk, sk.max_points + 1024, blocks, inlets)
        ctx.air_power_law(*c.power_law_params)
        ctx.set_states(pn, pnp1)
        ctx.integrate()
        orc.integrate()
        g, o = ctx.download(), orc.download()
        assert g.n == o.n, f"step {k}"
        m = min(pnp1.n, o.n)
        e_x = rel_rms(g.xi[nb:m] - pnp1.xi[nb:m], o.xi[nb:m] - pnp1.xi[nb:m])
        e_rho = rel_rms(g.rho[nb:m] - pnp1.rho[nb:m], o.rho[nb:m] - pnp1.rho[nb:m])
        assert e_x <= 1e-4 and e_rho <= 1e-4, f"step {k}: displacement {e_x:.2e}, density {e_rho:.2e}"
        ctx.close()
