"""Independent simulations in one context (the batched-droplet workload).

A batch of droplets stepped together must evolve as each droplet stepped alone in its own
context: same per-droplet time step, CFL number and time, and states equal to FP64 rounding
(FP64 form: displacements within 1e-8 relative, the difference being summation order in the
neighbour sums and the atomics of the per-group reductions; split-precision form: 1e-4).
The CUDA-graph replay of the step gives the same results as the ordinary launches.
"""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases
from tests._util import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib):
    return built_lib


def _batch():
    return cases.droplet_batch(n_drops=6, n_min=400, n_max=2500, seed=5)


def _grouped(b, prec, steps, graph, closure=None):
    from fjsph_gb300.api import Context
    s = b.case.settings.copy()
    s.precision = prec
    ctx = Context(s, b.case.state.n + 64, b.case.blocks)
    ctx.set_groups(b.first, b.v_inf)
    ctx.set_states(b.case.state, b.case.state)
    ctx.integrate_groups(steps, graph=graph)
    out = ctx.download(), ctx.group_report()
    ctx.close()
    return out


def _single(b, g, prec, steps):
    from fjsph_gb300.api import Context
    c = b.single(g)
    s = c.settings.copy()
    s.precision = prec
    ctx = Context(s, c.state.n + 64, c.blocks)
    ctx.set_states(c.state, c.state)
    for _ in range(steps):
        ctx.integrate()
    out = ctx.download(), ctx.settings
    ctx.close()
    return out, c


@pytest.mark.parametrize("prec,tol", [(d.PREC_FP64, 1e-8), (d.PREC_MIXED, 1e-4)])
def test_batch_equals_droplets_alone(prec, tol):
    b = _batch()
    steps = 3
    st, rep = _grouped(b, prec, steps, graph=False)
    assert np.all(rep["steps"] == steps)
    for g in range(len(b.counts)):
        (sg, sset), c = _single(b, g, prec, steps)
        sl = slice(b.first[g], b.first[g + 1])
        x0 = c.state.xi
        assert rel_err(st.xi[sl] - x0, sg.xi - x0) < tol, g
        assert rel_err(st.rho[sl] - c.state.rho, sg.rho - c.state.rho) < tol, g
        assert rep["dt"][g] == pytest.approx(sset.delta_t, rel=1e-9)
        assert rep["time"][g] == pytest.approx(sset.current_time, rel=1e-9)
        assert rep["cfl"][g] == pytest.approx(sset.cfl, rel=1e-12)


def test_graph_replay_matches_launches():
    b = _batch()
    a, ra = _grouped(b, d.PREC_MIXED, 5, graph=False)
    g, rg = _grouped(b, d.PREC_MIXED, 5, graph=True)
    assert rel_err(g.xi - b.case.state.xi, a.xi - b.case.state.xi) < 1e-6
    assert rel_err(g.rho - b.case.state.rho, a.rho - b.case.state.rho) < 1e-6
    np.testing.assert_allclose(rg["time"], ra["time"], rtol=1e-12)
    np.testing.assert_array_equal(rg["steps"], ra["steps"])


def test_autotune_choice_and_identical_results():
    """Every candidate launch configuration computes the same per-particle results (the sums of a
    particle run in one thread in list order), so the tuner only changes the time."""
    from fjsph_gb300.api import Context
    b = _batch()
    s = b.case.settings.copy()
    s.precision = d.PREC_MIXED
    ctx = Context(s, b.case.state.n + 64, b.case.blocks)
    ctx.set_groups(b.first, b.v_inf)
    ctx.set_states(b.case.state, b.case.state)
    ctx.update_neighbours()
    res = []
    for cfg in [(128, 128, 4), (64, 64, 2), (96, 32, 8)]:
        ctx.tuning(cfg)
        npd = ctx.dSPH_PreStep()
        ctx.get_aero_velocity()
        ctx.Detect_Surface()
        ctx.dissipation_terms()
        ctx.get_acc_and_Rrho(npd)
        res.append(ctx.download())
    for r in res[1:]:
        np.testing.assert_array_equal(r.Rrho, res[0].Rrho)
        np.testing.assert_array_equal(r.acc, res[0].acc)
        np.testing.assert_array_equal(r.norm, res[0].norm)
    out = ctx.autotune(2)
    ch = out["chosen"]
    assert ch["sweep_threads"] in (64, 128) and ch["resid_threads"] in (64, 128) and ch["list_ahead"] in (2, 4, 8)
    assert len(out["trials_ms"]) == 10 and all(t["ms"] > 0 for t in out["trials_ms"])
    assert ctx.tuning() == (ch["sweep_threads"], ch["resid_threads"], ch["list_ahead"])
    # the residual's work order: the faster of the two timed orders is kept
    grid_ms, sm_ms = (t["ms"] for t in out["trials_ms"][8:])
    assert ch["order"] == ("sm" if sm_ms < grid_ms else "grid")
    assert ctx.sweep_order() == (d.ORDER_SM if ch["order"] == "sm" else d.ORDER_GRID)
    ctx.close()


@pytest.mark.parametrize("graph", [False, True])
def test_one_group_with_walls_equals_context(graph):
    """A context holding one simulation with walls (the 2D dam break) as its only group steps as
    the ordinary context does: FP64 displacements and density changes within 1e-8 relative, the
    same time and CFL number; with and without the CUDA-graph replay."""
    from fjsph_gb300.api import Context
    c = cases.dam_break_2d(dx=0.04)
    steps = 20
    s = c.settings.copy()
    ctx = Context(s, c.state.n + 64, c.blocks)
    ctx.set_states(c.state, c.state)
    for _ in range(steps):
        ctx.integrate()
    ref, rset = ctx.download(), ctx.settings
    ctx.close()
    ctx = Context(s, c.state.n + 64, c.blocks)
    ctx.set_groups([0, c.state.n], [list(s.v_inf)])
    ctx.set_states(c.state, c.state)
    ctx.integrate_groups(steps, graph=graph)
    got, rep = ctx.download(), ctx.group_report()
    ctx.close()
    nb = c.state.n - c.n_fluid
    sl = slice(nb, None)
    assert rep["steps"][0] == steps
    assert rel_err(got.xi[sl] - c.state.xi[sl], ref.xi[sl] - c.state.xi[sl]) < 1e-8
    assert rel_err(got.rho[sl] - c.state.rho[sl], ref.rho[sl] - c.state.rho[sl]) < 1e-8
    np.testing.assert_array_equal(got.xi[:nb], ref.xi[:nb])  # the walls stay put
    assert rep["time"][0] == pytest.approx(rset.current_time, rel=1e-12)
    assert rep["cfl"][0] == pytest.approx(rset.cfl, rel=1e-12)
