"""The SM-local work order of the split-precision residual (FJSPH_ORDER_SM) against grid order.

The order only decides which SM computes which 32-particle chunk; every particle's arithmetic and
the warps' particle groups (the learned closure's network runs on whole warps) are the same.  The
two orders are separate kernels, each with its own copy of the particle body, and the compiler
may fuse a product and a sum into one multiply-add in one copy and not the other, so they agree
to FP32 rounding: residual fields (acc, Rrho, Af) within 1e-6 of the field's largest magnitude and
the state (positions, velocities, density, pressure) within 1e-9, after two whole steps of the 2D
and 3D (ALE) dam breaks and the droplet and one step of a jet under the learned closure.
"""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import closure as cl
from tests.test_gpu_mixed import _mixed
from tests.test_gpu_parity import _case

pytestmark = pytest.mark.gpu

STATE_FIELDS, STATE_TOL = ("xi", "v", "rho", "p"), 1e-9
RESID_FIELDS, RESID_TOL = ("acc", "Rrho", "Af"), 1e-6


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib):
    return built_lib


def _step(c, st, settings, order, weights=None, steps=1):
    from fjsph_gb300.api import Context
    ctx = Context(settings, st.n + 64, c.blocks, c.inlets)
    ctx.set_sweep_order(order)
    assert ctx.sweep_order() == order
    if weights is not None:
        ctx.closure_set_weights(weights, 1.0)
    ctx.set_states(st, st)
    for _ in range(steps):
        ctx.integrate()
    out = ctx.download()
    ctx.close()
    return out


def _same(a, b, label):
    assert a.n == b.n, label
    for fields, tol in ((STATE_FIELDS, STATE_TOL), (RESID_FIELDS, RESID_TOL)):
        for f in fields:
            x, y = np.asarray(getattr(a, f), np.float64), np.asarray(getattr(b, f), np.float64)
            scale = max(float(np.max(np.abs(y))), 1e-300)
            err = float(np.max(np.abs(x - y))) / scale
            assert err <= tol, f"{label}: {f} differs by {err:.2e} of its largest magnitude"


@pytest.mark.parametrize("name", ["2d", "3d", "drop"])
def test_sm_order_is_bit_identical(name):
    c, st = _case(name)
    s = _mixed(c.settings)
    _same(_step(c, st, s, d.ORDER_GRID, steps=2), _step(c, st, s, d.ORDER_SM, steps=2), name)


def test_sm_order_learned_closure():
    sp = cl.JetSpec(60_000, 14.0, 55.0, 77, D=1e-3)
    c = cl.jet_case(sp)
    s = c.settings.copy()
    s.precision = d.PREC_MIXED
    s.aero_closure = d.CLOSURE_LEARNED
    rng = np.random.default_rng(3)
    X = rng.normal(size=(4000, 12)).astype(np.float32)
    T = rng.normal(size=(4000, 2)).astype(np.float32)
    w = cl.init_params(X, T, seed=3)
    a = _step(c, c.state, s, d.ORDER_GRID, weights=w)
    b = _step(c, c.state, s, d.ORDER_SM, weights=w)
    _same(a, b, "jet, learned closure")
    assert np.any(a.Af != 0.0)


def test_sweep_order_argument():
    from fjsph_gb300.api import Context
    from fjsph_gb300._lib import FJSPHError
    c, st = _case("2d")
    ctx = Context(_mixed(c.settings), st.n + 64, c.blocks, c.inlets)
    with pytest.raises(FJSPHError):
        ctx.set_sweep_order(7)
    assert ctx.sweep_order() == d.ORDER_GRID
    ctx.close()


def test_sm_order_under_graph_replay():
    """Batched droplets stepped by CUDA-graph replay in the SM-local order (the region counters are
    zeroed by a captured memset before each residual) against grid order."""
    from fjsph_gb300 import cases
    from fjsph_gb300.api import Context
    b = cases.droplet_batch(n_drops=5, n_min=400, n_max=2000, seed=9)
    out = []
    for order in (d.ORDER_GRID, d.ORDER_SM):
        s = b.case.settings.copy()
        s.precision = d.PREC_MIXED
        ctx = Context(s, b.case.state.n + 64, b.case.blocks)
        ctx.set_groups(b.first, b.v_inf)
        ctx.set_sweep_order(order)
        ctx.set_states(b.case.state, b.case.state)
        ctx.integrate_groups(4, graph=True)
        out.append((ctx.download(), ctx.group_report()))
        ctx.close()
    (a, ra), (g, rg) = out
    _same(a, g, "droplet batch, graph replay")
    np.testing.assert_array_equal(ra["steps"], rg["steps"])
