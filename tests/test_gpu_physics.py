"""End-to-end physics against the analytic results the reference ships with its examples
(Examples/Standing_Column/Ideal.dat, Examples/Couette/SteadyState.dat), on the GPU in both forms.

  - standing column: after 0.5 s the depth-binned pressure follows p = rho g (H - y) (the
    reference plots p / (rho g H) against depth / H with the ideal line through (0,0), (1,1));
  - Couette flow: after 50 s (well past the viscous time, the slowest mode is down to 0.7 %) the
    velocity across the gap in the middle of the channel is linear, v_x = U y / h.
"""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases

from tests._util import hydrostatic_error

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib):
    return built_lib


def _run(c, precision, t_end):
    from fjsph_gb300.api import Context
    s = c.settings.copy()
    s.precision = precision
    ctx = Context(s, c.state.n + 64, c.blocks, c.inlets)
    ctx.set_states(c.state, c.state)
    steps = 0
    while ctx.settings.current_time < t_end and steps < 20000:
        ctx.integrate_n(50)
        steps += 50
    return ctx.download(), ctx.settings.current_time, steps


@pytest.mark.parametrize("precision", [d.PREC_FP64, d.PREC_MIXED])
def test_standing_column_hydrostatic(precision):
    c = cases.standing_column_2d()
    st, t, steps = _run(c, precision, 0.5)
    assert t >= 0.5
    nb = c.blocks[0].second
    s = c.settings
    assert hydrostatic_error(st, nb, s.rho_rest, 1.0 + 0.5 * s.particle_step) < 0.03
    assert np.all(np.isfinite(st.xi))
    assert np.abs(st.v[nb:]).max() < 0.05  # at rest up to the acoustic settling


@pytest.mark.parametrize("precision", [d.PREC_FP64, d.PREC_MIXED])
def test_couette_profile(precision):
    U, h = 1e-3, 1.0
    c = cases.couette_2d(wall_speed=U, gap=h)
    st, t, steps = _run(c, precision, 50.0)
    assert t >= 50.0
    nf0 = c.blocks[2].first
    x, y, vx = st.xi[nf0:, 0], st.xi[nf0:, 1], st.v[nf0:, 0]
    mid = (x > 1.2) & (x < 1.8)
    bins = np.linspace(0.05, 0.95, 10)
    idx = np.digitize(y[mid], bins)
    err = []
    for k in range(1, len(bins)):
        sel = idx == k
        if sel.sum() > 5:
            err.append(np.mean(vx[mid][sel]) - U * np.mean(y[mid][sel]) / h)
    err = np.array(err) / U
    assert np.sqrt(np.mean(err ** 2)) < 0.05, err
