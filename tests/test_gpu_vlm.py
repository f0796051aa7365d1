"""The vortex-lattice air source on the GPU against the FP64 oracle (restating src/VLM.cpp).

  - panels and circulations of the Examples/VLM wing (swept, tapered, flapped, 1400 panels):
    the panel corners bit for bit, circulations to 1e-9 of the largest (LU with partial against
    Gauss-Jordan pivoting);
  - VLM::getVelocity at scattered points: FP64 form to 1e-10 of the freestream speed; the
    split-precision form (FP32 sums) to 1e-4 at worst (points within millimetres of a trailing
    vortex, where single terms are large) and 1e-5 RMS;
  - inside the pre-step (get_aero_velocity, Detect_Surface with the Gissler occlusion): cellV and
    woccl of a droplet above a small wing, FP64 to 1e-9, split precision to 1e-4.
"""
import math

import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases
from tests._util import perturb

pytestmark = pytest.mark.gpu

EXAMPLE_WING = dict(span=22.275, chord=8.491, panels_span=50, panels_chord=14, aoa_deg=5.0, sweep_deg=32.5,
                    taper=0.6, flap_start=3, flap_width=24, flap_depth=6, flap_deg=20.0)
EXAMPLE_VINF = [89.69, 0.0, 7.8466]


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib, oracle_lib):
    return built_lib, oracle_lib


def _wing(**kw):
    from fjsph_gb300._lib import lib
    v = d.Vlm()
    lib().fjsph_vlm_defaults(v)
    for k, val in kw.items():
        setattr(v, k, val)
    return v


def _pair(c, st, s):
    from fjsph_gb300.api import Context
    from oracle.pyoracle import Oracle
    ctx = Context(s, st.n + 64, c.blocks, c.inlets)
    orc = Oracle(s, c.blocks, c.inlets)
    for h in (ctx, orc):
        h.set_states(st, st)
    return ctx, orc


def _settings(c, v_inf, precision, acase=None):
    s = c.settings.copy()
    for k in range(3):
        s.v_inf[k] = v_inf[k]
    s.asource = d.VLM_INFL
    s.precision = precision
    if acase is not None:
        s.acase = acase
    return s


def test_vlm_panels_and_circulations():
    c = cases.droplet_3d(diam=6e-4, dx=1e-4)
    ctx, orc = _pair(c, c.state, _settings(c, EXAMPLE_VINF, d.PREC_FP64))
    v = _wing(**EXAMPLE_WING)
    assert ctx.vlm_setup(v) == orc.vlm_setup(v) == 1400
    g, abc = ctx.vlm_panels()
    go, abco = orc.vlm_panels()
    assert np.max(np.abs(abc - abco)) <= 1e-12 * np.max(np.abs(abco))
    assert np.max(np.abs(g - go)) <= 1e-9 * np.max(np.abs(go))


@pytest.mark.parametrize("precision,tol,rms_tol", [(d.PREC_FP64, 1e-10, 1e-11), (d.PREC_MIXED, 1e-4, 1e-5)])
def test_vlm_velocity_at_points(precision, tol, rms_tol):
    c = cases.droplet_3d(diam=6e-4, dx=1e-4)
    ctx, orc = _pair(c, c.state, _settings(c, EXAMPLE_VINF, precision))
    v = _wing(**EXAMPLE_WING)
    ctx.vlm_setup(v)
    orc.vlm_setup(v)
    rng = np.random.Generator(np.random.PCG64(11))
    pts = np.column_stack([rng.uniform(-10, 40, 4000), rng.uniform(-30, 30, 4000), rng.uniform(-6, 6, 4000)])
    u, uo = ctx.vlm_velocity(pts), orc.vlm_velocity(pts)
    vinf = np.linalg.norm(EXAMPLE_VINF)
    e = np.linalg.norm(u - uo, axis=1) / vinf
    assert np.max(e) <= tol and np.sqrt(np.mean(e * e)) <= rms_tol, (np.max(e), np.sqrt(np.mean(e * e)))
    # the limit: no velocity above max_vel_fac x |v_inf|
    assert np.max(np.linalg.norm(u, axis=1)) <= 2.0 * vinf * (1 + 1e-12)


@pytest.mark.parametrize("precision,tol", [(d.PREC_FP64, 1e-9), (d.PREC_MIXED, 1e-4)])
def test_vlm_air_in_prestep(precision, tol):
    """A droplet 1.2 mm above a 4 mm x 2 mm wing: cellV of its aero-active particles and the
    Gissler occlusion, which uses the lattice velocity of every free particle."""
    c = cases.droplet_3d(diam=1.2e-3, dx=1e-4)
    st = perturb(c.state, 5, 0.5, 0.05e-4, 0)
    st.xi[:, 0] += 1.0e-3
    st.xi[:, 2] += 1.2e-3
    V, a = 30.0, math.radians(6.0)
    s = _settings(c, [V * math.cos(a), 0.0, V * math.sin(a)], precision, d.GISSLER)
    ctx, orc = _pair(c, st, s)
    v = _wing(span=2e-3, chord=2e-3, panels_span=8, panels_chord=4, taper=1.0)
    ctx.vlm_setup(v)
    orc.vlm_setup(v)
    for h in (ctx, orc):
        h.update_neighbours()
        h.dSPH_PreStep()
        h.get_aero_velocity()
        h.Detect_Surface()
    g, o = ctx.download(), orc.download()
    on = o.cellID == 1
    assert on.sum() > 50 and np.array_equal(g.cellID == 1, on)
    dv = np.linalg.norm(g.cellV[on] - o.cellV[on], axis=1) / V
    assert np.max(dv) <= tol, np.max(dv)
    # the lattice changes the air velocity noticeably over the droplet
    assert np.max(np.linalg.norm(o.cellV[on] - np.array(s.v_inf[:3]), axis=1)) > 0.02 * V
    werr = np.max(np.abs(g.woccl - o.woccl))
    assert werr <= (1e-9 if precision == d.PREC_FP64 else 2e-3), werr
