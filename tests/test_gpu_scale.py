"""The FP32 split-precision form against the FP64 oracle at the benchmark's spacing and coordinates.

Split precision loses accuracy as the ratio of coordinate to particle separation grows, so these
cases keep production spacing and production coordinates:
  - a cut of the config-2 benchmark workload (the live-inlet jet in crossflow, dx = 50 um,
    1/7-power-law air, ghost-walled pipe, pairwise surface tension, Gissler closure): the ~110k
    fluid particles nearest the pipe exit and the walls they touch;
  - a config-1 block: the 3D dam-break physics with ALE shifting at dx = 3 mm, lattice jittered by
    +-0.01 dx, placed at coordinates up to 1.6 m, with its walls.
On identical input states each pass of the FP32 form is compared with the oracle at the stated
tolerances (relative RMS over the particles the pass writes): residual density rate <= 1e-5 and
acceleration <= 1e-3 (the targets of the split-precision form), aero force <= 1e-3, pre-pass
fields <= 1e-4 (curvature and occlusion 1e-3), surface flags on at most 0.5 % of particles.  One
whole Runge-Kutta step from the same state: displacement and density change within 1e-4.
"""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases
from tests._util import assert_ints, n_bound, rel_rms
from tests.test_gpu_mixed import ACC_TOL, PASS_TOL, RRHO_TOL, _check, _mixed

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib, oracle_lib):
    return built_lib, oracle_lib


@pytest.fixture(scope="module")
def jet_cut():
    c = cases.jet_crossflow_live()
    return cases.cut(c, 110_000, centre=(0.0, 0.0, 0.0))


@pytest.fixture(scope="module")
def dam_block():
    """Config-1 physics (c0 from the 1.2 m column, ALE, jitter) on a 9 x 9 x 18 cm block of fluid
    in a wall corner, moved so that the block reaches x = 1.6 m, y = 0.6 m, z = 1.2 m."""
    c = cases.dam_break_3d(dx=0.003, column=(0.09, 0.09, 0.18), tank=(0.12, 0.12, 0.2), ale=True)
    s = cases.dam_break_3d_settings(dx=0.003, column_height=1.2, ale=True)
    st = c.state.copy()
    st.xi += np.array([1.6 - 0.12, 0.6 - 0.12, 1.2 - 0.2]) + 0.5 * 0.003
    rng = np.random.Generator(np.random.PCG64(5))
    nb = n_bound(c.blocks)
    st.v[nb:] += rng.normal(0.0, 0.2, size=(st.n - nb, 3))
    return cases.Case("dam_block", s, st, c.blocks)


def _ctx(c, st, settings):
    from fjsph_gb300.api import Context
    ctx = Context(settings, st.n + 64, c.blocks, c.inlets)
    if c.power_law_params:
        ctx.air_power_law(*c.power_law_params)
    ctx.set_states(st, st)
    return ctx


def _oracle(c, st):
    from oracle.pyoracle import Oracle
    o = Oracle(c.settings, c.blocks, c.inlets)
    if c.power_law_params:
        o.air_power_law(*c.power_law_params)
    o.set_states(st, st)
    return o


def _boundary(h, c):
    solvers = {b.bound_solver for b in c.blocks if not b.is_fluid}
    if d.GHOST in solvers:
        h.Boundary_Ghost()
    else:
        h.Get_Boundary_Pressure()


@pytest.mark.parametrize("which", ["jet_cut", "dam_block"])
def test_scale_prepasses(which, request):
    c = request.getfixturevalue(which)
    st = c.state
    o = _oracle(c, st)
    ctx = _ctx(c, st, _mixed(c.settings))
    nb = n_bound(c.blocks)
    npds = []
    for h in (ctx, o):
        h.update_neighbours()
        npds.append(h.dSPH_PreStep())
    assert npds[0] == pytest.approx(npds[1], rel=1e-6)
    g, r = ctx.download(), o.download()
    _check(g, r, ["L", "gradRho", "norm", "lam", "lam_nb", "kernsum", "colour"], PASS_TOL, slice(None),
           f"{which} dSPH_PreStep")
    for h in (ctx, o):
        h.get_aero_velocity()
        h.Detect_Surface()
    g, r = ctx.download(), o.download()
    assert_ints(g, r, ["surf", "surfzone"], slice(nb, None), max_frac=0.005, label=f"{which} Detect_Surface")
    _check(g, r, ["curve", "woccl"], 10 * PASS_TOL, slice(nb, None), f"{which} Detect_Surface")
    _check(g, r, ["cellV"], 1e-6, slice(nb, None), f"{which} get_aero_velocity")
    for h in (ctx, o):
        h.dissipation_terms()
        if c.settings.variant & d.VAR_ALE:
            h.particle_shift()
    g, r = ctx.download(), o.download()
    _check(g, r, ["aVisc", "deltaD"], PASS_TOL, slice(nb, None), f"{which} dissipation_terms")
    if c.settings.variant & d.VAR_ALE:
        _check(g, r, ["vPert"], 10 * PASS_TOL, slice(nb, None), f"{which} particle_shift")


@pytest.mark.parametrize("which", ["jet_cut", "dam_block"])
def test_scale_residual(which, request):
    """The residual alone, both sides from the oracle's pre-pass outputs."""
    c = request.getfixturevalue(which)
    o = _oracle(c, c.state)
    o.update_neighbours()
    npd = o.dSPH_PreStep()
    o.get_aero_velocity()
    o.Detect_Surface()
    o.dissipation_terms()
    if c.settings.variant & d.VAR_ALE:
        o.particle_shift()
    _boundary(o, c)
    prepared = o.download()
    o.get_acc_and_Rrho(npd)
    ref = o.download()
    nb = n_bound(c.blocks)
    for mode in (d.PAIRS_LISTS, d.PAIRS_TILES):
        ctx = _ctx(c, prepared, _mixed(c.settings))
        ctx.set_pair_mode(mode)
        ctx.update_neighbours()
        ctx.get_acc_and_Rrho(npd)
        g = ctx.download()
        tag = f"{which} ({'tiles' if mode == d.PAIRS_TILES else 'lists'})"
        _check(g, ref, ["Rrho"], RRHO_TOL, slice(nb, None), f"{tag} residual density rate")
        _check(g, ref, ["acc"], ACC_TOL, slice(nb, None), f"{tag} residual acceleration")
        if c.settings.acase != d.NOAERO:
            _check(g, ref, ["Af"], ACC_TOL, slice(nb, None), f"{tag} aero force")


@pytest.mark.parametrize("which", ["jet_cut", "dam_block"])
def test_scale_whole_step(which, request):
    """One Integrator::integrate step from the same state: FP32 form vs oracle, and the FP64 form
    vs oracle at the FP64 tolerance."""
    c = request.getfixturevalue(which)
    st = c.state
    o = _oracle(c, st)
    o.integrate()
    r = o.download()
    nb = n_bound(c.blocks)
    for prec, tol in ((d.PREC_MIXED, STEP_TOL), (d.PREC_FP64, 1e-7)):
        s = c.settings.copy()
        s.precision = prec
        ctx = _ctx(c, st, s)
        ctx.integrate()
        g = ctx.download()
        assert g.n == r.n
        e_x = rel_rms(g.xi[nb:] - st.xi[nb:], r.xi[nb:] - st.xi[nb:])
        e_rho = rel_rms(g.rho[nb:] - st.rho[nb:], r.rho[nb:] - st.rho[nb:])
        assert e_x <= tol and e_rho <= tol, f"{which} precision {prec}: displacement {e_x:.2e}, density {e_rho:.2e}"
