"""FP32 split-precision form against the FP64 oracle on identical input states.

Tolerances (stated as relative RMS over the particles the pass writes, field by field):
  - residual density rate (Rrho): <= 1e-5; residual acceleration: <= 1e-3 — the targets the
    split-precision form is built to;
  - pre-pass fields (L, gradRho, lam, normals, curvature, aVisc, deltaD, vPert): <= 1e-4;
  - one whole step (Runge-Kutta 4, Newmark-Beta): displacement and density change <= 1e-4;
  - integer flags (surf, surfzone): at most 0.5 % of particles may differ (an FP32 value within
    ~1e-6 of a threshold can fall on the other side);
  - neighbour lists: still bit-exact as sets (membership stays an FP64 decision).
"""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases
from tests._util import assert_ints, n_bound, perturb, rel_rms
from fjsph_gb300.settings import derive
from tests.test_gpu_parity import VARIANTS, _case

pytestmark = pytest.mark.gpu

RRHO_TOL = 1e-5
ACC_TOL = 1e-3
PASS_TOL = 1e-4


def _mixed(settings):
    s = settings.copy()
    s.precision = d.PREC_MIXED
    return s


def _ctx(c, st, s):
    from fjsph_gb300.api import Context
    ctx = Context(s, st.n + 64, c.blocks, c.inlets)
    ctx.set_states(st, st)
    return ctx


def _oracle(c, st):
    from oracle.pyoracle import Oracle
    o = Oracle(c.settings, c.blocks, c.inlets)
    o.set_states(st, st)
    return o


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib, oracle_lib):
    return built_lib, oracle_lib


def _check(g, o, fields, tol, sl, label):
    bad = []
    for f in fields:
        a, b = getattr(g, f)[sl], getattr(o, f)[sl]
        if not np.all(np.isfinite(a)):
            bad.append(f"{f} non-finite")
            continue
        e = rel_rms(a, b)
        if e > tol:
            bad.append(f"{f} rel-RMS {e:.2e}")
    assert not bad, f"{label} (tol {tol:g}): " + "; ".join(bad)


@pytest.mark.parametrize("name", ["2d", "3d", "drop"])
def test_mixed_neighbour_sets_exact(name):
    c, st = _case(name)
    ctx = _ctx(c, st, _mixed(c.settings))
    o = _oracle(c, st)
    assert ctx.update_neighbours() == o.update_neighbours()
    a, b = ctx.neighbours(), o.neighbours()
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("name", ["2d", "3d", "drop"])
def test_mixed_residual_on_oracle_state(name):
    """The residual alone: both sides start from the oracle's pre-pass outputs."""
    c, st = _case(name)
    o = _oracle(c, st)
    o.update_neighbours()
    npd = o.dSPH_PreStep()
    o.get_aero_velocity()
    o.Detect_Surface()
    o.dissipation_terms()
    if c.settings.variant & d.VAR_ALE:
        o.particle_shift()
    o.Get_Boundary_Pressure()
    prepared = o.download()
    o.get_acc_and_Rrho(npd)
    ref = o.download()
    ctx = _ctx(c, prepared, _mixed(c.settings))
    ctx.update_neighbours()
    ctx.get_acc_and_Rrho(npd)
    g = ctx.download()
    nb = n_bound(c.blocks)
    _check(g, ref, ["Rrho"], RRHO_TOL, slice(nb, None), f"{name} residual density rate")
    _check(g, ref, ["acc"], ACC_TOL, slice(nb, None), f"{name} residual acceleration")


@pytest.mark.parametrize("solver", [d.PRESSURE_G, d.GHOST, d.DBC])
def test_mixed_boundary_solvers(solver):
    """The boundary passes of the split-precision form from the oracle's pre-pass outputs (2D dam
    break, perturbed, no-slip walls): the no-slip mirror velocities (FP64 in both forms) to 1e-12,
    the pressure-gradient solver's wall pressure and density, the ghost solver's wall density rate
    (with the same near-inlet flags) and the DBC accelerations within the pre-pass tolerance."""
    c = cases.dam_break_2d(dx=0.04)
    for b in c.blocks:
        if not b.is_fluid:
            b.bound_solver = solver
            b.no_slip = 1
    nb = n_bound(c.blocks)
    st = perturb(c.state, 4, 0.3, 0.002, nb)
    o = _oracle(c, st)
    o.update_neighbours()
    o.dSPH_PreStep()
    o.get_aero_velocity()
    o.Detect_Surface()
    o.dissipation_terms()
    prepared = o.download()
    ctx = _ctx(c, prepared, _mixed(c.settings))
    ctx.update_neighbours()
    res = []
    for h in (ctx, o):
        h.Set_No_Slip()
        if solver == d.PRESSURE_G:
            h.Get_Boundary_Pressure()
            ni = None
        elif solver == d.GHOST:
            ni = h.Boundary_Ghost()
        else:
            h.Boundary_DBC()
            ni = None
        res.append((ni, h.download()))
    (n1, g), (n2, r) = res
    walls = slice(0, nb)
    _check(g, r, ["v"], 1e-12, walls, "Set_No_Slip")
    if solver == d.PRESSURE_G:
        _check(g, r, ["p", "rho"], PASS_TOL, walls, "Get_Boundary_Pressure")
    elif solver == d.GHOST:
        np.testing.assert_array_equal(n1, n2)
        _check(g, r, ["Rrho"], PASS_TOL, walls, "Boundary_Ghost")
    else:
        _check(g, r, ["acc"], PASS_TOL, walls, "Boundary_DBC")


@pytest.mark.parametrize("label,over", VARIANTS, ids=[v[0] for v in VARIANTS])
def test_mixed_variant_residual(label, over):
    """The residual under each build-flag variant the FP64 form is checked on (linear pressure,
    inline artificial viscosity, no delta-SPH, TIC, cubic spline, ALE with TIC, CSF and pairwise
    surface tension, isothermal EOS), from the oracle's pre-pass outputs on the 2D case."""
    c, st = _case("2d")
    s = c.settings.copy()
    for k, v in over.items():
        setattr(s, k, v)
    if s.st_model != d.ST_NOST:
        s.sig = 0.0728
    derive(s)
    c.settings = s
    o = _oracle(c, st)
    o.update_neighbours()
    npd = o.dSPH_PreStep()
    o.get_aero_velocity()
    o.Detect_Surface()
    o.dissipation_terms()
    if s.variant & d.VAR_ALE:
        o.particle_shift()
    o.Get_Boundary_Pressure()
    prepared = o.download()
    o.get_acc_and_Rrho(npd)
    ref = o.download()
    ctx = _ctx(c, prepared, _mixed(s))
    ctx.update_neighbours()
    ctx.get_acc_and_Rrho(npd)
    g = ctx.download()
    nb = n_bound(c.blocks)
    _check(g, ref, ["Rrho"], RRHO_TOL, slice(nb, None), f"{label} residual density rate")
    _check(g, ref, ["acc"], ACC_TOL, slice(nb, None), f"{label} residual acceleration")


@pytest.mark.parametrize("aero", [d.GISSLER, d.INDUCED_PRESSURE, d.SKIN_FRIC])
def test_mixed_aero_closures(aero):
    """The residual's aero force under each closure on the droplet, from the oracle's pre-pass
    outputs: the Gissler closure runs in FP32 in this form, the other two in FP64 on the same
    inputs; aero force and acceleration within the acceleration tolerance."""
    c, st = _case("drop")
    s = c.settings.copy()
    s.acase = aero
    c.settings = s
    o = _oracle(c, st)
    o.update_neighbours()
    npd = o.dSPH_PreStep()
    o.get_aero_velocity()
    o.Detect_Surface()
    o.dissipation_terms()
    prepared = o.download()
    o.get_acc_and_Rrho(npd)
    ref = o.download()
    assert np.any(ref.Af != 0.0), "the case exposes particles to the air"
    ctx = _ctx(c, prepared, _mixed(s))
    ctx.update_neighbours()
    ctx.get_acc_and_Rrho(npd)
    g = ctx.download()
    _check(g, ref, ["Af", "acc"], ACC_TOL, slice(None), f"aero closure {aero}")
    _check(g, ref, ["Rrho"], RRHO_TOL, slice(None), f"aero closure {aero}")


@pytest.mark.parametrize("name", ["2d", "3d", "drop"])
def test_mixed_prepasses(name):
    c, st = _case(name)
    o = _oracle(c, st)
    ctx = _ctx(c, st, _mixed(c.settings))
    nb = n_bound(c.blocks)
    npds = []
    for h in (ctx, o):
        h.update_neighbours()
        npds.append(h.dSPH_PreStep())
    assert npds[0] == pytest.approx(npds[1], rel=1e-6)
    g, r = ctx.download(), o.download()
    _check(g, r, ["L", "gradRho", "norm", "lam", "lam_nb", "kernsum", "colour"], PASS_TOL, slice(None), "dSPH_PreStep")
    for h in (ctx, o):
        h.get_aero_velocity()
        h.Detect_Surface()
    g, r = ctx.download(), o.download()
    assert_ints(g, r, ["surf", "surfzone"], slice(nb, None), max_frac=0.005, label="Detect_Surface")
    _check(g, r, ["curve", "woccl"], 10 * PASS_TOL, slice(nb, None), "Detect_Surface")
    for h in (ctx, o):
        h.dissipation_terms()
        if c.settings.variant & d.VAR_ALE:
            h.particle_shift()
    g, r = ctx.download(), o.download()
    _check(g, r, ["aVisc", "deltaD"], PASS_TOL, slice(nb, None), "dissipation_terms")
    if c.settings.variant & d.VAR_ALE:
        _check(g, r, ["vPert"], 10 * PASS_TOL, slice(nb, None), "particle_shift")


STEP_TOL = 1e-4


@pytest.mark.parametrize("name,solver", [("2d", d.RUNGE_KUTTA), ("3d", d.RUNGE_KUTTA), ("drop", d.RUNGE_KUTTA),
                                         ("2d", d.NEWMARK_BETA), ("drop", d.NEWMARK_BETA)])
def test_mixed_whole_step(name, solver):
    """One Integrator::integrate step (Runge-Kutta 4 or Newmark-Beta with its sub-iterations), mixed
    form vs oracle: displacements and density changes within 1e-4 relative RMS."""
    c, st = _case(name, solver=solver)
    o = _oracle(c, st)
    ctx = _ctx(c, st, _mixed(c.settings))
    o.integrate()
    ctx.integrate()
    g, r = ctx.download(), o.download()
    nb = n_bound(c.blocks)
    disp_g = g.xi[nb:] - st.xi[nb:]
    disp_r = r.xi[nb:] - st.xi[nb:]
    e_x = rel_rms(disp_g, disp_r)
    e_rho = rel_rms(g.rho[nb:] - st.rho[nb:], r.rho[nb:] - st.rho[nb:])
    assert e_x < STEP_TOL and e_rho < STEP_TOL, f"{name}: displacement {e_x:.2e}, density change {e_rho:.2e}"
    assert ctx.settings.delta_t == pytest.approx(o.settings.delta_t, rel=1e-3)


def test_mixed_matches_fp64_device_form():
    """Two steps of the 3D dam break: mixed vs FP64 form on the device."""
    from fjsph_gb300.api import Context
    c, st = _case("3d")
    outs = []
    for prec in (d.PREC_FP64, d.PREC_MIXED):
        s = c.settings.copy()
        s.precision = prec
        ctx = Context(s, st.n, c.blocks)
        ctx.set_states(st, st)
        for _ in range(2):
            ctx.integrate()
        outs.append(ctx.download())
    nb = n_bound(c.blocks)
    assert rel_rms(outs[1].xi[nb:] - st.xi[nb:], outs[0].xi[nb:] - st.xi[nb:]) < 1e-3
    assert rel_rms(outs[1].Rrho[nb:], outs[0].Rrho[nb:]) < 1e-3
