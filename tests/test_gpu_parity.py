"""Parity of the GB300 kernels with the CPU oracle on identical input states (FP64 form).

Each test uploads the same seeded state to a device context and to the oracle, runs the same
reference function on both, and compares:
  - neighbour lists: bit-exact as sets, and the squared distances bit-exact;
  - integer flags (surf, surfzone, cellID, near-inlet): exact;
  - floating-point fields: max |gpu - oracle| <= RTOL * max |oracle| per field.  Both sides are
    FP64; the differences come from summation order (cell order vs index order), fused
    multiply-adds and the order of operations inside each pair term.
"""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases
from fjsph_gb300.settings import derive
from tests._util import assert_fields, assert_ints, n_bound, perturb, rel_err

pytestmark = pytest.mark.gpu

RTOL = 1e-9          # single pass, FP64 vs FP64
RTOL_STEP = 1e-7     # whole integrator steps (differences grow through the stages)

PRESTEP_F = ["L", "gradRho", "norm", "lam", "lam_nb", "colourG", "kernsum", "colour"]
SURF_F = ["norm", "curve", "norm_curve", "woccl", "pDist"]
STATE_F = ["xi", "v", "rho", "p", "acc", "Rrho"]


def _case(name, **kw):
    if name == "2d":
        c = cases.dam_break_2d(dx=0.04, **kw)
        return c, perturb(c.state, 1, 0.3, 0.05 * 0.04, n_bound(c.blocks))
    if name == "3d":
        c = cases.dam_break_3d(dx=0.03, column=(0.3, 0.3, 0.6), tank=(0.8, 0.3, 0.6), **kw)
        return c, perturb(c.state, 2, 0.3, 0.05 * 0.03, n_bound(c.blocks))
    if name == "drop":
        c = cases.droplet_3d(diam=1.2e-3, dx=1e-4, **kw)
        return c, perturb(c.state, 3, 0.5, 0.05 * 1e-4, 0)
    raise KeyError(name)


def _pair(c, st, settings=None):
    from fjsph_gb300.api import Context
    from oracle.pyoracle import Oracle
    s = settings if settings is not None else c.settings
    ctx = Context(s, st.n + 64, c.blocks, c.inlets)
    orc = Oracle(s, c.blocks, c.inlets)
    for h in (ctx, orc):
        h.set_states(st, st)
    return ctx, orc


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib, oracle_lib):
    return built_lib, oracle_lib


@pytest.mark.parametrize("name", ["2d", "3d", "drop"])
def test_neighbour_lists_bit_exact(name):
    c, st = _case(name)
    ctx, orc = _pair(c, st)
    n1, n2 = ctx.update_neighbours(), orc.update_neighbours()
    assert n1 == n2
    o1, i1, d1 = ctx.neighbours()
    o2, i2, d2 = orc.neighbours()
    np.testing.assert_array_equal(o1, o2)
    np.testing.assert_array_equal(i1, i2)
    assert np.array_equal(d1.view(np.uint64), d2.view(np.uint64))


def test_neighbour_lists_wrapped_table():
    """Particles spread over a box with far more cells than hash buckets (wrap-around path)."""
    c, st = _case("drop")
    st = st.copy()
    rng = np.random.default_rng(9)
    st.xi[: st.n // 2] += rng.integers(-40, 40, size=(st.n // 2, 1)) * 0.05  # distant clusters
    ctx, orc = _pair(c, st)
    assert ctx.update_neighbours() == orc.update_neighbours()
    o1, i1, d1 = ctx.neighbours()
    o2, i2, d2 = orc.neighbours()
    np.testing.assert_array_equal(o1, o2)
    np.testing.assert_array_equal(i1, i2)


@pytest.mark.parametrize("name", ["2d", "3d", "drop"])
def test_prepasses(name):
    c, st = _case(name)
    ctx, orc = _pair(c, st)
    nb = n_bound(c.blocks)
    out = []
    for h in (ctx, orc):
        h.update_neighbours()
        npd = h.dSPH_PreStep()
        a = h.download()
        h.get_aero_velocity()
        h.Detect_Surface()
        b = h.download()
        h.dissipation_terms()
        if c.settings.variant & d.VAR_ALE:
            h.particle_shift()
        h.Check_Pipe_Outlet()
        out.append((npd, a, b, h.download()))
    (npd1, a1, b1, f1), (npd2, a2, b2, f2) = out
    assert abs(npd1 - npd2) <= 1e-12 * abs(npd2)
    assert_fields(a1, a2, PRESTEP_F, RTOL, label="dSPH_PreStep")
    assert_ints(b1, b2, ["cellID", "surf", "surfzone", "b"], label="Detect_Surface")
    assert_fields(b1, b2, SURF_F + ["cellV"], RTOL, slice(nb, None), label="Detect_Surface")
    assert_fields(f1, f2, ["aVisc", "deltaD"], RTOL, slice(nb, None), label="dissipation_terms")
    if c.settings.variant & d.VAR_ALE:
        assert_fields(f1, f2, ["vPert"], 1e-8, slice(nb, None), label="particle_shift")


def _prepared(c, st):
    ctx, orc = _pair(c, st)
    npds = []
    for h in (ctx, orc):
        h.update_neighbours()
        npds.append(h.dSPH_PreStep())
        h.get_aero_velocity()
        h.Detect_Surface()
        h.dissipation_terms()
        if c.settings.variant & d.VAR_ALE:
            h.particle_shift()
    return ctx, orc, npds


@pytest.mark.parametrize("name", ["2d", "3d", "drop"])
def test_residual(name):
    c, st = _case(name)
    ctx, orc, npds = _prepared(c, st)
    nb = n_bound(c.blocks)
    for h, npd in zip((ctx, orc), npds):
        h.Get_Boundary_Pressure()
        h.get_acc_and_Rrho(npd)
    g, o = ctx.download(), orc.download()
    assert_fields(g, o, ["p", "rho"], 1e-10, slice(0, nb), label="Get_Boundary_Pressure")
    assert_fields(g, o, ["acc", "Af", "Rrho"], RTOL, slice(nb, None), label="get_acc_and_Rrho")


@pytest.mark.parametrize("solver", [d.GHOST, d.DBC])
def test_boundary_solvers(solver):
    c = cases.dam_break_2d(dx=0.04)
    for b in c.blocks:
        if not b.is_fluid:
            b.bound_solver = solver
            b.no_slip = 1
    st = perturb(c.state, 4, 0.3, 0.002, n_bound(c.blocks))
    ctx, orc, npds = _prepared(c, st)
    nb = n_bound(c.blocks)
    res = []
    for h in (ctx, orc):
        h.Set_No_Slip()
        ni = h.Boundary_Ghost() if solver == d.GHOST else h.Boundary_DBC()
        res.append((ni, h.download()))
    (n1, g), (n2, o) = res
    assert_fields(g, o, ["v"], 1e-12, slice(0, nb), label="Set_No_Slip")
    if solver == d.GHOST:
        np.testing.assert_array_equal(n1, n2)
        assert_fields(g, o, ["Rrho"], RTOL, slice(0, nb), label="Boundary_Ghost")
    else:
        assert_fields(g, o, ["acc"], 0.0, slice(0, nb), label="Boundary_DBC")


VARIANTS = [
    ("linear", dict(variant=d.VAR_LINEAR)),
    ("nofrozen", dict(variant=d.VAR_NOFROZEN)),
    ("nodsph", dict(variant=d.VAR_NODSPH)),
    ("tic", dict(variant=d.VAR_TIC)),
    ("cubic", dict(variant=d.VAR_CUBIC)),
    ("ale_tic", dict(variant=d.VAR_ALE | d.VAR_TIC)),
    ("csf", dict(st_model=d.ST_CSF)),
    ("pairwise", dict(st_model=d.ST_PAIRWISE)),
    ("iso_eos", dict(pressure_rel=d.ISO_EOS)),
]


@pytest.mark.parametrize("label,over", VARIANTS, ids=[v[0] for v in VARIANTS])
def test_variant_residual(label, over):
    c, st = _case("2d")
    s = c.settings.copy()
    for k, v in over.items():
        setattr(s, k, v)
    if s.st_model != d.ST_NOST:
        s.sig = 0.0728
    derive(s)  # the derived settings follow the variant (kernel normalisation, pipe density, ycoef)
    c.settings = s
    ctx, orc, npds = _prepared(c, st)
    nb = n_bound(c.blocks)
    for h, npd in zip((ctx, orc), npds):
        h.Get_Boundary_Pressure()
        h.get_acc_and_Rrho(npd)
    g, o = ctx.download(), orc.download()
    assert_ints(g, o, ["surf", "surfzone"], label=label)
    assert_fields(g, o, ["acc", "Rrho", "aVisc", "deltaD"], RTOL, slice(nb, None), label=label)


@pytest.mark.parametrize("aero", [d.GISSLER, d.INDUCED_PRESSURE, d.SKIN_FRIC])
def test_aero_closures(aero):
    c, st = _case("drop")
    s = c.settings.copy()
    s.acase = aero
    c.settings = s
    ctx, orc, npds = _prepared(c, st)
    for h, npd in zip((ctx, orc), npds):
        h.get_acc_and_Rrho(npd)
    g, o = ctx.download(), orc.download()
    assert_fields(g, o, ["Af", "acc", "Rrho", "woccl"], RTOL, label=f"aero {aero}")


@pytest.mark.parametrize("name", ["2d", "3d", "drop"])
def test_find_timestep(name):
    c, st = _case(name)
    ctx, orc, npds = _prepared(c, st)
    for h, npd in zip((ctx, orc), npds):
        h.get_acc_and_Rrho(npd)
    dt1, dt2 = ctx.find_timestep(), orc.find_timestep()
    assert dt1 == pytest.approx(dt2, rel=1e-12)
    r1, r2 = ctx.step_report(), orc.step_report()
    for k in ("maxRho_pc", "maxf", "maxAf"):
        assert r1[k] == pytest.approx(r2[k], rel=1e-9), k


@pytest.mark.parametrize("name", ["2d", "3d", "drop"])
def test_runge_kutta_stages(name):
    """Get_First_RK, second search + pre-passes, Runge_Kutta4 (src/Integration.cpp:27-107)."""
    c, st = _case(name, solver=d.RUNGE_KUTTA)
    ctx, orc, npds = _prepared(c, st)
    nb = n_bound(c.blocks)
    dt = orc.find_timestep()
    logb, sts = [], []
    for h, npd in zip((ctx, orc), npds):
        s = h.settings
        s.delta_t = dt
        h.settings = s
        logb.append(h.Get_First_RK(npd))
        sts.append(h.download())
    assert logb[0] == pytest.approx(logb[1], abs=1e-9)
    assert_fields(sts[0], sts[1], STATE_F, RTOL, slice(nb, None), label="Get_First_RK")
    rms, fin = [], []
    for h, lb in zip((ctx, orc), logb):
        h.update_neighbours()
        npd = h.dSPH_PreStep()
        h.get_aero_velocity()
        h.Detect_Surface()
        h.dissipation_terms()
        if c.settings.variant & d.VAR_ALE:
            h.particle_shift()
        rms.append(h.Runge_Kutta4(npd, logb[1]))
        fin.append(h.download())
    assert rms[0] == pytest.approx(rms[1], abs=1e-7)
    assert_fields(fin[0], fin[1], STATE_F, RTOL_STEP, slice(nb, None), label="Runge_Kutta4")
    assert_fields(fin[0], fin[1], ["p", "rho"], RTOL_STEP, slice(0, nb), label="Runge_Kutta4 boundary")


@pytest.mark.parametrize("name", ["2d", "drop"])
def test_newmark_beta(name):
    c, st = _case(name, solver=d.NEWMARK_BETA)
    ctx, orc, npds = _prepared(c, st)
    nb = n_bound(c.blocks)
    dt = orc.find_timestep()
    out = []
    for h, npd in zip((ctx, orc), npds):
        s = h.settings
        s.delta_t = dt
        h.settings = s
        h.Do_NB_Iter(npd)
        a = h.download()
        r = h.Newmark_Beta(npd, 0.0, 1)
        out.append((a, r, h.download()))
    (a1, r1, f1), (a2, r2, f2) = out
    assert_fields(a1, a2, STATE_F, RTOL, slice(nb, None), label="Do_NB_Iter")
    assert r1[2] == r2[2], "sub-iteration counts differ"
    assert_fields(f1, f2, STATE_F, RTOL_STEP, slice(nb, None), label="Newmark_Beta")


@pytest.mark.parametrize("name,solver", [("2d", d.RUNGE_KUTTA), ("3d", d.RUNGE_KUTTA), ("drop", d.RUNGE_KUTTA),
                                         ("2d", d.NEWMARK_BETA)])
def test_integrate_steps(name, solver):
    """Three whole steps of Integrator::integrate from the same state."""
    c, st = _case(name, solver=solver)
    ctx, orc = _pair(c, st)
    errs = []
    for h in (ctx, orc):
        e = [h.integrate() for _ in range(3)]
        errs.append(e)
    g, o = ctx.download(), orc.download()
    np.testing.assert_allclose(errs[0], errs[1], atol=1e-6)
    assert ctx.settings.delta_t == pytest.approx(orc.settings.delta_t, rel=1e-9)
    assert ctx.settings.current_time == pytest.approx(orc.settings.current_time, rel=1e-9)
    nb = n_bound(c.blocks)
    assert_fields(g, o, ["xi", "v", "rho", "p"], RTOL_STEP, slice(nb, None), label="integrate")
    go, oo = ctx.download(d.PN), orc.download(d.PN)
    assert_fields(go, oo, ["xi", "v", "rho"], RTOL_STEP, slice(nb, None), label="integrate pn")


def test_reorder_interval_does_not_change_results():
    c, st = _case("3d")
    outs = []
    for interval in (0, 1, 3):
        s = c.settings.copy()
        s.reorder_interval = interval
        from fjsph_gb300.api import Context
        ctx = Context(s, st.n, c.blocks)
        ctx.set_states(st, st)
        for _ in range(2):
            ctx.integrate()
        outs.append(ctx.download())
    for o in outs[1:]:
        assert rel_err(o.xi, outs[0].xi) < 1e-12
        assert rel_err(o.rho, outs[0].rho) < 1e-12
