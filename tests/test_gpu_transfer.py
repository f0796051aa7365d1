"""Host <-> device state transfer: every field round-trips exactly (reference order in and out),
and uploading one state as both pn and pnp1 (FJSPH_BOTH) equals uploading it twice."""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300.state import ALL_FIELDS
from tests.test_gpu_parity import _case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib):
    return built_lib


@pytest.mark.parametrize("name", ["2d", "3d"])
def test_round_trip_and_both(name):
    from fjsph_gb300.api import Context
    c, st = _case(name)
    ctx = Context(c.settings, st.n + 64, c.blocks)
    ctx.upload(d.BOTH, st)
    for which in (d.PN, d.PNP1):
        g = ctx.download(which)
        for f in ALL_FIELDS:
            np.testing.assert_array_equal(getattr(g, f), getattr(st, f), err_msg=f)
    ctx.integrate()
    a = ctx.download()
    ctx2 = Context(c.settings, st.n + 64, c.blocks)
    ctx2.set_states(st, st)
    ctx2.integrate()
    b = ctx2.download()
    for f in ("xi", "v", "rho", "p", "acc", "Rrho"):
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)
    ctx.close()
    ctx2.close()


def _garbage(st, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    g = st.copy()
    for f in ALL_FIELDS:
        a = getattr(g, f)
        if a.dtype == np.float64:
            a[...] = rng.uniform(-1e3, 1e3, size=a.shape)
        else:
            a[...] = rng.integers(0, 4, size=a.shape)
    return g


def _cases():
    from fjsph_gb300 import cases
    out = []
    c, st = _case("2d")
    out.append(("dam2d_rk_fp64", c, st, None))
    c, st = _case("2d", solver=d.NEWMARK_BETA)
    out.append(("dam2d_nb_fp64", c, st, None))
    c, st = _case("3d")
    s = c.settings.copy()
    s.precision = d.PREC_MIXED
    out.append(("dam3d_ale_mixed", c, st, s))
    jet = cases.jet_crossflow(n_target=60_000)
    s = jet.settings.copy()
    s.precision = d.PREC_MIXED
    out.append(("jet_mixed", jet, jet.state, s))
    drop, mesh = cases.droplet_in_mesh(2)
    out.append(("mesh2d_fp64", drop, drop.state, mesh))
    c, st = _case("drop", solver=d.RUNGE_KUTTA)
    s = c.settings.copy()
    s.st_model = d.ST_CSF
    out.append(("drop_csf_fp64", c, st, s))
    c, st = _case("3d")
    s = c.settings.copy()
    s.variant |= d.VAR_TIC
    out.append(("dam3d_ale_tic_fp64", c, st, s))
    return out


@pytest.mark.parametrize("idx", range(7))
def test_step_fields_are_the_step_inputs(idx):
    """Two steps from a state whose non-step fields on the device are garbage equal two steps from
    the full upload, bit for bit: the other fields are recomputed before they are read."""
    from fjsph_gb300.api import Context
    from fjsph_gb300.mesh import CellMesh
    from fjsph_gb300.state import STEP_FIELDS
    label, c, st, extra = _cases()[idx]
    s = extra if isinstance(extra, d.Settings) else c.settings
    mesh = extra if isinstance(extra, CellMesh) else None
    res = []
    for partial in (False, True):
        ctx = Context(s, st.n + 4096, c.blocks, c.inlets)
        if mesh is not None:
            ctx.mesh_set(mesh)
        if partial:
            ctx.upload(d.BOTH, _garbage(st, 5))
            ctx.upload(d.BOTH, st, fields=STEP_FIELDS)
        else:
            ctx.upload(d.BOTH, st)
        for _ in range(2):
            ctx.integrate()
        res.append(ctx.download())
        ctx.close()
    a, b = res
    assert a.n == b.n
    # everything downstream of a step is a function of the step fields: were any other field read
    # before it is written, they would differ after two steps
    for f in STEP_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f"{label}: {f}")


def _prefix(big, n):
    """The first n particles of a state, sharing its memory."""
    from fjsph_gb300.state import SPHState
    out = SPHState.__new__(SPHState)
    out.n, out.dim = int(n), big.dim
    for f in ALL_FIELDS:
        setattr(out, f, getattr(big, f)[:n])
    return out


@pytest.mark.parametrize("idx", range(7))
def test_step_host_equals_separate_calls(idx):
    """fjsph_step_host (upload as pn and pnp1, step, download, the late fields in flight during the
    first search) equals the three calls, bit for bit, over three steps, on a context whose device
    state started as garbage: a late field read before it landed would show.  Its input and output
    share their arrays.  The first step re-orders at its first search, the others do not."""
    from fjsph_gb300.api import Context
    from fjsph_gb300.mesh import CellMesh
    from fjsph_gb300.state import SPHState, STEP_FIELDS
    label, c, st, extra = _cases()[idx]
    s = extra if isinstance(extra, d.Settings) else c.settings
    mesh = extra if isinstance(extra, CellMesh) else None
    cap = st.n + 4096
    ctxs = []
    for _ in range(2):
        ctx = Context(s, cap, c.blocks, c.inlets)
        if mesh is not None:
            ctx.mesh_set(mesh)
        ctx.upload(d.BOTH, _garbage(st, 5))
        ctxs.append(ctx)
    fused, plain = ctxs
    big = SPHState(cap, st.dim)
    for f in STEP_FIELDS:
        getattr(big, f)[:st.n] = getattr(st, f)
    cur_a = _prefix(big, st.n)
    cur_b = st
    for step in range(3):
        n_a = fused.step_host(cur_a, big, fields=STEP_FIELDS)
        cur_a = _prefix(big, n_a)
        plain.upload(d.BOTH, cur_b, fields=STEP_FIELDS)
        plain.integrate()
        cur_b = plain.download(fields=STEP_FIELDS)
        assert cur_a.n == cur_b.n
        for f in STEP_FIELDS:
            np.testing.assert_array_equal(getattr(cur_a, f), getattr(cur_b, f), err_msg=f"{label} step {step}: {f}")
    for ctx in ctxs:
        ctx.close()


def test_step_host_live_jet_inserts():
    """The live-inlet jet (FP32 form, power-law air): its first step inserts a layer, so the fields
    copied out after the pre-passes are copied again in the new order; the next steps keep them.
    fjsph_step_host equals the three calls bit for bit."""
    from fjsph_gb300 import cases
    from fjsph_gb300.api import Context
    from fjsph_gb300.state import SPHState, STEP_FIELDS
    c = cases.jet_crossflow_live(n_target=60_000, cap=70_000)
    s = c.settings.copy()
    s.precision = d.PREC_MIXED
    st = c.state
    cap = max(s.max_points, st.n) + 1024
    ctxs = []
    for _ in range(2):
        ctx = Context(s, cap, c.blocks, c.inlets)
        if c.power_law_params:
            ctx.air_power_law(*c.power_law_params)
        ctx.set_states(st, st)
        ctxs.append(ctx)
    fused, plain = ctxs
    big = SPHState(cap, st.dim)
    for f in STEP_FIELDS:
        getattr(big, f)[:st.n] = getattr(st, f)
    cur_a, cur_b = _prefix(big, st.n), st
    counts = []
    for step in range(3):
        n_a = fused.step_host(cur_a, big, fields=STEP_FIELDS)
        cur_a = _prefix(big, n_a)
        plain.upload(d.BOTH, cur_b, fields=STEP_FIELDS)
        plain.integrate()
        cur_b = plain.download(fields=STEP_FIELDS)
        assert cur_a.n == cur_b.n
        counts.append(cur_a.n)
        for f in STEP_FIELDS:
            np.testing.assert_array_equal(getattr(cur_a, f), getattr(cur_b, f), err_msg=f"step {step}: {f}")
    assert counts[0] > st.n  # the first step inserted
    for ctx in ctxs:
        ctx.close()


def test_step_host_then_plain_steps_and_capacity():
    """After fjsph_step_host the context holds the same pn and pnp1 as after the three calls: a
    plain fjsph_integrate that follows gives the same state bit for bit.  An output smaller than
    the particle count is refused with FJSPH_E_CAPACITY after the step, and the context steps on."""
    from fjsph_gb300._lib import FJSPHError
    from fjsph_gb300.api import Context
    from fjsph_gb300.state import SPHState, STEP_FIELDS
    label, c, st, s = _cases()[2]  # the 3D dam break, FP32 form, ALE
    cap = st.n + 4096
    fused = Context(s, cap, c.blocks, c.inlets)
    plain = Context(s, cap, c.blocks, c.inlets)
    for ctx in (fused, plain):
        ctx.upload(d.BOTH, _garbage(st, 7))
    big = SPHState(cap, st.dim)
    for f in STEP_FIELDS:
        getattr(big, f)[:st.n] = getattr(st, f)
    fused.step_host(_prefix(big, st.n), big, fields=STEP_FIELDS)
    plain.upload(d.BOTH, st, fields=STEP_FIELDS)
    plain.integrate()
    for ctx in (fused, plain):
        ctx.integrate()
    a, b = fused.download(), plain.download()
    for f in STEP_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f"{label} after a plain step: {f}")
    small = SPHState(st.n - 1, st.dim)
    with pytest.raises(FJSPHError, match="capacity"):
        fused.step_host(a, small, fields=STEP_FIELDS)
    fused.integrate()  # still usable
    assert np.isfinite(fused.download(fields=["xi"]).xi).all()
    fused.close()
    plain.close()
