"""The shared-memory tile path of the split-precision form (FJSPH_PAIRS_TILES) against the oracle.

The tile search keeps one member bit mask per particle instead of explicit pair lists; its
neighbour sets must be the reference's FP64 sets bit for bit, and the tile residual (staged
tile-relative positions and velocities, search-time squared distance from the in-cell positions)
must meet the same tolerances as the list residual: density rate <= 1e-5 and acceleration
<= 1e-3 relative RMS against the FP64 oracle on identical input states.
"""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from tests._util import n_bound, rel_rms
from tests.test_gpu_mixed import ACC_TOL, RRHO_TOL, _check, _mixed, _oracle
from tests.test_gpu_parity import _case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib, oracle_lib):
    return built_lib, oracle_lib


def _tile_ctx(c, st):
    from fjsph_gb300.api import Context
    ctx = Context(_mixed(c.settings), st.n + 64, c.blocks, c.inlets)
    ctx.set_pair_mode(d.PAIRS_TILES)
    ctx.set_states(st, st)
    return ctx


@pytest.mark.parametrize("name", ["2d", "3d", "drop"])
def test_tile_neighbour_sets_exact(name):
    c, st = _case(name)
    ctx = _tile_ctx(c, st)
    o = _oracle(c, st)
    o.update_neighbours()
    ctx.update_neighbours()
    assert ctx.pair_mode() == (d.PAIRS_TILES, True)
    a, b = ctx.neighbours(), o.neighbours()
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(a[2], b[2])  # squared distances recomputed in FP64


@pytest.mark.parametrize("name", ["2d", "3d", "drop"])
def test_tile_residual_on_oracle_state(name):
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
    ctx = _tile_ctx(c, prepared)
    ctx.update_neighbours()
    assert ctx.pair_mode() == (d.PAIRS_TILES, True)
    ctx.get_acc_and_Rrho(npd)
    g = ctx.download()
    nb = n_bound(c.blocks)
    _check(g, ref, ["Rrho"], RRHO_TOL, slice(nb, None), f"{name} tile residual density rate")
    _check(g, ref, ["acc"], ACC_TOL, slice(nb, None), f"{name} tile residual acceleration")


def test_tile_step_matches_list_step():
    """A whole step in tile mode stays within FP32 rounding of the same step on pair lists."""
    from fjsph_gb300.api import Context
    c, st = _case("3d")
    out = []
    for mode in (d.PAIRS_LISTS, d.PAIRS_TILES):
        ctx = Context(_mixed(c.settings), st.n + 64, c.blocks, c.inlets)
        ctx.set_pair_mode(mode)
        ctx.set_states(st, st)
        ctx.integrate()
        out.append(ctx.download())
    a, b = out
    nb = n_bound(c.blocks)
    e = rel_rms(b.xi[nb:] - st.xi[nb:], a.xi[nb:] - st.xi[nb:])
    assert e <= 1e-5, f"displacement: {e:.2e}"
    for f, tol in (("v", 1e-6), ("rho", 1e-8), ("acc", 1e-4), ("Rrho", 1e-4)):
        e = rel_rms(getattr(b, f), getattr(a, f))
        assert e <= tol, f"{f}: {e:.2e}"
