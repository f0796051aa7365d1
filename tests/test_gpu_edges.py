"""Edge cases of the device path against the oracle and the status codes of the C ABI.

  - a particle far outside the others makes the cell grid larger than the bucket table (2^26
    cells at most), so the search runs on the wrapped (hashed) table: lists bit-exact as sets in
    both forms all the same;
  - the split-precision lists grow past the fixed per-slot storage sized from the previous
    search (a state compressed by 0.7 between two searches): the fill detects the overflow,
    re-sizes and re-runs, and the lists are bit-exact;
  - a state larger than the context's capacity is refused (FJSPH_E_CAPACITY), and passes called
    before any state exists return FJSPH_E_STATE, leaving the context usable.
"""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases
from tests._util import n_bound

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib, oracle_lib):
    return built_lib, oracle_lib


def _ctx(c, st, prec):
    from fjsph_gb300.api import Context
    s = c.settings.copy()
    s.precision = prec
    ctx = Context(s, st.n + 64, c.blocks, c.inlets)
    ctx.set_states(st, st)
    return ctx


def _oracle_lists(c, st):
    from oracle.pyoracle import Oracle
    o = Oracle(c.settings, c.blocks, c.inlets)
    o.set_states(st, st)
    o.update_neighbours()
    return o.neighbours()


def _same_lists(a, b, label):
    for k in range(3):
        np.testing.assert_array_equal(a[k], b[k], err_msg=f"{label}: part {k}")


@pytest.mark.parametrize("prec", [d.PREC_FP64, d.PREC_MIXED])
def test_wrapped_bucket_table(prec):
    c = cases.dam_break_3d(dx=0.03, column=(0.3, 0.3, 0.6), tank=(0.8, 0.3, 0.6))
    st = c.state.copy()
    st.xi[-1] = (200.0, 200.0, 200.0)  # the last fluid particle, far from everything
    ctx = _ctx(c, st, prec)
    ctx.update_neighbours()
    _same_lists(ctx.neighbours(), _oracle_lists(c, st), "wrapped table")
    ctx.close()


def test_list_storage_outgrown():
    c = cases.dam_break_3d(dx=0.03, column=(0.3, 0.3, 0.6), tank=(0.8, 0.3, 0.6))
    st = c.state.copy()
    ctx = _ctx(c, st, d.PREC_MIXED)
    ctx.update_neighbours()
    m1 = int(ctx.neighbour_counts().max())
    dense = st.copy()
    nb = n_bound(c.blocks)
    centre = dense.xi[nb:].mean(axis=0)
    dense.xi[nb:] = centre + 0.7 * (dense.xi[nb:] - centre)  # ~3x the neighbours inside the column
    ctx.set_states(dense, dense)
    ctx.update_neighbours()
    m2 = int(ctx.neighbour_counts().max())
    assert m2 > 1.5 * m1  # past the storage sized from the first search (its maximum + 25 %)
    _same_lists(ctx.neighbours(), _oracle_lists(c, dense), "re-sized lists")
    ctx.close()


def test_capacity_and_state_errors():
    from fjsph_gb300._lib import FJSPHError
    from fjsph_gb300.api import Context
    c = cases.dam_break_2d(dx=0.04)
    st = c.state
    small = Context(c.settings, st.n - 1, c.blocks, c.inlets)
    with pytest.raises(FJSPHError, match="capacity"):
        small.set_states(st, st)
    small.close()
    ctx = Context(c.settings, st.n + 64, c.blocks, c.inlets)
    with pytest.raises(FJSPHError):
        ctx.update_neighbours()  # no state yet
    ctx.set_states(st, st)  # the context is still usable
    assert ctx.update_neighbours() > 0
    ctx.close()
