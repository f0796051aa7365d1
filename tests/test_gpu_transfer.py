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
