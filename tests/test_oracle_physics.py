"""The oracle on the standing water column (Examples/Standing_Column: Pressure-Gradient walls,
hydrostatic start, Newmark-Beta): after 0.5 s the pressure still follows p = rho g (H - y) and the
fluid is at rest up to the acoustic settling.  The GPU forms are held to the same bounds in
test_gpu_physics.py."""
import numpy as np
import pytest

from fjsph_gb300 import cases
from tests._util import hydrostatic_error


@pytest.fixture(scope="module", autouse=True)
def _libs(oracle_lib):
    return oracle_lib


def test_standing_column_hydrostatic_oracle():
    from oracle.pyoracle import Oracle
    c = cases.standing_column_2d()
    o = Oracle(c.settings, c.blocks, c.inlets)
    o.set_states(c.state, c.state)
    steps = 0
    while o.settings.current_time < 0.5 and steps < 5000:
        o.integrate()
        steps += 1
    st = o.download()
    s = c.settings
    nb = c.blocks[0].second
    assert o.settings.current_time >= 0.5
    assert hydrostatic_error(st, nb, s.rho_rest, 1.0 + 0.5 * s.particle_step) < 0.03
    assert np.all(np.isfinite(st.xi))
    assert np.abs(st.v[nb:]).max() < 0.05
