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


def test_power_law_air_field():
    """The analytic boundary-layer air field of the oracle: the aero velocity of every active free
    particle is v_inf * clamp((z - wall) / thickness, 0, 1)^(1/7) at its position."""
    import math

    from fjsph_gb300 import cases
    from fjsph_gb300 import _cdefs as d
    from oracle.pyoracle import Oracle
    c = cases.droplet_3d(diam=0.6e-3, dx=1e-4)
    s = c.settings.copy()
    s.asource = d.POWER_LAW
    st = c.state.copy()
    thick = 2e-3
    st.xi[:, 2] += 0.5e-3  # the droplet spans z in [0.2, 0.8] mm above the wall at z = 0
    o = Oracle(s, c.blocks, c.inlets)
    o.air_power_law(2, 0.0, thick, 1.0 / 7.0)
    o.set_states(st, st)
    o.update_neighbours()
    o.dSPH_PreStep()
    o.get_aero_velocity()
    r = o.download()
    act = r.cellID == 1
    assert act.sum() > 10
    z = r.xi[act, 2]
    want = np.array([s.v_inf[0] * math.pow(min(max(zz / thick, 0.0), 1.0), 1.0 / 7.0) for zz in z])
    np.testing.assert_allclose(r.cellV[act, 0], want, rtol=1e-14, atol=0)
    assert np.all(r.cellV[act, 1:] == 0.0)
