"""Restart files (src/H5IO.cpp Write_HDF5 / Read_HDF5 content and names): a context writes its state
after a few steps, the container holds the reference's groups, datasets and attributes, and a
fresh context reading it holds the same particles and integrator scalars bit for bit."""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import cases
from fjsph_gb300.restart import read_restart

pytestmark = pytest.mark.gpu

FIELDS_VEC = {"xi": "Position coordinate", "v": "Velocity", "acc": "Acceleration", "cellV": "Cell velocity"}
FIELDS_SCA = {"p": "Pressure", "rho": "Density", "Rrho": "Density gradient", "m": "Mass", "cellRho": "Cell density",
              "cellP": "Cell pressure"}


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib):
    return built_lib


@pytest.mark.parametrize("precision", [d.PREC_FP64, d.PREC_MIXED])
def test_restart_round_trip(tmp_path, precision):
    from fjsph_gb300.api import Context
    c = cases.dam_break_2d(dx=0.04) if precision == d.PREC_FP64 else cases.droplet_3d(diam=8e-4, dx=1e-4)
    s = c.settings.copy()
    s.precision = precision
    ctx = Context(s, c.state.n + 64, c.blocks, c.inlets)
    ctx.set_states(c.state, c.state)
    for _ in range(3):
        ctx.integrate()
    path = tmp_path / "run_particles.fjrst"
    ctx.restart_write(str(path), current_frame=7)
    st, s0 = ctx.download(), ctx.settings
    rec = read_restart(path)
    assert rec["Current frame"] == 7 and rec["Simulation current time"] == s0.current_time
    assert rec["SPH CFL condition"] == s0.cfl and rec["Grid scale"] == s0.scale
    nbb = sum(1 for b in c.blocks if not b.is_fluid)
    assert rec["Number of boundary blocks"] == nbb and rec["Number of fluid points"] == st.n - sum(
        b.second - b.first for b in c.blocks if not b.is_fluid)
    axes = "xyz"
    for bi, b in enumerate(c.blocks):
        z = f"Fluid {bi - nbb}/" if b.is_fluid else f"Boundary {bi}/"
        sl = slice(b.first, b.second)
        for f, name in FIELDS_VEC.items():
            for k in range(s.dim):
                want = getattr(st, f)[sl, k] / (s0.scale if f == "xi" else 1.0)
                np.testing.assert_array_equal(rec[z + f"{name} {axes[k]}"], want)
        for f, name in FIELDS_SCA.items():
            np.testing.assert_array_equal(rec[z + name], getattr(st, f)[sl])
        np.testing.assert_array_equal(rec[z + "Boundary condition"], st.b[sl])
        np.testing.assert_array_equal(rec[z + "Particle ID"], st.part_id[sl])
    # a fresh context from the file
    ctx2 = Context(s, c.state.n + 64, c.blocks, c.inlets)
    assert ctx2.restart_read(str(path)) == 7
    st2, s2 = ctx2.download(), ctx2.settings
    for f in list(FIELDS_VEC) + list(FIELDS_SCA) + ["b", "part_id", "cellID"]:
        np.testing.assert_array_equal(getattr(st2, f), getattr(st, f), err_msg=f)
    assert (s2.current_time, s2.cfl, s2.n_stable, s2.n_unstable) == (s0.current_time, s0.cfl, s0.n_stable,
                                                                     s0.n_unstable)
    ctx2.integrate()
    assert np.all(np.isfinite(ctx2.download().xi))
