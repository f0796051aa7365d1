"""Para-file reader: the reference's "Key: value" rules (src/IOFunctions.h:32-130, src/IO.cpp:305-720)."""
from pathlib import Path

import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import settings as S

HERE = Path(__file__).resolve().parent
from tests._util import reference_examples

REF_EXAMPLES = reference_examples()


def test_fixture_para(built_lib):
    s, extra = S.read_para(HERE / "golden" / "dam_break_2d.para", 2)
    assert s.rho_rest == 1000.0
    assert s.particle_step == 0.01
    assert s.H_fac == 1.3
    assert s.solver_type == d.RUNGE_KUTTA
    assert s.cfl == 0.2 and s.cfl_min == 0.2 and s.cfl_max == 0.2
    assert list(s.grav[:2]) == [0.0, -9.81]
    assert s.acase == d.NOAERO
    assert extra["input_fluid_file"] == "fluid.bmap"
    # the comment after '#' is dropped, the value kept
    assert s.visc_alpha == 0.01
    assert s.H == pytest.approx(0.013)


def test_unparsed_key_keeps_default(built_lib):
    # "SPH density variation (%)" is not a key GetInput reads; the default rho_var = 50 % stays
    s, _ = S.read_para(HERE / "golden" / "dam_break_2d.para", 2)
    assert s.rho_max == pytest.approx(1500.0)


@pytest.mark.skipif(REF_EXAMPLES is None, reason="FJSPH_REFERENCE_EXAMPLES is not set")
def test_reference_examples_parse(built_lib):
    s, extra = S.read_para(REF_EXAMPLES / "Dam_2D" / "para_n_1", 2)
    assert s.particle_step == 0.01 and s.speed_sound == 100.0 and s.visc_alpha == 0.01
    assert s.H_fac == 2.0 and s.mu == pytest.approx(8.94e-4)
    s3, extra3 = S.read_para(REF_EXAMPLES / "Crossflow" / "para3D", 3)
    assert s3.acase == d.GISSLER
    assert list(s3.v_inf) == [128.5, 0.0, 0.0]
    assert s3.rho_g == pytest.approx(1.2262)


def test_mesh_source_keys(tmp_path):
    """A TAU grid or an OpenFOAM directory in the para file selects the mesh-cell air source
    (src/IO.cpp:462-500); a VLM definition selects the vortex lattice only without them."""
    from fjsph_gb300 import _cdefs as d
    from fjsph_gb300.settings import read_para
    base = "SPH initial spacing: 0.01\nVLM definition filename: (thisfile)\n"
    cases = {"Primary grid face filename: mesh.grid\n2D offset vector (0 / x=1,y=2,z=3): 2\n": d.MESH_INFL,
             "OpenFOAM input directory: foam\nOpenFOAM solution directory: 100\n": d.MESH_INFL,
             "": d.VLM_INFL}
    for extra_lines, want in cases.items():
        p = tmp_path / "para"
        p.write_text(base + extra_lines)
        s, extra = read_para(p, 3)
        assert s.asource == want, extra_lines
    s, extra = read_para(p, 2)
    assert s.asource == d.CONST_VEL  # the vortex lattice is 3D only
