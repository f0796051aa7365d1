"""Initial particles from block files (src/Init.cpp:61-496, src/shapes/): the library's
fjsph_geometry_* path against the pure-Python restatement in oracle/shapes_ref.py, the perturbation
engine against the C++ library it restates, and known answers read off the reference's formulas.

The reference builds with -ffast-math -march=native, so its coordinates are defined only to
rounding: positions are compared to 1e-12 (absolute, extents of order 1-10); every integer
result (counts per block, culling, particle types, block ranges, inlet tables) is exact."""
import math
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300.settings import defaults, derive

ROOT = Path(__file__).resolve().parents[1]
GOLD = ROOT / "tests" / "golden" / "shapes"
from tests._util import reference_examples

REF_EXAMPLES = reference_examples()


@pytest.fixture(scope="module", autouse=True)
def _libs(built_lib):
    return built_lib


def _settings(dim, dx=0.1, **kw):
    s = defaults(dim)
    s.particle_step = dx
    s.rho_rest = 1000.0
    s.speed_sound = 50.0
    for k, v in kw.items():
        setattr(s, k, v)
    derive(s)
    return s


def _product(s, bound_text, fluid_text):
    from fjsph_gb300.geometry import build_particles
    return build_particles(s, bound_text, fluid_text)


def test_perturbation_engine_matches_libstdcxx(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    from oracle.shapes_ref import EPS, MinStd
    exe = tmp_path / "rng_check"
    subprocess.run([gxx, "-O2", "-o", str(exe), str(ROOT / "tests" / "native" / "rng_check.cpp")], check=True)
    got = [float(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = []
    for hi in (1.0, EPS * 0.01, EPS * 4e-4):
        U = MinStd(hi)
        want += [U() for _ in range(12)]
    assert got == want


def _compare(dim, bound, fluid, **kw):
    from oracle.shapes_ref import build as oracle_build
    s = _settings(dim, **kw)
    st, blocks, inlets, g = _product(s, bound, fluid)
    ref = oracle_build(s, bound, fluid)
    n = len(ref["xi"])
    assert st.n == n
    xi = np.array(ref["xi"])[:, :dim]
    assert np.max(np.abs(st.xi - xi)) <= 1e-12
    np.testing.assert_array_equal(st.b, ref["b"])
    np.testing.assert_allclose(st.v, np.array(ref["v"])[:, :dim], rtol=0, atol=1e-15)
    np.testing.assert_allclose(st.rho, ref["rho"], rtol=1e-14)
    np.testing.assert_allclose(st.p, ref["p"], rtol=1e-14)
    np.testing.assert_array_equal(st.m, ref["m"])
    assert [(b.first, b.second, b.is_fluid) for b in blocks] == ref["limits"]
    assert len(inlets) == len(ref["inlets"])
    for got, (back, buf) in zip(inlets, ref["inlets"]):
        np.testing.assert_array_equal(got.back, back)
        np.testing.assert_array_equal(got.buffer, np.array(buf, dtype=np.int64).reshape(-1, 4))
    info = g.block_info()
    for k, blk in enumerate(ref["blocks"]):
        assert info[k]["generated"] == len(blk.coords), blk.name
        assert info[k]["kept"] == blk.intersect.count(0), blk.name
    return st, blocks, inlets, g, ref


def test_2d_blocks_match_oracle():
    st, blocks, inlets, g, ref = _compare(2, (GOLD / "2d_bound.bmap").read_text(), (GOLD / "2d_fluid.bmap").read_text())
    info = {b["name"]: b for b in g.block_info()}
    # every shape produced particles, and the overlaps were culled
    for name in ("Floor", "Wall", "Bump", "Pipe", "PipeHCP", "Curve", "Curve3", "Points", "Pool", "Upper", "Jet", "Jet2"):
        assert info[name]["generated"] > 0, name
    assert info["Pool"]["kept"] < info["Pool"]["generated"]
    assert info["Points"]["generated"] == 3
    # the 2D arc takes its point count from the i-direction count (9 arc points + 3 + 2 straight, 2 layers)
    assert info["Curve"]["generated"] == (9 + 3 + 2) * 2
    # motion table from positions: velocities between the samples (get_boundary_velocity)
    mover = [b for b in blocks if b.name == "Mover"][0]
    assert mover.times == [0.0, 0.5, 1.0]
    assert mover.vels[0] == pytest.approx((0.2, 0.0, 0.0)) and mover.vels[1] == pytest.approx((0.0, 0.4, 0.0))
    assert len(inlets) == 2 and inlets[0].buffer.shape[1] == 4


def test_3d_blocks_match_oracle():
    st, blocks, inlets, g, ref = _compare(3, (GOLD / "3d_bound.bmap").read_text(), (GOLD / "3d_fluid.bmap").read_text())
    info = {b["name"]: b for b in g.block_info()}
    for name in ("Base", "Side", "Pipe", "PipeHCP", "Shell", "ShellHCP", "Box", "BoxHCP", "Ball", "JetS", "JetC"):
        assert info[name]["generated"] > 0, name
    assert info["Box"]["kept"] < info["Box"]["generated"]  # the layer next to the base plane
    # hollow cylinder: ni around, nj = ceil(L/dx) + 1 along, nk radial layers
    p = info["Pipe"]
    assert p["generated"] == p["ni"] * p["nj"] * p["nk"] and p["nj"] == 5 and p["nk"] == 2
    assert len(inlets) == 2


def test_known_answers_2d_line_and_square():
    """Coordinates read off line.cpp / square.cpp (perturbations are below 1e-17 at dx = 0.1)."""
    s = _settings(2)
    bound = "Name: L\nShape: Line\nStart coordinate: 0,0\nEnd coordinate: 0.3,0\nWall radial particle count: 2\nblock end\n"
    fluid = ("Name: S\nShape: Square\nParticle ordering (0=grid,1=HCP): 1\nStart coordinate: 0,1\n"
             "End coordinate: 0.2,1.2\nblock end\n")
    st, blocks, inlets, g = _product(s, bound, fluid)
    want_line = [(i * 0.1, -j * 0.1) for i in range(3) for j in range(2)]  # norm = (dy, -dx) of the direction
    np.testing.assert_allclose(st.xi[:6], want_line, atol=1e-15)
    h = math.sqrt(3.0) / 2 * 0.1
    want_sq = [(0.5 * (2 * i + (j % 2)) * 0.1, 1.0 + j * h) for j in range(3) for i in range(2)]
    np.testing.assert_allclose(st.xi[6:], want_sq, atol=1e-15)
    assert list(st.b) == [d.BOUND] * 6 + [d.FREE] * 6
    assert blocks[0].second == 6 and blocks[1].first == 6


def test_hydrostatic_start_and_masses():
    s = _settings(2, init_hydro_pressure=1, hydro_height=0.5)
    s.grav[:] = [0.0, -9.81, 0.0]
    fluid = "Name: S\nShape: Square\nStart coordinate: 0,0\nEnd coordinate: 0.3,0.5\nblock end\n"
    st, blocks, inlets, g = _product(s, "", fluid)
    p = np.maximum(0.0, 1000.0 * 9.81 * (0.5 - st.xi[:, 1]))
    np.testing.assert_allclose(st.p, p, rtol=1e-14)
    np.testing.assert_allclose(st.rho, 1000.0 * (p / s.B + 1.0) ** (1.0 / s.gam), rtol=1e-14)
    assert np.all(st.m == s.sim_mass)
    np.testing.assert_array_equal(st.cellP, s.p_ref)


def test_reference_quirks_kept():
    s = _settings(2)
    # a Circle without a particle spacing sets dx = 2r / 0 and raises the running spacing to
    # infinity (circle.cpp:29-40, shapes.cpp:158): a later Line's estimated count collapses to 1
    fluid = ("Name: C\nShape: Circle\nCentre coordinate: 0,0\nRadius: 0.3\nblock end\n"
             "Name: L\nShape: Line\nStart coordinate: 2,0\nEnd coordinate: 3,0\nWall radial particle count: 1\nblock end\n")
    st, blocks, inlets, g = _product(s, "", fluid)
    assert g.block_info()[1]["generated"] == 1
    # solid cylinders generate nothing (their loops never run upstream)
    bound = ("Name: Rod\nShape: Cylinder\nSub-shape: Solid\nStart coordinate: 0,0\nRight coordinate: 0,0.3\n"
             "End coordinate: 0.3,0.3\nLength: 0.5\nWall radial particle count: 1\nblock end\n")
    st, blocks, inlets, g = _product(s, bound, "Name: S\nShape: Square\nStart coordinate: 2,2\nEnd coordinate: 2.2,2.2\nblock end\n")
    assert g.block_info()[0]["generated"] == 0
    # a block with a starting pressure takes rho_rest ((p - p_pipe)/B + 1)^gam (shapes.cpp:141-148)
    fl = "Name: S\nShape: Square\nStart coordinate: 0,0\nEnd coordinate: 0.2,0.2\nStarting pressure: 1000\nblock end\n"
    st, *_ = _product(s, "", fl)
    np.testing.assert_allclose(st.rho, 1000.0 * (1000.0 / s.B + 1.0) ** s.gam, rtol=1e-14)


def test_errors_are_reported():
    from fjsph_gb300.geometry import Geometry
    s = _settings(2)
    g = Geometry(s)
    with pytest.raises(ValueError, match="is not a known shape"):
        g.read_text("Name: X\nShape: Hexagon\nblock end\n", False)
    g = Geometry(s)
    g.read_text("Name: X\nShape: Line\nStart coordinate: 0,0\nblock end\n", False)
    with pytest.raises(ValueError, match="end point missing"):
        g.build()
    s3 = _settings(3)
    g = Geometry(s3)  # HCP inlets: Init_Particles reads a buffer layer the generator never makes
    g.read_text("Name: J\nShape: Inlet\nSub-shape: Circle\nCentre coordinate: 0,0,0\nRadius: 0.3\nLength: 0.2\n"
                "Particle ordering (0=grid,1=HCP): 1\nblock end\n", True)
    with pytest.raises(ValueError, match="fifth buffer layer"):
        g.build()


def test_json_block_files(tmp_path):
    import json
    from fjsph_gb300.geometry import build_particles
    s = _settings(2)
    data = {"Walls": {"Shape": "Line", "Start coordinates": [0.0, 0.0], "End coordinates": [1.0, 0.0],
                      "Wall radial particle count": 2, "Boundary solver": "DBC"}}
    fl = {"Water": {"Shape": "Square", "Start coordinates": [0.0, 0.1], "End coordinates": [0.5, 0.5],
                    "Particle ordering (Grid/HCP)": True, "Start velocity": [1.0, 0.0]}}
    (tmp_path / "b.json").write_text(json.dumps(data))
    (tmp_path / "f.json").write_text(json.dumps(fl))
    st, blocks, inlets, g = build_particles(s, tmp_path / "b.json", tmp_path / "f.json")
    bm = ("Name: Walls\nShape: Line\nStart coordinate: 0,0\nEnd coordinate: 1,0\nWall radial particle count: 2\n"
          "Boundary solver: DBC\nblock end\n")
    fm = ("Name: Water\nShape: Square\nStart coordinate: 0,0.1\nEnd coordinate: 0.5,0.5\n"
          "Particle ordering (0=grid,1=HCP): 1\nStarting velocity: 1,0\nblock end\n")
    st2, *_ = build_particles(s, bm, fm)
    np.testing.assert_array_equal(st.xi, st2.xi)
    np.testing.assert_array_equal(st.v, st2.v)
    assert blocks[0].bound_solver == d.DBC and blocks[0].name == "Walls"


@pytest.mark.skipif(REF_EXAMPLES is None, reason="FJSPH_REFERENCE_EXAMPLES is not set")
def test_reference_examples_build():
    """Every shipped example whose para file names existing block files builds; the standing
    column's counts are the ones its block files give by hand (walls 210 x 4 and 105 x 4 at
    dx = 0.01, minus 3 bottom points inside the side walls; fluid 102 x 201 minus the columns
    and the row inside the walls: 99 x 200)."""
    from fjsph_gb300.geometry import load_case
    cases = {"Standing_Column/para": 2, "Dam_2D/para": 2, "Dam_2D/para_n_1": 2, "Poiseuille/para": 2,
             "Coflow/para2D": 2, "Coflow/para3D": 3, "Crossflow/para2D": 2, "Crossflow/para3D": 3,
             "Droplet/para2D": 2, "Droplet/para3D": 3, "Restart/para2D": 2, "VC10/para": 3, "VLM/para": 3,
             "RAE2822/para": 2}
    for rel, dim in cases.items():
        c = load_case(REF_EXAMPLES / rel, dim)
        assert c.state.n > 0 and np.all(np.isfinite(c.state.xi)), rel
    c = load_case(REF_EXAMPLES / "Standing_Column/para", 2)
    assert [b.second - b.first for b in c.blocks] == [840, 417, 840, 19800]


def test_grid_scale_matches_oracle():
    """A grid scale multiplies the block coordinates and plane constants (not radii or lengths,
    shapes.cpp:24-49)."""
    st, blocks, inlets, g, ref = _compare(2, (GOLD / "2d_bound.bmap").read_text(), (GOLD / "2d_fluid.bmap").read_text(),
                                          scale=1.5)
    jet = [b for b in blocks if b.name == "Jet"][0]
    assert jet.delconst == pytest.approx(4.5)  # 3.0 scaled


def test_json_coordinates_and_motion(tmp_path):
    import json
    from fjsph_gb300.geometry import build_particles
    s = _settings(2)
    data = {"Pts": {"Shape": "Coordinates", "Coordinate data": [[0.0, 0.0], [0.5, 0.25], [1.0, 0.5]]},
            "Lid": {"Shape": "Line", "Start coordinates": [0.0, 2.0], "End coordinates": [1.0, 2.0],
                    "Wall radial particle count": 1, "Time data": [0.0, 1.0, 2.0],
                    "Position data": [[0.0, 2.0], [0.5, 2.0], [0.5, 2.5]]}}
    fl = {"W": {"Shape": "Square", "Start coordinates": [3.0, 0.0], "End coordinates": [3.3, 0.3]}}
    (tmp_path / "b.json").write_text(json.dumps(data))
    (tmp_path / "f.json").write_text(json.dumps(fl))
    st, blocks, inlets, g = build_particles(s, tmp_path / "b.json", tmp_path / "f.json")
    np.testing.assert_allclose(st.xi[:3], [[0.0, 0.0], [0.5, 0.25], [1.0, 0.5]], atol=0)
    lid = blocks[1]
    assert lid.times == [0.0, 1.0, 2.0]
    assert lid.vels[0] == pytest.approx((0.5, 0.0, 0.0)) and lid.vels[1] == pytest.approx((0.0, 0.5, 0.0))
