"""Initial particles from the reference's block files (Init_Particles, src/Init.cpp:268-494).

`Geometry` drives the library's fjsph_geometry_* calls: block files in the reference's "bmap"
format (or its JSON format, translated to the same key/value text), check_input and
generate_points per block, Check_Intersection, and the state / LIMITS / inlet tables in reference
index order.  `load_case(para)` does what the reference does before its first step from a case
directory: read the para file (Set_Values applied), build the particles from the two block files
it names, and set the constant-velocity air source's cell values.

File names in the para file are taken relative to the para file's directory (the reference opens
them relative to its working directory, which is the case directory when it is run there).
"""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np

from . import _cdefs as d
from ._lib import check, lib
from .state import BlockSpec, InletSpec, SPHState

# read_shape_JSON keys (src/shapes/shapes.cpp:294-353) -> the bmap keys of read_shapes_bmap
_JSON_TO_BMAP = {
    "Shape": "Shape", "Sub-shape": "Sub-shape", "Boundary solver": "Boundary solver",
    "Aerodynamic entry normal": "Aerodynamic entry normal",
    "Fixed velocity or dynamic inlet BC": "Fixed velocity or dynamic inlet BC",
    "Deletion normal": "Deletion normal", "Insertion normal": "Insertion normal",
    "Aerodynamic entry plane constant": "Aerodynamic entry plane constant",
    "Deletion plane constant": "Deletion plane constant", "Insertion plane constant": "Insertion plane constant",
    "Pipe depth": "Pipe depth", "i-direction count": "i-direction count", "j-direction count": "j-direction count",
    "k-direction count": "k-direction count", "Normal vector": "Normal vector",
    "Rotation angles (degree)": "Rotation angles", "Rotation angle (degree)": "Rotation angle",
    "Start coordinates": "Start coordinate", "End coordinates": "End coordinate",
    "Right coordinates": "Right coordinate", "Midpoint coordinates": "Midpoint coordinate",
    "Centre coordinates": "Centre coordinate", "Arch normal": "Arch normal", "Radius": "Radius", "Length": "Length",
    "Arc start (degree)": "Arc start (degree)", "Arc end (degree)": "Arc end (degree)",
    "Arc length (degree)": "Arc length (degree)", "Start straight length": "Starting straight length",
    "End straight length": "Ending straight length", "Particle spacing": "Particle spacing",
    "Particle ordering (Grid/HCP)": "Particle ordering (0=grid,1=HCP)", "Wall thickness": "Wall thickness",
    "Wall radial particle count": "Wall radial particle count", "Wall is no-slip": "Wall is no slip (0/1)",
    "Start velocity": "Starting velocity", "Start jet velocity": "Starting jet velocity",
    "Start pressure": "Starting pressure", "Start density": "Starting density",
    "Coordinate filename": "Coordinate filename", "Time data filename": "Time data filename",
}


def _fmt(v) -> str:
    if isinstance(v, bool):
        return "1" if v else "0"
    if isinstance(v, (list, tuple)):
        return ",".join(_fmt(x) for x in v)
    if isinstance(v, float):
        return repr(v)
    return str(v)


def json_to_bmap(data: dict) -> str:
    """A JSON block file (block name -> parameters) as bmap text.  The JSON reader upstream leaves
    the motion table's length at zero (read_shape_JSON sets times and positions but not ntimes);
    here "Time data" with "Position data" becomes a full "Time position data" section."""
    out = []
    for name, blk in data.items():
        out.append(f"Name: {name}")
        for key, val in blk.items():
            if key in _JSON_TO_BMAP:
                out.append(f"{_JSON_TO_BMAP[key]}: {_fmt(val)}")
        if "Coordinate data" in blk:
            pts = blk["Coordinate data"]
            out.append("Coordinate data:")
            out.append("")  # the reader skips the line after the key
            out.append(" ".join([str(len(pts))] + [repr(float(x)) for p in pts for x in p]))
        if "Time data" in blk and "Position data" in blk:
            times, pos = blk["Time data"], blk["Position data"]
            out.append("Time position data")
            out.append(str(len(times)))
            for t, p in zip(times, pos):
                out.append(" ".join([repr(float(t))] + [repr(float(x)) for x in p]))
        out.append("block end")
    return "\n".join(out) + "\n"


class Geometry:
    """Init_Particles over the library: read block files, build, then read the results."""

    def __init__(self, settings: d.Settings):
        self.settings = settings.copy()
        self.dim = settings.dim
        h = C.c_void_p()
        check("fjsph_geometry_create", lib().fjsph_geometry_create(C.byref(self.settings), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if self._h:
            lib().fjsph_geometry_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def log(self) -> str:
        n = C.c_int64()
        lib().fjsph_geometry_log(self._h, None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value + 1)
        lib().fjsph_geometry_log(self._h, buf, n.value + 1, C.byref(n))
        return buf.value.decode(errors="replace")

    def _check(self, fn: str, status: int) -> None:
        if status != d.OK:
            raise ValueError(f"{fn} failed ({status}):\n{self.log}")

    def read_text(self, text: str, fluid: bool) -> None:
        self._check("fjsph_geometry_read", lib().fjsph_geometry_read(self._h, text.encode(), int(fluid)))

    def read_file(self, path, fluid: bool) -> None:
        path = Path(path)
        if path.suffix.lower() == ".json":
            self.read_text(json_to_bmap(json.loads(path.read_text())), fluid)
        else:
            self._check("fjsph_geometry_read_file",
                        lib().fjsph_geometry_read_file(self._h, str(path).encode(), int(fluid)))

    def build(self) -> None:
        self._check("fjsph_geometry_build", lib().fjsph_geometry_build(self._h))

    def sizes(self) -> dict:
        n, nbp = C.c_int64(), C.c_int64()
        nbb, nfb, ni = C.c_int32(), C.c_int32(), C.c_int32()
        check("fjsph_geometry_sizes", lib().fjsph_geometry_sizes(self._h, C.byref(n), C.byref(nbp), C.byref(nbb),
                                                                 C.byref(nfb), C.byref(ni)))
        return {"n": n.value, "n_bound_points": nbp.value, "n_bound_blocks": nbb.value,
                "n_fluid_blocks": nfb.value, "n_inlets": ni.value}

    def state(self) -> SPHState:
        st = SPHState(self.sizes()["n"], self.dim)
        check("fjsph_geometry_state", lib().fjsph_geometry_state(self._h, C.byref(st.view())))
        return st

    def block_info(self) -> list[dict]:
        sz = self.sizes()
        out = []
        for k in range(sz["n_bound_blocks"] + sz["n_fluid_blocks"]):
            g = d.GeometryBlock()
            check("fjsph_geometry_block_info", lib().fjsph_geometry_block_info(self._h, k, C.byref(g)))
            info = {f: getattr(g, f) for f, _ in d.GeometryBlock._fields_}
            info["name"] = g.name.decode(errors="replace")
            for f in ("start", "end", "right", "centre", "normal"):
                info[f] = tuple(info[f][:self.dim])
            out.append(info)
        return out

    def blocks(self) -> list[BlockSpec]:
        sz = self.sizes()
        nb = sz["n_bound_blocks"] + sz["n_fluid_blocks"]
        arr = (d.Block * max(nb, 1))()
        check("fjsph_geometry_blocks", lib().fjsph_geometry_blocks(self._h, arr, nb))
        info = self.block_info()
        out = []
        for k in range(nb):
            b = arr[k]
            nt = b.n_times
            vels = [tuple(b.vels[t][:3]) for t in range(max(nt, 1))]
            out.append(BlockSpec(
                int(b.first), int(b.second), bool(b.is_fluid), name=info[k]["name"], bound_solver=b.bound_solver,
                no_slip=b.no_slip, block_type=b.block_type, fixed_vel_or_dynamic=b.fixed_vel_or_dynamic,
                times=[b.times[t] for t in range(nt)], vels=vels,
                delete_norm=tuple(b.delete_norm), delconst=b.delconst, insert_norm=tuple(b.insert_norm),
                insconst=b.insconst, aero_norm=tuple(b.aero_norm), aeroconst=b.aeroconst))
        return out

    def inlets(self) -> list[InletSpec]:
        out = []
        for k in range(self.sizes()["n_inlets"]):
            q = d.Inlet()
            check("fjsph_geometry_inlet", lib().fjsph_geometry_inlet(self._h, k, C.byref(q)))
            back = np.zeros(q.n_back, dtype=np.int64)
            buf = np.zeros((q.n_back, q.depth), dtype=np.int64)
            q.back = back.ctypes.data_as(C.POINTER(C.c_int64))
            q.buffer = buf.ctypes.data_as(C.POINTER(C.c_int64))
            check("fjsph_geometry_inlet", lib().fjsph_geometry_inlet(self._h, k, C.byref(q)))
            out.append(InletSpec(int(q.block), back, buf))
        return out


def build_particles(settings: d.Settings, boundary, fluid):
    """Init_Particles from two block files (paths, or bmap text when given as str with newlines):
    returns (state, blocks, inlets, geometry)."""
    g = Geometry(settings)
    for src, is_fluid in ((boundary, False), (fluid, True)):
        if isinstance(src, str) and "\n" in src:
            g.read_text(src, is_fluid)
        else:
            g.read_file(src, is_fluid)
    g.build()
    return g.state(), g.blocks(), g.inlets(), g


def load_case(para, dim: int, variant: int = 0, st_model: int = d.ST_PAIRWISE, name: str | None = None,
              tau_solution: str | None = None):
    """A reference case directory's starting point: settings from `para` and the particles of the
    fluid and boundary block files it names; for a 2D TAU mesh case also the air mesh (the
    solution file from the para's "Restart-data prefix", or `tau_solution`)."""
    from .cases import Case
    from .settings import read_para
    para = Path(para)
    s, extra = read_para(para, dim, variant=variant, st_model=st_model)
    root = para.parent
    bound_file = extra.get("input_bound_file")
    fluid_file = extra.get("input_fluid_file")
    if not bound_file or not fluid_file:
        raise ValueError("the para file names no fluid or boundary definition file")
    st, blocks, inlets, g = build_particles(s, root / bound_file, root / fluid_file)
    g.close()
    mesh = None
    if s.asource == d.MESH_INFL and extra.get("foam_dir"):
        from .foam import read_foam
        if dim != 3:
            raise ValueError("OpenFOAM meshes are read in 3D only (as upstream)")
        mesh = read_foam(root / extra["foam_dir"], extra.get("foam_sol", ""),
                         buoyant=str(extra.get("foam_buoyant", "0")).strip().startswith("1"), rho=s.rho_g,
                         scale=s.scale)
    elif s.asource == d.MESH_INFL and dim == 2:
        from .tau import read_tau_2d
        sol = tau_solution or extra.get("tau_sol")
        if not sol:
            raise ValueError("the para file names a TAU grid but no solution file")
        axis = int(str(extra.get("offset_axis", "2")).split()[0] or 2)
        mesh = read_tau_2d(root / extra["tau_mesh"], root / sol, offset_axis=axis, scale=s.scale)
    return Case(name or para.parent.name, s, st, blocks, inlets, mesh)
