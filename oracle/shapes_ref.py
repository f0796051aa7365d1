"""Pure-Python restatement of the reference's initial-particle generation (TEST INFRASTRUCTURE ONLY).

Follows src/shapes/shapes.cpp:400-600 (read_shapes_bmap, with src/IOFunctions.h's Get_* rules),
the check_input / generate_points pairs of src/shapes/{line,square,circle,arc,cylinder,inlet,
coordinates}.cpp, src/Init.cpp:61-233 (Check_Intersection, brute-force distances here) and
src/Init.cpp:268-494 (Init_Particles' layout and hydrostatic start), for small cases.  The
perturbation engine restates libstdc++'s std::default_random_engine (minstd_rand0: x <- 16807 x mod
2^31 - 1, seed 1) and generate_canonical<double, 53> (two draws: (x1 - 1) + (x2 - 1) r over r^2,
r = 2^31 - 2), pinned against the C++ library in tests/test_shapes.py.

Parity status: unpinned against the reference itself (it cannot be built here; its -ffast-math
-march=native build defines coordinates only to rounding).  Only tests/ import this module.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field

import numpy as np

DV = 9999999.0
EPS = 2.220446049250313e-16
PI = math.pi
BOUND, BUFFER, BACK, PIPE, FREE = 0, 2, 3, 4, 5
LINE, SQUARE, CIRCLE, CYLINDER, ARC, COORD, INLET, HOLLOW, SOLID = range(9)


class MinStd:
    """minstd_rand0 with libstdc++'s generate_canonical<double, 53> and uniform_real_distribution."""
    R = 2147483646.0

    def __init__(self, hi: float):
        self.x = 1
        self.hi = hi

    def _next(self) -> int:
        self.x = (16807 * self.x) % 2147483647
        return self.x

    def canonical(self) -> float:
        s = float(self._next() - 1)
        s = s + float(self._next() - 1) * self.R
        tmp = self.R * self.R
        ret = s / tmp
        return ret if ret < 1.0 else math.nextafter(1.0, 0.0)

    def __call__(self) -> float:
        return self.canonical() * (self.hi - 0.0) + 0.0


# ---- small vector helpers (tuples of length 3; 2D keeps z = 0) ----
def add(a, b): return (a[0] + b[0], a[1] + b[1], a[2] + b[2])
def sub(a, b): return (a[0] - b[0], a[1] - b[1], a[2] - b[2])
def mul(a, s): return (a[0] * s, a[1] * s, a[2] * s)
def div(a, s): return (a[0] / s, a[1] / s, a[2] / s)
def dot(a, b): return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]
def norm(a): return math.sqrt(dot(a, a))
def cross(a, b): return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def normalized(a):
    n = dot(a, a)
    return div(a, math.sqrt(n)) if n > 0 else a


def matvec(m, v):
    return tuple(m[i][0] * v[0] + m[i][1] * v[1] + m[i][2] * v[2] for i in range(3))


IDENT = ((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0))


def rotation(ang, D):
    """GetRotationMat (src/Geometry.h:14-43)."""
    if D == 2:
        c, s = math.cos(ang[0]), math.sin(ang[0])
        return ((c, -s, 0.0), (s, c, 0.0), (0.0, 0.0, 1.0))

    def q_axis(angle, k):
        h = 0.5 * angle
        q = [math.cos(h), 0.0, 0.0, 0.0]
        q[1 + k] = math.sin(h)
        return q

    def q_mul(a, b):
        return [a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3],
                a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2],
                a[0] * b[2] + a[2] * b[0] + a[3] * b[1] - a[1] * b[3],
                a[0] * b[3] + a[3] * b[0] + a[1] * b[2] - a[2] * b[1]]
    w, x, y, z = q_mul(q_mul(q_axis(ang[0], 0), q_axis(-ang[1], 1)), q_axis(ang[2], 2))
    tx, ty, tz = 2 * x, 2 * y, 2 * z
    twx, twy, twz = tx * w, ty * w, tz * w
    txx, txy, txz = tx * x, ty * x, tz * x
    tyy, tyz, tzz = ty * y, tz * y, tz * z
    return ((1 - (tyy + tzz), txy - twz, txz + twy), (txy + twz, 1 - (txx + tzz), tyz - twx),
            (txz - twy, tyz + twx, 1 - (txx + tyy)))


def is_ident(m, D):
    return all(m[i][j] == (1.0 if i == j else 0.0) for i in range(D) for j in range(D))


# ---- reading ----
def _value(line):
    return line[line.find(":") + 1:].strip(" \n\r\t\f\v")


def _key(line):
    p = line.find(":")
    return None if p < 0 else line[:p].lstrip(" \n\r\t\f\v")


_NUM = re.compile(r"[-+]?((\d+\.?\d*)|(\.\d+))([eE][-+]?\d+)?")


def _num(t):
    """istream >> double: the longest numeric prefix, 0 when there is none."""
    mm = _NUM.match(t.lstrip(" \n\r\t\f\v"))
    return float(mm.group(0)) if mm else 0.0


def _int(t):
    t = t.lstrip(" \n\r\t\f\v")
    n = 0
    while n < len(t) and (t[n].isdigit() or (n == 0 and t[n] in "+-")):
        n += 1
    try:
        return int(t[:n])
    except ValueError:
        return 0


@dataclass
class Block:
    D: int
    name: str = ""
    shape: str = ""
    subshape: str = ""
    filename: str = ""
    position_filename: str = ""
    solver_name: str = ""
    write_data: bool = False
    no_slip: bool = False
    particle_order: bool = False
    bound_type: int = -1
    sub_bound_type: int = -1
    fixed_vel_or_dynamic: int = 0
    inlet_bc_type: str = ""
    bound_solver: int = 1
    ni: int = 0
    nj: int = 0
    nk: int = 0
    npts: int = 0
    ntimes: int = 0
    insconst: float = DV
    delconst: float = DV
    aeroconst: float = DV
    dx: float = -1.0
    radius: float = -1.0
    arc_start: float = -1.0
    arc_end: float = -1.0
    arclength: float = DV
    thickness: float = -1.0
    length: float = -1.0
    sstraight: float = 0.0
    estraight: float = 0.0
    vmag: float = 0.0
    press: float = 0.0
    dens: float = 1000.0
    insert_norm: tuple = (1.0, 0.0, 0.0)
    delete_norm: tuple = (1.0, 0.0, 0.0)
    aero_norm: tuple = (1.0, 0.0, 0.0)
    normal: tuple = (1.0, 0.0, 0.0)
    angles: tuple = (0.0, 0.0, 0.0)
    rotmat: tuple = IDENT
    start: tuple = None
    end: tuple = None
    right: tuple = None
    mid: tuple = None
    centre: tuple = None
    vel: tuple = (0.0, 0.0, 0.0)
    back: list = field(default_factory=list)
    buffer: list = field(default_factory=list)
    bc: list = field(default_factory=list)
    intersect: list = field(default_factory=list)
    times: list = field(default_factory=list)
    pos: list = field(default_factory=list)
    vels: list = field(default_factory=list)
    coords: list = field(default_factory=list)

    def __post_init__(self):
        z = DV if self.D == 3 else 0.0
        for f in ("start", "end", "right", "mid", "centre"):
            setattr(self, f, (DV, DV, z))


SHAPES2 = {"Line": LINE, "Square": SQUARE, "Circle": CIRCLE, "Arc": ARC}
SHAPES3 = {"Plane": LINE, "Cube": SQUARE, "Sphere": CIRCLE, "Arch": ARC}
SHAPES = {"Cylinder": CYLINDER, "Inlet": INLET, "Coordinates": COORD}

_STR = {"Name": "name", "Shape": "shape", "Sub-shape": "subshape", "Boundary solver": "solver_name",
        "Coordinate filename": "filename", "Time data filename": "position_filename",
        "Fixed velocity or dynamic inlet BC": "inlet_bc_type"}
_BOOL = {"Write surface data (0/1)": "write_data", "Particle ordering (0=grid,1=HCP)": "particle_order",
         "Wall is no slip (0/1)": "no_slip"}
_INT = {"Fixed velocity or dynamic inlet BC (0/1)": "fixed_vel_or_dynamic", "i-direction count": "ni",
        "j-direction count": "nj", "k-direction count": "nk", "Wall radial particle count": "nk"}
_DBL = {"Aerodynamic entry plane constant": "aeroconst", "Deletion plane constant": "delconst",
        "Insertion plane constant": "insconst", "Pipe depth": "thickness", "Radius": "radius", "Length": "length",
        "Arc start (degree)": "arc_start", "Arc end (degree)": "arc_end", "Arc length (degree)": "arclength",
        "Starting straight length": "sstraight", "Ending straight length": "estraight",
        "Particle spacing": "dx", "Wall thickness": "thickness", "Starting jet velocity": "vmag",
        "Starting pressure": "press", "Starting density": "dens"}
_VEC = {"Aerodynamic entry normal": "aero_norm", "Deletion normal": "delete_norm",
        "Insertion normal": "insert_norm", "Normal vector": "normal", "Rotation angles": "angles",
        "Start coordinate": "start", "End coordinate": "end", "Right coordinate": "right",
        "Midpoint coordinate": "mid", "Centre coordinate": "centre", "Arch normal": "right",
        "Starting velocity": "vel"}


def read_bmap(text: str, D: int) -> list[Block]:
    lines = text.split("\n")
    blocks = []
    shape = ""
    for raw in lines:
        c = raw.find("#")
        line = raw[:c + 1] if c >= 0 else raw
        if _key(line) == "Shape":
            shape = _value(line)
        if "block end" in line:
            b = Block(D)
            table = SHAPES2 if D == 2 else SHAPES3
            b.bound_type = table.get(shape, SHAPES.get(shape, -1))
            if b.bound_type == -1:
                raise ValueError(f"unrecognised shape {shape!r}")
            blocks.append(b)
            shape = ""
    if not blocks:
        return blocks
    k, i = 0, 0
    while i < len(lines):
        raw = lines[i]
        i += 1
        c = raw.find("#")
        line = raw[:c] if c >= 0 else raw
        b = blocks[k]
        key = _key(line)
        if key in _STR:
            setattr(b, _STR[key], _value(line))
        elif key in _BOOL:
            setattr(b, _BOOL[key], _int(_value(line)) != 0)
        elif key in _INT:
            setattr(b, _INT[key], _int(_value(line)))
        elif key in _DBL:
            setattr(b, _DBL[key], _num(_value(line)))
        elif key == "Rotation angle":
            b.angles = (_num(_value(line)), b.angles[1], b.angles[2])
        elif key in _VEC:
            parts = _value(line).split(",")
            vals = list(getattr(b, _VEC[key]))
            for d in range(D):
                vals[d] = _num(parts[d]) if d < len(parts) else 0.0
            setattr(b, _VEC[key], tuple(vals))
        if "Coordinate data:" in line:
            i += 1  # the line after the key is skipped
            toks = " ".join(lines[i:]).split()
            n = int(toks[0])
            vals = [float(t) for t in toks[1:1 + n * D]]
            b.coords = [tuple(vals[p * D:(p + 1) * D]) + ((0.0,) if D == 2 else ()) for p in range(n)]
            b.npts = n
            used = 1 + n * D  # skip the lines the tokens came from
            cnt = 0
            while i < len(lines) and cnt < used:
                cnt += len(lines[i].split())
                i += 1
        if "Time position data" in line or "Time velocity data" in line:
            nt = _int(lines[i]); i += 1
            b.ntimes = nt
            b.times, rows = [], []
            for _ in range(nt):
                t = [float(x) for x in lines[i].split()]
                i += 1
                b.times.append(t[0])
                rows.append(tuple(t[1:1 + D]) + ((0.0,) if D == 2 else ()))
            if "Time position data" in line:
                b.pos = rows
            else:
                b.vels = rows
        if "block end" in line:
            k += 1
            if k == len(blocks):
                break
    return blocks


# ---- check_input ----
class Gen:
    def __init__(self, s):
        self.s = s
        self.D = s.dim
        self.gs = s.dx

    def cv(self, v):
        return all(v[k] != DV for k in range(self.D))

    def unit_x(self, v):
        return all(v[k] == (1.0 if k == 0 else 0.0) for k in range(self.D))

    def base(self, b):
        s = self.s
        if s.scale != 1.0:
            for f in ("start", "end", "right", "mid", "centre"):
                if self.cv(getattr(b, f)):
                    setattr(b, f, mul(getattr(b, f), s.scale))
            for f in ("aeroconst", "insconst", "delconst"):
                if getattr(b, f) != DV:
                    setattr(b, f, getattr(b, f) * s.scale)
        b.bound_solver = {"DBC": 0, "Pressure-Gradient": 1, "Ghost": 2}.get(b.solver_name, b.bound_solver)
        if b.inlet_bc_type:
            b.fixed_vel_or_dynamic = {"Fixed Velocity": 0, "Dynamic": 1}.get(b.inlet_bc_type, b.fixed_vel_or_dynamic)
        if b.press != 0:
            B = s.rho_rest * (s.speed_sound * s.speed_sound) / s.gam
            b.dens = math.pow(((b.press - s.press_pipe) / B + 1.0), s.gam) * s.rho_rest
        else:
            b.dens = s.rho_rest

    def post(self, b):
        self.gs = b.dx if b.dx > self.gs else self.gs
        b.npts = max(b.npts, 1)

    def check(self, b):
        self.base(b)
        getattr(self, {LINE: "c_line", SQUARE: "c_square", CIRCLE: "c_circle", CYLINDER: "c_cyl", ARC: "c_arc",
                       INLET: "c_inlet", COORD: "c_coord"}[b.bound_type])(b)
        self.post(b)

    def c_line(self, b):
        gs, D = self.gs, self.D
        if D == 2:
            if b.ni > 0 and b.dx < 0:
                b.dx = norm(sub(b.end, b.start)) / float(b.ni)
        elif b.ni > 0 and b.nj > 0:
            b.dx = min(norm(sub(b.right, b.start)) / float(b.ni), norm(sub(b.end, b.right)) / float(b.nj))
        if b.thickness >= 0 and b.nk < 0:
            b.nk = math.ceil(b.thickness / b.dx / math.sqrt(3.0) * 2.0) if b.particle_order else math.ceil(b.thickness / b.dx)
        b.nk = max(b.nk, 1)
        if b.ni > 0:
            if D == 3 and b.nj < 1:
                b.nj = max(math.ceil(norm(sub(b.end, b.right)) / gs), 1)
            b.npts = b.ni * b.nk * (b.nj if D == 3 else 1)
        elif D == 2:
            b.ni = max(math.ceil(norm(sub(b.end, b.start)) / gs), 1)
            b.npts = b.ni * b.nk
        else:
            b.ni = max(math.ceil(norm(sub(b.right, b.start)) / gs), 1)
            e = norm(sub(b.end, b.right))
            b.nj = max(math.ceil(e / gs / math.sqrt(3.0) * 2.0) if b.particle_order else math.ceil(e / gs), 1)
            b.npts = b.ni * b.nj * b.nk

    def counts(self, b, gs):
        D = self.D
        if b.particle_order:
            ni = math.ceil((b.end[0] - b.start[0]) / gs)
            nj = math.ceil((b.end[1] - b.start[1]) / gs / math.sqrt(3.0) * 2.0)
            nk = math.ceil((b.end[2] - b.start[2]) / gs / math.sqrt(6.0) * 3.0) if D == 3 else 1
        else:
            ni = math.ceil((b.end[0] - b.start[0]) / gs)
            nj = math.ceil((b.end[1] - b.start[1]) / gs)
            nk = math.ceil((b.end[2] - b.start[2]) / gs) if D == 3 else 1
        return max(ni, 1), max(nj, 1), max(nk, 1)

    def c_square(self, b):
        if b.ni > 0 and b.nj > 0 and (self.D == 2 or b.nk > 0) and b.dx < 0:
            dd = sub(b.end, b.start)
            di, dj = dd[0] / float(b.ni), dd[1] / float(b.nj)
            b.dx = min(di, dj) if self.D == 2 else min(di, min(dj, dd[1] / float(b.nk)))
        ni, nj, nk = self.counts(b, self.gs)
        b.ni, b.nj = ni, nj
        if self.D == 3:
            b.nk = nk
        b.npts = ni * nj * (nk if self.D == 3 else 1)

    def c_circle(self, b):
        D = self.D
        b.start = tuple(b.centre[k] - b.radius if k < D else 0.0 for k in range(3))
        b.end = tuple(b.centre[k] + b.radius if k < D else 0.0 for k in range(3))
        if b.dx < 0:
            b.dx = self.gs if b.ni < 0 else _fdiv(2.0 * b.radius, float(b.ni))
        ni, nj, nk = self.counts(b, self.gs)
        n = max(ni * nj * (nk if D == 3 else 1), 1)
        b.npts = math.ceil(float(n) * PI / (4.0 if D == 2 else 6.0))

    def _normal_branch(self, b, shift):
        b.normal = normalized(b.normal)
        if self.D == 2:
            b.angles = (math.atan2(b.normal[1], b.normal[0]) + shift, b.angles[1], b.angles[2])

    def _rotate_from_angles(self, b):
        b.angles = mul(b.angles, PI / 180.0)
        b.rotmat = rotation(b.angles, self.D)
        b.normal = matvec(b.rotmat, (1.0, 0.0, 0.0))

    def c_cyl(self, b):
        D, gs = self.D, self.gs
        cfg = 0

        def from_cr():
            st, en = list(b.centre), list(b.centre)
            st[1] -= b.radius
            en[1] += b.radius
            if D == 3:
                st[2] -= b.radius
                en[2] += b.radius
                rt = list(b.centre)
                rt[1] += b.radius
                rt[2] -= b.radius
                b.right = tuple(rt)
            b.start, b.end = tuple(st), tuple(en)

        def from_cre():
            v, u = sub(b.right, b.centre), sub(b.end, b.right)
            b.start = sub(sub(b.centre, v), u)
            b.right = add(b.start, mul(v, 2.0))
            b.end = add(b.right, mul(u, 2.0))
            b.radius = norm(v)
        if b.subshape == "Hollow":
            b.sub_bound_type = HOLLOW
            if self.cv(b.centre):
                if b.radius > 0:
                    cfg = 3
                    from_cr()
                elif D == 3 and self.cv(b.right) and self.cv(b.end):
                    cfg = 4
                    from_cre()
            elif self.cv(b.start) and self.cv(b.end) and (D == 2 or self.cv(b.right)):
                cfg = 1
                b.centre = mul(add(b.start, b.end), 0.5)
                v = sub(b.right, b.start)
                b.radius = 0.5 * norm(v)
                b.right = add(b.centre, mul(v, 0.5))
        elif b.subshape == "Solid":
            b.sub_bound_type = SOLID
            if self.cv(b.start) and self.cv(b.right) and self.cv(b.end):
                cfg = 1
                b.centre = mul(add(b.start, b.end), 0.5)
                b.radius = 0.5 * norm(sub(b.right, b.start))
            elif self.cv(b.centre):
                if b.radius > 0:
                    cfg = 3
                    from_cr()
                if self.cv(b.right) and self.cv(b.end):
                    cfg = 4
                    from_cre()
            elif self.cv(b.start) and b.ni > 0 and b.nj > 0:
                cfg = 2
        if cfg == 0:
            raise ValueError("cylinder geometry not defined")
        if norm(b.angles) != 0:
            self._rotate_from_angles(b)
        elif not self.unit_x(b.normal):
            self._normal_branch(b, 0.0)
        if cfg == 1:
            ab = normalized(sub(b.end, b.start))
            if D == 3:
                b.normal = normalized(cross(ab, normalized(sub(b.right, b.start))))
            else:
                a = math.atan2(ab[1], ab[0])
                b.angles = (a, b.angles[1], b.angles[2])
                b.normal = (math.cos(a), -math.sin(a), 0.0)
        if cfg == 2:
            c = list(b.start)
            b.radius = 0.5 * gs * b.ni
            c[1] += b.radius
            if D == 3:
                r = list(b.start)
                r[1] += gs * b.ni
                e = list(r)
                e[2] += gs * b.nj
                c[2] += b.radius
                b.right, b.end = tuple(r), tuple(e)
            else:
                e = list(b.start)
                e[1] += gs * b.ni
                b.end = tuple(e)
            b.centre = tuple(c)
            if not is_ident(b.rotmat, D):
                b.centre = add(matvec(b.rotmat, sub(b.centre, b.start)), b.start)
                b.end = add(matvec(b.rotmat, sub(b.end, b.start)), b.start)
                if D == 3:
                    b.right = add(matvec(b.rotmat, sub(b.right, b.start)), b.start)
        elif cfg in (3, 4) and not is_ident(b.rotmat, D):
            b.start = add(matvec(b.rotmat, sub(b.start, b.centre)), b.centre)
            b.end = add(matvec(b.rotmat, sub(b.end, b.centre)), b.centre)
            if D == 3:
                b.right = add(matvec(b.rotmat, sub(b.right, b.centre)), b.centre)
        b.dx = gs
        if b.sub_bound_type == HOLLOW:
            if b.thickness < 0:
                b.thickness = float(b.nk) * gs * (math.sqrt(3.0) * 2.0 if b.particle_order else 1.0)
            elif b.nk < 0:
                b.nk = max(math.ceil(b.thickness / (gs * math.sqrt(3.0) * 2.0)) if b.particle_order
                           else math.ceil(b.thickness / gs), 1)
            if D == 3:
                b.ni = max(math.ceil((2 * PI) / (gs / b.radius)), 1)
            b.nj = max(math.ceil(b.length / gs) + 1, 1)
            b.npts = b.nj * b.nk * (b.ni if D == 3 else 2)
        else:
            b.ni = max(math.ceil(2.0 * b.radius / gs), 1)
            b.nj = max(math.ceil(b.length / gs), 1)
            if D == 3:
                b.nk = math.ceil(2.0 * b.radius / gs)
            b.nk = max(b.nk, 1)
            b.npts = int(b.nj * b.nk * (PI / 4.0) * b.ni) * b.ni if D == 3 else b.ni * b.nj

    def c_arc(self, b):
        D, gs = self.D, self.gs
        cfg, arc_defined = 0, 0
        if D == 2 and self.cv(b.centre):
            if b.arc_start >= 0 and b.arc_end >= 0 and b.radius > 0:
                cfg = 1
            elif b.arc_start >= 0 and b.ni > 0 and b.radius > 0:
                cfg = 1
            elif b.arc_start >= 0 and b.arclength != DV and b.radius > 0:
                cfg, arc_defined = 1, 1
        if not cfg and self.cv(b.centre) and self.cv(b.start) and self.cv(b.end):
            cfg = 1
            self._centrepoint(b)
        if not cfg:
            if D == 3:
                if self.cv(b.centre) and self.cv(b.start) and self.cv(b.mid) and b.arclength != DV:
                    cfg, arc_defined = 1, 1
            elif self.cv(b.start) and self.cv(b.end) and self.cv(b.mid):
                cfg = 1
                self._midpoint(b)
        if not cfg and self.cv(b.centre) and self.cv(b.start) and b.arclength != DV and (D == 2 or self.cv(b.right)):
            cfg, arc_defined = 1, 1
        if not cfg:
            raise ValueError("arc geometry not defined")
        if b.dx < 0:
            b.dx = gs if b.ni < 0 else _fdiv(2.0 * b.radius, float(b.ni))
        if b.thickness >= 0 and b.nk < 0:
            b.nk = math.ceil(b.thickness / gs / math.sqrt(3.0) * 2.0) if b.particle_order else math.ceil(b.thickness / gs)
        dth = gs / b.radius
        if arc_defined:
            if D == 3:
                u = sub(b.start, b.centre)
                b.radius = norm(u)
                u = div(u, b.radius)
                w = normalized(b.right)
                v = normalized(cross(u, w))
                al = b.arclength * PI / 180.0
                b.end = add(mul(add(mul(u, math.cos(al)), mul(v, math.sin(al))), b.radius), b.centre)
        else:
            if b.arc_end < 0 and b.ni > 0:
                b.arc_end = 180.0 / PI * (b.arc_start * PI / 180 + float(b.ni) * dth)
            b.arclength = b.arc_end - b.arc_start
        ni = max(math.ceil((abs(b.arclength) * PI / 180) / dth), 1)
        smax = math.ceil(b.sstraight / gs) if b.sstraight > 0 else 0
        emax = math.ceil(b.estraight / gs) if b.estraight > 0 else 0
        b.npts = (ni + smax + emax) * b.nk
        if D == 3:
            if b.length >= 0 and b.nj < 0:
                b.nj = max(math.ceil(b.length / gs / math.sqrt(6.0) * 3.0) if b.particle_order else math.ceil(b.length / gs), 1)
            b.npts *= b.nj

    def _centrepoint(self, b):
        d0, d1 = sub(b.start, b.centre), sub(b.end, b.centre)
        r = dot(d0, d0)
        if abs(dot(d1, d1) - r) > 0.001:
            raise ValueError("arc radii differ")
        b.radius = math.sqrt(r)
        if self.D == 2:
            b.arc_start = math.atan2(d0[1], d0[0]) * 180 / PI
            b.arc_end = math.atan2(d1[1], d1[0]) * 180 / PI
            return
        d0, d1 = normalized(d0), normalized(d1)
        w = normalized(cross(d1, d0))
        v = normalized(cross(w, d0))
        mx = abs(d0[0]) + abs(v[0]); my = abs(d0[1]) + abs(v[1]); mz = abs(d0[2]) + abs(v[2])
        r0, r1 = 0, 1
        if mx < my and mx < mz:
            r0, r1 = 1, 2
        elif my < mx and my < mz:
            r0, r1 = 0, 2
        a, bb = _solve2(d0[r0], v[r0], d0[r1], v[r1], v[0], v[1])
        b.arc_start = math.atan2(1.0, 0.0) * 180 / PI
        b.arc_end = math.atan2(a, bb) * 180 / PI
        b.right = w

    def _midpoint(self, b):
        s, e, m = b.start, b.end, b.mid
        r1x, r1y, r2x, r2y, r3x, r3y = s[0] * s[0], s[1] * s[1], m[0] * m[0], m[1] * m[1], e[0] * e[0], e[1] * e[1]
        cx, cy = _solve2(2.0 * (s[0] - e[0]), 2.0 * (s[1] - e[1]), 2.0 * (s[0] - m[0]), 2.0 * (s[1] - m[1]),
                         r1x - r3x + r1y - r3y, r1x - r2x + r1y - r2y)
        b.centre = (cx, cy, 0.0)
        self._centrepoint(b)

    def c_inlet(self, b):
        D, gs = self.D, self.gs
        cfg = 0
        if D == 3:
            if b.subshape == "Square":
                b.sub_bound_type = SQUARE
                if self.cv(b.start) and self.cv(b.right) and self.cv(b.end):
                    cfg = 1
                if self.cv(b.start) and b.ni > 0 and b.nj > 0:
                    cfg = 2
            elif b.subshape == "Circle":
                b.sub_bound_type = CIRCLE
                if self.cv(b.centre):
                    if self.cv(b.right) and self.cv(b.end):
                        cfg = 4
                        v, u = sub(b.right, b.centre), sub(b.end, b.right)
                        b.start = sub(sub(b.centre, v), u)
                        b.right = add(b.start, mul(v, 2.0))
                        b.end = add(b.right, mul(u, 2.0))
                    if b.radius > 0:
                        cfg = 3
                        c, r = b.centre, b.radius
                        b.start = (c[0], c[1] - r, c[2] - r)
                        b.end = (c[0], c[1] + r, c[2] + r)
                        b.right = (c[0], c[1] + r, c[2] - r)
                elif self.cv(b.start) and self.cv(b.right) and self.cv(b.end):
                    cfg = 1
                    b.centre = mul(add(b.start, b.end), 0.5)
                    v = sub(b.right, b.start)
                    b.radius = 0.5 * norm(v)
                    b.right = add(b.centre, mul(v, 0.5))
        else:
            if self.cv(b.start) and self.cv(b.end):
                cfg = 1
                b.centre = mul(add(b.start, b.end), 0.5)
                b.radius = norm(sub(b.centre, b.start))
            elif self.cv(b.centre) and b.radius > 0:
                cfg = 3
                b.start = (b.centre[0], b.centre[1] - b.radius, 0.0)
                b.end = (b.centre[0], b.centre[1] + b.radius, 0.0)
        if cfg == 0:
            raise ValueError("inlet geometry not defined")
        b.dx = gs
        if norm(b.angles) != 0:
            self._rotate_from_angles(b)
            b.insert_norm = b.normal
        elif not self.unit_x(b.normal):
            self._normal_branch(b, 0.0)
            b.insert_norm = b.normal
        elif not self.unit_x(b.insert_norm):
            b.normal = b.insert_norm
            self._normal_branch(b, -PI / 2.0)
        if cfg == 1:
            ab = normalized(sub(b.end, b.start))
            if D == 3:
                b.normal = normalized(cross(ab, normalized(sub(b.right, b.start))))
            else:
                a = math.atan2(ab[1], ab[0])
                b.angles = (a, b.angles[1], b.angles[2])
                b.normal = (math.sin(a), math.cos(a), 0.0)
            b.insert_norm = b.normal
            b.insconst = dot(b.insert_norm, sub(b.start, mul(b.insert_norm, b.length - 0.01 * gs)))
        elif cfg == 2:
            if D == 3:
                r = list(b.start); r[1] += gs * b.ni
                e = list(r); e[2] += gs * b.nj
                b.right, b.end = tuple(r), tuple(e)
            else:
                e = list(b.start); e[1] += gs * b.ni
                b.end = tuple(e)
            if not is_ident(b.rotmat, D):
                b.end = add(matvec(b.rotmat, sub(b.end, b.start)), b.start)
                if D == 3:
                    b.right = add(matvec(b.rotmat, sub(b.right, b.start)), b.start)
        elif not is_ident(b.rotmat, D):
            b.start = add(matvec(b.rotmat, sub(b.start, b.centre)), b.centre)
            b.end = add(matvec(b.rotmat, sub(b.end, b.centre)), b.centre)
            if D == 3:
                b.right = add(matvec(b.rotmat, sub(b.right, b.centre)), b.centre)
        xl = norm(sub(b.right, b.start)) if D == 3 else norm(sub(b.end, b.start))
        b.ni = max(math.ceil(xl / gs), 1)
        if D == 3:
            b.nj = max(math.ceil(norm(sub(b.end, b.right)) / gs), 1)
        b.nk = max(math.ceil(b.length / gs), 1)
        if D == 3:
            if b.sub_bound_type == CIRCLE:
                if not self.cv(b.centre):
                    b.centre = mul(add(b.start, b.end), 0.5)
                if b.radius < 0:
                    b.radius = norm(sub(b.centre, b.start)) * math.cos(PI / 4.0)
                b.npts = int(b.ni * b.nj * (PI / 4.0) * (b.nk + 5))
            else:
                b.npts = b.ni * b.nj * (b.nk + 5)
        else:
            b.npts = b.ni * (b.nk + 4)
        if b.vmag != 0:
            b.vel = mul(b.insert_norm, b.vmag)

    def c_coord(self, b):
        if not b.filename:
            if not b.coords:
                raise ValueError("no coordinates")
            b.npts = len(b.coords)


def _fdiv(a, b):
    """IEEE a / b (a division by zero gives a signed infinity or NaN)"""
    if b != 0.0:
        return a / b
    if a == 0.0 or a != a:
        return math.nan
    return math.copysign(math.inf, a) * math.copysign(1.0, b)


def _solve2(m00, m01, m10, m11, v0, v1):
    if abs(m10) > abs(m00):
        m00, m10, m01, m11, v0, v1 = m10, m00, m11, m01, v1, v0
    f = m10 / m00
    a11, w1 = m11 - f * m01, v1 - f * v0
    x1 = w1 / a11
    return (v0 - m01 * x1) / m00, x1


# ---- generate_points ----
def _lattice(hcp, D, i, j, k):
    if D == 2:
        return mul((float(2 * i + (j % 2)), math.sqrt(3.0) * float(j), 0.0), 0.5) if hcp else (float(i), float(j), 0.0)
    if hcp:
        return mul((float(2 * i + ((j + k) % 2)), math.sqrt(3.0) * (float(j) + float(k % 2) / 3.0),
                    2.0 / 3.0 * math.sqrt(6.0) * float(k)), 0.5)
    return (float(i), float(j), float(k))


def _one(U, D):
    u = U()
    return (u, u, u if D == 3 else 0.0)


def _each(U, D):
    r = [0.0, 0.0, 0.0]
    for k in range(D):
        r[k] = U()
    return tuple(r)


def _rings(radius, gs, at):
    rad = radius
    while rad > 0.99 * gs:
        dth = math.atan(gs / rad)
        ncirc = math.floor(abs(2.0 * PI / dth))
        dth = 2.0 * PI / float(ncirc)
        th = 0.0
        while th < 2 * PI - 0.5 * dth:
            at(rad * math.sin(th), rad * math.cos(th))
            th += dth
        rad -= gs


def generate(g: Gen, b: Block):
    gs, D = g.s.dx, g.D
    U = MinStd(EPS * gs)
    out = b.coords
    if b.bound_type == LINE:
        s3, s6 = math.sqrt(3.0), math.sqrt(6.0)
        if D == 2:
            de = mul(normalized(sub(b.end, b.start)), gs)
            nm = (de[1], -de[0], 0.0)
            for ii in range(b.ni):
                for jj in range(b.nk):
                    if b.particle_order:
                        p = add(mul(de, float(ii + 0.5 * (jj % 2))), mul(mul(mul(nm, 0.5), s3), float(jj)))
                    else:
                        p = add(mul(de, float(ii)), mul(nm, float(jj)))
                    out.append(add(add(p, _one(U, 2)), b.start))
        else:
            di = mul(normalized(sub(b.right, b.start)), gs)
            dj = mul(normalized(sub(b.end, b.right)), gs)
            nm = mul(normalized(cross(dj, di)), gs)
            for jj in range(b.nj):
                for ii in range(b.ni):
                    for kk in range(b.nk):
                        if b.particle_order:
                            p = mul(add(add(mul(di, float(2 * ii + ((jj + kk) % 2))),
                                            mul(dj, s3 * (float(jj) + float(kk % 2) / 3))),
                                        mul(div(mul(mul(nm, 2.0), s6), 3.0), float(kk))), 0.5)
                        else:
                            p = add(add(mul(di, float(ii)), mul(dj, float(jj))), mul(nm, float(kk)))
                        out.append(add(add(p, _one(U, 3)), b.start))
    elif b.bound_type == SQUARE:
        for k in range(b.nk if D == 3 else 1):
            for j in range(b.nj):
                for i in range(b.ni):
                    p = mul(_lattice(b.particle_order, D, i, j, k), gs)
                    out.append(add(add(p, _one(U, D)), b.start))
    elif b.bound_type == CIRCLE:
        if D == 2:
            _rings(b.radius, gs, lambda x, y: out.append(add(matvec(b.rotmat, add((x, y, 0.0), _each(U, 2))), b.centre)))
            out.append(add(matvec(b.rotmat, _each(U, 2)), b.centre))
        else:
            ni, nj, nk = g.counts(b, gs)
            rsq = b.radius * b.radius
            for k in range(nk):
                for j in range(nj):
                    for i in range(ni):
                        p = matvec(b.rotmat, mul(_lattice(b.particle_order, 3, i, j, k), gs))
                        p = add(add(p, _each(U, 3)), b.start)
                        d = sub(p, b.centre)
                        if dot(d, d) > rsq:
                            continue
                        out.append(p)
    elif b.bound_type == CYLINDER and b.sub_bound_type == HOLLOW:
        if D == 2:
            nm = normalized(b.normal)
            left = (nm[1], -nm[0], 0.0)
            for sg in (1.0, -1.0):
                for ii in range(b.nj):
                    for kk in range(b.nk):
                        if b.particle_order:
                            p = mul(add(mul(nm, float(-ii + 0.5 * (kk % 2))), mul(mul(mul(left, 0.5), math.sqrt(3.0)), sg * float(kk))), gs)
                        else:
                            p = mul(add(mul(nm, float(-ii)), mul(left, sg * float(kk))), gs)
                        p = add(p, mul(left, sg * b.radius))
                        out.append(add(add(p, _each(U, 2)), b.centre))
        else:
            dth = 2 * PI / float(b.ni)
            for jj in range(b.nj):
                for kk in range(b.nk):
                    r, l, doff = b.radius, float(jj) * gs, 0.0
                    if b.particle_order:
                        r += 1.0 / 3.0 * math.sqrt(6.0) * float(kk) * gs
                        l = 0.5 * math.sqrt(3.0) * (float(jj) + float(kk % 2) / 3.0) * gs
                        doff = 0.5 * dth * ((kk + jj) % 2)
                    else:
                        r += float(kk) * gs
                    for ii in range(b.ni):
                        th = float(ii) * dth + (doff if b.particle_order else 0.0)
                        p = add((-l, math.cos(th) * r, math.sin(th) * r), _each(U, 3))
                        out.append(add(matvec(b.rotmat, p), b.centre))
    elif b.bound_type == ARC:
        _gen_arc(b, gs, D, U, out)
    elif b.bound_type == INLET:
        _gen_inlet(b, gs, D, U, out)


def _gen_arc(b, gs, D, U, out):
    if D == 2:
        th0, dth = b.arc_start * PI / 180.0, gs / b.radius
        ni = b.ni
        sv = (math.cos(th0), math.sin(th0), 0.0)
        sn = (sv[1], -sv[0], 0.0)
        smax = math.ceil(b.sstraight / gs)
        ev = (math.cos(th0 + float(ni - 1) * dth), math.sin(th0 + float(ni - 1) * dth), 0.0)
        en = (-ev[1], ev[0], 0.0)
        emax = math.ceil(b.estraight / gs)
        for jj in range(b.nk):
            if b.sstraight > 0:
                for ii in range(smax, 0, -1):
                    p = add(mul(sv, b.radius - float(jj) * gs), mul(sn, float(ii) * gs))
                    out.append(add(p, add(_each(U, 2), b.centre)))
            for ii in range(ni):
                th, r = th0 + float(ii) * dth, b.radius
                if b.particle_order:
                    th += 0.5 * dth * (jj % 2)
                    r -= 0.5 * math.sqrt(3.0) * float(jj) * gs
                else:
                    r -= float(jj) * gs
                out.append(add(add((math.cos(th) * r, math.sin(th) * r, 0.0), _each(U, 2)), b.centre))
            if b.estraight > 0:
                for ii in range(1, emax + 1):
                    p = add(mul(ev, b.radius - float(jj) * gs), mul(en, float(ii) * gs))
                    out.append(add(p, add(_each(U, 2), b.centre)))
        return
    dth = gs / b.radius
    nrad = math.ceil(b.arclength * PI / 180.0 / dth)
    u = normalized(sub(b.start, b.centre))
    w = normalized(b.right)
    v = normalized(cross(u, w))
    smax, emax = math.ceil(b.sstraight / gs), math.ceil(b.estraight / gs)
    ev = add(mul(u, math.cos(float(nrad - 1) * dth)), mul(v, math.sin(float(nrad - 1) * dth)))
    en = cross(ev, w)
    for kk in range(b.nj):
        for jj in range(b.nk):
            r, l, doff = b.radius, float(kk) * gs, 0.0
            if b.particle_order:
                r += 1.0 / 3.0 * math.sqrt(6.0) * float(jj) * gs
                l = 0.5 * math.sqrt(3.0) * (float(kk) + float(jj % 2) / 3.0) * gs
                doff = 0.5 * dth * ((jj + kk) % 2)
            else:
                r += float(jj) * gs
            if b.sstraight > 0:
                for ii in range(smax, 0, -1):
                    dist = float(ii) * gs + doff
                    p = add(sub(mul(u, r), mul(v, dist)), mul(w, l))
                    out.append(add(p, add(_each(U, 3), b.centre)))
            for ii in range(nrad):
                th = float(ii) * dth + (doff if b.particle_order else 0.0)
                p = add(add(mul(u, math.cos(th) * r), mul(v, math.sin(th) * r)), mul(w, float(kk) * gs))
                out.append(add(add(p, _each(U, 3)), b.centre))
            if b.estraight > 0:
                for ii in range(1, emax + 1):
                    dist = float(ii) * gs + doff
                    p = add(add(mul(ev, r), mul(en, dist)), mul(w, l))
                    out.append(add(p, add(_each(U, 3), b.centre)))


def _disk(b, dx, kk):
    U = MinStd(EPS * dx)
    pts = []
    if b.particle_order:
        x = -dx * kk
        _rings(b.radius, dx, lambda y, z: pts.append(add(matvec(b.rotmat, add((x, y, z), _each(U, 3))), b.centre)))
        pts.append(add(matvec(b.rotmat, add((x, 0.0, 0.0), _each(U, 3))), b.centre))
        return pts
    rsq = b.radius * b.radius
    for jj in range(b.nj):
        for ii in range(b.ni):
            p = mul((-float(kk), float(ii), float(jj)), dx)
            a, c = p[1] - b.radius, p[2] - b.radius
            if a * a + c * c > rsq:
                continue
            pts.append(add(matvec(b.rotmat, add(p, _each(U, 3))), b.start))
    return pts


def _gen_inlet(b, gs, D, U, out):
    def put(p, t):
        out.append(p)
        b.bc.append(t)
    if D == 2:
        de = div(sub(b.end, b.start), float(b.ni))
        nm = (de[1], -de[0], 0.0)

        def at(ii, jj):
            return add(add(add(mul(de, float(ii)), mul(nm, float(-jj))), _one(U, 2)), b.start)
        for jj in range(b.nk):
            for ii in range(b.ni):
                put(at(ii, jj), PIPE)
        for ii in range(b.ni):
            put(at(ii, b.nk), BACK)
            b.back.append(len(out) - 1)
        b.buffer = [[0] * 4 for _ in range(b.ni)]
        for buff, jj in enumerate(range(b.nk + 1, b.nk + 5)):
            for ii in range(b.ni):
                put(at(ii, jj), BUFFER)
                b.buffer[ii][buff] = len(out) - 1
        return
    if b.sub_bound_type == SQUARE:
        def at3(x, y, z):
            return add(matvec(b.rotmat, add(mul((float(x), float(y), float(z)), gs), _each(U, 3))), b.start)
        for kk in range(b.nk):
            for jj in range(b.nj):
                for ii in range(b.ni):
                    put(at3(-kk, ii, jj), PIPE)
        for jj in range(b.nj):
            for ii in range(b.ni):
                put(at3(-b.nk, jj, ii), BACK)
                b.back.append(len(out) - 1)
        b.buffer = [[0] * 4 for _ in b.back]
        for buff, kk in enumerate(range(b.nk + 1, b.nk + 5)):
            q = 0
            for jj in range(b.nj):
                for ii in range(b.ni):
                    put(at3(-kk, ii, jj), BUFFER)
                    b.buffer[q][buff] = len(out) - 1
                    q += 1
    elif b.sub_bound_type == CIRCLE:
        for kk in range(b.nk):
            for p in _disk(b, gs, kk):
                put(p, PIPE)
        for p in _disk(b, gs, b.nk):
            b.back.append(len(out))
            put(p, BACK)
        b.buffer = [[0] * 4 for _ in b.back]
        for buff, kk in enumerate(range(b.nk + 1, b.nk + 5)):
            for ii, p in enumerate(_disk(b, gs, kk)):
                b.buffer[ii][buff] = len(out)
                put(p, BUFFER)


# ---- Check_Intersection and Init_Particles ----
def _matches(pts, q, r2, D):
    """indices of pts (an (n, 3) array) with squared distance to q below r2, accumulated x, y[, z]"""
    if len(pts) == 0:
        return []
    d2 = np.zeros(len(pts))
    for k in range(D):
        dd = q[k] - pts[:, k]
        d2 = d2 + dd * dd
    return np.nonzero(d2 < r2)[0].tolist()


def intersect(g: Gen, bound, fluid):
    r2 = (0.9 * g.s.dx) * (0.9 * g.s.dx)
    D = g.D
    for b in bound + fluid:
        b.arr = np.array(b.coords, dtype=np.float64).reshape(-1, 3)
    for b in bound:
        b.intersect = [0] * len(b.coords)
    for i, bi in enumerate(bound):
        for bj in bound[i:]:
            for jj, q in enumerate(bj.coords):
                if bj.intersect[jj] == 0:
                    for m in _matches(bi.arr, q, r2, D):
                        if m != jj:
                            bi.intersect[m] = 1
    for f in fluid:
        f.intersect = [0] * len(f.coords)
    for i, fi in enumerate(fluid):
        for bj in bound:
            for jj, q in enumerate(bj.coords):
                if bj.intersect[jj] == 0:
                    for m in _matches(fi.arr, q, r2, D):
                        fi.intersect[m] = 1
        for fj in fluid[i + 1:]:
            for jj, q in enumerate(fj.coords):
                if fj.intersect[jj] == 0:
                    for m in _matches(fi.arr, q, r2, D):
                        fi.intersect[m] = 1
    for f in fluid:
        for k, bk in enumerate(f.back):
            if f.intersect[bk] or any(f.intersect[q] for q in f.buffer[k]):
                f.intersect[bk] = 1
                for q in f.buffer[k]:
                    f.intersect[q] = 1


def build(settings, bound_text: str, fluid_text: str):
    """Particles, block ranges and inlet tables of Init_Particles for two bmap texts:
    returns dict(xi, v, rho, p, m, b, limits=[(first, second, is_fluid)], inlets=[(back, buffer)],
    blocks=[Block])."""
    g = Gen(settings)
    D = g.D
    bound, fluid = read_bmap(bound_text, D), read_bmap(fluid_text, D)
    for b in bound + fluid:
        g.check(b)
    for b in bound + fluid:
        generate(g, b)
    intersect(g, bound, fluid)
    s = settings
    xi, v, rho, p, m, typ, limits, inlets = [], [], [], [], [], [], [], []

    def push(x, blk, mass, t):
        xi.append(x); v.append(blk.vel); rho.append(blk.dens); p.append(blk.press); m.append(mass); typ.append(t)
    for blk in bound:
        first = len(xi)
        for i, x in enumerate(blk.coords):
            if not blk.intersect[i]:
                push(x, blk, s.bnd_mass, BOUND)
        limits.append((first, len(xi), False))
    for blk in fluid:
        first = len(xi)
        if blk.bound_type == INLET:
            i = 0
            while i < len(blk.bc) and blk.bc[i] == PIPE:
                if not blk.intersect[i]:
                    push(blk.coords[i], blk, s.bnd_mass, PIPE)
                i += 1
            keep = [not blk.intersect[bk] for bk in blk.back]
            back, buf = [], []
            for k, bk in enumerate(blk.back):
                if keep[k]:
                    back.append(len(xi))
                    buf.append([0] * 4)
                    push(blk.coords[bk], blk, s.sim_mass, BACK)
            for layer in range(4):
                col = 0
                for k in range(len(blk.back)):
                    if keep[k]:
                        buf[col][layer] = len(xi)
                        push(blk.coords[blk.buffer[k][layer]], blk, s.sim_mass, BUFFER)
                        col += 1
            inlets.append((back, buf))
        else:
            for i, x in enumerate(blk.coords):
                if not blk.intersect[i]:
                    push(x, blk, s.sim_mass, FREE)
        limits.append((first, len(xi), True))
    if s.init_hydro_pressure:
        for i, x in enumerate(xi):
            pr = max(0.0, -s.rho_rest * s.grav[1] * (s.hydro_height - x[1]))
            p[i] = pr
            if s.pressure_rel == 1:
                rho[i] = (pr - s.press_back) / (s.speed_sound * s.speed_sound) + s.rho_rest
            else:
                rho[i] = s.rho_rest * math.pow(((pr - s.press_back) / s.B) + 1.0, 1.0 / s.gam)
    return {"xi": xi, "v": v, "rho": rho, "p": p, "m": m, "b": typ, "limits": limits, "inlets": inlets,
            "blocks": bound + fluid}
