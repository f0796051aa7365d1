"""Synthetic input states for the hot path.

These builders stand in for the reference's geometry files (src/shapes/*, src/Init.cpp); they
produce the particle layouts that the benchmark configurations describe:

  dam_break_2d   water column in a 2D tank, square lattice, hydrostatic density (config 0)
  dam_break_3d   3D dam break, jittered lattice, ALE (config 1); hydrostatic along z
  droplet_3d     spherical droplet in a uniform air stream, Gissler aero + pairwise surface
                 tension (the droplets of config 4)
  jet_crossflow  liquid column leaving a pipe into an analytic crossflow, broken into ligaments and
                 droplets downstream (configs 2-3); the air field is uniform v_inf, as the
                 reference's constant-velocity source supplies it

Boundary particles form `layers` rows outside the fluid region at the lattice spacing.  All
random numbers come from numpy's PCG64 with the given seed.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _cdefs as d
from .settings import defaults, derive
from .state import BlockSpec, InletSpec, SPHState


@dataclass
class Case:
    name: str
    settings: d.Settings
    state: SPHState
    blocks: list[BlockSpec]
    inlets: list[InletSpec] = field(default_factory=list)
    mesh: object = None  # the air mesh of a mesh-source case (fjsph_gb300.mesh.CellMesh)
    power_law_params: tuple = None  # (axis, wall, thickness, exponent) of an FJSPH_POWER_LAW case

    @property
    def n_fluid(self) -> int:
        return self.state.n - sum(b.second - b.first for b in self.blocks if not b.is_fluid)


def _eos_density(s: d.Settings, p: np.ndarray) -> np.ndarray:
    if s.pressure_rel == d.ISO_EOS:
        return (p - s.press_back) / (s.speed_sound ** 2) + s.rho_rest
    return s.rho_rest * np.power((p - s.press_back) / s.B + 1.0, 1.0 / s.gam)


def _assemble(s: d.Settings, bound: np.ndarray, fluid: np.ndarray, b_fluid: int = d.FREE):
    dim = s.dim
    nb, nf = len(bound), len(fluid)
    st = SPHState(nb + nf, dim)
    if nb:
        st.xi[:nb] = bound
    st.xi[nb:] = fluid
    st.m[:] = s.sim_mass
    st.rho[:] = s.rho_rest
    st.b[:nb] = d.BOUND
    st.b[nb:] = b_fluid
    st.cellRho[:] = s.rho_g
    st.cellP[:] = s.p_ref
    st.cellV[:] = np.asarray(s.v_inf[:dim])
    st.part_id[:] = np.arange(nb + nf)
    return st


def _blocks(nb: int, n: int, bound_solver: int = d.PRESSURE_G, no_slip: int = 0) -> list[BlockSpec]:
    out = []
    if nb:
        out.append(BlockSpec(0, nb, False, name="walls", bound_solver=bound_solver, no_slip=no_slip))
    out.append(BlockSpec(nb, n, True, name="fluid"))
    return out


def _hydrostatic(s: d.Settings, st: SPHState, axis: int, height: float) -> None:
    """Init_Particles' hydrostatic option (src/Init.cpp:480-493) along `axis`."""
    g = abs(s.grav[axis])
    p = np.maximum(0.0, s.rho_rest * g * (height - st.xi[:, axis]))
    st.p[:] = p
    st.rho[:] = _eos_density(s, p)


def dam_break_2d_settings(dx: float = 0.01, column_height: float = 2.0, solver: int = d.RUNGE_KUTTA,
                          cfl: float = 0.2) -> d.Settings:
    """Settings of config 0: Wendland C2 at H = 1.3 dx, Cole EOS (rho0 1000, gamma 7,
    c0 = 10 sqrt(2 g H_column)), delta-SPH 0.1, artificial viscosity 0.01, no surface tension,
    fixed CFL."""
    s = defaults(2)
    s.st_model = d.ST_NOST
    s.particle_step = dx
    s.H_fac = 1.3
    s.rho_rest = 1000.0
    s.gam = 7.0
    s.speed_sound = 10.0 * math.sqrt(2.0 * 9.81 * column_height)
    s.dsph_delta = 0.1
    s.visc_alpha = 0.01
    s.sig = 0.0
    s.grav[:] = [0.0, -9.81, 0.0]
    s.solver_type = solver
    s.cfl = s.cfl_min = s.cfl_max = cfl
    s.delta_t_min = 1e-9
    return derive(s)


def dam_break_2d(dx: float = 0.01, column=(1.0, 2.0), tank=(4.0, 3.0), layers: int = 3,
                 solver: int = d.RUNGE_KUTTA, cfl: float = 0.2) -> Case:
    """Config 0: 1.0 x 2.0 m column in a 4.0 x 3.0 m tank, dx = 0.01 (20,000 fluid particles)."""
    s = dam_break_2d_settings(dx, column[1], solver, cfl)
    nx, ny = int(round(column[0] / dx)), int(round(column[1] / dx))
    fx, fy = np.meshgrid((np.arange(nx) + 0.5) * dx, (np.arange(ny) + 0.5) * dx, indexing="ij")
    fluid = np.stack([fx.ravel(), fy.ravel()], axis=1)
    tx, ty = int(round(tank[0] / dx)), int(round(tank[1] / dx))
    walls = []
    for k in range(layers):
        xs = (np.arange(-layers, tx + layers) + 0.5) * dx
        walls.append(np.stack([xs, np.full_like(xs, -(k + 0.5) * dx)], axis=1))
    ys = (np.arange(ty) + 0.5) * dx
    for k in range(layers):
        walls.append(np.stack([np.full_like(ys, -(k + 0.5) * dx), ys], axis=1))
        walls.append(np.stack([np.full_like(ys, tank[0] + (k + 0.5) * dx), ys], axis=1))
    bound = np.concatenate(walls)
    st = _assemble(s, bound, fluid)
    _hydrostatic(s, st, 1, column[1])
    return Case("dam_break_2d", s, st, _blocks(len(bound), st.n))


def _line_wall(start, end, dx: float, layers: int) -> np.ndarray:
    """A Line block (src/shapes/line.cpp, grid ordering, 2D): ceil(|end - start| / dx) points
    along the line from start, `layers` rows offset along (dy, -dx) of the line direction."""
    start, end = np.asarray(start, float), np.asarray(end, float)
    delta = (end - start) / np.linalg.norm(end - start) * dx
    norm = np.array([delta[1], -delta[0]])
    ni = max(int(math.ceil(np.linalg.norm(end - start) / dx)), 1)
    ii, kk = np.meshgrid(np.arange(ni), np.arange(layers), indexing="ij")
    return start + ii.ravel()[:, None] * delta + kk.ravel()[:, None] * norm


def _square(start, end, dx: float) -> np.ndarray:
    """A Square block (src/shapes/square.cpp, grid ordering, 2D): ceil(extent / dx) points per
    axis from start, x fastest."""
    start, end = np.asarray(start, float), np.asarray(end, float)
    ni, nj = (max(int(math.ceil((end[k] - start[k]) / dx)), 1) for k in range(2))
    jj, ii = np.meshgrid(np.arange(nj), np.arange(ni), indexing="ij")
    return start + np.stack([ii.ravel(), jj.ravel()], axis=1) * dx


def standing_column_2d(dx: float = 0.02, width: float = 0.5, height: float = 1.0, layers: int = 4,
                       cfl: float = 1.0) -> Case:
    """Examples/Standing_Column's layout and settings at a coarser spacing: a water column at rest
    between Line walls (left, bottom, right; Pressure-Gradient), hydrostatic initial pressure
    (src/Init.cpp:480-493), smoothing length factor 2, artificial viscosity 0.1, no surface
    tension, the default Newmark-Beta integrator (src/Integration.h:52).  The reference compares
    p / (rho g H) against depth / H (Ideal.dat: the line through (0, 0) and (1, 1)).  The speed
    of sound is ten times the column's free-fall speed."""
    s = defaults(2)
    s.st_model = d.ST_NOST
    s.particle_step = dx
    s.H_fac = 2.0
    s.rho_rest = 1000.0
    s.mu = 8.94e-4
    s.gam = 7.0
    s.speed_sound = 10.0 * math.sqrt(2.0 * 9.81 * height)
    s.visc_alpha = 0.1
    s.sig = 0.0
    s.grav[:] = [0.0, -9.81, 0.0]
    s.solver_type = d.NEWMARK_BETA
    s.cfl = s.cfl_max = cfl
    s.cfl_min = 0.1 * cfl
    s.delta_t_min = 1e-9
    derive(s)
    top = height + 0.1
    walls = [_line_wall((0.0, top), (0.0, 0.0), dx, layers),             # left, layers towards -x
             _line_wall((-(layers - 1) * dx, 0.0), (width + (layers - 1) * dx, 0.0), dx, layers),  # bottom
             _line_wall((width + dx, 0.0), (width + dx, top), dx, layers)]  # right, layers towards +x
    fluid = _square((dx, dx), (width + 0.5 * dx, height), dx)
    bound = np.concatenate(walls)
    keep = np.ones(len(bound), bool)  # drop wall points that coincide (corner overlaps)
    _, first = np.unique(np.round(bound / (0.1 * dx)).astype(np.int64), axis=0, return_index=True)
    keep[:] = False
    keep[np.sort(first)] = True
    bound = bound[keep]
    st = _assemble(s, bound, fluid)
    _hydrostatic(s, st, 1, height + 0.5 * dx)
    return Case("standing_column_2d", s, st, _blocks(len(bound), st.n))


def couette_2d(dx: float = 0.02, length: float = 3.0, gap: float = 1.0, wall_speed: float = 1e-3,
               layers: int = 4, cfl: float = 1.0) -> Case:
    """Examples/Couette's layout: fluid between a fixed bottom wall and a top wall moving at
    wall_speed along x (Line blocks, Pressure-Gradient, no-slip off), rho = 1, mu = 0.01, c = 1,
    no gravity.  The steady profile is v_x = wall_speed * y / gap (SteadyState.dat)."""
    s = defaults(2)
    s.st_model = d.ST_NOST
    s.particle_step = dx
    s.H_fac = 2.0
    s.rho_rest = 1.0
    s.mu = 1e-2
    s.gam = 7.0
    s.speed_sound = 1.0
    s.visc_alpha = 0.01
    s.sig = 0.0
    s.rho_var = 20.0
    s.grav[:] = [0.0, 0.0, 0.0]
    s.solver_type = d.RUNGE_KUTTA
    s.cfl = s.cfl_min = s.cfl_max = cfl
    s.delta_t_min = 1e-9
    s.delta_t_max = 0.5
    derive(s)
    bottom = _line_wall((-0.18, 0.0), (length + 0.2, 0.0), dx, layers)
    top = _line_wall((length + 0.2, gap), (-0.2, gap), dx, layers)
    fluid = _square((0.0, dx), (length, gap), dx)
    bound = np.concatenate([bottom, top])
    st = _assemble(s, bound, fluid)
    nb0 = len(bottom)
    blocks = [BlockSpec(0, nb0, False, name="Bottom", bound_solver=d.PRESSURE_G),
              BlockSpec(nb0, len(bound), False, name="Top", bound_solver=d.PRESSURE_G,
                        vels=[(wall_speed, 0.0, 0.0)]),
              BlockSpec(len(bound), st.n, True, name="Fluid")]
    st.v[nb0:len(bound), 0] = wall_speed
    return Case("couette_2d", s, st, blocks)


def dam_break_3d_settings(dx: float = 0.003, column_height: float = 1.2, ale: bool = True,
                          solver: int = d.RUNGE_KUTTA, cfl: float = 0.2) -> d.Settings:
    """Settings of config 1: config 0's physics in 3D, with ALE shifting."""
    s = defaults(3)
    s.variant = d.VAR_ALE if ale else 0
    s.st_model = d.ST_NOST
    s.particle_step = dx
    s.H_fac = 1.3
    s.speed_sound = 10.0 * math.sqrt(2.0 * 9.81 * column_height)
    s.dsph_delta = 0.1
    s.visc_alpha = 0.01
    s.sig = 0.0
    s.grav[:] = [0.0, 0.0, -9.81]
    s.solver_type = solver
    s.cfl = s.cfl_min = s.cfl_max = cfl
    s.delta_t_min = 1e-9
    s.max_shift_vel = 5.0
    return derive(s)


def dam_break_3d(dx: float = 0.003, column=(0.6, 0.6, 1.2), tank=(1.6, 0.6, 1.2), layers: int = 3,
                 jitter: float = 0.01, seed: int = 12345, ale: bool = True, solver: int = d.RUNGE_KUTTA,
                 cfl: float = 0.2) -> Case:
    """Config 1: 0.6 x 0.6 x 1.2 m column in a 1.6 x 0.6 x 1.2 m tank (dx = 3 mm: 16M fluid)."""
    s = dam_break_3d_settings(dx, column[2], ale, solver, cfl)
    rng = np.random.Generator(np.random.PCG64(seed))
    n = [int(round(column[k] / dx)) for k in range(3)]
    g = np.meshgrid(*[(np.arange(n[k]) + 0.5) * dx for k in range(3)], indexing="ij")
    fluid = np.stack([a.ravel() for a in g], axis=1)
    fluid += rng.uniform(-jitter * dx, jitter * dx, size=fluid.shape)
    t = [int(round(tank[k] / dx)) for k in range(3)]
    walls = []
    # floor: z < 0, covering the tank footprint plus the side walls
    gx, gy = np.meshgrid((np.arange(-layers, t[0] + layers) + 0.5) * dx, (np.arange(-layers, t[1] + layers) + 0.5) * dx,
                         indexing="ij")
    for k in range(layers):
        walls.append(np.stack([gx.ravel(), gy.ravel(), np.full(gx.size, -(k + 0.5) * dx)], axis=1))
    zs = (np.arange(t[2]) + 0.5) * dx
    # x walls (full y extent incl. corners), y walls (tank x extent)
    ay, az = np.meshgrid((np.arange(-layers, t[1] + layers) + 0.5) * dx, zs, indexing="ij")
    for k in range(layers):
        walls.append(np.stack([np.full(ay.size, -(k + 0.5) * dx), ay.ravel(), az.ravel()], axis=1))
        walls.append(np.stack([np.full(ay.size, tank[0] + (k + 0.5) * dx), ay.ravel(), az.ravel()], axis=1))
    bx, bz = np.meshgrid((np.arange(t[0]) + 0.5) * dx, zs, indexing="ij")
    for k in range(layers):
        walls.append(np.stack([bx.ravel(), np.full(bx.size, -(k + 0.5) * dx), bz.ravel()], axis=1))
        walls.append(np.stack([bx.ravel(), np.full(bx.size, tank[1] + (k + 0.5) * dx), bz.ravel()], axis=1))
    bound = np.concatenate(walls)
    st = _assemble(s, bound, fluid)
    _hydrostatic(s, st, 2, column[2])
    return Case("dam_break_3d", s, st, _blocks(len(bound), st.n))


def _air(s: d.Settings, speed: float) -> None:
    s.acase = d.GISSLER
    s.v_inf[:] = [speed, 0.0, 0.0]
    s.rho_g = 1.225
    s.mu_g = 1.8e-5
    s.p_ref = 101325.0


def _liquid(s: d.Settings) -> None:
    s.rho_rest = 800.0
    s.mu = 1.5e-3
    s.sig = 0.025
    s.st_model = d.ST_PAIRWISE


def _sphere_points(diam: float, dx: float, centre=(0.0, 0.0, 0.0)) -> np.ndarray:
    r = 0.5 * diam
    m = int(math.ceil(r / dx)) + 1
    ax = np.arange(-m, m + 1) * dx
    g = np.meshgrid(ax, ax, ax, indexing="ij")
    pts = np.stack([a.ravel() for a in g], axis=1)
    pts = pts[np.einsum("ij,ij->i", pts, pts) <= r * r]
    return pts + np.asarray(centre)


def droplet_settings(dx: float = 5e-5, air_speed: float = 30.0, solver: int = d.RUNGE_KUTTA, cfl: float = 0.5,
                     ale: bool = False) -> d.Settings:
    """Settings of a config-4 droplet: the config-2 liquid and air, no gravity."""
    s = defaults(3)
    _liquid(s)
    _air(s, air_speed)
    s.variant = d.VAR_ALE if ale else 0
    s.particle_step = dx
    s.H_fac = 1.3
    s.speed_sound = 40.0
    s.visc_alpha = 0.05
    s.grav[:] = [0.0, 0.0, 0.0]
    s.solver_type = solver
    s.cfl = cfl
    s.cfl_min = 0.1
    s.cfl_max = cfl
    s.delta_t_min = 1e-12
    s.delta_t_max = 1e-5
    return derive(s)


def droplet_3d(diam: float = 1e-3, dx: float = 5e-5, air_speed: float = 30.0, seed: int = 7,
               solver: int = d.RUNGE_KUTTA, cfl: float = 0.5, ale: bool = False) -> Case:
    """A spherical droplet of the config-2 liquid in a uniform air stream (config 4 unit)."""
    s = droplet_settings(dx, air_speed, solver, cfl, ale)
    rng = np.random.Generator(np.random.PCG64(seed))
    pts = _sphere_points(diam, dx)
    pts += rng.uniform(-0.01 * dx, 0.01 * dx, size=pts.shape)
    st = _assemble(s, np.zeros((0, 3)), pts)
    return Case("droplet_3d", s, st, _blocks(0, st.n))


def jet_settings(dx: float = 5e-5, jet_speed: float = 10.0, air_speed: float = 50.0, ale: bool = False,
                 solver: int = d.RUNGE_KUTTA, max_points: int = 2_000_000) -> d.Settings:
    """Settings of config 2: the liquid (rho 800, mu 1.5e-3, sigma 0.025, pairwise surface
    tension), air at air_speed with the Gissler closure, c0 = 10 x the jet speed."""
    s = defaults(3)
    _liquid(s)
    _air(s, air_speed)
    s.variant = d.VAR_ALE if ale else 0
    s.particle_step = dx
    s.H_fac = 1.3
    s.speed_sound = 10.0 * jet_speed
    s.visc_alpha = 0.05
    s.grav[:] = [0.0, 0.0, -9.81]
    s.solver_type = solver
    s.cfl = 0.5
    s.cfl_min = 0.1
    s.cfl_max = 0.5
    s.delta_t_min = 1e-12
    s.delta_t_max = 1e-5
    s.max_points = max_points
    return derive(s)


def settings_for(config: int) -> d.Settings:
    """Settings of the five benchmark configurations: 0 the 2D dam break, 1 the 3D dam break with
    ALE, 2 the jet in crossflow, 3 the same jet in the FP32 form with the learned closure, 4 a
    droplet of the batched breakup sweep."""
    if config == 0:
        return dam_break_2d_settings()
    if config == 1:
        return dam_break_3d_settings()
    if config == 2:
        return jet_settings()
    if config == 3:
        s = jet_settings()
        s.precision = d.PREC_MIXED
        s.aero_closure = d.CLOSURE_LEARNED
        return s
    if config == 4:
        return droplet_settings()
    raise ValueError(f"no configuration {config}")


def jet_crossflow(n_target: int = 2_000_000, D: float = 2e-3, dx: float = 5e-5, jet_speed: float = 10.0,
                  air_speed: float = 50.0, seed: int = 2024, ale: bool = False, solver: int = d.RUNGE_KUTTA,
                  pipe_layers: int = 2) -> Case:
    """Config-2 liquid jet in crossflow, ~n_target particles.

    A ghost-walled pipe (diameter D) feeds a column that rises along +z and bends downstream along
    +x with the crossflow; past the bend the column is broken into ligaments and droplets of
    log-uniform diameter.  Liquid rho = 800, mu = 1.5e-3, sigma = 0.025; air 1.225 kg/m^3 moving at
    air_speed along +x.  Fluid particles carry the jet velocity plus the local crossflow drift.
    """
    s = jet_settings(dx, jet_speed, air_speed, ale, solver)
    rng = np.random.Generator(np.random.PCG64(seed))
    disk = _disk(0.5 * D, dx)
    # pipe walls: rings from R + dx/2 outward, z in [-4D, 0)
    pipe_len = 4.0 * D
    zs = (np.arange(int(pipe_len / dx)) + 0.5) * dx - pipe_len
    bound = _pipe_walls(0.5 * D, dx, zs, pipe_layers)
    parts, vels, types = [], [], []
    # liquid inside the pipe: PIPE particles
    for z in zs:
        parts.append(np.concatenate([disk, np.full((len(disk), 1), z)], axis=1))
        vels.append(np.tile([0.0, 0.0, jet_speed], (len(disk), 1)))
        types.append(np.full(len(disk), d.PIPE))
    n_now = sum(len(p) for p in parts)
    col, colv, drops, dropv = _jet_free_parts(disk, D, dx, jet_speed, air_speed, n_target - n_now, rng)
    parts += [col, drops]
    vels += [colv, dropv]
    types += [np.full(len(col), d.FREE), np.full(len(drops), d.FREE)]
    fluid = np.concatenate(parts)
    v = np.concatenate(vels)
    b = np.concatenate(types)
    fluid += rng.uniform(-0.01 * dx, 0.01 * dx, size=fluid.shape)
    st = _assemble(s, bound, fluid)
    st.v[len(bound):] = v
    st.b[len(bound):] = b
    blocks = _blocks(len(bound), st.n, bound_solver=d.GHOST)
    fl = blocks[-1]
    fl.aero_norm = (0.0, 0.0, 1.0)
    fl.aeroconst = 0.0
    return Case("jet_crossflow", s, st, blocks)


def _disk(R: float, dx: float) -> np.ndarray:
    """Lattice points of spacing dx inside a disk of radius R (the pipe's cross-section)."""
    m = int(math.ceil(R / dx)) + 1
    ax = np.arange(-m, m + 1) * dx
    gx, gy = np.meshgrid(ax, ax, indexing="ij")
    disk = np.stack([gx.ravel(), gy.ravel()], axis=1)
    return disk[np.einsum("ij,ij->i", disk, disk) <= R * R]


def _pipe_walls(R: float, dx: float, zs: np.ndarray, layers: int) -> np.ndarray:
    """Ghost-wall rings of a pipe along z: `layers` rings from R + dx/2 outward at every z."""
    wall = []
    for k in range(layers):
        rr = R + (k + 0.5) * dx
        nth = int(round(2 * math.pi * rr / dx))
        th = np.arange(nth) * 2 * math.pi / nth
        ring = np.stack([rr * np.cos(th), rr * np.sin(th)], axis=1)
        for z in zs:
            wall.append(np.concatenate([ring, np.full((nth, 1), z)], axis=1))
    return np.concatenate(wall)


def _jet_free_parts(disk: np.ndarray, D: float, dx: float, jet_speed: float, air_speed: float, n_free: int,
                    rng) -> tuple:
    """The emitted jet above the pipe exit: an intact column whose centreline bends from +z to +x
    over a quarter circle of radius 5D, then droplets of log-uniform diameter (6 dx .. 0.9 D)
    downstream of the bend, x in [5.5D, 20D], |y| < 4D, z in [3D, 9D], kept 2 dx apart, until
    about n_free particles.  Returns (column points, their velocities, droplet points, velocities);
    the column is ordered from the exit outward."""
    Rb = 5.0 * D
    arc = 0.5 * math.pi * Rb
    nlay = int(arc / dx)
    col, colv = [], []
    for k in range(nlay):
        phi = (k * dx) / Rb
        c = np.array([Rb * (1 - math.cos(phi)), 0.0, Rb * math.sin(phi)])
        t = np.array([math.sin(phi), 0.0, math.cos(phi)])
        e1 = np.array([math.cos(phi), 0.0, -math.sin(phi)])
        e2 = np.array([0.0, 1.0, 0.0])
        pts = c + disk[:, :1] * e1 + disk[:, 1:2] * e2
        col.append(pts)
        colv.append(np.tile(jet_speed * t + np.array([0.2 * air_speed * math.sin(phi), 0.0, 0.0]), (len(pts), 1)))
    n_now = sum(len(p) for p in col)
    lo = np.array([Rb + 0.5 * D - D, -5 * D, 2 * D])
    hi = np.array([21 * D, 5 * D, 10 * D])
    shape = tuple(np.ceil((hi - lo) / dx).astype(int) + 1)
    occ = np.zeros(shape, dtype=bool)
    tries = 0
    drops, dropv = [], []
    while n_now < n_free and tries < 200000:
        tries += 1
        dd = math.exp(rng.uniform(math.log(6 * dx), math.log(0.9 * D)))
        centre = np.array([rng.uniform(Rb + 0.5 * D, 20 * D), rng.uniform(-4 * D, 4 * D), rng.uniform(3 * D, 9 * D)])
        pts = _sphere_points(dd, dx, centre)
        if len(pts) == 0:
            continue
        gi = np.floor((pts - lo) / dx).astype(np.int64)
        if np.any(occ[gi[:, 0], gi[:, 1], gi[:, 2]]):
            continue
        for ox in (-2, -1, 0, 1, 2):
            for oy in (-2, -1, 0, 1, 2):
                for oz in (-2, -1, 0, 1, 2):
                    g2 = gi + np.array([ox, oy, oz])
                    g2 = np.clip(g2, 0, np.array(shape) - 1)
                    occ[g2[:, 0], g2[:, 1], g2[:, 2]] = True
        drops.append(pts)
        drift = 0.5 * air_speed * (centre[0] - Rb) / (20 * D - Rb)
        dropv.append(np.tile([jet_speed * 0.3 + drift, 0.0, 0.2 * jet_speed], (len(pts), 1)))
        n_now += len(pts)
    cat = lambda a, w: np.concatenate(a) if a else np.zeros((0, w))
    return cat(col, 3), cat(colv, 3), cat(drops, 3), cat(dropv, 3)


BL_THICKNESS = 5e-3  # boundary-layer thickness of the config-2 crossflow (m)


def jet_crossflow_live(n_target: int = 2_000_000, D: float = 2e-3, dx: float = 5e-5, jet_speed: float = 10.0,
                       air_speed: float = 50.0, seed: int = 2024, cap: int = 2_000_000, headroom: int = 50_000,
                       pipe_layers: int = 80, depth: int = 4, solver: int = d.RUNGE_KUTTA) -> Case:
    """Config 2 as specified: the jet in crossflow fed by a live inlet.

    One fluid block of type inletZone (src/shapes/inlet.cpp): a pipe of diameter D along +z with
    ghost walls, `depth` BUFFER layers below the BACK layer at z_b = -pipe_layers dx, PIPE layers
    up to the exit at z = 0, and above it the jet already emitted (the bent column and droplets of
    jet_crossflow), about n_target - headroom particles in all.  The insertion plane lies 0.02 dx
    above BACK, so every column inserts a BUFFER particle whenever its BACK particle crosses it;
    particles crossing x = 20.5 D (the downstream end of the 20D x 20D x 10D domain) are deleted;
    insertions stop at `cap` particles (max_points; raised to the start's count + headroom when the
    emitted column alone exceeds it).  The air is the analytic crossflow: 50 m/s
    along +x with a 1/7-power-law boundary layer of thickness 5 mm over the wall z = 0 (settings
    asource FJSPH_POWER_LAW; apply with Context.air_power_law(*power_law_params)).  Fluid order is by
    age as insertion produces it (the reference's table bookkeeping depends on it): droplets, the
    column from its far end, the PIPE layers from the top, BACK, the BUFFER layers.
    """
    s = jet_settings(dx, jet_speed, air_speed, False, solver, max_points=cap)
    s.asource = d.POWER_LAW
    rng = np.random.Generator(np.random.PCG64(seed))
    R = 0.5 * D
    disk = _disk(R, dx)
    nd = len(disk)
    z_b = -pipe_layers * dx
    zs = z_b - depth * dx + np.arange(pipe_layers + depth + 1) * dx
    bound = _pipe_walls(R, dx, zs, 2)

    def layer(z):
        return np.concatenate([disk, np.full((nd, 1), z)], axis=1)

    n_inlet = (pipe_layers + depth) * nd
    col, colv, drops, dropv = _jet_free_parts(disk, D, dx, jet_speed, air_speed,
                                              n_target - headroom - n_inlet - len(bound), rng)
    # oldest first: droplets furthest downstream first, then the column from its far end
    order = np.argsort(-drops[:, 0], kind="stable") if len(drops) else np.zeros(0, dtype=np.int64)
    drops, dropv = drops[order], dropv[order]
    col, colv = col[::-1], colv[::-1]
    parts = [drops, col]
    vels = [dropv, colv]
    types = [np.full(len(drops), d.FREE), np.full(len(col), d.FREE)]
    for k in reversed(range(1, pipe_layers)):
        parts.append(layer(z_b + k * dx))
        vels.append(np.tile([0.0, 0.0, jet_speed], (nd, 1)))
        types.append(np.full(nd, d.PIPE))
    parts.append(layer(z_b))
    vels.append(np.tile([0.0, 0.0, jet_speed], (nd, 1)))
    types.append(np.full(nd, d.BACK))
    for j in range(depth):  # buffer layer j is (j + 1) dx below BACK
        parts.append(layer(z_b - (j + 1) * dx))
        vels.append(np.tile([0.0, 0.0, jet_speed], (nd, 1)))
        types.append(np.full(nd, d.BUFFER))
    fluid = np.concatenate(parts)
    fluid[:, :2] += rng.uniform(-0.01 * dx, 0.01 * dx, size=(len(fluid), 2))
    st = _assemble(s, bound, fluid)
    nb = len(bound)
    st.v[nb:] = np.concatenate(vels)
    st.b[nb:] = np.concatenate(types)
    s.max_points = max(cap, st.n + headroom)  # the emitted column alone may exceed a small cap
    blocks = _blocks(nb, st.n, bound_solver=d.GHOST)
    fl = blocks[-1]
    fl.block_type = 6  # inletZone
    fl.insert_norm = (0.0, 0.0, 1.0)
    fl.insconst = z_b + 0.02 * dx
    fl.delete_norm = (1.0, 0.0, 0.0)
    fl.delconst = 20.5 * D
    fl.aero_norm = (0.0, 0.0, 1.0)
    fl.aeroconst = 0.0
    first_back = nb + len(drops) + len(col) + (pipe_layers - 1) * nd
    back = first_back + np.arange(nd)
    buffer = np.stack([first_back + (j + 1) * nd + np.arange(nd) for j in range(depth)], axis=1)
    c = Case("jet_crossflow_live", s, st, blocks, [InletSpec(len(blocks) - 1, back, buffer)])
    c.power_law_params = (2, 0.0, BL_THICKNESS, 1.0 / 7.0)
    return c


def jet_inlet(D: float = 1e-3, dx: float = 5e-5, jet_speed: float = 10.0, air_speed: float = 50.0,
              pipe_layers: int = 30, column_layers: int = 40, depth: int = 4, seed: int = 77,
              max_points: int | None = None, solver: int = d.RUNGE_KUTTA) -> Case:
    """A live inlet feeding a straight jet (the insertion and deletion paths of config 2).

    One fluid block of type inletZone (src/shapes/inlet.cpp): per disk column, `depth` BUFFER
    layers below one BACK layer at z_b, PIPE layers above it inside ghost-walled pipe walls, and
    a FREE column above the pipe exit at z = 0.  The insertion plane sits 0.02 dx above the BACK
    layer, so every column advances in the first step and a new BUFFER particle is inserted one
    dx upstream of each column's last; the deletion plane sits half a dx below the column top, so
    the top layer is deleted at the first update.  max_points caps the insertions.
    """
    s = defaults(3)
    _liquid(s)
    _air(s, air_speed)
    s.particle_step = dx
    s.H_fac = 1.3
    s.speed_sound = 10.0 * jet_speed
    s.visc_alpha = 0.05
    s.grav[:] = [0.0, 0.0, -9.81]
    s.solver_type = solver
    s.cfl = 0.5
    s.cfl_min = 0.1
    s.cfl_max = 0.5
    s.delta_t_min = 1e-12
    s.delta_t_max = 1e-5
    derive(s)
    rng = np.random.Generator(np.random.PCG64(seed))
    R = 0.5 * D
    m = int(math.ceil(R / dx)) + 1
    ax = np.arange(-m, m + 1) * dx
    gx, gy = np.meshgrid(ax, ax, indexing="ij")
    disk = np.stack([gx.ravel(), gy.ravel()], axis=1)
    disk = disk[np.einsum("ij,ij->i", disk, disk) <= R * R]
    nd = len(disk)
    z_b = -pipe_layers * dx
    # pipe walls (two ghost rings) from below the deepest buffer layer to the pipe exit
    zs = z_b - depth * dx + np.arange(pipe_layers + depth + 1) * dx
    wall = []
    for k in range(2):
        rr = R + (k + 0.5) * dx
        nth = int(round(2 * math.pi * rr / dx))
        th = np.arange(nth) * 2 * math.pi / nth
        ring = np.stack([rr * np.cos(th), rr * np.sin(th)], axis=1)
        for z in zs:
            wall.append(np.concatenate([ring, np.full((nth, 1), z)], axis=1))
    bound = np.concatenate(wall)

    def layer(z):
        return np.concatenate([disk, np.full((nd, 1), z)], axis=1)

    # fluid order by age, as insertion produces it: downstream (oldest) first -- the FREE column
    # from the top, the PIPE layers, BACK, then the BUFFER layers (newest last).  The reference's
    # bookkeeping relies on it: deletion shifts the inlet tables by every deletion in the block.
    parts, types = [], []
    for k in reversed(range(column_layers)):
        parts.append(layer(k * dx))
        types.append(np.full(nd, d.FREE))
    for k in reversed(range(1, pipe_layers)):
        parts.append(layer(z_b + k * dx))
        types.append(np.full(nd, d.PIPE))
    parts.append(layer(z_b))
    types.append(np.full(nd, d.BACK))
    for j in range(depth):  # buffer layer j is (j + 1) dx below BACK
        parts.append(layer(z_b - (j + 1) * dx))
        types.append(np.full(nd, d.BUFFER))
    fluid = np.concatenate(parts)
    fluid[:, :2] += rng.uniform(-0.01 * dx, 0.01 * dx, size=(len(fluid), 2))
    st = _assemble(s, bound, fluid)
    nb = len(bound)
    st.b[nb:] = np.concatenate(types)
    st.v[nb:] = [0.0, 0.0, jet_speed]
    free = st.b == d.FREE
    st.v[free, 0] = 0.05 * air_speed
    s.max_points = max_points if max_points is not None else st.n + 4 * nd
    blocks = _blocks(nb, st.n, bound_solver=d.GHOST)
    fl = blocks[-1]
    fl.block_type = 6  # inletZone
    fl.insert_norm = (0.0, 0.0, 1.0)
    fl.insconst = z_b + 0.02 * dx
    fl.delete_norm = (0.0, 0.0, 1.0)
    fl.delconst = (column_layers - 1) * dx - 0.5 * dx
    fl.aero_norm = (0.0, 0.0, 1.0)
    fl.aeroconst = 0.0
    # columns: BACK index and buffer indices, buffer[ii][0] the layer next to BACK
    first_back = nb + (column_layers + pipe_layers - 1) * nd
    back = first_back + np.arange(nd)
    buffer = np.stack([first_back + (j + 1) * nd + np.arange(nd) for j in range(depth)], axis=1)
    return Case("jet_inlet", s, st, blocks, [InletSpec(len(blocks) - 1, back, buffer)])


@dataclass
class DropletBatch:
    """Independent droplets in one state: droplet g is reference indices first[g]..first[g+1]-1
    with free-stream velocity v_inf[g]."""

    case: Case
    first: np.ndarray
    v_inf: np.ndarray
    counts: np.ndarray
    diam: np.ndarray
    we: np.ndarray

    def subset(self, ids) -> "DropletBatch":
        """The droplets `ids` (in that order) as a batch of their own."""
        ids = np.asarray(ids, dtype=np.int64)
        idx = np.concatenate([np.arange(self.first[g], self.first[g + 1]) for g in ids]) if len(ids) else \
            np.zeros(0, dtype=np.int64)
        st = self.case.state.take(idx)
        st.part_id[:] = np.arange(st.n)
        first = np.concatenate([[0], np.cumsum(self.counts[ids])]).astype(np.int64)
        s = self.case.settings.copy()
        s.max_points = st.n
        return DropletBatch(Case(self.case.name, s, st, _blocks(0, st.n)), first, self.v_inf[ids].copy(),
                            self.counts[ids].copy(), self.diam[ids].copy(), self.we[ids].copy())

    def single(self, g: int) -> Case:
        """Droplet g alone, as its own case (same settings, its own free stream)."""
        s = self.case.settings.copy()
        s.v_inf[:] = list(self.v_inf[g])
        st = self.case.state.take(np.arange(self.first[g], self.first[g + 1]))
        st.part_id[:] = np.arange(st.n)
        return Case(f"droplet_{g}", s, st, _blocks(0, st.n))


def droplet_batch(n_drops: int = 256, n_min: int = 2000, n_max: int = 60000, dx: float = 5e-5,
                  we_range=(10.0, 500.0), seed: int = 4242, cfl: float = 0.5) -> DropletBatch:
    """Config-4 batch: n_drops spherical droplets of the config-2 liquid, particle counts
    log-uniform in [n_min, n_max] (diameter from the count at spacing dx), each in its own air
    stream along +x with speed set by a Weber number drawn from we_range (We = rho_air U^2 d / sigma).
    Droplets sit on a cubic grid with gaps of 8 smoothing lengths, so no two interact."""
    base = droplet_3d(diam=4 * dx, dx=dx, cfl=cfl)
    s = base.settings
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_drops)).astype(np.int64)
    diam = dx * np.cbrt(6.0 * counts / math.pi)
    we = rng.uniform(we_range[0], we_range[1], n_drops)
    speed = np.sqrt(we * s.sig / (s.rho_g * diam))
    pitch = diam.max() + 8.0 * s.H + 2 * dx
    side = int(math.ceil(n_drops ** (1.0 / 3.0)))
    parts, first, vinf = [], [0], []
    for g in range(n_drops):
        ix, iy, iz = g % side, (g // side) % side, g // (side * side)
        centre = np.array([ix, iy, iz], dtype=np.float64) * pitch
        pts = _sphere_points(diam[g], dx, centre)
        pts += rng.uniform(-0.01 * dx, 0.01 * dx, size=pts.shape)
        parts.append(pts)
        first.append(first[-1] + len(pts))
        vinf.append([speed[g], 0.0, 0.0])
    st = _assemble(s, np.zeros((0, 3)), np.concatenate(parts))
    vinf = np.array(vinf)
    first = np.array(first, dtype=np.int64)
    for g in range(n_drops):
        st.cellV[first[g]:first[g + 1]] = vinf[g]
    s.max_points = st.n
    case = Case("droplet_batch", s, st, _blocks(0, st.n))
    return DropletBatch(case, first, vinf, np.diff(first), diam, we)


def shard_ids(n_drops: int, counts, rank: int, world: int) -> np.ndarray:
    """Droplets of one rank when a batch is split over `world` GPUs with no exchange between them:
    greedy balance of particle counts (largest droplet to the least-loaded rank, ties to the lower
    rank), identical on every rank."""
    counts = np.asarray(counts)
    order = np.argsort(-counts, kind="stable")
    load = np.zeros(world, dtype=np.int64)
    owner = np.empty(n_drops, dtype=np.int64)
    for g in order:
        r = int(np.argmin(load))
        owner[g] = r
        load[r] += counts[g]
    return np.flatnonzero(owner == rank)


def droplet_in_mesh(dim: int = 2, diam: float = 1.2e-3, dx: float = 1e-4, air_speed: float = 30.0, seed: int = 11):
    """A droplet of the config-2 liquid inside a CFD mesh whose cells carry a seeded air solution
    (the mesh-cell air source, Gissler aero): 2D, a quad mesh with a square hole (inner boundary)
    downstream of the drop; 3D, a box of tetrahedra.  Returns (case, mesh)."""
    from .mesh import quad_mesh_2d, tet_mesh_3d
    s = defaults(dim)
    _liquid(s)
    _air(s, air_speed)
    s.asource = d.MESH_INFL
    s.particle_step = dx
    s.H_fac = 1.3
    s.speed_sound = 40.0
    s.visc_alpha = 0.05
    s.grav[:] = [0.0, 0.0, 0.0]
    s.solver_type = d.RUNGE_KUTTA
    s.cfl = s.cfl_max = 0.5
    s.cfl_min = 0.1
    s.delta_t_min = 1e-12
    s.delta_t_max = 1e-5
    derive(s)
    rng = np.random.Generator(np.random.PCG64(seed))
    if dim == 2:
        r = 0.5 * diam
        g = np.arange(-r, r + 1e-12, dx)
        gx, gy = np.meshgrid(g, g, indexing="ij")
        pts = np.stack([gx.ravel(), gy.ravel()], axis=1)
        pts = pts[np.sum(pts ** 2, axis=1) <= r * r]
        mesh = quad_mesh_2d(lo=(-2e-3, -2e-3), hi=(6e-3, 3e-3), n=(56, 35), hole=((3.5e-3, -0.6e-3), (4.6e-3, 0.6e-3)),
                            u0=air_speed, seed=seed)
    else:
        pts = _sphere_points(diam, dx)
        mesh = tet_mesh_3d(lo=(-1.5e-3, -1.5e-3, -1.5e-3), hi=(2.5e-3, 1.5e-3, 1.5e-3), n=(12, 9, 9), u0=air_speed,
                           seed=seed)
    pts = pts + rng.uniform(-0.01 * dx, 0.01 * dx, size=pts.shape)
    st = _assemble(s, np.zeros((0, dim)), pts)
    return Case(f"droplet_in_mesh_{dim}d", s, st, _blocks(0, st.n)), mesh


def cut(c: Case, n_sample: int, centre=(0.0, 0.0, 0.0)) -> Case:
    """A spatially contiguous cut of a case at the same spacing and coordinates: the fluid
    particles nearest `centre` (about n_sample of them) and the boundary particles within reach of
    them, as one boundary block (the case's first boundary solver) and one plain fluid block (the
    case's aero plane; no inlet).  Particle types, velocities and densities are kept."""
    st = c.state
    nb = sum(b.second - b.first for b in c.blocks if not b.is_fluid)
    ctr = np.asarray(centre, dtype=np.float64)[: st.dim]
    fl = np.arange(nb, st.n)
    dist = np.linalg.norm(st.xi[fl] - ctr, axis=1)
    keep_f = np.sort(fl[np.argsort(dist, kind="stable")[:n_sample]])
    reach = np.linalg.norm(st.xi[keep_f] - ctr, axis=1).max() + 4 * c.settings.H
    wb = np.arange(nb)
    keep_b = wb[np.linalg.norm(st.xi[wb] - ctr, axis=1) < reach]
    sub = st.take(np.concatenate([keep_b, keep_f]))
    sub.part_id[:] = np.arange(sub.n)
    blocks = []
    if len(keep_b):
        b0 = [b for b in c.blocks if not b.is_fluid][0]
        blocks.append(BlockSpec(0, len(keep_b), False, bound_solver=b0.bound_solver))
    fb = [b for b in c.blocks if b.is_fluid][0]
    blocks.append(BlockSpec(len(keep_b), sub.n, True, aero_norm=fb.aero_norm, aeroconst=fb.aeroconst))
    s = c.settings.copy()
    s.max_points = sub.n
    out = Case(c.name + "_cut", s, sub, blocks)
    out.power_law_params = c.power_law_params
    return out

