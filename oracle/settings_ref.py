"""Settings defaults and derivations restated for the oracle (TEST INFRASTRUCTURE ONLY).

An independent restatement, in plain Python, of what the reference derives from a case's inputs
before its first step, so that the oracle no longer takes derived settings from the library it
checks:
  - the member defaults of FLUID, AERO, SIM and INTEG_SETT (src/Var.h:63-92, 159-236, 240-310,
    337-394);
  - Set_Values (src/IO.cpp:26-128): Cole factor B, pipe density, density limits, dx, masses, gas
    speed of sound and Mach, the initial time step, H, H^2, the search radius, delta-SPH factor,
    kinematic viscosity, the kernel normalisation W_correc and W(dx), A_plate;
  - AERO::GetYcoef (src/Var.h:244-266): L, A_sphere, td, omega, tmax, Cdef, ycoef;
  - get_n_full (src/Geometry.cpp:282-308): lattice points within the search radius, the lattice
    walked from -2(H + dx) to 2(H + dx) by adding dx, distances accumulated as the radius search
    accumulates them (fused multiply-adds; evaluated here exactly with rationals).

Works on the ctypes mirror of the C-ABI settings struct (fjsph_gb300._cdefs.Settings, a layout
declaration) without loading any compiled library.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

from fjsph_gb300 import _cdefs as d

PI = math.pi


def _fma(a: float, b: float, c: float) -> float:
    """a * b + c with one rounding (exact rational arithmetic, rounded to nearest)."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def defaults(dim: int) -> d.Settings:
    """Member defaults of the reference's settings structs (src/Var.h)."""
    if dim not in (2, 3):
        raise ValueError("dim must be 2 or 3")
    s = d.Settings()
    s.dim = dim
    s.variant = 0
    s.st_model = d.ST_PAIRWISE
    s.precision = d.PREC_FP64
    s.aero_closure = d.CLOSURE_PLAIN
    s.solver_type = d.NEWMARK_BETA
    # FLUID (src/Var.h:159-200)
    s.pressure_rel = d.COLE_EOS
    s.H = s.H_sq = s.sr = -1.0
    s.H_fac = 2.0
    s.W_dx = -1.0
    s.rho_rest = s.rho_pipe = 1000.0
    s.press_pipe = s.press_back = 0.0
    s.rho_max, s.rho_min, s.rho_var, s.rho_max_iter = 1500.0, 500.0, 50.0, 1.0
    s.sim_mass = s.bnd_mass = s.W_correc = -1.0
    s.visc_alpha = 0.1
    s.speed_sound = 300.0
    s.mu = 8.94e-4
    s.nu = s.mu / s.rho_rest
    s.sig = 0.0708
    s.gam = 7.0
    s.B = -1.0
    s.contangb = 150.0
    s.dsph_delta = 0.1
    s.dsph_cont = -1.0
    # SIM (src/Var.h:337-394)
    s.particle_step = s.dx = -1.0
    s.scale = 1.0
    s.grav[0] = 0.0
    s.grav[1] = 0.0 if dim == 3 else -9.81
    s.grav[2] = -9.81 if dim == 3 else 0.0
    s.asource = 0
    s.init_hydro_pressure = 0
    s.hydro_height = -1.0
    s.max_points = 9999999
    # AERO (src/Var.h:240-310)
    s.acase = d.NOAERO
    s.use_lam, s.use_TAB_def, s.use_dx = 1, 0, 0
    s.L = s.td = s.omega = s.tmax = s.ycoef = -1.0
    s.Cf, s.Ck, s.Cd, s.Cb = 1.0 / 3.0, 8.0, 5.0, 0.5
    s.Cdef = s.A_sphere = s.A_plate = -1.0
    s.v_ref, s.p_ref = 0.0, 101353.0
    s.rho_g, s.mu_g = 1.29251, 1.716e-5
    s.mass_g = -1.0
    s.temp_g, s.R_g, s.gamma_g = 298.0, 287.0, 1.403
    s.sos = math.sqrt(s.temp_g * s.R_g * s.gamma_g)
    s.i_sos_sq = 1.0 / (s.sos * s.sos)
    s.M_ref = -1.0
    s.lam_cutoff, s.interp_fac, s.i_interp_fac = 0.75, 2.0, 0.5
    s.n_full = 30.0 if dim == 2 else 200.0
    s.i_n_full = 1.0 / s.n_full
    s.i_n_count = 1.0 / (s.i_interp_fac * s.n_full)
    # INTEG_SETT (src/Var.h:63-92)
    s.max_subits = 20
    s.n_stable, s.n_stable_limit, s.n_unstable, s.n_unstable_limit = 0, 10, 0, 3
    s.subits_factor = 0.333
    s.cfl, s.cfl_step, s.cfl_max, s.cfl_min = 1.0, 0.05, 2.0, 0.1
    s.current_time = s.last_frame_time = 0.0
    s.frame_time_interval = 1e30  # no default upstream: the para file sets it
    s.min_residual = -7.0
    s.delta_t, s.delta_t_max, s.delta_t_min = 2e-10, 1.0, 0.0
    s.nb_beta, s.nb_gamma = 0.25, 0.5
    s.max_shift_vel = 9999999.0
    s.reorder_interval = 8
    s.learned_judge_interval = 50
    return s


def get_density(s: d.Settings, press: float) -> float:
    """FLUID::get_density (src/Var.h:219-236)."""
    if s.pressure_rel == d.ISO_EOS:
        return (press - s.press_back) / (s.speed_sound * s.speed_sound) + s.rho_rest
    return s.rho_rest * math.pow(((press - s.press_back) / s.B) + 1.0, 1.0 / s.gam)


def kernel(dist: float, H: float, Wc: float, cubic: bool) -> float:
    """Kernel (src/Kernel.h:11-21 cubic spline, :37-45 Wendland C2)."""
    if cubic:
        q = dist / H
        if q < 1.0:
            return Wc * (1.0 - 1.5 * q * q * (1 - 0.5 * q))
        if q < 2.0:
            return Wc * 0.25 * math.pow(2.0 - q, 3.0)
        return 0.0
    return math.pow(1 - 0.5 * dist / H, 4) * (2 * dist / H + 1) * Wc


def n_full(dx: float, H: float, dim: int) -> float:
    """get_n_full (src/Geometry.cpp:282-308): lattice points with d^2 < 4 H^2 of the origin."""
    sr = 4.0 * H * H
    lim = 2.0 * (H + dx)
    axis = []
    x = -lim
    while x <= lim:
        axis.append(x)
        x += dx
    count = 0
    for a in axis:
        r0 = a * a
        for b in axis:
            r1 = _fma(b, b, r0)
            if dim == 3:
                for c in axis:
                    if _fma(c, c, r1) < sr:
                        count += 1
            elif r1 < sr:
                count += 1
    return float(count)


def get_ycoef(s: d.Settings, diam: float) -> None:
    """AERO::GetYcoef (src/Var.h:244-266).  IEEE semantics as in C: a zero surface tension or
    viscosity gives infinities and NaNs, not errors (numpy float64 scalars, libm functions)."""
    D = s.dim
    f = np.float64
    with np.errstate(all="ignore"):
        if D == 3:
            L = f(diam) * np.cbrt(f(3.0) / (f(4.0) * f(PI)))
            s.A_sphere = float(f(PI) * L * L)
            s.A_plate = diam * diam
        else:
            L = f(diam) / np.sqrt(f(PI))
            s.A_sphere = float(2 * L)
            s.A_plate = diam
        s.L = float(L)
        td = (f(2.0) * f(s.rho_rest) * np.power(L, f(D - 1))) / (f(s.Cd) * f(s.mu))
        omega = np.sqrt((f(s.Ck) * f(s.sig)) / (f(s.rho_rest) * np.power(L, f(D))) - f(1.0) / np.power(td, f(2.0)))
        tmax = f(-2.0) * (np.arctan(np.sqrt(np.power(td * omega, f(2.0)) + f(1)) + td * omega) - f(PI)) / omega
        Cdef = f(1.0) - np.exp(-tmax / td) * (np.cos(omega * tmax) + f(1) / (omega * td) * np.sin(omega * tmax))
        ycoef = f(0.5) * Cdef * (f(s.Cf) / (f(s.Ck) * f(s.Cb))) * (f(s.rho_g) * L) / f(s.sig)
    s.td, s.omega, s.tmax, s.Cdef, s.ycoef = float(td), float(omega), float(tmax), float(Cdef), float(ycoef)


def derive(s: d.Settings) -> d.Settings:
    """Set_Values (src/IO.cpp:26-128) on s, in place; returns s."""
    if s.dim not in (2, 3) or not s.particle_step > 0:
        raise ValueError("dim 2 or 3 and a positive particle step are required")
    D = s.dim
    cubic = bool(s.variant & d.VAR_CUBIC)
    s.B = s.rho_rest * math.pow(s.speed_sound, 2) / s.gam
    s.rho_pipe = get_density(s, s.press_pipe)
    if s.rho_max == 1500 and s.rho_min == 500:
        s.rho_max = s.rho_rest * (1.0 + s.rho_var * 0.01)
        s.rho_min = s.rho_rest * (1.0 - s.rho_var * 0.01)
    s.dx = s.particle_step * math.pow(s.rho_pipe / s.rho_rest, 1.0 / D)
    s.nb_beta, s.nb_gamma = 0.25, 0.5
    s.sim_mass = s.rho_rest * math.pow(s.particle_step, D)
    s.bnd_mass = s.sim_mass
    s.mass_g = s.rho_g * math.pow(s.particle_step, D)
    s.sos = math.sqrt(s.temp_g * s.R_g * s.gamma_g)
    s.i_sos_sq = 1.0 / (s.sos * s.sos)
    if s.M_ref != -1:
        s.v_ref = s.sos * s.M_ref
    else:
        s.M_ref = s.v_ref / s.sos
    s.delta_t = s.delta_t_min if s.delta_t_min > 0 else 2e-10
    s.H = s.H_fac * s.particle_step
    s.H_sq = s.H * s.H
    s.sr = 4 * s.H_sq
    s.dsph_cont = 2.0 * s.dsph_delta * s.H * s.speed_sound
    s.nu = s.mu / s.rho_rest
    if D == 2:
        s.W_correc = 10.0 / (7.0 * PI * s.H * s.H) if cubic else 7.0 / (4.0 * PI * s.H * s.H)
    else:
        s.W_correc = (1.0 / (PI * s.H * s.H * s.H)) if cubic else (21 / (16 * PI * s.H * s.H * s.H))
    s.W_dx = kernel(s.particle_step, s.H, s.W_correc, cubic)
    get_ycoef(s, s.particle_step)
    s.n_full = n_full(s.particle_step, s.H, D)
    s.i_n_full = 1.0 / s.n_full
    s.interp_fac = 1.0 / s.i_interp_fac
    s.A_plate = s.particle_step * s.particle_step if D == 3 else s.particle_step
    return s


# fields Set_Values (and GetYcoef, get_n_full) writes
DERIVED = ["B", "rho_pipe", "rho_max", "rho_min", "dx", "nb_beta", "nb_gamma", "sim_mass", "bnd_mass", "mass_g",
           "sos", "i_sos_sq", "v_ref", "M_ref", "delta_t", "H", "H_sq", "sr", "dsph_cont", "nu", "W_correc", "W_dx",
           "L", "A_sphere", "A_plate", "td", "omega", "tmax", "Cdef", "ycoef", "n_full", "i_n_full", "interp_fac"]
