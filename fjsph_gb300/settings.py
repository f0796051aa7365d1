"""Settings (SIM / FLUID / AERO / INTEG_SETT of src/Var.h) and the para-file reader.

`defaults(dim)` and `derive(s)` call the library's fjsph_settings_defaults / _derive (the
reference's defaults and its Set_Values derivations, src/IO.cpp:26-128).  `read_para` parses the
reference's "Key: value" settings file with the same rules as src/IOFunctions.h:32-130: leading
whitespace trimmed, '#' ends the value, exact key match before the first ':'.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import _cdefs as d
from ._lib import check, lib


def defaults(dim: int) -> d.Settings:
    s = d.Settings()
    check("fjsph_settings_defaults", lib().fjsph_settings_defaults(C.byref(s), dim))
    return s


def derive(s: d.Settings) -> d.Settings:
    check("fjsph_settings_derive", lib().fjsph_settings_derive(C.byref(s)))
    return s


# key -> (field, kind); kinds: f float, i int, v vector, s string (kept aside)
PARA_KEYS = {
    "Reference dispersed density": ("rho_rest", "f"),
    "Sutherland reference viscosity": ("mu_g", "f"),
    "Reference dispersed viscosity": ("mu", "f"),
    "Reference surface tension": ("sig", "f"),
    "SPH surface tension contact angle": ("contangb", "f"),
    "Init hydrostatic pressure (0/1)": ("init_hydro_pressure", "i"),
    "Hydrostatic height": ("hydro_height", "f"),
    "Grid scale": ("scale", "f"),
    "SPH integration solver": ("solver_name", "s"),
    "SPH equation of state (0=Cole/1=Isothermal)": ("pressure_rel", "i"),
    "SPH solver minimum residual": ("min_residual", "f"),
    "SPH maximum timestep": ("delta_t_max", "f"),
    "SPH minimum timestep": ("delta_t_min", "f"),
    "SPH maximum CFL": ("cfl_max", "f"),
    "SPH minimum CFL": ("cfl_min", "f"),
    "SPH CFL condition": ("cfl", "f"),
    "SPH unstable CFL step": ("cfl_step", "f"),
    "SPH unstable CFL count limit": ("n_unstable_limit", "i"),
    "SPH stable CFL count limit": ("n_stable_limit", "i"),
    "SPH stable CFL count iteration factor": ("subits_factor", "f"),
    "SPH maximum shifting velocity": ("max_shift_vel", "f"),
    "SPH background pressure": ("press_back", "f"),
    "SPH starting pressure": ("press_pipe", "f"),
    "SPH maximum absolute density variation (%)": ("rho_var", "f"),
    "SPH density variation to reduce timestep (%)": ("rho_max_iter", "f"),
    "SPH maximum density": ("rho_max", "f"),
    "SPH minimum density": ("rho_min", "f"),
    "SPH delta coefficient": ("dsph_delta", "f"),
    "SPH artificial viscosity factor": ("visc_alpha", "f"),
    "SPH speed of sound": ("speed_sound", "f"),
    "SPH Newmark-Beta iteration limit": ("max_subits", "i"),
    "SPH gravity vector": ("grav", "v"),
    "SPH initial spacing": ("particle_step", "f"),
    "SPH smoothing length factor": ("H_fac", "f"),
    "SPH maximum particle count": ("max_points", "i"),
    "SPH frame time interval": ("frame_time_interval", "f"),
    "SPH aerodynamic case": ("aero_case", "s"),
    "SPH SP diameter definition (0=dx/1=h)": ("use_dx", "i"),
    "SPH use TAB deformation (0/1)": ("use_TAB_def", "i"),
    "SPH interpolation factor (0=ncount/1=lambda)": ("use_lam", "i"),
    "SPH aerodynamic cutoff value": ("lam_cutoff", "f"),
    "SPH aerodynamic interpolation factor": ("i_interp_fac", "f"),
    "SPH freestream velocity": ("v_inf", "v"),
    "Reference velocity": ("v_ref", "f"),
    "Reference pressure": ("p_ref", "f"),
    "Reference Mach number": ("M_ref", "f"),
    "Reference density": ("rho_g", "f"),
    "Reference temperature": ("temp_g", "f"),
    "Gas constant gamma": ("gamma_g", "f"),
    "VLM definition filename": ("vlm_file", "s"),
    "Input fluid definition filename": ("input_fluid_file", "s"),
    "Input boundary definition filename": ("input_bound_file", "s"),
    "Primary grid face filename": ("tau_mesh", "s"),
    "Restart-data prefix": ("tau_sol", "s"),
    "Boundary mapping filename": ("tau_bmap", "s"),
    "2D offset vector (0 / x=1,y=2,z=3)": ("offset_axis", "s"),
    "OpenFOAM input directory": ("foam_dir", "s"),
    "OpenFOAM solution directory": ("foam_sol", "s"),
    "OpenFOAM buoyant (0/1)": ("foam_buoyant", "s"),
}

AERO_CASES = {"(none)": d.NOAERO, "Gissler": d.GISSLER, "Induced_pressure": d.INDUCED_PRESSURE,
              "Skin_friction": d.SKIN_FRIC}


def _value(line: str) -> str:
    """Get_Parameter_Value (src/IOFunctions.h:32-45)."""
    pos = line.find(":")
    end = line.find("#", pos + 1)
    if end != -1:
        value = line[pos + 1: pos + 1 + (end - pos + 2)]
    else:
        value = line[pos + 1:]
    return value.strip(" \n\r\t\f\v")


def parse_para_text(text: str) -> dict:
    """Key/value pairs of a para file, following GetInput's line handling (src/IO.cpp:337-456)."""
    out: dict = {}
    for raw in text.splitlines(keepends=True):
        line = raw.lstrip(" \n\r\t\f\v")
        end = line.find("#")
        if end != -1:
            line = line[: end + 1]
        pos = line.find(":")
        if pos == -1:
            continue
        key = line[:pos].lstrip(" \n\r\t\f\v")
        if key in PARA_KEYS:
            out[key] = _value(line)
    return out


def _num(tok: str) -> float:
    """istringstream >> value: leading numeric prefix, 0 when none."""
    import re
    m = re.match(r"\s*[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?", tok)
    return float(m.group(0)) if m else 0.0


def apply_para(s: d.Settings, kv: dict) -> dict:
    """Write parsed values into s; returns the string-valued entries (file names, solver, aero case)."""
    extra = {}
    for key, val in kv.items():
        field, kind = PARA_KEYS[key]
        if kind == "s":
            extra[field] = val
        elif kind == "f":
            setattr(s, field, _num(val))
        elif kind == "i":
            setattr(s, field, int(_num(val)))
        elif kind == "v":
            parts = [p for p in val.replace(" ", "").split(",") if p != ""]
            arr = getattr(s, field)
            for k in range(min(len(parts), s.dim)):
                arr[k] = _num(parts[k])
    solver = extra.get("solver_name", "")
    if solver == "Newmark-Beta":
        s.solver_type = d.NEWMARK_BETA
    elif solver == "Runge-Kutta":
        s.solver_type = d.RUNGE_KUTTA
    elif solver:
        raise ValueError(f"unrecognised solver name {solver!r}")
    if "aero_case" in extra:
        if extra["aero_case"] not in AERO_CASES:
            raise ValueError("Aerodynamic coupling model is not defined or correct.")
        s.acase = AERO_CASES[extra["aero_case"]]
    # air source (src/IO.cpp:462-500): a TAU grid file selects the mesh cells, else a VLM
    # definition file the vortex lattice (3D)
    if extra.get("tau_mesh") or extra.get("foam_dir"):
        s.asource = d.MESH_INFL
    elif extra.get("vlm_file") and s.dim == 3:
        s.asource = d.VLM_INFL
    return extra


# VLM::Init keys (src/VLM.cpp:27-44) -> (field, kind); "v2" = two values into two fields
VLM_KEYS = {
    "VLM wing dimensions": (("span", "chord"), "v2"),
    "VLM panel counts": (("panels_span", "panels_chord"), "v2i"),
    "VLM angle alpha (degree)": ("aoa_deg", "f"),
    "VLM sweep angle (degree)": ("sweep_deg", "f"),
    "VLM taper ratio": ("taper", "f"),
    "VLM flap start (panels)": ("flap_start", "i"),
    "VLM flap width (panels)": ("flap_width", "i"),
    "VLM flap depth (panels)": ("flap_depth", "i"),
    "VLM flap angle (degree)": ("flap_deg", "f"),
    "VLM maximum velocity factor": ("max_vel_fac", "f"),
    "VLM maximum velocity": ("max_vel", "f"),
}


def read_vlm(path: str | Path) -> d.Vlm:
    """The wing of a VLM definition file (the para file itself for "(thisfile)")."""
    v = d.Vlm()
    check("fjsph_vlm_defaults", lib().fjsph_vlm_defaults(C.byref(v)))
    for raw in Path(path).read_text().splitlines():
        line = raw.lstrip(" \n\r\t\f\v")
        pos = line.find(":")
        if pos == -1:
            continue
        key = line[:pos].lstrip(" \n\r\t\f\v")
        if key not in VLM_KEYS:
            continue
        field, kind = VLM_KEYS[key]
        val = _value(line)
        if kind in ("v2", "v2i"):
            parts = [p for p in val.replace(" ", "").split(",") if p != ""]
            for f, p in zip(field, parts[:2]):
                setattr(v, f, int(_num(p)) if kind == "v2i" else _num(p))
        elif kind == "f":
            setattr(v, field, _num(val))
        else:
            setattr(v, field, int(_num(val)))
    return v


def read_para(path: str | Path, dim: int, variant: int = 0, st_model: int = d.ST_PAIRWISE,
              apply_set_values: bool = True) -> tuple[d.Settings, dict]:
    """Settings from a reference para file, with Set_Values applied (unless apply_set_values is
    false: the file's values over the defaults, before any derivation)."""
    s = defaults(dim)
    s.variant = variant
    s.st_model = st_model
    extra = apply_para(s, parse_para_text(Path(path).read_text()))
    if extra.get("vlm_file") == "(thisfile)":
        extra["vlm_file"] = str(path)
    if s.delta_t_min > 0.0:
        s.delta_t = s.delta_t_min
    if apply_set_values:
        derive(s)
    return s, extra
