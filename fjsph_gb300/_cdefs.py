"""ctypes mirrors of the plain-C structures in include/fjsph_gb300.h."""
from __future__ import annotations

import ctypes as C

# status codes
OK = 0
E_ARG, E_CUDA, E_CAPACITY, E_NEIGHBOUR, E_NONFINITE, E_UNSUPPORTED, E_STATE = -1, -2, -3, -4, -5, -6, -7

# particle types (src/VarDefs.h:92-102)
BOUND, PISTON, BUFFER, BACK, PIPE, FREE, OUTLET, LOST = range(8)

# variant bits: one per reference -D flag
VAR_ALE, VAR_LINEAR, VAR_NOFROZEN, VAR_NODSPH, VAR_TIC, VAR_CUBIC = (1 << k for k in range(6))
ST_PAIRWISE, ST_NOST, ST_CSF = 0, 1, 2
NEWMARK_BETA, RUNGE_KUTTA = 0, 1
DBC, PRESSURE_G, GHOST = 0, 1, 2
COLE_EOS, ISO_EOS = 0, 1
NOAERO, GISSLER, INDUCED_PRESSURE, SKIN_FRIC = 0, 1, 2, 3
CONST_VEL, MESH_INFL, VLM_INFL = 0, 1, 2  # fjsph_aero_source
POWER_LAW = 100  # analytic boundary-layer air field (fjsph_air_power_law)
PREC_FP64, PREC_MIXED = 0, 1
PAIRS_TILES, PAIRS_LISTS = 0, 1
ORDER_GRID, ORDER_SM = 0, 1
CLOSURE_PLAIN, CLOSURE_LEARNED = 0, 1
CLOSURE_ARM_JUDGE, CLOSURE_ARM_LOG = 1, 2
MLP_INPUTS, MLP_OUTPUTS = 12, 2
PN, PNP1, BOTH = 0, 1, 2
INLET_ZONE = 6
MAX_TIMES = 16
DEFAULT_VAL = 9999999.0

_d = C.c_double
_i32 = C.c_int32
_u32 = C.c_uint32
_i64 = C.c_int64


class Settings(C.Structure):
    _fields_ = [
        ("dim", _i32), ("variant", _u32), ("st_model", _i32), ("precision", _i32),
        ("aero_closure", _i32), ("solver_type", _i32),
        ("pressure_rel", _i32),
        ("H", _d), ("H_sq", _d), ("sr", _d), ("H_fac", _d), ("W_dx", _d), ("W_correc", _d),
        ("rho_rest", _d), ("rho_pipe", _d), ("press_pipe", _d), ("press_back", _d), ("rho_max", _d),
        ("rho_min", _d), ("rho_var", _d), ("rho_max_iter", _d),
        ("sim_mass", _d), ("bnd_mass", _d), ("visc_alpha", _d), ("speed_sound", _d), ("mu", _d), ("nu", _d),
        ("sig", _d), ("gam", _d), ("B", _d), ("contangb", _d),
        ("dsph_delta", _d), ("dsph_cont", _d),
        ("particle_step", _d), ("dx", _d), ("scale", _d),
        ("grav", _d * 3),
        ("asource", _i32), ("init_hydro_pressure", _i32),
        ("hydro_height", _d),
        ("max_points", _i64),
        ("acase", _i32), ("use_lam", _i32), ("use_TAB_def", _i32), ("use_dx", _i32),
        ("v_inf", _d * 3),
        ("L", _d), ("td", _d), ("omega", _d), ("tmax", _d), ("ycoef", _d), ("Cf", _d), ("Ck", _d), ("Cd", _d),
        ("Cb", _d), ("Cdef", _d), ("A_sphere", _d), ("A_plate", _d),
        ("v_ref", _d), ("p_ref", _d), ("rho_g", _d), ("mu_g", _d), ("mass_g", _d), ("temp_g", _d), ("R_g", _d),
        ("gamma_g", _d), ("sos", _d), ("i_sos_sq", _d), ("M_ref", _d),
        ("lam_cutoff", _d), ("interp_fac", _d), ("i_interp_fac", _d), ("n_full", _d), ("i_n_full", _d),
        ("i_n_count", _d),
        ("max_subits", _i32), ("n_stable", _i32), ("n_stable_limit", _i32), ("n_unstable", _i32),
        ("n_unstable_limit", _i32),
        ("subits_factor", _d), ("cfl", _d), ("cfl_step", _d), ("cfl_max", _d), ("cfl_min", _d),
        ("current_time", _d), ("last_frame_time", _d),
        ("frame_time_interval", _d), ("min_residual", _d), ("delta_t", _d), ("delta_t_max", _d),
        ("delta_t_min", _d),
        ("nb_beta", _d), ("nb_gamma", _d), ("max_shift_vel", _d),
        ("reorder_interval", _i32), ("learned_judge_interval", _i32),
    ]

    def copy(self) -> "Settings":
        out = Settings()
        C.memmove(C.byref(out), C.byref(self), C.sizeof(Settings))
        return out


class Block(C.Structure):
    _fields_ = [
        ("first", _i64), ("second", _i64),
        ("is_fluid", _i32), ("bound_solver", _i32), ("no_slip", _i32), ("block_type", _i32),
        ("fixed_vel_or_dynamic", _i32), ("n_times", _i32),
        ("times", _d * MAX_TIMES), ("vels", (_d * 3) * MAX_TIMES),
        ("delete_norm", _d * 3), ("delconst", _d),
        ("insert_norm", _d * 3), ("insconst", _d),
        ("aero_norm", _d * 3), ("aeroconst", _d),
    ]


class Inlet(C.Structure):
    _fields_ = [("block", _i32), ("n_back", _i64), ("depth", _i64), ("back", C.POINTER(_i64)),
                ("buffer", C.POINTER(_i64))]


VIEW_F64 = ["xi", "v", "acc", "Af", "aVisc", "cellV", "gradRho", "norm", "vPert", "L", "Rrho", "rho", "p", "m",
            "curve", "norm_curve", "woccl", "pDist", "deltaD", "cellP", "cellRho", "colourG", "colour", "lam",
            "lam_nb", "kernsum"]
VIEW_I64 = ["part_id", "cellID"]
VIEW_I32 = ["b", "surf", "surfzone"]


class StateView(C.Structure):
    _fields_ = ([("n", _i64)] + [(f, C.POINTER(_d)) for f in VIEW_F64] + [(f, C.POINTER(_i64)) for f in VIEW_I64]
                + [(f, C.POINTER(_i32)) for f in VIEW_I32])


class ClosureReport(C.Structure):
    _fields_ = [("judged", _i64), ("judged_particles", _i64), ("last_rel_rms", _d), ("max_rel_rms", _d),
                ("judge_tol", _d), ("logged", _i64), ("log_capacity", _i64), ("steps", _i64),
                ("learned_active", _i32), ("fallback", _i32)]


class Vlm(C.Structure):
    """fjsph_vlm: the vortex-lattice wing of the air source (src/VLM.h)."""
    _fields_ = [("span", _d), ("chord", _d), ("panels_span", _i32), ("panels_chord", _i32), ("aoa_deg", _d),
                ("sweep_deg", _d), ("taper", _d), ("flap_start", _i32), ("flap_width", _i32),
                ("flap_depth", _i32), ("pad", _i32), ("flap_deg", _d), ("max_vel_fac", _d), ("max_vel", _d)]


class GeometryBlock(C.Structure):
    """fjsph_geometry_block: one block of the initial-particle generator after check_input."""
    _fields_ = [("name", C.c_char * 64), ("is_fluid", _i32), ("shape", _i32), ("sub_shape", _i32),
                ("particle_order", _i32), ("write_data", _i32), ("ni", _i32), ("nj", _i32), ("nk", _i32),
                ("estimated", _i64), ("generated", _i64), ("kept", _i64), ("radius", _d),
                ("start", _d * 3), ("end", _d * 3), ("right", _d * 3), ("centre", _d * 3), ("normal", _d * 3)]


# shape_type (src/VarDefs.h:116-127)
LINE_PLANE, SQUARE_CUBE, CIRCLE_SPHERE, CYLINDER, ARC_SECTION, COORD_DEF, INLET_ZONE, HOLLOW, SOLID = range(9)


class Mesh(C.Structure):
    """fjsph_mesh: a CFD mesh with a solution per cell (the mesh-cell air source)."""
    _fields_ = [("dim", _i32), ("n_verts", _i64), ("verts", C.POINTER(_d)), ("n_faces", _i64),
                ("face_offsets", C.POINTER(_i64)), ("face_verts", C.POINTER(_i64)), ("face_right", C.POINTER(_i32)),
                ("n_cells", _i64), ("cell_face_offsets", C.POINTER(_i64)), ("cell_faces", C.POINTER(_i64)),
                ("cell_centres", C.POINTER(_d)), ("cell_vel", C.POINTER(_d)), ("cell_p", C.POINTER(_d)),
                ("cell_rho", C.POINTER(_d))]
