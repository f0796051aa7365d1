"""Loader of the in-tree C-ABI library libfjsph_gb300.so.

The product path has no CPU fallback: if the library is missing, importing a Context raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from . import _cdefs as d

LIB_PATH = Path(__file__).resolve().parent / "libfjsph_gb300.so"

_P = C.c_void_p
_pp = C.POINTER(C.c_void_p)
_i32 = C.c_int32
_i64 = C.c_int64
_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_fp = C.POINTER(C.c_float)

PROTOTYPES = {
    "fjsph_settings_defaults": (C.c_int, [C.POINTER(d.Settings), _i32]),
    "fjsph_settings_derive": (C.c_int, [C.POINTER(d.Settings)]),
    "fjsph_ctx_create": (C.c_int, [C.POINTER(d.Settings), _i64, _pp]),
    "fjsph_ctx_destroy": (C.c_int, [_P]),
    "fjsph_set_settings": (C.c_int, [_P, C.POINTER(d.Settings)]),
    "fjsph_get_settings": (C.c_int, [_P, C.POINTER(d.Settings)]),
    "fjsph_set_limits": (C.c_int, [_P, C.POINTER(d.Block), _i32, _i64]),
    "fjsph_set_inlet": (C.c_int, [_P, C.POINTER(d.Inlet)]),
    "fjsph_get_inlet": (C.c_int, [_P, C.POINTER(d.Inlet)]),
    "fjsph_state_upload": (C.c_int, [_P, _i32, C.POINTER(d.StateView)]),
    "fjsph_state_download": (C.c_int, [_P, _i32, C.POINTER(d.StateView)]),
    "fjsph_particle_count": (C.c_int, [_P, _i64p, _i64p]),
    "fjsph_update_neighbours": (C.c_int, [_P, _i64p]),
    "fjsph_neighbours_export": (C.c_int, [_P, _i64p, _i64p, _dp]),
    "fjsph_dsph_prestep": (C.c_int, [_P, _dp]),
    "fjsph_get_aero_velocity": (C.c_int, [_P]),
    "fjsph_detect_surface": (C.c_int, [_P]),
    "fjsph_dissipation_terms": (C.c_int, [_P]),
    "fjsph_particle_shift": (C.c_int, [_P]),
    "fjsph_check_pipe_outlet": (C.c_int, [_P]),
    "fjsph_get_boundary_pressure": (C.c_int, [_P]),
    "fjsph_boundary_ghost": (C.c_int, [_P, _i32p]),
    "fjsph_boundary_dbc": (C.c_int, [_P]),
    "fjsph_set_no_slip": (C.c_int, [_P]),
    "fjsph_get_acc_and_rrho": (C.c_int, [_P, C.c_double]),
    "fjsph_find_timestep": (C.c_int, [_P, _dp]),
    "fjsph_get_first_rk": (C.c_int, [_P, C.c_double, _dp]),
    "fjsph_runge_kutta4": (C.c_int, [_P, C.c_double, C.c_double, _dp]),
    "fjsph_nb_iter": (C.c_int, [_P, C.c_double]),
    "fjsph_newmark_beta": (C.c_int, [_P, C.c_double, _dp, _i32p, _dp]),
    "fjsph_integrate_no_update": (C.c_int, [_P, _dp]),
    "fjsph_integrate": (C.c_int, [_P, _dp]),
    "fjsph_step_host": (C.c_int, [_P, C.POINTER(d.StateView), C.POINTER(d.StateView), _dp]),
    "fjsph_integrate_n": (C.c_int, [_P, _i32, _dp]),
    "fjsph_step_report": (C.c_int, [_P, _dp]),
    "fjsph_timestep_maxima": (C.c_int, [_P, _dp]),
    "fjsph_set_pair_mode": (C.c_int, [_P, _i32]),
    "fjsph_air_power_law": (C.c_int, [_P, _dp]),
    "fjsph_neighbour_counts": (C.c_int, [_P, _i32p]),
    "fjsph_get_pair_mode": (C.c_int, [_P, _i32p, _i32p]),
    "fjsph_set_sweep_order": (C.c_int, [_P, _i32]),
    "fjsph_get_sweep_order": (C.c_int, [_P, _i32p]),
    "fjsph_autotune_order": (C.c_int, [_P, _i32, _i32p, _dp]),
    "fjsph_launch_stats": (C.c_int, [_P, _i64p, _i32]),
    "fjsph_ctx_stream": (C.c_int, [_P, _pp]),
    "fjsph_status_string": (C.c_char_p, [C.c_int]),
    "fjsph_abi_sizes": (C.c_int, [_i64p]),
    "fjsph_event_record": (C.c_int, [_P, _i32]),
    "fjsph_event_elapsed": (C.c_int, [_P, _i32, _i32, _dp]),
    "fjsph_profile_enable": (C.c_int, [_P, _i32]),
    "fjsph_profile_read": (C.c_int, [_P, _dp, _i64p]),
    "fjsph_profile_pass_name": (C.c_char_p, [_i32]),
    "fjsph_get_limits": (C.c_int, [_P, C.POINTER(d.Block), _i32, _i32p]),
    "fjsph_set_groups": (C.c_int, [_P, _i32, _i64p, _dp]),
    "fjsph_set_tuning": (C.c_int, [_P, _i32p]),
    "fjsph_get_tuning": (C.c_int, [_P, _i32p]),
    "fjsph_autotune": (C.c_int, [_P, _i32, _i32p, _dp]),
    "fjsph_integrate_groups": (C.c_int, [_P, _i32, _i32]),
    "fjsph_group_report": (C.c_int, [_P, _dp, _dp, _dp, _dp, _i64p]),
    "fjsph_update_counts": (C.c_int, [_P, _i64p, _i64p]),
    "fjsph_mlp_num_params": (C.c_int, []),
    "fjsph_mlp_forward": (C.c_int, [_fp, _fp, _i64, _fp]),
    "fjsph_mlp_gradient": (C.c_int, [_fp, _fp, _fp, _i64, _fp, _dp]),
    "fjsph_mlp_train": (C.c_int, [_fp, _fp, _fp, _i64, _i32, _i32, C.c_float, C.c_uint64, _dp]),
    "fjsph_closure_set_weights": (C.c_int, [_P, _fp, C.c_double]),
    "fjsph_closure_get_weights": (C.c_int, [_P, _fp]),
    "fjsph_closure_log": (C.c_int, [_P, _i64, _i32]),
    "fjsph_closure_log_read": (C.c_int, [_P, _fp, _fp, _i64, _i64p, _i32]),
    "fjsph_closure_arm": (C.c_int, [_P, _i32]),
    "fjsph_closure_report_get": (C.c_int, [_P, C.POINTER(d.ClosureReport)]),
    "fjsph_closure_reset": (C.c_int, [_P]),
    "fjsph_vlm_defaults": (C.c_int, [C.POINTER(d.Vlm)]),
    "fjsph_vlm_setup": (C.c_int, [_P, C.POINTER(d.Vlm), _i32p]),
    "fjsph_vlm_panels": (C.c_int, [_P, _dp, _dp, _i32p]),
    "fjsph_vlm_velocity": (C.c_int, [_P, _i64, _dp, _dp]),
    "fjsph_restart_write": (C.c_int, [_P, C.c_char_p, _i64]),
    "fjsph_restart_read": (C.c_int, [_P, C.c_char_p, _i64p]),
    "fjsph_mesh_set": (C.c_int, [_P, C.POINTER(d.Mesh)]),
    "fjsph_geometry_create": (C.c_int, [C.POINTER(d.Settings), _pp]),
    "fjsph_geometry_destroy": (C.c_int, [_P]),
    "fjsph_geometry_read": (C.c_int, [_P, C.c_char_p, _i32]),
    "fjsph_geometry_read_file": (C.c_int, [_P, C.c_char_p, _i32]),
    "fjsph_geometry_build": (C.c_int, [_P]),
    "fjsph_geometry_sizes": (C.c_int, [_P, _i64p, _i64p, _i32p, _i32p, _i32p]),
    "fjsph_geometry_state": (C.c_int, [_P, C.POINTER(d.StateView)]),
    "fjsph_geometry_blocks": (C.c_int, [_P, C.POINTER(d.Block), _i32]),
    "fjsph_geometry_block_info": (C.c_int, [_P, _i32, C.POINTER(d.GeometryBlock)]),
    "fjsph_geometry_inlet": (C.c_int, [_P, _i32, C.POINTER(d.Inlet)]),
    "fjsph_geometry_log": (C.c_int, [_P, C.c_char_p, _i64, _i64p]),
    "fjsph_find_timestep_noalloc": (C.c_int, [C.POINTER(d.Settings), _i64, C.POINTER(_dp), C.POINTER(_dp), _dp, _dp,
                                              _dp, C.POINTER(_dp), C.POINTER(_dp), _P, _dp, _dp]),
}

_lib = None


class FJSPHError(RuntimeError):
    def __init__(self, fn: str, status: int):
        msg = lib().fjsph_status_string(status).decode() if _lib is not None else str(status)
        super().__init__(f"{fn} failed: {msg} ({status})")
        self.status = status


def lib() -> C.CDLL:
    """Load the library once; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        h = C.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | getattr(os, "RTLD_LOCAL", 0))
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        sizes = (C.c_int64 * 4)()
        h.fjsph_abi_sizes(sizes)
        expect = [C.sizeof(d.Settings), C.sizeof(d.Block), C.sizeof(d.Inlet), C.sizeof(d.StateView)]
        if list(sizes) != expect:
            raise RuntimeError(f"ABI mismatch between libfjsph_gb300.so {list(sizes)} and bindings {expect}")
        _lib = h
    return _lib


def check(fn: str, status: int) -> None:
    if status != d.OK:
        raise FJSPHError(fn, status)
