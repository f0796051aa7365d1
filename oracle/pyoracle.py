"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Mirrors fjsph_gb300.api.Context method by method so that parity tests call both the same way.
Loads only oracle/libfjsph_oracle.so; the derived settings come from oracle/settings_ref.py, not
from the library under test.
Parity status: unpinned (see oracle.cpp).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from fjsph_gb300 import _cdefs as d
from fjsph_gb300.state import BlockSpec, InletSpec, SPHState, blocks_to_c

from .build import build
from .settings_ref import derive as derive_settings

_lib = None
_P = C.c_void_p
_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)

_PROTO = {
    "orc_create": (_P, [C.POINTER(d.Settings)]),
    "orc_destroy": (None, [_P]),
    "orc_set_settings": (None, [_P, C.POINTER(d.Settings)]),
    "orc_get_settings": (None, [_P, C.POINTER(d.Settings)]),
    "orc_set_limits": (C.c_int, [_P, C.POINTER(d.Block), C.c_int32, C.c_int64]),
    "orc_set_inlet": (C.c_int, [_P, C.POINTER(d.Inlet)]),
    "orc_get_inlet": (C.c_int, [_P, C.POINTER(d.Inlet)]),
    "orc_get_limits": (C.c_int, [_P, C.POINTER(d.Block), C.c_int32, C.POINTER(C.c_int32)]),
    "orc_update_counts": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "orc_set_state": (C.c_int, [_P, C.c_int32, C.POINTER(d.StateView)]),
    "orc_get_state": (C.c_int, [_P, C.c_int32, C.POINTER(d.StateView)]),
    "orc_particle_count": (C.c_int64, [_P]),
    "orc_set_threads": (None, [C.c_int32]),
    "orc_update_neighbours": (C.c_int64, [_P]),
    "orc_neighbours_export": (None, [_P, _i64p, _i64p, _dp]),
    "orc_dsph_prestep": (C.c_double, [_P]),
    "orc_get_aero_velocity": (None, [_P]),
    "orc_detect_surface": (None, [_P]),
    "orc_dissipation_terms": (None, [_P]),
    "orc_particle_shift": (None, [_P]),
    "orc_check_pipe_outlet": (None, [_P]),
    "orc_get_boundary_pressure": (None, [_P]),
    "orc_boundary_ghost": (None, [_P, _i32p]),
    "orc_boundary_dbc": (None, [_P]),
    "orc_set_no_slip": (None, [_P]),
    "orc_get_acc_and_rrho": (None, [_P, C.c_double]),
    "orc_find_timestep": (C.c_double, [_P]),
    "orc_get_first_rk": (C.c_double, [_P, C.c_double]),
    "orc_runge_kutta4": (C.c_double, [_P, C.c_double, C.c_double]),
    "orc_nb_iter": (None, [_P, C.c_double]),
    "orc_newmark_beta": (C.c_double, [_P, C.c_double, _dp, _i32p]),
    "orc_integrate_no_update": (C.c_double, [_P]),
    "orc_integrate": (C.c_double, [_P]),
    "orc_step_report": (None, [_P, _dp]),
    "orc_kernel": (C.c_double, [C.c_double, C.c_double, C.c_double, C.c_int32]),
    "orc_gradk": (None, [_dp, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32, _dp]),
    "orc_min_eig": (C.c_double, [_dp, C.c_int32]),
    "orc_qr_inverse": (C.c_int32, [_dp, C.c_int32, _dp]),
    "orc_get_cd": (C.c_double, [C.c_double]),
    "orc_vlm_setup": (C.c_int, [_P, C.c_void_p]),
    "orc_air_power_law": (C.c_int, [_P, _dp]),
    "orc_mesh_set": (C.c_int, [_P, C.c_void_p]),
    "orc_vlm_panels": (C.c_int, [_P, _dp, _dp]),
    "orc_vlm_velocity": (None, [_P, C.c_int64, _dp, _dp]),
}


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        h = C.CDLL(str(build()))
        for name, (res, args) in _PROTO.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


class Oracle:
    """CPU restatement with the Context interface."""

    def __init__(self, settings: d.Settings, blocks: list[BlockSpec], inlets: list[InletSpec] = ()):
        self._l = lib()
        self.dim = settings.dim
        # the oracle derives the reference's derived settings itself (Set_Values, GetYcoef,
        # get_n_full: oracle/settings_ref.py) from the case's inputs
        own = derive_settings(settings.copy())
        self._h = self._l.orc_create(C.byref(own))
        self.blocks = list(blocks)
        arr = blocks_to_c(self.blocks)
        nbb = sum(1 for b in blocks if not b.is_fluid)
        self._l.orc_set_limits(self._h, arr, len(self.blocks), nbb)
        for inl in inlets:
            back = np.ascontiguousarray(inl.back, dtype=np.int64)
            buf = np.ascontiguousarray(inl.buffer, dtype=np.int64)
            c = d.Inlet()
            c.block, c.n_back = inl.block, back.shape[0]
            c.depth = buf.shape[1] if buf.ndim == 2 else 0
            c.back = back.ctypes.data_as(_i64p)
            c.buffer = buf.ctypes.data_as(_i64p)
            self._l.orc_set_inlet(self._h, C.byref(c))
        self._n_pairs = 0

    def close(self):
        if getattr(self, "_h", None):
            self._l.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def settings(self) -> d.Settings:
        s = d.Settings()
        self._l.orc_get_settings(self._h, C.byref(s))
        return s

    @settings.setter
    def settings(self, s: d.Settings) -> None:
        self._l.orc_set_settings(self._h, C.byref(s))

    def upload(self, which: int, st: SPHState) -> None:
        v = st.view()
        self._l.orc_set_state(self._h, which, C.byref(v))

    def download(self, which: int = d.PNP1) -> SPHState:
        n = self._l.orc_particle_count(self._h)
        st = SPHState(n, self.dim)
        v = st.view()
        self._l.orc_get_state(self._h, which, C.byref(v))
        return st

    def set_states(self, pn: SPHState, pnp1: SPHState) -> None:
        self.upload(d.PNP1, pnp1)
        self.upload(d.PN, pn)

    def particle_count(self) -> int:
        return int(self._l.orc_particle_count(self._h))

    def update_neighbours(self) -> int:
        self._n_pairs = int(self._l.orc_update_neighbours(self._h))
        return self._n_pairs

    def neighbours(self):
        n = self._l.orc_particle_count(self._h)
        off = np.zeros(n + 1, dtype=np.int64)
        idx = np.zeros(self._n_pairs, dtype=np.int64)
        d2 = np.zeros(self._n_pairs, dtype=np.float64)
        self._l.orc_neighbours_export(self._h, off.ctypes.data_as(_i64p), idx.ctypes.data_as(_i64p),
                                      d2.ctypes.data_as(_dp))
        return off, idx, d2

    def dSPH_PreStep(self) -> float:
        return self._l.orc_dsph_prestep(self._h)

    def air_power_law(self, axis: int, wall: float, thickness: float, exponent: float = 1.0 / 7.0) -> None:
        """The analytic boundary-layer air field (settings asource = FJSPH_POWER_LAW)."""
        p = (C.c_double * 4)(float(axis), wall, thickness, exponent)
        if self._l.orc_air_power_law(self._h, p) != 0:
            raise ValueError("air_power_law: the settings do not name the power-law source")

    def mesh_set(self, mesh) -> None:
        """The mesh-cell air source's mesh (mesh: fjsph_gb300.mesh.CellMesh)."""
        m = mesh.to_c()
        rc = lib().orc_mesh_set(self._h, C.byref(m))
        if rc != 0:
            raise RuntimeError(f"orc_mesh_set failed ({rc})")

    def vlm_setup(self, vlm) -> int:
        """VLM::Init + GetGamma for the settings' v_inf (vlm: fjsph_gb300._cdefs.Vlm)."""
        n = lib().orc_vlm_setup(self._h, C.byref(vlm))
        if n < 0:
            raise RuntimeError(f"orc_vlm_setup failed ({n})")
        return n

    def vlm_panels(self):
        n = lib().orc_vlm_panels(self._h, None, None)
        g = np.zeros(n)
        abc = np.zeros((n, 3, 3))
        lib().orc_vlm_panels(self._h, g.ctypes.data_as(_dp), abc.ctypes.data_as(_dp))
        return g, abc

    def vlm_velocity(self, pos):
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        out = np.zeros_like(p)
        lib().orc_vlm_velocity(self._h, p.shape[0], p.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
        return out

    def get_aero_velocity(self):
        self._l.orc_get_aero_velocity(self._h)

    def Detect_Surface(self):
        self._l.orc_detect_surface(self._h)

    def dissipation_terms(self):
        self._l.orc_dissipation_terms(self._h)

    def particle_shift(self):
        self._l.orc_particle_shift(self._h)

    def Check_Pipe_Outlet(self):
        self._l.orc_check_pipe_outlet(self._h)

    def Get_Boundary_Pressure(self):
        self._l.orc_get_boundary_pressure(self._h)

    def Boundary_Ghost(self) -> np.ndarray:
        n = self._l.orc_particle_count(self._h)
        out = np.zeros(max(n, 1), dtype=np.int32)
        self._l.orc_boundary_ghost(self._h, out.ctypes.data_as(_i32p))
        nb = sum(b.second - b.first for b in self.blocks if not b.is_fluid)
        return out[:nb]

    def Boundary_DBC(self):
        self._l.orc_boundary_dbc(self._h)

    def Set_No_Slip(self):
        self._l.orc_set_no_slip(self._h)

    def get_acc_and_Rrho(self, npd: float):
        self._l.orc_get_acc_and_rrho(self._h, float(npd))

    def find_timestep(self) -> float:
        return self._l.orc_find_timestep(self._h)

    def Get_First_RK(self, npd: float) -> float:
        return self._l.orc_get_first_rk(self._h, float(npd))

    def Runge_Kutta4(self, npd: float, logbase: float) -> float:
        return self._l.orc_runge_kutta4(self._h, float(npd), float(logbase))

    def Do_NB_Iter(self, npd: float):
        self._l.orc_nb_iter(self._h, float(npd))

    def Newmark_Beta(self, npd: float, logbase: float, iteration: int):
        lb, it = C.c_double(logbase), C.c_int32(iteration)
        r = self._l.orc_newmark_beta(self._h, float(npd), C.byref(lb), C.byref(it))
        return r, lb.value, it.value

    def integrate_no_update(self) -> float:
        return self._l.orc_integrate_no_update(self._h)

    def integrate(self) -> float:
        return self._l.orc_integrate(self._h)

    def integrate_n(self, n_steps: int) -> float:
        r = 0.0
        for _ in range(n_steps):
            r = self.integrate()
        return r

    def limits(self) -> list:
        """(first, second) of every LIMITS entry as update_data left them."""
        nb = C.c_int32()
        self._l.orc_get_limits(self._h, None, 0, C.byref(nb))
        arr = (d.Block * nb.value)()
        self._l.orc_get_limits(self._h, arr, nb.value, C.byref(nb))
        return [(arr[i].first, arr[i].second) for i in range(nb.value)]

    def get_inlet(self, block: int, n_back: int, depth: int):
        back = np.zeros(n_back, dtype=np.int64)
        buf = np.zeros(n_back * depth, dtype=np.int64)
        c = d.Inlet()
        c.block, c.n_back, c.depth = block, n_back, depth
        c.back = back.ctypes.data_as(_i64p)
        c.buffer = buf.ctypes.data_as(_i64p)
        self._l.orc_get_inlet(self._h, C.byref(c))
        return back, buf.reshape(n_back, depth)

    def deleted(self) -> int:
        v = C.c_int64()
        self._l.orc_update_counts(self._h, C.byref(v))
        return v.value

    def step_report(self) -> dict:
        out = (C.c_double * 5)()
        self._l.orc_step_report(self._h, out)
        return dict(maxRho_pc=out[0], maxf=out[1], maxAf=out[2], maxShift=out[3], iteration=int(out[4]))


def kernel(r, H, Wc, cubic=False):
    return lib().orc_kernel(r, H, Wc, int(cubic))


def gradk(Rij, r, H, Wc, cubic=False):
    Rij = np.ascontiguousarray(Rij, dtype=np.float64)
    out = np.zeros_like(Rij)
    lib().orc_gradk(Rij.ctypes.data_as(_dp), r, H, Wc, int(cubic), len(Rij), out.ctypes.data_as(_dp))
    return out


def min_eig(A):
    A = np.ascontiguousarray(A, dtype=np.float64)
    return lib().orc_min_eig(A.ctypes.data_as(_dp), A.shape[0])


def qr_inverse(A):
    A = np.ascontiguousarray(A, dtype=np.float64)
    out = np.zeros_like(A)
    ok = lib().orc_qr_inverse(A.ctypes.data_as(_dp), A.shape[0], out.ctypes.data_as(_dp))
    return bool(ok), out


def get_cd(Re):
    return lib().orc_get_cd(float(Re))
