"""Host-side mirror of FJSPH's hot-path interface, backed by the GB300 C-ABI library.

Method names follow the reference functions they replace; each operates on the context's
working state `pnp1` (and reads `pn`), as the reference functions do on SPHState references:

  update_neighbours      src/Neighbours.cpp:7        dSPH_PreStep        src/Shifting.cpp:12
  get_aero_velocity      src/Resid.cpp:471            Detect_Surface      src/Geometry.cpp:14
  dissipation_terms      src/Shifting.cpp:126         particle_shift      src/Shifting.cpp:189
  Check_Pipe_Outlet      src/Containment.cpp:822      Get_Boundary_Pressure src/Resid.cpp:21
  Boundary_Ghost         src/Resid.cpp:122            Boundary_DBC        src/Resid.cpp:78
  Set_No_Slip            src/Resid.cpp:162            get_acc_and_Rrho    src/Resid.cpp:426
  find_timestep          src/Integration.cpp:370      Get_First_RK        src/Runge_Kutta.cpp:462
  Runge_Kutta4           src/Runge_Kutta.cpp:480      Do_NB_Iter          src/Newmark_Beta.cpp:54
  Newmark_Beta           src/Newmark_Beta.cpp:303     integrate_no_update src/Integration.cpp:27
  integrate              src/Integration.cpp:233

Errors raise FJSPHError (the reference prints and exits instead).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _cdefs as d
from ._lib import check, lib
from .state import BlockSpec, InletSpec, SPHState, blocks_to_c


class Context:
    """One device context: two particle states (pn, pnp1), neighbour lists, integrator scratch."""

    def __init__(self, settings: d.Settings, capacity: int, blocks: list[BlockSpec],
                 inlets: list[InletSpec] = ()):
        self._lib = lib()
        self.dim = settings.dim
        h = C.c_void_p()
        check("fjsph_ctx_create", self._lib.fjsph_ctx_create(C.byref(settings), int(capacity), C.byref(h)))
        self._h = h
        self.blocks = list(blocks)
        self.n_bound_blocks = sum(1 for b in blocks if not b.is_fluid)
        arr = blocks_to_c(self.blocks)
        check("fjsph_set_limits", self._lib.fjsph_set_limits(self._h, arr, len(self.blocks), self.n_bound_blocks))
        self._inlets = list(inlets)
        for inl in self._inlets:
            self._set_inlet(inl)

    def _set_inlet(self, inl: InletSpec) -> None:
        back = np.ascontiguousarray(inl.back, dtype=np.int64)
        buf = np.ascontiguousarray(inl.buffer, dtype=np.int64)
        c = d.Inlet()
        c.block = inl.block
        c.n_back = back.shape[0]
        c.depth = buf.shape[1] if buf.ndim == 2 else 0
        c.back = back.ctypes.data_as(C.POINTER(C.c_int64))
        c.buffer = buf.ctypes.data_as(C.POINTER(C.c_int64))
        check("fjsph_set_inlet", self._lib.fjsph_set_inlet(self._h, C.byref(c)))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.fjsph_ctx_destroy(self._h)
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

    # ---- settings and state ------------------------------------------------------------------
    @property
    def settings(self) -> d.Settings:
        s = d.Settings()
        check("fjsph_get_settings", self._lib.fjsph_get_settings(self._h, C.byref(s)))
        return s

    @settings.setter
    def settings(self, s: d.Settings) -> None:
        check("fjsph_set_settings", self._lib.fjsph_set_settings(self._h, C.byref(s)))

    def upload(self, which: int, st: SPHState, fields=None) -> None:
        """fields: names to transfer (None = all); the device keeps its copy of the others."""
        v = st.view(fields)
        check("fjsph_state_upload", self._lib.fjsph_state_upload(self._h, which, C.byref(v)))

    def download(self, which: int = d.PNP1, fields=None, out: SPHState | None = None) -> SPHState:
        """The state (fields: names to transfer, None = all; out: a state of the right size to
        fill in place)."""
        if out is None:
            n = C.c_int64()
            check("fjsph_particle_count", self._lib.fjsph_particle_count(self._h, C.byref(n), None))
            out = SPHState(n.value, self.dim)
        v = out.view(fields)
        check("fjsph_state_download", self._lib.fjsph_state_download(self._h, which, C.byref(v)))
        return out

    def set_states(self, pn: SPHState, pnp1: SPHState) -> None:
        self.upload(d.PNP1, pnp1)
        self.upload(d.PN, pn)

    # ---- neighbour search --------------------------------------------------------------------
    def update_neighbours(self) -> int:
        n = C.c_int64()
        check("fjsph_update_neighbours", self._lib.fjsph_update_neighbours(self._h, C.byref(n)))
        self._n_pairs = n.value
        return n.value

    def neighbours(self):
        """(offsets, neighbour indices, squared distances) in reference order, lists sorted."""
        n = C.c_int64()
        self._lib.fjsph_particle_count(self._h, C.byref(n), None)
        off = np.zeros(n.value + 1, dtype=np.int64)
        idx = np.zeros(self._n_pairs, dtype=np.int64)
        d2 = np.zeros(self._n_pairs, dtype=np.float64)
        check("fjsph_neighbours_export", self._lib.fjsph_neighbours_export(
            self._h, off.ctypes.data_as(C.POINTER(C.c_int64)), idx.ctypes.data_as(C.POINTER(C.c_int64)),
            d2.ctypes.data_as(C.POINTER(C.c_double))))
        return off, idx, d2

    # ---- pre-passes ----------------------------------------------------------------------------
    def dSPH_PreStep(self) -> float:
        npd = C.c_double()
        check("fjsph_dsph_prestep", self._lib.fjsph_dsph_prestep(self._h, C.byref(npd)))
        return npd.value

    def get_aero_velocity(self) -> None:
        check("fjsph_get_aero_velocity", self._lib.fjsph_get_aero_velocity(self._h))

    def Detect_Surface(self) -> None:
        check("fjsph_detect_surface", self._lib.fjsph_detect_surface(self._h))

    def dissipation_terms(self) -> None:
        check("fjsph_dissipation_terms", self._lib.fjsph_dissipation_terms(self._h))

    def particle_shift(self) -> None:
        check("fjsph_particle_shift", self._lib.fjsph_particle_shift(self._h))

    def Check_Pipe_Outlet(self) -> None:
        check("fjsph_check_pipe_outlet", self._lib.fjsph_check_pipe_outlet(self._h))

    # ---- boundary passes and residual ----------------------------------------------------------
    def Get_Boundary_Pressure(self) -> None:
        check("fjsph_get_boundary_pressure", self._lib.fjsph_get_boundary_pressure(self._h))

    def Boundary_Ghost(self) -> np.ndarray:
        n, nb = C.c_int64(), C.c_int64()
        self._lib.fjsph_particle_count(self._h, C.byref(n), C.byref(nb))
        out = np.zeros(max(nb.value, 1), dtype=np.int32)
        check("fjsph_boundary_ghost", self._lib.fjsph_boundary_ghost(self._h, out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out[: nb.value]

    def Boundary_DBC(self) -> None:
        check("fjsph_boundary_dbc", self._lib.fjsph_boundary_dbc(self._h))

    def Set_No_Slip(self) -> None:
        check("fjsph_set_no_slip", self._lib.fjsph_set_no_slip(self._h))

    def get_acc_and_Rrho(self, npd: float) -> None:
        check("fjsph_get_acc_and_rrho", self._lib.fjsph_get_acc_and_rrho(self._h, float(npd)))

    # ---- integrators ----------------------------------------------------------------------------
    def find_timestep(self) -> float:
        dt = C.c_double()
        check("fjsph_find_timestep", self._lib.fjsph_find_timestep(self._h, C.byref(dt)))
        return dt.value

    def Get_First_RK(self, npd: float) -> float:
        lb = C.c_double()
        check("fjsph_get_first_rk", self._lib.fjsph_get_first_rk(self._h, float(npd), C.byref(lb)))
        return lb.value

    def Runge_Kutta4(self, npd: float, logbase: float) -> float:
        r = C.c_double()
        check("fjsph_runge_kutta4", self._lib.fjsph_runge_kutta4(self._h, float(npd), float(logbase), C.byref(r)))
        return r.value

    def Do_NB_Iter(self, npd: float) -> None:
        check("fjsph_nb_iter", self._lib.fjsph_nb_iter(self._h, float(npd)))

    def Newmark_Beta(self, npd: float, logbase: float, iteration: int):
        lb, it, r = C.c_double(logbase), C.c_int32(iteration), C.c_double()
        check("fjsph_newmark_beta", self._lib.fjsph_newmark_beta(self._h, float(npd), C.byref(lb), C.byref(it),
                                                                  C.byref(r)))
        return r.value, lb.value, it.value

    def integrate_no_update(self) -> float:
        r = C.c_double()
        check("fjsph_integrate_no_update", self._lib.fjsph_integrate_no_update(self._h, C.byref(r)))
        return r.value

    def integrate(self) -> float:
        r = C.c_double()
        check("fjsph_integrate", self._lib.fjsph_integrate(self._h, C.byref(r)))
        return r.value

    def step_host(self, st_in: SPHState, out: SPHState, fields=None) -> int:
        """One step on a host state: upload st_in as pn and pnp1, integrate, download pnp1 into
        `out` (fields: names to transfer both ways, None = all; out's arrays must hold the
        particle count after the step).  Returns the particle count after the step."""
        vi = st_in.view(fields)
        vo = out.view(fields)
        r = C.c_double()
        check("fjsph_step_host", self._lib.fjsph_step_host(self._h, C.byref(vi), C.byref(vo), C.byref(r)))
        return int(vo.n)

    def integrate_n(self, n_steps: int) -> float:
        r = C.c_double()
        check("fjsph_integrate_n", self._lib.fjsph_integrate_n(self._h, int(n_steps), C.byref(r)))
        return r.value

    def neighbour_counts(self) -> np.ndarray:
        """Neighbours (self included) of every particle in reference order, from the last search."""
        out = np.zeros(self.particle_count(), dtype=np.int32)
        check("fjsph_neighbour_counts", self._lib.fjsph_neighbour_counts(self._h, out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out

    def particle_count(self) -> int:
        """Particles in the context now (insertions and deletions included)."""
        n = C.c_int64()
        check("fjsph_particle_count", self._lib.fjsph_particle_count(self._h, C.byref(n), None))
        return n.value

    def limits(self) -> list:
        """(first, second) of every LIMITS entry as update_data left them."""
        nb = C.c_int32()
        check("fjsph_get_limits", self._lib.fjsph_get_limits(self._h, None, 0, C.byref(nb)))
        arr = (d.Block * nb.value)()
        check("fjsph_get_limits", self._lib.fjsph_get_limits(self._h, arr, nb.value, C.byref(nb)))
        return [(arr[i].first, arr[i].second) for i in range(nb.value)]

    def get_inlet(self, block: int, n_back: int, depth: int):
        """The inlet's back and buffer tables (reference indices) as they are now."""
        back = np.zeros(n_back, dtype=np.int64)
        buf = np.zeros(n_back * depth, dtype=np.int64)
        c = d.Inlet()
        c.block, c.n_back, c.depth = block, n_back, depth
        c.back = back.ctypes.data_as(C.POINTER(C.c_int64))
        c.buffer = buf.ctypes.data_as(C.POINTER(C.c_int64))
        check("fjsph_get_inlet", self._lib.fjsph_get_inlet(self._h, C.byref(c)))
        return back, buf.reshape(n_back, depth)

    # ---- independent simulations sharing the context --------------------------------------------
    def set_groups(self, first, v_inf) -> None:
        """Groups of reference indices [first[g], first[g+1]) with their free-stream velocities."""
        f = np.ascontiguousarray(first, dtype=np.int64)
        vi = np.ascontiguousarray(np.asarray(v_inf, dtype=np.float64).reshape(-1, 3))
        self._ngroups = len(f) - 1
        check("fjsph_set_groups", self._lib.fjsph_set_groups(
            self._h, self._ngroups, f.ctypes.data_as(C.POINTER(C.c_int64)), vi.ctypes.data_as(C.POINTER(C.c_double))))

    def integrate_groups(self, n_steps: int, graph: bool = True) -> None:
        check("fjsph_integrate_groups", self._lib.fjsph_integrate_groups(self._h, int(n_steps), int(graph)))

    def group_report(self) -> dict:
        g = self._ngroups
        out = {k: np.zeros(g) for k in ("time", "dt", "cfl", "err")}
        steps = np.zeros(g, dtype=np.int64)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        check("fjsph_group_report", self._lib.fjsph_group_report(
            self._h, dp(out["time"]), dp(out["dt"]), dp(out["cfl"]), dp(out["err"]),
            steps.ctypes.data_as(C.POINTER(C.c_int64))))
        out["steps"] = steps
        return out

    # ---- launch-configuration autotuner --------------------------------------------------------
    def autotune(self, repeats: int = 3) -> dict:
        """Pick the fastest pair-sweep / residual launch configuration on the current state, then
        the faster work order of the residual with it."""
        cfg = (C.c_int32 * 3)()
        ms = (C.c_double * 8)()
        check("fjsph_autotune", self._lib.fjsph_autotune(self._h, int(repeats), cfg, ms))
        tried = [("sweep", b, None) for b in (64, 128)] + [("resid", b, a) for b in (64, 128) for a in (2, 4, 8)]
        trials = [dict(kind=k, threads=b, list_ahead=a, ms=ms[i]) for i, (k, b, a) in enumerate(tried)]
        order, oms = C.c_int32(), (C.c_double * 2)()
        check("fjsph_autotune_order", self._lib.fjsph_autotune_order(self._h, int(repeats), C.byref(order), oms))
        trials += [dict(kind="resid order", order=name, ms=oms[i]) for i, name in enumerate(("grid", "sm"))]
        return {"chosen": {"sweep_threads": cfg[0], "resid_threads": cfg[1], "list_ahead": cfg[2],
                           "order": "sm" if order.value == d.ORDER_SM else "grid"},
                "trials_ms": trials}

    def tuning(self, cfg=None):
        """Get (cfg None) or set the launch configuration (sweep threads, residual threads, rows ahead)."""
        arr = (C.c_int32 * 3)()
        if cfg is None:
            check("fjsph_get_tuning", self._lib.fjsph_get_tuning(self._h, arr))
            return tuple(arr)
        arr[:] = list(cfg)
        check("fjsph_set_tuning", self._lib.fjsph_set_tuning(self._h, arr))
        return tuple(cfg)

    def update_counts(self) -> tuple[int, int]:
        """Particles inserted and deleted by update_data since the context was created."""
        a, b = C.c_int64(), C.c_int64()
        check("fjsph_update_counts", self._lib.fjsph_update_counts(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def step_report(self) -> dict:
        out = (C.c_double * 5)()
        check("fjsph_step_report", self._lib.fjsph_step_report(self._h, out))
        return dict(maxRho_pc=out[0], maxf=out[1], maxAf=out[2], maxShift=out[3], iteration=int(out[4]))

    def air_power_law(self, axis: int, wall: float, thickness: float, exponent: float = 1.0 / 7.0) -> None:
        """The analytic boundary-layer air field of a context with asource = FJSPH_POWER_LAW:
        v_inf * clamp((x[axis] - wall) / thickness, 0, 1)^exponent."""
        p = (C.c_double * 4)(float(axis), wall, thickness, exponent)
        check("fjsph_air_power_law", self._lib.fjsph_air_power_law(self._h, p))

    def set_pair_mode(self, mode: int) -> None:
        """d.PAIRS_LISTS (pair lists, default) or d.PAIRS_TILES (shared-memory tiles for the residual)."""
        check("fjsph_set_pair_mode", self._lib.fjsph_set_pair_mode(self._h, int(mode)))

    def pair_mode(self) -> tuple[int, bool]:
        """(mode, whether the last search built tiles)."""
        m, t = C.c_int32(), C.c_int32()
        check("fjsph_get_pair_mode", self._lib.fjsph_get_pair_mode(self._h, C.byref(m), C.byref(t)))
        return m.value, bool(t.value)

    def set_sweep_order(self, order: int) -> None:
        """d.ORDER_GRID (grid order, default) or d.ORDER_SM (SM-local chunks) for the residual."""
        check("fjsph_set_sweep_order", self._lib.fjsph_set_sweep_order(self._h, int(order)))

    def sweep_order(self) -> int:
        o = C.c_int32()
        check("fjsph_get_sweep_order", self._lib.fjsph_get_sweep_order(self._h, C.byref(o)))
        return o.value

    def timestep_maxima(self) -> list[float]:
        """maxf, maxAf, maxdrho, maxRhoi, minST, maxU, maxShift of the last find_timestep."""
        out = (C.c_double * 7)()
        check("fjsph_timestep_maxima", self._lib.fjsph_timestep_maxima(self._h, out))
        return list(out)

    def launch_stats(self, reset: bool = False) -> int:
        n = C.c_int64()
        check("fjsph_launch_stats", self._lib.fjsph_launch_stats(self._h, C.byref(n), int(reset)))
        return n.value

    def event_record(self, slot: int) -> None:
        check("fjsph_event_record", self._lib.fjsph_event_record(self._h, int(slot)))

    def event_elapsed(self, a: int, b: int) -> float:
        ms = C.c_double()
        check("fjsph_event_elapsed", self._lib.fjsph_event_elapsed(self._h, int(a), int(b), C.byref(ms)))
        return ms.value

    def profile(self, on: bool) -> None:
        check("fjsph_profile_enable", self._lib.fjsph_profile_enable(self._h, int(on)))

    def profile_read(self) -> dict:
        """{pass name: (milliseconds, section count)} accumulated since the last read."""
        npass = 13
        ms = (C.c_double * npass)()
        cnt = (C.c_int64 * npass)()
        check("fjsph_profile_read", self._lib.fjsph_profile_read(self._h, ms, cnt))
        return {self._lib.fjsph_profile_pass_name(k).decode(): (ms[k], cnt[k]) for k in range(npass)}

    def stream(self) -> int:
        p = C.c_void_p()
        check("fjsph_ctx_stream", self._lib.fjsph_ctx_stream(self._h, C.byref(p)))
        return p.value or 0

    # ---- learned aerodynamic closure -----------------------------------------------------------
    def closure_set_weights(self, params: np.ndarray, judge_tol: float = 0.05) -> None:
        """Weights of the learned closure (used when settings.aero_closure == CLOSURE_LEARNED)."""
        w = np.ascontiguousarray(params, dtype=np.float32)
        if w.size != self._lib.fjsph_mlp_num_params():
            raise ValueError(f"expected {self._lib.fjsph_mlp_num_params()} parameters, got {w.size}")
        check("fjsph_closure_set_weights",
              self._lib.fjsph_closure_set_weights(self._h, _fptr(w), float(judge_tol)))

    def closure_get_weights(self) -> np.ndarray:
        w = np.empty(self._lib.fjsph_mlp_num_params(), dtype=np.float32)
        check("fjsph_closure_get_weights", self._lib.fjsph_closure_get_weights(self._h, _fptr(w)))
        return w

    def closure_log(self, capacity: int, every_n_steps: int = 1) -> None:
        """Log (inputs, targets) of the plain closure on the device; capacity 0 frees the log."""
        check("fjsph_closure_log", self._lib.fjsph_closure_log(self._h, int(capacity), int(every_n_steps)))

    def closure_log_read(self, reset: bool = True) -> tuple[np.ndarray, np.ndarray]:
        rep = self.closure_report()
        m = int(rep["logged"])
        X = np.empty((m, d.MLP_INPUTS), dtype=np.float32)
        T = np.empty((m, d.MLP_OUTPUTS), dtype=np.float32)
        cnt = C.c_int64()
        check("fjsph_closure_log_read",
              self._lib.fjsph_closure_log_read(self._h, _fptr(X), _fptr(T), m, C.byref(cnt), int(reset)))
        return X[:cnt.value], T[:cnt.value]

    def closure_arm(self, what: int) -> None:
        """One-shot: the next residual judges (CLOSURE_ARM_JUDGE) or logs (CLOSURE_ARM_LOG)."""
        check("fjsph_closure_arm", self._lib.fjsph_closure_arm(self._h, int(what)))

    def closure_report(self) -> dict:
        r = d.ClosureReport()
        check("fjsph_closure_report_get", self._lib.fjsph_closure_report_get(self._h, C.byref(r)))
        return {f: getattr(r, f) for f, _ in d.ClosureReport._fields_}

    def closure_reset(self) -> None:
        check("fjsph_closure_reset", self._lib.fjsph_closure_reset(self._h))

    # ---- restart files (src/H5IO.cpp) ----
    def restart_write(self, path: str, current_frame: int = 0) -> None:
        check("fjsph_restart_write", self._lib.fjsph_restart_write(self._h, str(path).encode(), int(current_frame)))

    def restart_read(self, path: str) -> int:
        """Load a restart file into pn and pnp1; returns the stored frame."""
        f = C.c_int64(0)
        check("fjsph_restart_read", self._lib.fjsph_restart_read(self._h, str(path).encode(), C.byref(f)))
        return f.value

    # ---- vortex-lattice air source (src/VLM.h) ----
    def mesh_set(self, mesh) -> None:
        """The mesh-cell air source's mesh (mesh: fjsph_gb300.mesh.CellMesh); the context must have
        been created with asource = MESH_INFL."""
        m = mesh.to_c()
        check("fjsph_mesh_set", self._lib.fjsph_mesh_set(self._h, C.byref(m)))

    def vlm_setup(self, vlm: "d.Vlm") -> int:
        """VLM::Init + GetGamma for the context's v_inf; returns the panel count."""
        n = C.c_int32(0)
        check("fjsph_vlm_setup", self._lib.fjsph_vlm_setup(self._h, C.byref(vlm), C.byref(n)))
        return n.value

    def vlm_panels(self):
        """(gamma[np], abc[np, 3, 3]): circulations and the vortex ends A, B and control point C."""
        n = C.c_int32(0)
        check("fjsph_vlm_panels", self._lib.fjsph_vlm_panels(self._h, None, None, C.byref(n)))
        g = np.zeros(n.value)
        abc = np.zeros((n.value, 3, 3))
        check("fjsph_vlm_panels", self._lib.fjsph_vlm_panels(self._h, _dptr(g), _dptr(abc), C.byref(n)))
        return g, abc

    def vlm_velocity(self, pos: np.ndarray) -> np.ndarray:
        """VLM::getVelocity at the rows of pos (n x 3), on the device in the context's precision."""
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        out = np.zeros_like(p)
        check("fjsph_vlm_velocity", self._lib.fjsph_vlm_velocity(self._h, p.shape[0], _dptr(p), _dptr(out)))
        return out


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))
