"""Host-side particle state (SPHState, src/Var.h:499-642) as numpy structure-of-arrays.

Vector fields have shape (n, dim), the renormalisation matrix L has shape (n, dim, dim), scalar
fields shape (n,).  Particle order is the reference's: boundary blocks first, then fluid blocks.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._cdefs import VIEW_F64, VIEW_I32, VIEW_I64, StateView, Block, DEFAULT_VAL, MAX_TIMES

# the fields a step reads before writing them (FJSPH_STEP_FIELDS of the C header)
STEP_FIELDS = ("xi", "v", "acc", "Rrho", "rho", "p", "m", "cellV", "cellP", "cellRho", "vPert", "aVisc", "deltaD",
               "woccl", "lam", "lam_nb", "curve", "norm", "norm_curve", "b", "part_id", "cellID", "surf", "surfzone")

VECTOR_FIELDS = ["xi", "v", "acc", "Af", "aVisc", "cellV", "gradRho", "norm", "vPert"]
MATRIX_FIELDS = ["L"]
SCALAR_FIELDS = ["Rrho", "rho", "p", "m", "curve", "norm_curve", "woccl", "pDist", "deltaD", "cellP", "cellRho",
                 "colourG", "colour", "lam", "lam_nb", "kernsum"]
INT64_FIELDS = list(VIEW_I64)
INT32_FIELDS = list(VIEW_I32)
ALL_FIELDS = VECTOR_FIELDS + MATRIX_FIELDS + SCALAR_FIELDS + INT64_FIELDS + INT32_FIELDS


class SPHState:
    """Structure-of-arrays particle state with the reference's field names."""

    def __init__(self, n: int, dim: int):
        self.n = int(n)
        self.dim = int(dim)
        for f in VECTOR_FIELDS:
            setattr(self, f, np.zeros((n, dim), dtype=np.float64))
        self.L = np.zeros((n, dim, dim), dtype=np.float64)
        for f in SCALAR_FIELDS:
            setattr(self, f, np.zeros(n, dtype=np.float64))
        self.part_id = np.arange(n, dtype=np.int64)
        self.cellID = np.full(n, -3, dtype=np.int64)  # c_no_cell
        for f in INT32_FIELDS:
            setattr(self, f, np.zeros(n, dtype=np.int32))

    def copy(self) -> "SPHState":
        out = SPHState.__new__(SPHState)
        out.n, out.dim = self.n, self.dim
        for f in ALL_FIELDS:
            setattr(out, f, getattr(self, f).copy())
        return out

    def view(self, fields=None) -> StateView:
        """ctypes view over this state's arrays (valid while the arrays are alive and unchanged);
        with `fields`, only those names (the others stay null: transfers skip them)."""
        v = StateView()
        v.n = self.n
        if fields is not None:
            unknown = set(fields) - set(VIEW_F64) - set(VIEW_I64) - set(VIEW_I32)
            if unknown:
                raise KeyError(f"unknown state fields {sorted(unknown)}")
        for f in VIEW_F64:
            if fields is not None and f not in fields:
                continue
            a = getattr(self, f)
            assert a.dtype == np.float64 and a.flags.c_contiguous
            setattr(v, f, a.ctypes.data_as(C.POINTER(C.c_double)))
        for f in VIEW_I64:
            if fields is not None and f not in fields:
                continue
            a = getattr(self, f)
            assert a.dtype == np.int64 and a.flags.c_contiguous
            setattr(v, f, a.ctypes.data_as(C.POINTER(C.c_int64)))
        for f in VIEW_I32:
            if fields is not None and f not in fields:
                continue
            a = getattr(self, f)
            assert a.dtype == np.int32 and a.flags.c_contiguous
            setattr(v, f, a.ctypes.data_as(C.POINTER(C.c_int32)))
        return v

    def take(self, idx) -> "SPHState":
        out = SPHState.__new__(SPHState)
        out.dim = self.dim
        for f in ALL_FIELDS:
            setattr(out, f, np.ascontiguousarray(getattr(self, f)[idx]))
        out.n = len(out.rho)
        return out


@dataclass
class BlockSpec:
    """One LIMITS entry (src/Var.h:820-881) in Python form."""

    first: int
    second: int
    is_fluid: bool
    name: str = ""
    bound_solver: int = 1  # pressure_G, the default of src/shapes/shapes.h:33
    no_slip: int = 0
    block_type: int = 1  # squareCube
    fixed_vel_or_dynamic: int = 0
    times: list = field(default_factory=list)
    vels: list = field(default_factory=lambda: [(0.0, 0.0, 0.0)])
    delete_norm: tuple = (DEFAULT_VAL, DEFAULT_VAL, DEFAULT_VAL)
    delconst: float = DEFAULT_VAL
    insert_norm: tuple = (DEFAULT_VAL, DEFAULT_VAL, DEFAULT_VAL)
    insconst: float = DEFAULT_VAL
    aero_norm: tuple = (DEFAULT_VAL, DEFAULT_VAL, DEFAULT_VAL)
    aeroconst: float = DEFAULT_VAL

    def to_c(self) -> Block:
        b = Block()
        b.first, b.second = self.first, self.second
        b.is_fluid = int(self.is_fluid)
        b.bound_solver, b.no_slip, b.block_type = self.bound_solver, self.no_slip, self.block_type
        b.fixed_vel_or_dynamic = self.fixed_vel_or_dynamic
        b.n_times = len(self.times)
        if b.n_times > MAX_TIMES:
            raise ValueError("boundary motion table longer than FJSPH_MAX_TIMES")
        for t, tv in enumerate(self.times):
            b.times[t] = tv
        for t, vel in enumerate(self.vels[:MAX_TIMES]):
            for k, x in enumerate(vel):
                b.vels[t][k] = x
        for k in range(3):
            b.delete_norm[k] = self.delete_norm[k] if k < len(self.delete_norm) else 0.0
            b.insert_norm[k] = self.insert_norm[k] if k < len(self.insert_norm) else 0.0
            b.aero_norm[k] = self.aero_norm[k] if k < len(self.aero_norm) else 0.0
        b.delconst, b.insconst, b.aeroconst = self.delconst, self.insconst, self.aeroconst
        return b


@dataclass
class InletSpec:
    """Inlet back/buffer tables of one inletZone block (src/shapes/inlet.cpp)."""

    block: int
    back: np.ndarray  # (n_back,) reference indices
    buffer: np.ndarray  # (n_back, depth) reference indices


def blocks_to_c(blocks: list[BlockSpec]):
    arr = (Block * len(blocks))()
    for i, b in enumerate(blocks):
        arr[i] = b.to_c()
    return arr
