"""Learned aerodynamic closure: parameter set-up, GPU training, sample collection.

The network (12 -> 64 -> 64 -> 64 -> 2, GELU, BF16 weights, FP32 accumulation) replaces the Gissler
occlusion factor and drag coefficient of the plain closure (src/Aero.h:37-98, occlusion from
src/Geometry.cpp:233-255) inside the split-precision residual.  Its inputs and outputs per particle
are documented in fjsph_gb300/csrc/closure.cuh.  Everything here calls the C ABI: training runs on
the GPU through the library's own forward/backward kernels.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _cdefs as d
from ._lib import check, lib

N_IN, N_IN_PAD, N_HID, N_OUT, N_OUT_PAD = 12, 16, 64, 2, 8
INPUT_NAMES = ["occ_up_sum", "occ_down_sum", "occ_sq_sum", "occ_max", "n_neigh_frac", "log_speed", "log_We",
               "log_Re", "normal_mag", "normal_dot_wind", "lam_nb", "lam"]
OUTPUT_NAMES = ["log10_CdA", "woccl"]

# offsets of the parameter vector (include/fjsph_gb300.h)
O_W1 = 0
O_B1 = O_W1 + N_HID * N_IN_PAD
O_W2 = O_B1 + N_HID
O_B2 = O_W2 + N_HID * N_HID
O_W3 = O_B2 + N_HID
O_B3 = O_W3 + N_HID * N_HID
O_W4 = O_B3 + N_HID
O_B4 = O_W4 + N_OUT_PAD * N_HID
N_WEIGHTS = O_B4 + N_OUT_PAD
O_IN_SHIFT = N_WEIGHTS
O_IN_SCALE = O_IN_SHIFT + N_IN_PAD
O_OUT_SHIFT = O_IN_SCALE + N_IN_PAD
O_OUT_SCALE = O_OUT_SHIFT + N_OUT
N_PARAMS = O_OUT_SCALE + N_OUT


def _f(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def unpack(params: np.ndarray) -> dict:
    """Named views (W1 [64,16], b1, W2, b2, W3, b3, W4 [8,64], b4, in_shift, in_scale, out_shift,
    out_scale) of a parameter vector."""
    p = np.asarray(params)
    return dict(
        W1=p[O_W1:O_B1].reshape(N_HID, N_IN_PAD), b1=p[O_B1:O_W2],
        W2=p[O_W2:O_B2].reshape(N_HID, N_HID), b2=p[O_B2:O_W3],
        W3=p[O_W3:O_B3].reshape(N_HID, N_HID), b3=p[O_B3:O_W4],
        W4=p[O_W4:O_B4].reshape(N_OUT_PAD, N_HID), b4=p[O_B4:N_WEIGHTS],
        in_shift=p[O_IN_SHIFT:O_IN_SCALE], in_scale=p[O_IN_SCALE:O_OUT_SHIFT],
        out_shift=p[O_OUT_SHIFT:O_OUT_SCALE], out_scale=p[O_OUT_SCALE:N_PARAMS])


def init_params(X: np.ndarray, T: np.ndarray, seed: int = 0) -> np.ndarray:
    """Normalisation from the samples (mean / standard deviation per input and output) and a
    seeded LeCun-normal initialisation of the weights; padding rows and columns stay zero."""
    if lib().fjsph_mlp_num_params() != N_PARAMS:
        raise RuntimeError("parameter layout of the library and of fjsph_gb300.closure differ")
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.zeros(N_PARAMS, dtype=np.float32)
    v = unpack(p)
    v["W1"][:, :N_IN] = rng.normal(0.0, 1.0 / np.sqrt(N_IN), (N_HID, N_IN))
    v["W2"][:] = rng.normal(0.0, 1.0 / np.sqrt(N_HID), (N_HID, N_HID))
    v["W3"][:] = rng.normal(0.0, 1.0 / np.sqrt(N_HID), (N_HID, N_HID))
    v["W4"][:N_OUT] = rng.normal(0.0, 1.0 / np.sqrt(N_HID), (N_OUT, N_HID))
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    mu, sd = X.mean(axis=0), X.std(axis=0)
    v["in_shift"][:N_IN] = mu
    v["in_scale"][:N_IN] = np.where(sd > 1e-6, 1.0 / np.maximum(sd, 1e-6), 1.0)
    v["in_scale"][N_IN:] = 1.0
    tm, ts = T.mean(axis=0), T.std(axis=0)
    v["out_shift"][:] = tm
    v["out_scale"][:] = np.maximum(ts, 1e-3)
    return p


def forward(params: np.ndarray, X: np.ndarray) -> np.ndarray:
    """Network outputs for the rows of X (GPU, the library's inference kernel)."""
    p = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    Y = np.empty((X.shape[0], N_OUT), dtype=np.float32)
    check("fjsph_mlp_forward", lib().fjsph_mlp_forward(_f(p), _f(X), X.shape[0], _f(Y)))
    return Y


def gradient(params: np.ndarray, X: np.ndarray, T: np.ndarray) -> tuple[np.ndarray, float]:
    """Mean-squared-error loss (normalised outputs) and its gradient w.r.t. the trainable part."""
    p = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    g = np.empty(N_WEIGHTS, dtype=np.float32)
    loss = C.c_double()
    check("fjsph_mlp_gradient", lib().fjsph_mlp_gradient(_f(p), _f(X), _f(T), X.shape[0], _f(g), C.byref(loss)))
    return g, loss.value


def train(params: np.ndarray, X: np.ndarray, T: np.ndarray, epochs: int = 20, batch: int = 4096,
          lr: float = 2e-3, seed: int = 0) -> tuple[np.ndarray, float]:
    """Adam on the GPU; returns the trained parameters and the last epoch's mean loss."""
    p = np.array(params, dtype=np.float32, copy=True)
    X = np.ascontiguousarray(X, dtype=np.float32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    loss = C.c_double()
    check("fjsph_mlp_train", lib().fjsph_mlp_train(_f(p), _f(X), _f(T), X.shape[0], int(epochs), int(batch),
                                                   float(lr), int(seed), C.byref(loss)))
    return p, loss.value


def plain_closure_outputs(T: np.ndarray) -> np.ndarray:
    """The targets are the plain closure's own outputs (log10 Cd A / A_sphere, woccl)."""
    return np.asarray(T)


def aero_scale(Y: np.ndarray) -> np.ndarray:
    """Force factor Cd_i A_i (1 - woccl) / A_sphere of closure outputs Y[:, 2]."""
    Y = np.asarray(Y, dtype=np.float64)
    return 10.0 ** Y[:, 0] * (1.0 - np.clip(Y[:, 1], 0.0, 1.0))


@dataclass
class JetSpec:
    n_target: int
    jet_speed: float
    air_speed: float
    seed: int
    D: float = 2e-3
    live: bool = False  # config 2 as specified: live inlet and power-law crossflow


def jet_specs(n_runs: int, n_target: int, seed: int = 0, D: float = 2e-3, live: bool = False) -> list[JetSpec]:
    """Seeded jet-in-crossflow runs with jet speed ~ U(5, 20) m/s and crossflow ~ U(30, 80) m/s."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return [JetSpec(n_target, float(rng.uniform(5.0, 20.0)), float(rng.uniform(30.0, 80.0)),
                    int(rng.integers(1 << 30)), D, live) for _ in range(n_runs)]


def jet_case(sp: JetSpec, closure: int = d.CLOSURE_PLAIN):
    """The split-precision jet of a spec, with the given closure selected: the live-inlet jet in
    the power-law crossflow (cases.jet_crossflow_live) or the static jet (cases.jet_crossflow)."""
    from .cases import jet_crossflow, jet_crossflow_live
    if sp.live:
        c = jet_crossflow_live(n_target=sp.n_target, D=sp.D, jet_speed=sp.jet_speed, air_speed=sp.air_speed,
                               seed=sp.seed, cap=sp.n_target)
    else:
        c = jet_crossflow(n_target=sp.n_target, D=sp.D, jet_speed=sp.jet_speed, air_speed=sp.air_speed,
                          seed=sp.seed)
    c.settings.precision = d.PREC_MIXED
    c.settings.aero_closure = closure
    return c


def collect_samples(specs: list[JetSpec], n_samples: int, steps: int = 6, capacity: int | None = None,
                    every: int = 1) -> tuple[np.ndarray, np.ndarray]:
    """Inputs and targets logged from plain-closure runs of the split-precision form (GPU): each
    spec runs `steps` integrate() steps with logging every `every` steps, until n_samples are held."""
    from .api import Context
    Xs, Ts, held = [], [], 0
    for sp in specs:
        c = jet_case(sp)
        cap = c.settings.max_points + 1024 if c.inlets else c.state.n + 64  # room for insertions
        ctx = Context(c.settings, cap, c.blocks, c.inlets)
        try:
            if c.power_law_params:
                ctx.air_power_law(*c.power_law_params)
            ctx.set_states(c.state, c.state)
            ctx.closure_log(capacity or 4 * c.state.n, every)
            for _ in range(steps):
                ctx.integrate()
                if held + int(ctx.closure_report()["logged"]) >= n_samples:
                    break
            X, T = ctx.closure_log_read(reset=True)
        finally:
            ctx.close()
        Xs.append(X)
        Ts.append(T)
        held += len(X)
        if held >= n_samples:
            break
    X = np.concatenate(Xs)[:n_samples]
    T = np.concatenate(Ts)[:n_samples]
    return X, T
