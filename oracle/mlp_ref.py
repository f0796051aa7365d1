"""CPU FP64 reference of the learned-closure network -- test infrastructure only.

Checks the library's BF16 tensor-core forward and backward kernels (fjsph_gb300/csrc/mlp.cuh,
mlp_train.cu).  The network has no counterpart in the reference code base; what it restates is
the published mathematics: a 12 -> 64 -> 64 -> 64 -> 2 perceptron with GELU in its tanh form
(Hendrycks & Gimpel 2016), mean-squared-error loss on normalised outputs, and backpropagation.

`bf16=True` rounds to BF16 (round to nearest even) at the points where the device kernels hold
BF16 values: normalised inputs, weights, hidden activations and the back-propagated errors;
everything else is FP64.  `bf16=False` is the exact FP64 network.
"""
from __future__ import annotations

import numpy as np

N_IN, N_IN_PAD, N_HID, N_OUT, N_OUT_PAD = 12, 16, 64, 2, 8
_S = np.sqrt(2.0 / np.pi)
_C = 0.044715


def bf16(a: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    return np.where(np.isfinite(f), out, f.astype(np.float64))


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(_S * (x + _C * x ** 3)))


def gelu_grad(x):
    th = np.tanh(_S * (x + _C * x ** 3))
    return 0.5 * (1.0 + th) + 0.5 * x * (1.0 - th * th) * _S * (1.0 + 3.0 * _C * x * x)


def unpack(p: np.ndarray) -> dict:
    p = np.asarray(p, dtype=np.float64)
    o = 0
    out = {}
    for name, shape in (("W1", (N_HID, N_IN_PAD)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
                        ("W3", (N_HID, N_HID)), ("b3", (N_HID,)), ("W4", (N_OUT_PAD, N_HID)), ("b4", (N_OUT_PAD,)),
                        ("in_shift", (N_IN_PAD,)), ("in_scale", (N_IN_PAD,)), ("out_shift", (N_OUT,)),
                        ("out_scale", (N_OUT,))):
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    out["n_weights"] = sum(int(np.prod(out[k].shape)) for k in ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"))
    return out


def _prep(p: dict, X: np.ndarray, rnd):
    x = np.zeros((X.shape[0], N_IN_PAD))
    # the device normalises in FP32 before rounding to BF16
    xn = (np.asarray(X, np.float32) - p["in_shift"][:N_IN].astype(np.float32)) * p["in_scale"][:N_IN].astype(np.float32)
    x[:, :N_IN] = rnd(xn)
    Ws = [rnd(p[k]) for k in ("W1", "W2", "W3", "W4")]
    bs = [p[k] for k in ("b1", "b2", "b3", "b4")]
    return x, Ws, bs


def forward(params: np.ndarray, X: np.ndarray, bf16_points: bool = True):
    """Outputs (un-normalised) and the intermediate values of the forward pass."""
    rnd = bf16 if bf16_points else (lambda a: np.asarray(a, np.float64))
    p = unpack(params)
    h, Ws, bs = _prep(p, X, rnd)
    Z, H = [], [h]
    for l in range(3):
        z = H[-1] @ Ws[l].T + bs[l]
        Z.append(z)
        H.append(rnd(gelu(z)))
    y = H[-1] @ Ws[3].T + bs[3]
    out = y[:, :N_OUT] * p["out_scale"] + p["out_shift"]
    return out, dict(Z=Z, H=H, y=y, Ws=Ws)


def loss_and_grad(params: np.ndarray, X: np.ndarray, T: np.ndarray, bf16_points: bool = True):
    """Mean over samples of sum over outputs of (y_norm - t_norm)^2, and its gradient w.r.t. the
    trainable parameters (W1, b1, ..., W4, b4 in the library's order)."""
    rnd = bf16 if bf16_points else (lambda a: np.asarray(a, np.float64))
    p = unpack(params)
    n = X.shape[0]
    _, c = forward(params, X, bf16_points)
    tn = (np.asarray(T, np.float64) - p["out_shift"]) / p["out_scale"]
    e = c["y"][:, :N_OUT] - tn
    loss = float(np.sum(e * e) / n)
    dy = np.zeros((n, N_OUT_PAD))
    dy[:, :N_OUT] = 2.0 * e / n
    # mirrors the device: weight gradients and back-propagation take BF16 errors, bias gradients
    # the FP32 ones
    Ws, H, Z = c["Ws"], c["H"], c["Z"]
    gW, gb = [None] * 4, [None] * 4
    dz = dy
    for l in (3, 2, 1, 0):
        dzb = rnd(dz)
        gW[l] = dzb.T @ H[l]
        gb[l] = dz.sum(axis=0)
        if l == 0:
            break
        dz = (dzb @ Ws[l]) * gelu_grad(Z[l - 1])
    g = np.concatenate([gW[0].ravel(), gb[0], gW[1].ravel(), gb[1], gW[2].ravel(), gb[2], gW[3].ravel(), gb[3]])
    return loss, g
