"""Shared helpers of the parity tests: matched oracle / device pairs and field comparison."""
from __future__ import annotations

import os
from pathlib import Path

import numpy as np

from fjsph_gb300 import _cdefs as d
from fjsph_gb300.state import SPHState


def perturb(st: SPHState, seed: int, vscale: float, xscale: float, fluid_from: int) -> SPHState:
    """Seeded random velocity and position noise on the fluid particles (makes every branch of the
    pair terms active: approaching and receding pairs, non-zero shifting, occlusion)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = st.copy()
    nf = st.n - fluid_from
    out.v[fluid_from:] += rng.normal(0.0, vscale, size=(nf, st.dim))
    out.xi[fluid_from:] += rng.uniform(-xscale, xscale, size=(nf, st.dim))
    out.rho[fluid_from:] *= 1.0 + rng.uniform(-2e-3, 2e-3, size=nf)
    return out


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max |a-b| / max(|b|, tiny) over all entries."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.max(np.abs(b)) if b.size else 0.0, 1e-300)
    return float(np.max(np.abs(a - b)) / scale) if b.size else 0.0


def rel_rms(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    den = np.sqrt(np.mean(b * b)) if b.size else 0.0
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(den, 1e-300)) if b.size else 0.0


def assert_fields(a: SPHState, b: SPHState, fields, rtol: float, sl=slice(None), label=""):
    bad = []
    for f in fields:
        x, y = getattr(a, f)[sl], getattr(b, f)[sl]
        e = rel_err(x, y)
        if not np.all(np.isfinite(x)) or e > rtol:
            bad.append(f"{f}: rel err {e:.3e}")
    assert not bad, f"{label} mismatches (rtol {rtol:g}): " + "; ".join(bad)


def assert_ints(a: SPHState, b: SPHState, fields, sl=slice(None), max_frac=0.0, label=""):
    for f in fields:
        x, y = getattr(a, f)[sl], getattr(b, f)[sl]
        diff = np.count_nonzero(x != y)
        assert diff <= max_frac * max(len(x), 1), f"{label} {f}: {diff} of {len(x)} differ"


def n_bound(blocks) -> int:
    return sum(b.second - b.first for b in blocks if not b.is_fluid)


def hydrostatic_error(st: SPHState, fluid_from: int, rho_rest: float, top: float, g: float = 9.81) -> float:
    """RMS over depth bins of p / (rho g H) - depth / H (Examples/Standing_Column/Ideal.dat is the
    line through (0, 0) and (1, 1)); bins away from the free surface and the floor."""
    y, p = st.xi[fluid_from:, 1], st.p[fluid_from:]
    depth = (top - y) / top
    pn = p / (rho_rest * g * top)
    bins = np.linspace(0.1, 0.95, 12)
    idx = np.digitize(depth, bins)
    err = [np.mean(pn[idx == k]) - np.mean(depth[idx == k])
           for k in range(1, len(bins)) if np.count_nonzero(idx == k) > 10]
    return float(np.sqrt(np.mean(np.square(err))))


def reference_examples() -> Path | None:
    """The reference's Examples folder, named by the FJSPH_REFERENCE_EXAMPLES environment variable;
    None when the variable is unset or names no folder (the tests that read it then skip)."""
    p = os.environ.get("FJSPH_REFERENCE_EXAMPLES")
    return Path(p) if p and Path(p).is_dir() else None
