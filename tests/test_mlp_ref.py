"""The CPU FP64 network that checks the learned-closure kernels: pinned by finite differences and
by the BF16 rounding rule (round to nearest, ties to even)."""
import numpy as np

from fjsph_gb300 import closure
from oracle import mlp_ref as m


def _params(seed=1):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(48, 12))
    T = rng.normal(size=(48, 2))
    p = closure.init_params(X, T, seed=seed)
    v = closure.unpack(p)
    v["b1"][:] = rng.normal(0, 0.1, 64)
    v["b3"][:] = rng.normal(0, 0.1, 64)
    v["b4"][:2] = rng.normal(0, 0.1, 2)
    return p, X, T


def test_bf16_rounding_rule():
    one = 1.0
    ulp = 2.0 ** -7  # BF16 spacing at 1
    vals = np.array([one, one + ulp / 2, one + 1.5 * ulp, one + ulp / 2 + 2.0 ** -20, -3.0, 0.0])
    out = m.bf16(vals)
    # ties go to the even mantissa: 1 + ulp/2 -> 1, 1 + 1.5 ulp -> 1 + 2 ulp; above the tie rounds up
    np.testing.assert_array_equal(out, [1.0, 1.0, one + 2 * ulp, one + ulp, -3.0, 0.0])


def test_layout_matches_header_constants():
    assert closure.N_PARAMS == 9964
    assert closure.N_WEIGHTS == m.unpack(np.zeros(closure.N_PARAMS))["n_weights"]


def test_fp64_gradient_matches_finite_differences():
    p, X, T = _params()
    loss, g = m.loss_and_grad(p, X, T, bf16_points=False)
    rng = np.random.default_rng(3)
    idx = rng.choice(closure.N_WEIGHTS, 60, replace=False)
    pp = p.astype(np.float64)
    eps = 1e-6
    for i in idx:
        a, b = pp.copy(), pp.copy()
        a[i] += eps
        b[i] -= eps
        fd = (m.loss_and_grad(a, X, T, False)[0] - m.loss_and_grad(b, X, T, False)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(fd), (i, fd, g[i])
    # padding rows / columns carry no gradient
    v = m.unpack(np.concatenate([g, np.zeros(closure.N_PARAMS - closure.N_WEIGHTS)]))
    assert np.all(v["W1"][:, 12:] == 0.0)
    assert np.all(v["W4"][2:] == 0.0) and np.all(v["b4"][2:] == 0.0)


def test_bf16_points_change_gradient_by_bf16_order():
    p, X, T = _params()
    _, g = m.loss_and_grad(p, X, T, bf16_points=False)
    _, gb = m.loss_and_grad(p, X, T, bf16_points=True)
    rel = np.linalg.norm(g - gb) / np.linalg.norm(g)
    assert 1e-4 < rel < 3e-2
