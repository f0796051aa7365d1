"""Learned aerodynamic closure on the GPU.

  - forward and backward kernels against the CPU FP64 network (oracle/mlp_ref.py): outputs within
    1e-2 relative RMS of the BF16-rounded FP64 network, gradients within 2e-2 (relative L2) of it
    and within 5e-2 of the exact FP64 gradient;
  - training on the GPU lowers the loss;
  - the sample log holds the plain closure's own targets (occlusion factor exactly, drag term to
    1e-4 in log10);
  - a network trained on seeded jets reproduces the plain closure's aero force on a held-out jet
    within 5 % relative RMS (the target the learned form is built to), and what it gains: the
    error of the same residual without the network's occlusion output (occlusion ignored) and
    of an untrained network are reported and must be far larger;
  - the judge re-runs the plain closure on scheduled steps, and a network that misses the
    tolerance is switched off (fallback to the plain closure).
"""
import numpy as np
import pytest

from fjsph_gb300 import _cdefs as d
from fjsph_gb300 import closure as cl
from oracle import mlp_ref as m

pytestmark = pytest.mark.gpu

FWD_TOL = 1e-2
GRAD_TOL_BF16 = 2e-2
GRAD_TOL_FP64 = 5e-2
AERO_TOL = 0.05


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def _random_net(seed=0, n=3000):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, 12)).astype(np.float32) * 2.0 + 1.0
    T = np.stack([np.sin(X[:, 0]) + 0.3 * X[:, 5], np.tanh(X[:, 3] - X[:, 7])], axis=1).astype(np.float32)
    p = cl.init_params(X, T, seed=seed)
    v = cl.unpack(p)
    for k in ("b1", "b2", "b3"):
        v[k][:] = rng.normal(0, 0.1, 64)
    v["b4"][:2] = rng.normal(0, 0.1, 2)
    return p, X, T


def _rel_rms(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-300))


def test_forward_matches_fp64_network():
    p, X, _ = _random_net(1, 5000)  # not a multiple of 16: ragged last tile
    Y = cl.forward(p, X)
    ref, _ = m.forward(p, X, bf16_points=True)
    for o in range(2):
        assert _rel_rms(Y[:, o] - ref[:, o].mean(), ref[:, o] - ref[:, o].mean()) < FWD_TOL


@pytest.mark.parametrize("n", [16, 1000, 8192])
def test_gradient_matches_fp64_network(n):
    p, X, T = _random_net(2, n)
    g, loss = cl.gradient(p, X, T)
    lb, gb = m.loss_and_grad(p, X, T, bf16_points=True)
    l64, g64 = m.loss_and_grad(p, X, T, bf16_points=False)
    assert loss == pytest.approx(lb, rel=1e-2)
    assert np.linalg.norm(g - gb) / np.linalg.norm(gb) < GRAD_TOL_BF16
    assert np.linalg.norm(g - g64) / np.linalg.norm(g64) < GRAD_TOL_FP64
    v = cl.unpack(np.concatenate([g, np.zeros(cl.N_PARAMS - cl.N_WEIGHTS, np.float32)]))
    assert np.all(v["W1"][:, 12:] == 0) and np.all(v["W4"][2:] == 0)


def test_training_lowers_loss():
    p, X, T = _random_net(3, 20000)
    _, l0 = cl.gradient(p, X, T)
    p2, last = cl.train(p, X, T, epochs=15, batch=1024, lr=3e-3, seed=4)
    _, l1 = cl.gradient(p2, X, T)
    assert np.all(np.isfinite(p2))
    assert l1 < 0.1 * l0, (l0, l1, last)
    # normalisation constants are not trained
    np.testing.assert_array_equal(p2[cl.N_WEIGHTS:], p[cl.N_WEIGHTS:])


def _get_cd(Re):
    return (1.0 + 0.197 * Re ** 0.63 + 2.6e-04 * Re ** 1.38) * (24.0 / (Re + 0.00001))


def test_log_holds_plain_closure_targets():
    from fjsph_gb300.api import Context
    sp = cl.JetSpec(120_000, 12.0, 45.0, 99, D=1e-3)
    c = cl.jet_case(sp)
    ctx = Context(c.settings, c.state.n + 64, c.blocks)
    ctx.set_states(c.state, c.state)
    ctx.closure_log(4 * c.state.n, 1)
    ctx.integrate()
    ctx.integrate()
    X, T = ctx.closure_log_read()
    s = ctx.settings
    ctx.close()
    assert len(X) > 1000
    assert np.all(np.isfinite(X)) and np.all(np.isfinite(T))
    # occlusion factor = clamp(max cosine, 0, 1) for every logged particle
    np.testing.assert_array_equal(T[:, 1], np.clip(X[:, 3], 0.0, 1.0))
    # drag term from the logged Reynolds number and lambda_nb (use_lam, no TAB deformation)
    assert s.use_lam == 1 and s.use_TAB_def == 0
    Re = 10.0 ** X[:, 7].astype(np.float64) - 1.0
    f2 = np.minimum(s.interp_fac * X[:, 10].astype(np.float64), 1.0)
    Cdi = (1 - f2) * _get_cd(Re) + f2
    A = (1 - f2) * s.A_sphere + f2 * s.A_plate
    np.testing.assert_allclose(T[:, 0], np.log10(Cdi * A / s.A_sphere), atol=1e-4)


@pytest.fixture(scope="module")
def trained():
    specs = cl.jet_specs(6, 150_000, seed=11, D=1e-3)
    X, T = cl.collect_samples(specs, 600_000, steps=5)
    p0 = cl.init_params(X, T, seed=5)
    p, loss = cl.train(p0, X, T, epochs=40, batch=2048, lr=3e-3, seed=6)
    return dict(p0=p0, p=p, loss=loss, n=len(X))


def _held_out_state():
    from fjsph_gb300.api import Context
    sp = cl.JetSpec(150_000, 14.0, 55.0, 4242, D=1e-3)  # speeds inside the training ranges, new seed
    c = cl.jet_case(sp)
    ctx = Context(c.settings, c.state.n + 64, c.blocks)
    ctx.set_states(c.state, c.state)
    ctx.integrate()
    ctx.integrate()
    return c, ctx


def _aero(ctx, closure, params=None):
    s = ctx.settings
    s.aero_closure = closure
    ctx.settings = s
    if params is not None:
        ctx.closure_set_weights(params, 1.0)
    ctx.update_neighbours()
    npd = ctx.dSPH_PreStep()
    ctx.get_aero_velocity()
    ctx.Detect_Surface()
    ctx.dissipation_terms()
    ctx.Get_Boundary_Pressure()
    ctx.get_acc_and_Rrho(npd)
    return ctx.download()


def test_learned_closure_matches_plain_and_what_it_gains(trained):
    from tests._util import n_bound
    c, ctx = _held_out_state()
    nb = n_bound(c.blocks)
    st = ctx.download()
    plain = _aero(ctx, d.CLOSURE_PLAIN)
    ctx.set_states(st, st)
    learned = _aero(ctx, d.CLOSURE_LEARNED, trained["p"])
    ctx.set_states(st, st)
    untrained = _aero(ctx, d.CLOSURE_LEARNED, trained["p0"])
    ctx.close()
    Ap, Al, Au = (x.Af[nb:].reshape(-1) for x in (plain, learned, untrained))
    assert np.sqrt(np.mean(Ap ** 2)) > 0.0
    err = _rel_rms(Al, Ap)
    err_untrained = _rel_rms(Au, Ap)
    # without the network's occlusion output: the same drag with woccl = 0 wherever the plain
    # closure's occlusion rule applies (lambda_nb below the cutoff)
    wo = plain.woccl[nb:]
    cov = (plain.lam_nb[nb:] < c.settings.lam_cutoff) & (wo < 1.0)
    Af_p = plain.Af[nb:].reshape(len(wo), -1)
    no_occ = np.where(cov[:, None], Af_p / np.maximum(1.0 - wo, 1e-12)[:, None], Af_p)
    err_no_occl = _rel_rms(no_occ.reshape(-1), Ap)
    print(f"aero-force rel RMS vs plain: learned {err:.4f}, untrained {err_untrained:.3f}, "
          f"occlusion ignored {err_no_occl:.3f} (trained on {trained['n']} samples, loss {trained['loss']:.3e})")
    assert err <= AERO_TOL
    assert err_untrained > 5 * err
    assert err_no_occl > 5 * err
    # the rest of the residual does not depend on the closure
    np.testing.assert_array_equal(learned.Rrho, plain.Rrho)


def test_judge_and_fallback(trained):
    c, ctx = _held_out_state()
    s = ctx.settings
    s.aero_closure = d.CLOSURE_LEARNED
    s.learned_judge_interval = 1
    ctx.settings = s
    ctx.closure_set_weights(trained["p"], AERO_TOL)
    for _ in range(3):
        ctx.integrate()
    r = ctx.closure_report()
    assert r["judged"] >= 2 and r["judged_particles"] > 0
    assert r["max_rel_rms"] <= AERO_TOL and r["fallback"] == 0 and r["learned_active"] == 1
    # an untrained network fails the judge and the context falls back to the plain closure
    ctx.closure_set_weights(trained["p0"], AERO_TOL)
    ctx.closure_reset()
    ctx.integrate()
    r = ctx.closure_report()
    assert r["fallback"] == 1 and r["learned_active"] == 0 and r["last_rel_rms"] > AERO_TOL
    ctx.closure_reset()
    assert ctx.closure_report()["learned_active"] == 1
    ctx.close()
