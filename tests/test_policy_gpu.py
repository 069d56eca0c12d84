"""The learned proposal's CUDA kernels against the CPU oracle (forward, gradient, Adam,
training), and the solver hook: proposals that equal the defaults change nothing, a
proposal that fails its checks falls back to the reference's beta, and the committed
policy solves held-out instances of its family to the default solver's optimum."""
import importlib
import os

import numpy as np
import pytest

from oracle import mlp

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def learned(sdpg):
    return importlib.import_module("sdpa-gmp_gb300.learned")


def _data(seed, count):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 2, (count, mlp.IN)).astype(np.float32)
    t = rng.normal(0, 1, (count, mlp.OUT)).astype(np.float32)
    mask = ((rng.random((count, mlp.OUT)) < 0.7) * rng.choice([1.0, 4.0], (count, mlp.OUT))).astype(np.float32)
    sc = np.concatenate([rng.normal(0, 0.3, mlp.IN), rng.uniform(0.5, 2, mlp.IN), rng.normal(0, 0.3, mlp.OUT),
                         rng.uniform(0.5, 2, mlp.OUT)]).astype(np.float32)
    return x, t, mask, sc


def _policy(sdpg, seed):
    w = mlp.glorot_params(seed).astype(np.float32)
    pol = sdpg.Policy()
    return pol, w


@pytest.mark.parametrize("count", [1, 31, 100])
def test_forward_matches_oracle(sdpg, count):
    x, _, _, sc = _data(10 + count, count)
    pol, w = _policy(sdpg, 11)
    pol.set(w, sc)
    y = pol.forward(x)
    ref = mlp.forward(w.astype(np.float64), sc.astype(np.float64), x.astype(np.float64))
    # FP32 against FP64: three tanh layers of 64-term sums
    assert np.max(np.abs(y - ref)) <= 2e-5 * max(1.0, np.max(np.abs(ref)))
    w2, sc2 = pol.get()
    assert np.array_equal(w2, w) and np.array_equal(sc2, sc)


@pytest.mark.parametrize("count", [7, 100])
def test_gradient_matches_oracle(sdpg, count):
    x, t, mask, sc = _data(20 + count, count)
    pol, w = _policy(sdpg, 21)
    pol.set(w, sc)
    g, loss = pol.gradient(x, t, mask)
    rloss, rg = mlp.loss_and_grad(w.astype(np.float64), sc.astype(np.float64), x.astype(np.float64),
                                  t.astype(np.float64), mask.astype(np.float64))
    assert abs(loss - rloss) <= 1e-5 * rloss
    # FP32 gradients accumulated by atomics over 32-sample tiles
    assert np.max(np.abs(g - rg)) <= 1e-4 * np.max(np.abs(rg))


def test_one_adam_step_matches_oracle(sdpg):
    x, t, mask, sc = _data(30, 64)
    pol, w = _policy(sdpg, 31)
    pol.set(w, sc)
    lr = 1e-3
    pol.train(x, t, mask, epochs=1, batch=64, lr=lr, seed=0)  # one batch = one step
    w1, _ = pol.get()
    _, rg = mlp.loss_and_grad(w.astype(np.float64), sc.astype(np.float64), x.astype(np.float64),
                              t.astype(np.float64), mask.astype(np.float64))
    rw, _, _ = mlp.adam_step(w.astype(np.float64), rg, np.zeros_like(rg), np.zeros_like(rg), 1, lr)
    big = np.abs(rg) > 1e-4 * np.max(np.abs(rg))  # where the step's sign is well defined
    assert np.max(np.abs(w1 - rw)[big]) <= 1e-3 * lr + 1e-7
    assert np.max(np.abs(w1 - w)) <= lr * (1 + 1e-3) + 1e-7


def test_training_fits_a_smooth_target(sdpg):
    rng = np.random.default_rng(40)
    x = rng.uniform(-1, 1, (2048, mlp.IN)).astype(np.float32)
    t = np.stack([np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2], 0.5 * np.tanh(x[:, 3] - x[:, 4]) + x[:, 5]], 1)
    mask = np.ones_like(t)
    pol, _ = _policy(sdpg, 41)
    sc = np.concatenate([np.zeros(6), np.ones(6), np.zeros(2), np.ones(2)]).astype(np.float32)
    pol.set(scale=sc)
    losses = pol.train(x, t.astype(np.float32), mask, epochs=60, batch=128, lr=3e-3, seed=1)
    assert losses[-1] < 0.05 * losses[0]
    y = pol.forward(x[:256])
    assert np.mean((y - t[:256]) ** 2) < 0.02


def _constant_policy(sdpg, lam, beta):
    """All weights zero: outputs are the scaling's means (log10 lambda, beta)."""
    pol = sdpg.Policy()
    sc = np.concatenate([np.zeros(6), np.ones(6), [np.log10(lam), beta], [1.0, 1.0]]).astype(np.float32)
    pol.set(np.zeros(sdpg.POLICY_PARAMS, np.float32), sc)
    return pol


def test_default_valued_proposals_leave_the_solve_unchanged(sdpg, learned):
    prob = learned.instance(7)
    prm = learned.param()
    base = learned.solve(prob, prm)
    # lambdaStar = the default, beta = 1.0: every corrector beta proposal is then checked
    # and either kept or replaced; with lambda only, the solve must match exactly
    pol = _constant_policy(sdpg, prm.lambdaStar, 0.1)
    s = sdpg.Solver(prob, prm)
    s.set_policy(pol, beta=False, lam=True)
    s.run()
    st = s.policy_stats()
    assert st["proposals"] == 0 and abs(st["lambda_proposed"] - prm.lambdaStar) <= 1e-3 * prm.lambdaStar
    hist = s.history()
    s.close()
    assert hist.shape == base["history"].shape
    assert np.allclose(hist, base["history"], rtol=1e-12, atol=0)


def test_bad_beta_proposals_fall_back(sdpg, learned):
    """beta = 1 stalls mu: the gap check rejects every such proposal in the feasible
    phase, and the solve still reaches the default optimum."""
    prob = learned.instance(8)
    base = learned.solve(prob, learned.param())
    pol = _constant_policy(sdpg, learned.param().lambdaStar, 1.0)
    r = learned.solve(prob, learned.param(), policy=pol)
    assert r["phase"] == "pdOPT"
    assert r["policy"]["fallbacks"] > 0
    assert learned.objective_rel_error(r, base) <= 1e-25


def test_features_rows_follow_the_history(sdpg, learned):
    r = learned.solve(learned.instance(9), learned.param())
    f, h = r["features"], r["history"]
    assert f.shape == (h.shape[0] + 1, 6)
    assert np.isclose(f[0, 0], 8.0, atol=1e-6)  # log10 mu0 = log10 lambdaStar^2 at lambdaStar 1e4
    assert np.allclose(f[1:, 5], h[:, 8], rtol=1e-6)  # the rule's beta is what the default run used


def test_committed_policy_on_held_out_seeds(sdpg, learned):
    path = learned.POLICY_FILE
    if not os.path.exists(path):
        pytest.skip("no trained policy committed")
    pol = sdpg.Policy.load(path)
    ev = learned.evaluate(pol, range(learned.HOLDOUT_BASE + 500, learned.HOLDOUT_BASE + 506), workers=3)
    assert all(r["default_phase"] == "pdOPT" for r in ev["rows"])
    # the plain solver's optimum judges the learned path's error
    assert ev["max_objective_rel_error"] <= 1e-25
    assert ev["mean_iterations_learned"] < ev["mean_iterations_default"]
