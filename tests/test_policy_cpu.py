"""The learned proposal's CPU oracle: analytic gradient against finite differences,
and the network layout against the C header."""
import os
import re
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import mlp  # noqa: E402


def _batch(seed, count=40):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1, (count, mlp.IN))
    t = rng.normal(0, 1, (count, mlp.OUT))
    mask = (rng.random((count, mlp.OUT)) < 0.7).astype(float) * rng.choice([1.0, 3.0], (count, mlp.OUT))
    sc = np.concatenate([rng.normal(0, 0.3, mlp.IN), rng.uniform(0.5, 2, mlp.IN), rng.normal(0, 0.3, mlp.OUT),
                         rng.uniform(0.5, 2, mlp.OUT)])
    return x, t, mask, sc


def test_layout_matches_header():
    text = open(os.path.join(ROOT, "include", "sdpg.h")).read()
    vals = {k: int(v) for k, v in re.findall(r"#define SDPG_POLICY_(\w+) (\d+)", text)}
    assert vals["INPUTS"] == mlp.IN and vals["OUTPUTS"] == mlp.OUT
    assert vals["PARAMS"] == mlp.N_PARAMS == 8898
    assert vals["SCALE"] == mlp.N_SCALE


def test_gradient_matches_finite_differences():
    x, t, mask, sc = _batch(1)
    w = mlp.glorot_params(2)
    loss, g = mlp.loss_and_grad(w, sc, x, t, mask)
    assert loss > 0
    rng = np.random.default_rng(3)
    # every bias and a sample of every weight matrix
    idx = np.unique(np.concatenate([rng.integers(0, mlp.N_PARAMS, 200), np.arange(mlp.N_PARAMS - 2, mlp.N_PARAMS)]))
    fd = mlp.finite_difference(w, sc, x, t, mask, idx)
    scale = np.max(np.abs(g))
    assert np.max(np.abs(fd - g[idx])) <= 1e-7 * scale + 1e-10


def test_masked_outputs_carry_no_gradient():
    x, t, mask, sc = _batch(4)
    mask[:, 1] = 0.0
    w = mlp.glorot_params(5)
    _, g1 = mlp.loss_and_grad(w, sc, x, t, mask)
    t2 = t.copy()
    t2[:, 1] += 100.0  # targets of a masked output do not matter
    _, g2 = mlp.loss_and_grad(w, sc, x, t2, mask)
    assert np.array_equal(g1, g2)
    p = mlp.unpack(g1)
    assert np.all(p["W4"][1] == 0) and p["b4"][1] == 0


def test_adam_first_step_is_signed_learning_rate():
    g = np.array([1e-2, -3.0, 5e-4])
    w, m1, m2 = mlp.adam_step(np.zeros(3), g, np.zeros(3), np.zeros(3), 1, lr=1e-3)
    assert np.allclose(w, -1e-3 * np.sign(g), rtol=1e-4)
