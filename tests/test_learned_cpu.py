"""Host side of the learned proposal: the family's generator, the dataset built from
traces, the standardisation, and the objective comparison used to accept a run."""
import importlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
learned = importlib.import_module("sdpa-gmp_gb300.learned")
problems = importlib.import_module("sdpa-gmp_gb300.problems")


def _run(iters, lam, beta_rule, phase="pdOPT", obj="-1.2345678901234567890123456789012345678901e+02"):
    feats = np.zeros((iters + 1, 6), np.float32)
    feats[:, 0] = np.log10(lam * lam) - np.arange(iters + 1)
    feats[:, 5] = beta_rule
    hist = np.zeros((iters, 9))
    hist[:, 0] = np.arange(iters)
    hist[:, 8] = beta_rule
    return {"iterations": iters, "phase": phase, "objP_text": obj, "features": feats, "history": hist}


def test_dataset_and_scaling():
    tr = []
    for seed in range(3):
        runs = {(lam, learned.BETA_GRID[0]): _run(40 - int(np.log10(lam)), lam, 0.1) for lam in learned.LAMBDA_GRID}
        tr.append({"seed": seed, "runs": runs, "best": (1.0, learned.BETA_GRID[0]),
                   "default": (learned.LAMBDA_GRID[-1], learned.BETA_GRID[0])})
    x, t, m = learned.dataset(tr, lambda_weight=8.0)
    best_iters = tr[0]["runs"][(1.0, learned.BETA_GRID[0])]["iterations"]
    assert x.shape == (3 * (1 + best_iters), 6) and t.shape == m.shape == (x.shape[0], 2)
    lam_rows = m[:, 0] > 0
    assert lam_rows.sum() == 3 and np.all(m[lam_rows, 0] == 8.0) and np.all(m[lam_rows, 1] == 0)
    assert np.allclose(t[lam_rows, 0], 0.0)  # log10 of the best lambdaStar, 1
    assert np.allclose(x[lam_rows, 0], 8.0)  # features at the default initial point (mu0 = 1e8)
    assert np.allclose(t[~lam_rows, 1], 0.1)
    sc = learned.scaling(x, t, m)
    assert sc.shape == (16,) and np.all(sc[6:12] >= 1e-3) and np.all(sc[14:] >= 1e-3)
    assert np.isclose(sc[13], 0.1)  # the mean beta target


def test_objective_comparison():
    a = {"objP_text": "-1.2345678901234567890123456789012345678901e+02"}
    b = {"objP_text": " -1.2345678901234567890123456789012345678900e+02"}
    assert 0 < learned.objective_rel_error(a, b) < 1e-39
    c = {"objP_text": "-1.2345678901234567890123456789e+02"}
    assert not learned._agrees(c, {"objP_text": "-1.2345678901234567990123456789e+02"})


def test_family_generator():
    p = learned.edge_probability(7)
    assert 0.02 <= p <= 0.2 and p == learned.edge_probability(7)
    text = problems.maxcut(n=learned.N_VERTICES, p=p, seed=7, signed=True)
    assert text.m == 124 and text.block_struct == [124]
    vals = {v for k, b, i, j, v in text.entries if k == 0 and i != j}
    assert vals <= {"0.25", "-0.25"}  # Laplacian / 4 off the diagonal, weights +-1
