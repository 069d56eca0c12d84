"""Learned lambdaStar / beta proposal for the signed MaxCut family.

Family: MaxCut relaxations of G(n=124, p) with p ~ U[0.02, 0.2] and edge weights +1 or
-1 with probability one half each, 256-bit mantissa, the reference's default
parameters otherwise.  Everything a user needs to rebuild the committed policy:

* ``instance(seed)``: the problem of one seed;
* ``collect(seeds)``: trace collection with the plain solver.  Per seed the solver
  runs at every lambdaStar of ``LAMBDA_GRID`` (default centering), then at every
  (betaStar, betaBar) of ``BETA_GRID`` for the best lambdaStar; the run with the fewest
  iterations that reaches pdOPT with the default run's objective is the label source;
* ``dataset(traces)``: one lambdaStar sample per seed (the features at the default
  initial point, target log10 of the best lambdaStar) and one beta sample per iteration
  of the best run (its features, target the beta it used);
* ``train(x, t, mask)``: standardisation and Adam on the library's CUDA kernels;
* ``evaluate(policy, seeds)``: default against proposed parameters on held-out seeds,
  with the defaults as the fallback of a solve that does not reach pdOPT.

Command line (one GPU): ``python sdpa-gmp_gb300/learned.py --train 256 --holdout 64``
writes ``policy_mcp124.npz`` beside this file and prints the evaluation as JSON.
"""
from __future__ import annotations

import argparse
import decimal
import importlib
import json
import os
import sys
import threading
import time

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
if os.path.dirname(PKG_DIR) not in sys.path:
    sys.path.insert(0, os.path.dirname(PKG_DIR))

POLICY_FILE = os.path.join(PKG_DIR, "policy_mcp124.npz")
N_VERTICES = 124
PRECISION = 256
LAMBDA_GRID = (0.3, 1.0, 3.0, 10.0, 100.0, 1.0e3, 1.0e4)
BETA_GRID = ((0.1, 0.3), (0.05, 0.15), (0.02, 0.1))
HOLDOUT_BASE = 1_000_000  # held-out seeds start here; training seeds start at 0
# The best single configuration of the label grid on the training seeds (fewest mean
# iterations over all training seeds, reaching pdOPT with the default objective): every
# training seed's best lambdaStar was 1 (X0 = I already meets diag(X) = 1 for MaxCut) and
# the default centering pair.  The ablation compares the network with this constant.
BEST_CONSTANT = (1.0, BETA_GRID[0])


def _sdpg():
    return importlib.import_module("sdpa-gmp_gb300")


def _problems():
    return importlib.import_module("sdpa-gmp_gb300.problems")


def edge_probability(seed: int) -> float:
    return float(np.random.default_rng([seed, 5]).uniform(0.02, 0.2))


def instance(seed: int):
    """The family's problem for `seed` (a Problem of the library)."""
    sdpg = _sdpg()
    text = _problems().maxcut(n=N_VERTICES, p=edge_probability(seed), seed=seed, signed=True)
    prob = sdpg.Problem.new(text.m, text.block_struct)
    for k, v in enumerate(text.c):
        prob.set_c(k + 1, v)
    for k, block, i, j, v in text.entries:
        prob.add_entry(k, block, i, j, v)
    return prob


def param(lambda_star: float | None = None, beta: tuple[float, float] | None = None):
    sdpg = _sdpg()
    p = sdpg.Param.default()
    p.precision = PRECISION
    if lambda_star is not None:
        p.lambdaStar = lambda_star
    if beta is not None:
        p.betaStar, p.betaBar = beta
    return p


def solve(prob, prm, policy=None, device: int = 0) -> dict:
    """One solve; returns iterations, phase, objectives, history, features, policy stats."""
    sdpg = _sdpg()
    s = sdpg.Solver(prob, prm, device=device)
    try:
        if policy is not None:
            s.set_policy(policy)
        s.run()
        info = s.info()
        out = {"iterations": info["iteration"], "phase": info["phase"], "objP": info["objValPrimal"],
               "objD": info["objValDual"], "objP_text": s.text(0, 40), "history": s.history(),
               "features": s.features()}
        if policy is not None:
            out["policy"] = s.policy_stats()
        return out
    finally:
        s.close()


def _parallel(items, fn, workers: int):
    """fn(item) for every item on `workers` host threads (each solver has its own streams)."""
    results = [None] * len(items)
    errors = []
    nxt = [0]
    lock = threading.Lock()

    def work():
        while True:
            with lock:
                if nxt[0] >= len(items) or errors:
                    return
                i = nxt[0]
                nxt[0] += 1
            try:
                results[i] = fn(items[i])
            except Exception as exc:  # reported after the join
                with lock:
                    errors.append(exc)

    threads = [threading.Thread(target=work) for _ in range(max(1, workers))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return results


def objective_rel_error(a: dict, b: dict) -> float:
    """|objP(a) - objP(b)| / |objP(b)| from the 40-digit texts of the two solves."""
    with decimal.localcontext() as ctx:
        ctx.prec = 60
        x, y = decimal.Decimal(a["objP_text"].strip()), decimal.Decimal(b["objP_text"].strip())
        return float(abs(x - y) / max(abs(y), decimal.Decimal("1e-300")))


def _agrees(a: dict, b: dict, tol: float = 1e-25) -> bool:
    return objective_rel_error(a, b) <= tol


def trace_seed(seed: int, device: int = 0) -> dict:
    """The coordinate search of one seed; returns the runs and the chosen configuration."""
    prob = instance(seed)
    runs = {}
    default_key = (LAMBDA_GRID[-1], BETA_GRID[0])
    for lam in LAMBDA_GRID:
        runs[(lam, BETA_GRID[0])] = solve(prob, param(lam, BETA_GRID[0]), device=device)
    ref = runs[default_key]

    def good(k):
        r = runs[k]
        return r["phase"] == "pdOPT" and _agrees(r, ref)

    lam_best = min((k for k in runs if good(k)), key=lambda k: (runs[k]["iterations"], k != default_key))[0]
    for beta in BETA_GRID[1:]:
        runs[(lam_best, beta)] = solve(prob, param(lam_best, beta), device=device)
    best = min((k for k in runs if good(k)), key=lambda k: (runs[k]["iterations"], k != default_key))
    return {"seed": seed, "runs": runs, "best": best, "default": default_key}


def collect(seeds, workers: int = 8, device: int = 0) -> list[dict]:
    return _parallel(list(seeds), lambda s: trace_seed(s, device), workers)


def dataset(traces, lambda_weight: float = 8.0):
    """(x, t, mask) float32 arrays from the traces (see the module docstring)."""
    xs, ts, ms = [], [], []
    for tr in traces:
        d = tr["runs"][tr["default"]]
        lam, _ = tr["best"]
        xs.append(d["features"][0])
        ts.append([np.log10(lam), 0.0])
        ms.append([lambda_weight, 0.0])
        b = tr["runs"][tr["best"]]
        feats, hist = b["features"], b["history"]
        for k in range(hist.shape[0]):
            xs.append(feats[k + 1])
            ts.append([0.0, hist[k, 8]])
            ms.append([0.0, 1.0])
    return (np.asarray(xs, dtype=np.float32), np.asarray(ts, dtype=np.float32),
            np.asarray(ms, dtype=np.float32))


def scaling(x, t, mask) -> np.ndarray:
    """x_mean, x_std, y_mean, y_std of the standardisation (std floored at 1e-3)."""
    xm = x.mean(0)
    xsd = np.maximum(x.std(0), 1e-3)
    ym, ysd = np.zeros(2), np.ones(2)
    for o in range(2):
        sel = mask[:, o] > 0
        if sel.any():
            ym[o] = t[sel, o].mean()
            ysd[o] = max(t[sel, o].std(), 1e-3)
    return np.concatenate([xm, xsd, ym, ysd]).astype(np.float32)


def train(x, t, mask, epochs: int = 300, batch: int = 256, lr: float = 1e-3, seed: int = 0, device: int = 0):
    """A policy trained on (x, t, mask) by the library's kernels; returns (policy, losses)."""
    pol = _sdpg().Policy(device)
    pol.set(scale=scaling(x, t, mask))
    losses = pol.train(x, t, mask, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return pol, losses


def evaluate(policy, seeds, workers: int = 8, device: int = 0, constant=None) -> dict:
    """Default parameters against the proposal on `seeds`; the defaults also serve as the
    fallback of any proposed solve that does not reach pdOPT.  With `constant` =
    (lambdaStar, (betaStar, betaBar)) the same seeds are also solved with that fixed
    configuration (the ablation: what the network adds beyond the best constant)."""

    def one(seed):
        prob = instance(seed)
        base = solve(prob, param(), device=device)
        lrn = solve(prob, param(), policy=policy, device=device)
        fell_back = lrn["phase"] != "pdOPT"
        used = base if fell_back else lrn
        spent = lrn["iterations"] + (base["iterations"] if fell_back else 0)
        err = objective_rel_error(used, base)
        row = {"seed": seed, "default": base["iterations"], "learned": spent, "fallback_solve": fell_back,
               "beta_fallbacks": lrn["policy"]["fallbacks"], "beta_proposals": lrn["policy"]["proposals"],
               "lambda": lrn["policy"]["lambda_star"], "objective_rel_error": err,
               "default_phase": base["phase"]}
        if constant is not None:
            cst = solve(prob, param(constant[0], constant[1]), device=device)
            c_fell = cst["phase"] != "pdOPT"
            row["constant"] = cst["iterations"] + (base["iterations"] if c_fell else 0)
            row["constant_fallback"] = c_fell
            row["constant_objective_rel_error"] = objective_rel_error(base if c_fell else cst, base)
        return row

    rows = _parallel(list(seeds), one, workers)
    d = np.array([r["default"] for r in rows], dtype=float)
    lr = np.array([r["learned"] for r in rows], dtype=float)
    extra = {}
    if constant is not None:
        c = np.array([r["constant"] for r in rows], dtype=float)
        extra = {"constant": {"lambda_star": constant[0], "beta": list(constant[1])},
                 "mean_iterations_constant": float(c.mean()),
                 "constant_reduction": float(1.0 - c.mean() / d.mean()),
                 "learned_vs_constant": float(1.0 - lr.mean() / c.mean()),
                 "seeds_learned_better": int(np.sum(lr < c)), "seeds_constant_better": int(np.sum(c < lr)),
                 "constant_fallback_solves": int(sum(r["constant_fallback"] for r in rows)),
                 "max_constant_objective_rel_error": float(max(r["constant_objective_rel_error"] for r in rows))}
    return {"seeds": len(rows), "mean_iterations_default": float(d.mean()),
            "mean_iterations_learned": float(lr.mean()),
            "iteration_reduction": float(1.0 - lr.mean() / d.mean()), **extra,
            "fallback_solves": int(sum(r["fallback_solve"] for r in rows)),
            "beta_fallback_rate": float(sum(r["beta_fallbacks"] for r in rows)
                                        / max(1, sum(r["beta_proposals"] for r in rows))),
            "mean_lambda": float(np.mean([r["lambda"] for r in rows])),
            "max_objective_rel_error": float(max(r["objective_rel_error"] for r in rows)),
            "rows": rows}


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--train", type=int, default=256, help="training seeds (0..N-1)")
    ap.add_argument("--holdout", type=int, default=64, help="held-out seeds")
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--out", default=POLICY_FILE)
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    t0 = time.time()
    traces = collect(range(args.train), workers=args.workers, device=args.device)
    t1 = time.time()
    x, t, mask = dataset(traces)
    pol, losses = train(x, t, mask, epochs=args.epochs, device=args.device)
    t2 = time.time()
    pol.save(args.out)
    ev = evaluate(pol, range(HOLDOUT_BASE, HOLDOUT_BASE + args.holdout), workers=args.workers, device=args.device)
    t3 = time.time()
    best = [tr["best"] for tr in traces]
    summary = {k: v for k, v in ev.items() if k != "rows"}
    summary.update({"train_seeds": args.train, "samples": int(x.shape[0]), "epochs": args.epochs,
                    "loss_first": float(losses[0]), "loss_last": float(losses[-1]),
                    "best_lambda_counts": {str(l): sum(1 for b in best if b[0] == l) for l in LAMBDA_GRID},
                    "best_beta_counts": {str(bb): sum(1 for b in best if b[1] == bb) for bb in BETA_GRID},
                    "mean_iterations_best_config": float(np.mean([tr["runs"][tr["best"]]["iterations"]
                                                                  for tr in traces])),
                    "mean_iterations_default_train": float(np.mean([tr["runs"][tr["default"]]["iterations"]
                                                                    for tr in traces])),
                    "seconds": {"collect": t1 - t0, "train": t2 - t1, "evaluate": t3 - t2}})
    print(json.dumps(summary))


if __name__ == "__main__":
    main()
