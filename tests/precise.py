"""Errors of a solve against a high-precision golden fixture (the reference solver's
xVec / xMat / yMat printed with 80 or 160 significant digits, and the objectives
recomputed exactly from them; tests/golden/make_golden.py, PRECISE cases).

Shared by the parity tests and bench.py's error_vs_reference field.  Every error is
relative in the sense SDPA prints its own figures:

  objValPrimal / objValDual : |ours - ref| / max(1, |ref|)
  relgap                    : |gap_ours - gap_ref| / max(1, (|P| + |D|) / 2), i.e. the
                              gap difference on the objectives' scale
  xVec                      : max_i |ours_i - ref_i| / max(1, max_i |ref_i|)
  xMat / yMat               : the same over the digest entries (first column and
                              diagonal of every block) or the whole matrix

The high-precision cases have SDP blocks only.
"""
from __future__ import annotations

import math
from decimal import Decimal, getcontext

getcontext().prec = 400


def _d(s) -> Decimal:
    return Decimal(str(s))


def _log2(x: Decimal) -> float:
    if x == 0:
        return -math.inf
    return math.log2(float(x)) if float(x) > 0 else float(x.ln() / Decimal(2).ln())


def errors(sdpg, solver, golden: dict, digits: int | None = None) -> dict:
    """Relative errors of `solver` (after run()) against `golden`; values are floats and
    their log2 under "<key>_log2".  The solver's values are read as decimal text with
    `digits` significant digits (default: 20 more than the golden's precision holds, so
    the text itself adds nothing to the error)."""
    if digits is None:
        digits = int(int(golden.get("precision", 256)) * 0.30103) + 20
    P = _d(solver.text(0, digits))
    D = _d(solver.text(1, digits))
    Pr, Dr = _d(golden["objValPrimal_hp"]), _d(golden["objValDual_hp"])
    scale = max(Decimal(1), (abs(Pr) + abs(Dr)) / 2)
    gap = abs(P - D) / max(Decimal(1), (abs(P) + abs(D)) / 2)
    # the reference's gap from its objectives (stored to more digits than relgap_hp in
    # older fixtures)
    gapr = abs(Pr - Dr) / max(Decimal(1), (abs(Pr) + abs(Dr)) / 2)
    out = {
        "objValPrimal": abs(P - Pr) / max(Decimal(1), abs(Pr)),
        "objValDual": abs(D - Dr) / max(Decimal(1), abs(Dr)),
        "relgap": abs(gap - gapr) * max(Decimal(1), (abs(P) + abs(D)) / 2) / scale,
    }
    x = [_d(s) for s in sdpg.ml_format(solver.xvec(ml=True), digits)]
    xr = [_d(s) for s in golden["xVec"]]
    xs = max(Decimal(1), max(abs(v) for v in xr))
    out["xVec"] = max(abs(a - b) for a, b in zip(x, xr)) / xs
    # printed xMat = the solver's Z, printed yMat = its X (REVERSE_PRIMAL_DUAL)
    for key, which in (("xMat", 1), ("yMat", 0)):
        worst, big = Decimal(0), Decimal(1)
        if "digest" in golden:
            dig = golden["digest"][key]
            for t, l in enumerate(range(len(solver.block_sizes))):
                n = solver.block_sizes[l]
                vals = sdpg.ml_format(solver.block(which, l, ml=True), digits)  # column-major
                for i in range(n):
                    for got, ref in ((vals[i + n * i], dig["diag"][t][i]), (vals[i], dig["col0"][t][i])):
                        r = _d(ref)
                        big = max(big, abs(r))
                        worst = max(worst, abs(_d(got) - r))
        elif key in golden:
            ref = [_d(s) for s in golden[key]]
            got = []
            for l, n in enumerate(solver.block_sizes):
                # printed row by row; symmetric, so the column-major order reads the same
                got += sdpg.ml_format(solver.block(which, l, ml=True), digits)
            for a, r in zip(got, ref):
                big = max(big, abs(r))
                worst = max(worst, abs(_d(a) - r))
        out[key] = worst / big
    res = {}
    for k, v in out.items():
        res[k] = float(v)
        res[k + "_log2"] = _log2(v) if v > 0 else -math.inf
    return res


def golden_errors(golden: dict, yardstick: dict) -> dict:
    """The same errors between two reference fixtures of one problem and iteration count
    (e.g. the reference at 256 bits against itself at 512 bits): objectives, gap and xVec,
    and xMat / yMat over the digest entries both fixtures hold."""
    P, D = _d(golden["objValPrimal_hp"]), _d(golden["objValDual_hp"])
    Pr, Dr = _d(yardstick["objValPrimal_hp"]), _d(yardstick["objValDual_hp"])
    scale = max(Decimal(1), (abs(Pr) + abs(Dr)) / 2)
    gap = abs(P - D) / max(Decimal(1), (abs(P) + abs(D)) / 2)
    gapr = abs(Pr - Dr) / max(Decimal(1), (abs(Pr) + abs(Dr)) / 2)
    out = {
        "objValPrimal": abs(P - Pr) / max(Decimal(1), abs(Pr)),
        "objValDual": abs(D - Dr) / max(Decimal(1), abs(Dr)),
        "relgap": abs(gap - gapr) * max(Decimal(1), (abs(P) + abs(D)) / 2) / scale,
    }
    x = [_d(v) for v in golden["xVec"]]
    xr = [_d(v) for v in yardstick["xVec"]]
    out["xVec"] = max(abs(a - b) for a, b in zip(x, xr)) / max(Decimal(1), max(abs(v) for v in xr))
    for key in ("xMat", "yMat"):
        worst, big = Decimal(0), Decimal(1)
        for part in ("diag", "col0"):
            for blk, blkr in zip(golden["digest"][key][part], yardstick["digest"][key][part]):
                for a, b in zip(blk, blkr):
                    r = _d(b)
                    big = max(big, abs(r))
                    worst = max(worst, abs(_d(a) - r))
        out[key] = worst / big
    res = {}
    for k, v in out.items():
        res[k] = float(v)
        res[k + "_log2"] = _log2(v) if v > 0 else -math.inf
    return res
