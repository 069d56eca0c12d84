"""Helpers shared by the parity tests: load a golden fixture (the reference
solver's own output, see tests/golden/make_golden.py) and write its input."""
import hashlib
import importlib
import json
import math
import os

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


def write_inputs(name, directory):
    """Write <name>.dat-s and <name>.param for a golden case; returns (dat, param, golden)."""
    g = load(name)
    if name.startswith("example1"):  # the reference's own input (and initial points)
        return os.path.join(GOLDEN, "example1.dat-s"), os.path.join(GOLDEN, "example1.param"), g
    problems = importlib.import_module("sdpa-gmp_gb300.problems")
    kw = {k: (tuple(v) if isinstance(v, list) else v) for k, v in g["kwargs"].items()}
    text = getattr(problems, g["generator"])(**kw).text()
    assert hashlib.sha256(text.encode()).hexdigest() == g["sha256"], "generator drifted from the golden input"
    dat = os.path.join(directory, name + ".dat-s")
    par = os.path.join(directory, name + ".param")
    with open(dat, "w") as f:
        f.write(text)
    with open(par, "w") as f:
        f.write(problems.param_text(precision=g["precision"], **g.get("param", {})))
    return dat, par, g


def fnum(s):
    return float(s)


def init_file(g):
    """(path, sparse) of a golden case's initial-point file, or None."""
    ini = g.get("init")
    if not ini:
        return None
    return os.path.join(GOLDEN, ini["file"]), bool(ini["sparse"])


def close_printed(a: float, b_str: str, digits: int) -> bool:
    """`a` agrees with the reference's printed value `b_str` (printed with `digits`
    digits after the point) to within two units of the last printed digit."""
    b = float(b_str)
    if b == 0.0:
        return abs(a) < 1e-300 or a == 0.0
    if abs(b) < 1e-60:  # residual ratios at rounding-noise level differ by construction
        return abs(a) < 1e-55
    ulp = 10.0 ** (math.floor(math.log10(abs(b))) - digits)
    return abs(a - b) <= 2.0 * ulp + 1e-12 * abs(b)
