"""The SDPLIB-style sweep runner (sdpa-gmp_gb300/sdplib.py), CPU side: it reads the
reference's result file (tests/golden/maxcut20.result.xz, written by the reference solver
for the seeded MaxCut n = 20 problem), pairs data and result files in a directory, and maps
the result's parameter block onto the solver's parameters."""
import importlib
import os
import shutil
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sdplib = importlib.import_module("sdpa-gmp_gb300.sdplib")
problems = importlib.import_module("sdpa-gmp_gb300.problems")
GOLDEN = os.path.join(ROOT, "tests", "golden")

from golden_cases import load  # noqa: E402


def test_parse_reference_result():
    r = sdplib.parse_result(sdplib.read_text(os.path.join(GOLDEN, "maxcut20.result.xz")))
    g = load("maxcut20")
    assert r["phase"] == g["phase"] and r["iteration"] == g["iteration"]
    assert r["objValPrimal"] == float(g["objValPrimal"]) and r["objValDual"] == float(g["objValDual"])
    assert r["params"]["precision"] == 256 and r["params"]["maxIteration"] == 200
    assert r["params"]["epsilonStar"] == 1e-30 and r["params"]["lambdaStar"] == 1e4
    assert set(r["params"]) == set(sdplib.PARAM_KEYS)
    assert r["main_loop_time"] > 0


def test_pairs_and_sizes(tmp_path):
    text = problems.maxcut(n=20, p=0.3, seed=1).text()
    (tmp_path / "maxcut20.dat-s").write_text(text)
    shutil.copy(os.path.join(GOLDEN, "maxcut20.result.xz"), tmp_path / "maxcut20.result.xz")
    (tmp_path / "lonely.dat-s").write_text(text)  # no result beside it: not a pair
    (tmp_path / "other.result").write_text("phase.value = pdOPT\n")
    found = sdplib.pairs(str(tmp_path))
    assert [f[0] for f in found] == ["maxcut20"]
    assert sdplib.data_size(text) == (20, [20])
