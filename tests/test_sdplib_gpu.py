"""The SDPLIB-style sweep runner on the GPU: a directory holding the seeded MaxCut n = 20
problem and the reference's result file for it is swept, and the solve matches the
recorded phase, iteration count and objectives."""
import importlib
import os
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.mark.gpu
def test_sweep_matches_reference_result(sdpg, tmp_path):
    sdplib = importlib.import_module("sdpa-gmp_gb300.sdplib")
    problems = importlib.import_module("sdpa-gmp_gb300.problems")
    (tmp_path / "maxcut20.dat-s").write_text(problems.maxcut(n=20, p=0.3, seed=1).text())
    shutil.copy(os.path.join(GOLDEN, "maxcut20.result.xz"), tmp_path / "maxcut20.result.xz")
    rows = sdplib.sweep(str(tmp_path))
    assert len(rows) == 1 and "error" not in rows[0], rows
    r = rows[0]
    assert r["same_phase"] and r["iteration_difference"] == 0, r
    assert r["objective_rel_difference"] <= 1e-15, r
