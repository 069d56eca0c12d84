"""The C++ class surface (include/sdpa_gb300.hpp): a driver in the shape of the
reference's pinpal main loop (tests/cxx/pinpal_loop.cpp), compiled with g++ against
that header and libsdpg.so only, solves the reference's example1 and the control-type
m = 231 problem and matches the reference solver's goldens: final phase, iteration
count, objectives to the printed 17 digits, and every row of the iteration table.

The same driver is built without a GPU by test_cxx_surface_builds (CPU suite).
"""
import os
import subprocess

import pytest

from golden_cases import close_printed, write_inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_driver(sdpg, out_dir):
    lib_dir = os.path.dirname(sdpg.LIB_PATH)
    exe = os.path.join(out_dir, "pinpal_loop")
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cxx", "pinpal_loop.cpp"), "-o", exe, "-L" + lib_dir, "-lsdpg",
           "-Wl,-rpath," + lib_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cxx_surface_builds(sdpg, tmp_path):
    assert os.path.exists(build_driver(sdpg, str(tmp_path)))


def summary(text):
    res = {}
    for ln in text.splitlines():
        if "=" in ln:
            k, v = (s.strip() for s in ln.split("=", 1))
            if k in ("phase.value", "Iteration", "objValPrimal", "objValDual"):
                res[k] = v
    return res


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["example1", "control231"])
def test_pinpal_loop_matches_reference(sdpg, name, tmp_path):
    exe = build_driver(sdpg, str(tmp_path))
    dat, par, g = write_inputs(name, str(tmp_path))
    out = tmp_path / (name + ".out")
    r = subprocess.run([exe, dat, par, str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-2000:])
    res = summary(r.stdout)
    assert res["phase.value"] == g["phase"], (res, g["phase"])
    assert int(res["Iteration"]) == g["iteration"]
    for key in ("objValPrimal", "objValDual"):
        got, ref = float(res[key]), float(g[key])
        assert abs(got - ref) <= 1e-15 * max(1.0, abs(ref)), (key, res[key], g[key])
    rows = [ln.split() for ln in out.read_text().splitlines()]
    rows = [x for x in rows if len(x) == 9 and x[0].isdigit()]
    table = g["iterations_table"]
    assert len(rows) == len(table), (len(rows), len(table))
    for row, ref in zip(rows, table):
        assert row[0] == ref[0]
        for col, digits in ((1, 1), (4, 2), (5, 2), (8, 2)):  # mu, objP, objD, beta as printed
            assert close_printed(float(row[col]), ref[col], digits), (row[0], col, row[col], ref[col])
    assert "lal: block" in r.stdout  # the Lal helper ran on the final iterate
