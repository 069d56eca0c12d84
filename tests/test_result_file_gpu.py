"""The result file of a whole solve (the reference driver's output: header, iteration
table, summary, parameters, time table, xVec / xMat / yMat, final times) against the
reference's own file for its known-answer input example1.dat-s and for a problem with
an LP block: the same lines once
numbers, the start time and file names are masked, and the 40-digit solution within
1e-20 relative to max(1, |x|) (the solves stop at relative gap 1e-30)."""
import importlib.util
import os
import subprocess
from decimal import Decimal, getcontext

import pytest

from golden_cases import GOLDEN, init_file, load, write_inputs

pytestmark = pytest.mark.gpu


def _make_golden():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _close(got, ref, tol=1e-20):
    getcontext().prec = 80
    worst = 0.0
    assert len(got) == len(ref)
    for a, b in zip(got, ref):
        d = abs(Decimal(a) - Decimal(b))
        worst = max(worst, float(d / max(Decimal(1), abs(Decimal(b)))))
    return worst <= tol, worst


def _check(text, g, mg):
    assert mg.result_layout(text) == g["layout"]
    r = mg.parse_result(text)
    assert r["phase"] == g["phase"] and r["iteration"] == g["iteration"]
    for key in ("xVec", "xMat", "yMat"):
        ok, worst = _close(r[key], g[key])
        assert ok, (key, worst)


@pytest.mark.parametrize("name", ["example1", "controllp20"])
def test_solve_file_writes_the_reference_layout(sdpg, tmp_path, name):
    """example1 (one SDP block) and a problem with an LP block, whose solution prints
    as one braced row per LP block."""
    g = load(name)
    mg = _make_golden()
    dat, par, _ = write_inputs(name, str(tmp_path))
    out = str(tmp_path / (name + ".result"))
    info = sdpg.solve_file(dat, par, out)
    assert info["phase"] == "pdOPT"
    with open(out) as f:
        _check(f.read(), g, mg)


def test_command_line_driver(sdpg, tmp_path):
    exe = os.path.join(os.path.dirname(sdpg.LIB_PATH), "sdpa_gmp_gb300")
    assert os.path.exists(exe), "the driver is built with the library"
    g = load("example1")
    mg = _make_golden()
    dat, par, _ = write_inputs("example1", str(tmp_path))
    out = str(tmp_path / "cli.result")
    r = subprocess.run([exe, "-ds", dat, "-o", out, "-p", par], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "phase.value = pdOPT" in r.stdout
    with open(out) as f:
        _check(f.read(), g, mg)
    # an initial point (-is / -id), as the reference ran it
    for name, opt in (("example1_is", "-is"), ("example1_id", "-id")):
        gi = load(name)
        path, _ = init_file(gi)
        outi = str(tmp_path / (name + ".result"))
        r = subprocess.run([exe, "-ds", dat, "-o", outi, "-p", par, opt, path], capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr
        with open(outi) as f:
            _check(f.read(), gi, mg)
    # the dense data format (-dd)
    gd = load("example1_dd")
    outd = str(tmp_path / "dd.result")
    r = subprocess.run([exe, "-dd", os.path.join(GOLDEN, "example1.dat"), "-o", outd, "-p", par],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    with open(outd) as f:
        _check(f.read(), gd, mg)
    # the positional form, and a call that fails (no such data file)
    out2 = str(tmp_path / "cli2.result")
    assert subprocess.run([exe, dat, out2, par], capture_output=True, timeout=300).returncode == 0
    with open(out2) as f:
        _check(f.read(), g, mg)
    assert subprocess.run([exe, "-ds", str(tmp_path / "missing.dat-s"), "-o", out2], capture_output=True,
                          timeout=60).returncode != 0
