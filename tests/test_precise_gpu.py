"""High-precision parity with the reference solver on the benchmark configuration
(graph-partition n = 500, m = 501) and on the other BASELINE shapes.

The reference printed its final xVec / xMat / yMat with 80 significant digits (160
at 512 bits), so its final iterate is known far below 2^-p; the fixtures hold the
objectives recomputed exactly from that output (tests/golden/make_golden.py).  For
every case the measured errors (tests/precise.py: objectives, relative gap, xVec,
xMat, yMat) are printed as log2 and asserted against the bounds below.

Why the bounds are not all 2^-(p-16).  The reference computes in GMP mpf (precision
256 holds 5 64-bit limbs, 257-320 significant bits) and this solver in a fixed
256-bit mantissa, with a different order of operations (exact GEMM sums, left-looking
Cholesky, Newton instead of QL for the tridiagonal eigenvalue).  Each iteration's
Newton system has a condition number near 1/mu^2, so rounding differences of 2^-256
in an iterate grow by that factor in the next direction.  Agreement is therefore at
the 2^-(p-16) level for the first iterations and degrades as mu falls: the
fixed-iteration cases (5, 10, 20 iterations) show where; the full solves agree to
the digits the bounds state.  The objectives of a full solve stop at relative gap
1e-30 (epsilonStar), so both implementations' optimal objectives agree far below
the gap itself.
"""
import math
import os

import pytest

from golden_cases import GOLDEN, close_printed, load, write_inputs
from precise import errors, golden_errors

# case -> (max log2 relative error of objectives / gap, of xVec, of xMat / yMat).  Each
# bound sits a few bits above the error measured on a GB300 (in brackets: objValPrimal,
# objValDual, relgap; xVec; xMat, yMat).
BOUNDS = {
    # after 5 iterations: [-218.8, -218.8, exact; -218.8; -218.3, -218.8] (-225.9 .. -234.2
    # with the earlier tridiagonal Newton ladder: the agreement moves by a few bits with
    # the rounding of the step lengths, amplified by the iterations)
    "gpp500_it5": (-214, -214, -214),
    # after 10: [-135.3, -135.6, -134.5; -133.4; -133.4, -133.9]
    "gpp500_it10": (-128, -128, -128),
    # after 20: [-153.5, -147.0, -147.0; -131.1; -131.1, -145.3]
    "gpp500_it20": (-140, -125, -125),
    # 512 bits after 10: [-491.8, -491.8, -490.9; -484.3; -484.3, -490.4]
    "gpp500_p512_it10": (-480, -475, -475),
    "gpp500_hp": (-100, -64, -64),
    # full solve, 43 iterations to pdOPT: [-119.9, -118.5, -118.0; -89.9; -84.8, -93.9]
    "control231_hp": (-110, -80, -75),
    # full solve, 42 iterations to pdOPT: [-118.9, -118.0, -119.2; -106.3; -105.6, -84.8]
    "maxcut124pm_hp": (-110, -95, -75),
    # full solve, 41 iterations to pdOPT: [-131.3, -111.3, -111.3; -90.1; -88.4, -76.5]
    "maxcut100_hp": (-105, -85, -70),
}
# the full graph-partition solve stops in pFEAS when the step collapses (no strictly
# feasible primal point); where exactly depends on rounding, so its iteration count
# may differ by a few
DEGENERATE = {"gpp500_hp"}
# The same ten graph-partition iterations run by the reference at 256, 512 and 1024 bits:
# (run, yardstick, margin) triples in which the yardstick holds the more precise iterate.
# The reference's own distance from the yardstick shows how far rounding at the run's
# precision moves the iterate; this solver's distance is held to that, within a factor of
# 2^margin.  GMP at precision 256 / 512 carries 5 / 9 limbs of 64 bits (at least 64 bits
# beyond the nominal precision), this solver exactly 256 / 512 bits.  Measured on a GB300
# (log2, objValPrimal .. yMat): at 256 bits this solver -135.1 .. -133.2 against the
# reference's -137.9 .. -136.0 (2.8 bits); at 512 bits -491.8 .. -484.3 against
# -507.9 .. -493.6 (9.3 to 16.1 bits).
YARDSTICKS = [("gpp500_it10", "gpp500_p512_it10", 6), ("gpp500_it10", "gpp500_p1024_it10", 6),
              ("gpp500_p512_it10", "gpp500_p1024_it10", 20)]
KEYS = ("objValPrimal", "objValDual", "relgap", "xVec", "xMat", "yMat")


def cases():
    return [c for c in BOUNDS if os.path.exists(os.path.join(GOLDEN, c + ".json"))]


def have(name):
    return os.path.exists(os.path.join(GOLDEN, name + ".json"))


def solve(sdpg, name, tmp_path):
    dat, par, g = write_inputs(name, str(tmp_path))
    solver = sdpg.Solver(sdpg.Problem.read(dat), sdpg.Param.read(par))
    solver.run()
    return solver, g


def fmt(e):
    return "  ".join(f"{k}={e[k + '_log2']:.1f}" for k in KEYS)


@pytest.mark.gpu
@pytest.mark.parametrize("name", cases())
def test_precise_parity(sdpg, name, tmp_path):
    solver, g = solve(sdpg, name, tmp_path)
    info = solver.info()
    assert info["phase"] == g["phase"], (info["phase"], g["phase"])
    if name in DEGENERATE:
        assert abs(info["iteration"] - g["iteration"]) <= 10, (info["iteration"], g["iteration"])
    else:
        assert info["iteration"] == g["iteration"], (info["iteration"], g["iteration"])
    if info["iteration"] != g["iteration"]:
        # a degenerate solve that stopped elsewhere: the iterates are compared through the
        # printed table while mu > 1e-12, and the final objectives to the stop's own scale
        hist = solver.history()
        for row, ref in zip(hist, g["iterations_table"]):
            if float(ref[1]) < 1e-12:
                break
            for col, digits in ((1, 1), (4, 2), (5, 2)):  # mu, objP, objD as printed
                assert close_printed(row[col], ref[col], digits), (int(row[0]), col, row[col], ref[col])
        for key in ("objValPrimal", "objValDual"):
            ref = float(g[key])
            assert abs(info[key] - ref) <= 1e-9 * max(1.0, abs(ref)), (key, info[key], ref)
        print(f"\n{name}: stopped at iteration {info['iteration']} ({info['phase']}), the reference at "
              f"{g['iteration']}; table and objectives agree (final iterates not comparable digit by digit)")
        return
    e = errors(sdpg, solver, g)
    print(f"\n{name} ({g['precision']}-bit, {info['iteration']} iterations, {info['phase']}): log2 error {fmt(e)}")
    b_obj, b_x, b_mat = BOUNDS[name]
    for key in ("objValPrimal", "objValDual", "relgap"):
        assert e[key + "_log2"] <= b_obj, (key, e[key + "_log2"], b_obj)
    assert e["xVec_log2"] <= b_x, ("xVec", e["xVec_log2"], b_x)
    for key in ("xMat", "yMat"):
        assert e[key + "_log2"] <= b_mat, (key, e[key + "_log2"], b_mat)


@pytest.mark.gpu
@pytest.mark.parametrize("run,yardstick,margin", [p for p in YARDSTICKS if have(p[0]) and have(p[1])])
def test_precise_against_higher_precision(sdpg, run, yardstick, margin, tmp_path):
    """This solver at the run's precision is no further from the higher-precision iterate
    than the reference at the same precision is (within 2^margin)."""
    solver, g = solve(sdpg, run, tmp_path)
    y = load(yardstick)
    assert solver.info()["iteration"] == y["iteration"]
    ours = errors(sdpg, solver, y)
    ref = golden_errors(g, y)
    print(f"\n{run} vs {yardstick}: this solver {fmt(ours)}\n{'':>{len(run) + len(yardstick) + 4}}"
          f"  reference   {fmt(ref)}")
    for key in KEYS:
        assert ours[key + "_log2"] <= ref[key + "_log2"] + margin, (key, ours[key + "_log2"], ref[key + "_log2"])


def test_precise_fixtures_present():
    """The benchmark configuration's fixtures are committed (CPU-side check of the set)."""
    have_ = cases()
    for need in ("gpp500_hp", "gpp500_it5", "gpp500_it10", "gpp500_it20", "gpp500_p512_it10"):
        assert need in have_, need
    g = load("gpp500_it5")
    assert g["param"]["print_format"] == "%+.80Fe" and g["iteration"] == 5
    assert not math.isnan(float(g["objValPrimal_hp"]))


def test_reference_precision_ladder():
    """The reference's own 256-bit iterate after ten graph-partition iterations lies within
    2^-120 of its 512-bit one (CPU-side: fixtures only).  This is the scale on which the
    256-bit parity bounds above are set."""
    if not (have("gpp500_it10") and have("gpp500_p512_it10")):
        pytest.skip("fixtures absent")
    e = golden_errors(load("gpp500_it10"), load("gpp500_p512_it10"))
    for key in KEYS:
        assert e[key + "_log2"] <= -120, (key, e[key + "_log2"])
