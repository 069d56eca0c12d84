"""Failure detection of the bounded waits, without a GPU fault.

A child process shortens the tensor-core GEMM's primary wait budget (TMA data, free
ring stages) to fewer cycles than a copy takes, so those waits give up while the data
is still legitimately on its way.  The kernel then records the time-out, waits with
the full budget for the copies and products it already issued, frees its tensor
memory and returns; nothing is left running and the context stays usable.  The same
budget bounds the Cholesky panel's row waits (the rows of a panel wait for the
columns of its diagonal block), which then give up with info = -1.  Checked:

  * a standalone product reports the time-out in the sticky device flag;
  * a standalone Cholesky returns SDPG_ERR_TIMEOUT;
  * a solver fails with SDPG_ERR_TIMEOUT at the first iteration;
  * with the default budget restored, a new product is exact again, the Cholesky
    succeeds, and a new solver (its own, fresh error word) solves the problem as the
    reference does, although the device-wide flag stays set.

It runs in a child process so that the sticky flag does not reach the other tests.
"""
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent("""
    import importlib, os, random, sys
    sys.path.insert(0, {root!r}); sys.path.insert(0, os.path.join({root!r}, "tests"))
    sdpg = importlib.import_module("sdpa-gmp_gb300")
    exact = importlib.import_module("oracle.exact")
    from golden_cases import write_inputs
    rng = random.Random(5)
    m = n = k = 64
    A = exact.random_ml(m * k, 8, rng, -20, 20)
    B = exact.random_ml(k * n, 8, rng, -20, 20)
    C = exact.random_ml(m * n, 8, rng, -2, 2)
    one = sdpg.ml_parse(["1"], 8)
    zero = sdpg.ml_parse(["0"], 8)
    sdpg.set_gemm_method(2)          # every 256-bit product on the tensor-core path
    assert sdpg.tensor_error(0) == 0
    sdpg.set_tensor_wait_budget(16)  # far shorter than a TMA copy takes
    sdpg.rgemm("N", "N", m, n, k, one, A, m, B, k, zero, C, m)
    assert sdpg.tensor_error(0) != 0, "the time-out was not recorded"
    import numpy as np
    nc = 64                          # two panels: the first one's rows wait on its diagonal block
    S = sdpg.ml_from_double((np.ones((nc, nc)) + nc * np.eye(nc)).reshape(-1), 8)
    try:
        sdpg.rpotrf(S, nc, nc)
        raise SystemExit("the Cholesky panel did not report the time-out")
    except sdpg.SdpgError as e:
        assert e.code == -8, e.code
    dat, par, g = write_inputs("maxcut20", {tmp!r})
    s = sdpg.Solver(sdpg.Problem.read(dat), sdpg.Param.read(par))
    try:
        s.run()
        raise SystemExit("the solver did not report the time-out")
    except sdpg.SdpgError as e:
        assert e.code == -8, e.code
    s.close()
    sdpg.set_tensor_wait_budget(0)   # default budget again
    got = sdpg.rgemm("N", "N", m, n, k, one, A, m, B, k, zero, C, m)
    ref, scale = exact.gemm("N", "N", m, n, k, (1, 0), exact.ml_decode(A), m, exact.ml_decode(B), k,
                            exact.ml_decode(zero)[0], exact.ml_decode(C), m)
    err = exact.max_rel_err(got, ref, scale)
    assert err <= 2.0 ** -240, err
    assert sdpg.rpotrf(S, nc, nc)[1] == 0
    s = sdpg.Solver(sdpg.Problem.read(dat), sdpg.Param.read(par))
    s.run()
    info = s.info()
    assert info["phase"] == g["phase"] and info["iteration"] == g["iteration"], (info, g["phase"], g["iteration"])
    assert sdpg.tensor_error(0) != 0  # sticky for the life of the process
    print("TIMEOUT-TEST-OK", err)
""")


def test_tensor_wait_timeout_reported_and_recovered(sdpg, tmp_path):
    code = CHILD.format(root=ROOT, tmp=str(tmp_path))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "TIMEOUT-TEST-OK" in r.stdout, (r.stdout[-2000:], r.stderr[-4000:])
