"""Host check of the integer summation helpers (sdpa-gmp_gb300/csrc/mlfix.cuh).

The exact fixed-point group sums behind every warp / block reduction, and the
block-floating-point dots of the Cholesky panel update, are compiled for the host with
g++ (tests/cxx/mlfix_check.cpp) and compared with sums in a wider format: errors within
2^-250 of the group's scale at 256 bits and 2^-500 at 512 bits, with zeros, exponent
spreads up to 300 binades and exact cancellation among the cases.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_mlfix_host(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "mlfix_check")
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-Wextra", "-Werror",
           "-I" + os.path.join(ROOT, "sdpa-gmp_gb300", "csrc"),
           os.path.join(ROOT, "tests", "cxx", "mlfix_check.cpp"), "-o", exe]
    b = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert b.returncode == 0, b.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
