"""Multi-limb GEMM (replaces Rgemm, mplapack/Rgemm_omp.cpp:41-127) on the GPU
against the exact-arithmetic oracle.

Tolerance: |C - C_exact| <= 2^-(p-16) * (|alpha| K max_k|a_ik| max_k|b_kj| + |beta c_ij|)
per entry, p = 32 * limbs (256 or 512) -- the normwise form of the bound GMP's
truncated sequential summation in Rgemm obeys."""
import random

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("limbs,ta,tb,m,n,k", [
    (8, "N", "N", 37, 29, 53),
    (8, "T", "N", 33, 40, 17),
    (8, "N", "T", 64, 64, 64),
    (8, "T", "T", 5, 70, 31),
    (8, "N", "N", 1, 1, 1),
    (8, "N", "N", 12, 9, 0),
    (16, "N", "N", 23, 31, 45),
    (16, "T", "T", 17, 19, 33),
])
@pytest.mark.parametrize("method", [1, 2])
def test_rgemm_matches_exact(sdpg, exact, limbs, ta, tb, m, n, k, method):
    """method 1: integer digit GEMM; 2: residue-number-system path on the tensor cores
    (256-bit operands; 512-bit ones always take the digit GEMM)."""
    old = sdpg.set_gemm_method(method)
    try:
        _rgemm_case(sdpg, exact, limbs, ta, tb, m, n, k)
    finally:
        sdpg.set_gemm_method(old)


def _rgemm_case(sdpg, exact, limbs, ta, tb, m, n, k):
    rng = random.Random(hash((limbs, ta, tb, m, n, k)) & 0xFFFF)
    lda = (k if ta == "T" else m) + 3
    ldb = (n if tb == "T" else k) + 2
    ldc = m + 1
    acols = m if ta == "T" else k
    bcols = k if tb == "T" else n
    A = exact.random_ml(max(lda * acols, 1), limbs, rng, -30, 30, zero_frac=0.05)
    B = exact.random_ml(max(ldb * bcols, 1), limbs, rng, -30, 30, zero_frac=0.05)
    C = exact.random_ml(ldc * n, limbs, rng, -10, 10)
    alpha = exact.random_ml(1, limbs, rng, -2, 2)
    beta = exact.random_ml(1, limbs, rng, -2, 2)
    got = sdpg.rgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc)
    ref, scale = exact.gemm(ta, tb, m, n, k, exact.ml_decode(alpha)[0], exact.ml_decode(A), lda,
                            exact.ml_decode(B), ldb, exact.ml_decode(beta)[0], exact.ml_decode(C), ldc)
    rows = [i + j * ldc for j in range(n) for i in range(m)]
    err = exact.max_rel_err(got[rows], [ref[r] for r in rows], [scale[r] for r in rows])
    assert err <= 2.0 ** -(32 * limbs - 16), err
    # padding rows of C (i >= m) untouched
    pad = [m + j * ldc for j in range(n)]
    assert (got[pad] == C[pad]).all()


@pytest.mark.parametrize("method", [1, 2])
def test_rgemm_wide_dynamic_range(sdpg, exact, method):
    """Rows whose entries span 2^-200..2^200 (late-iteration Z^-1 shapes)."""
    old = sdpg.set_gemm_method(method)
    try:
        _wide_case(sdpg, exact)
    finally:
        sdpg.set_gemm_method(old)


def _wide_case(sdpg, exact):
    rng = random.Random(7)
    m = n = k = 24
    A = exact.random_ml(m * k, 8, rng, -200, 200)
    B = exact.random_ml(k * n, 8, rng, -200, 200)
    C = exact.random_ml(m * n, 8, rng, 0, 0)
    one = sdpg.ml_parse(["1"], 8)
    zero = sdpg.ml_parse(["0"], 8)
    got = sdpg.rgemm("N", "N", m, n, k, one, A, m, B, k, zero, C, m)
    ref, scale = exact.gemm("N", "N", m, n, k, (1, 0), exact.ml_decode(A), m, exact.ml_decode(B), k, (0, 0),
                            exact.ml_decode(C), m)
    assert exact.max_rel_err(got, ref, scale) <= 2.0 ** -240


@pytest.mark.parametrize("m,n,k", [(500, 500, 500), (257, 131, 1024), (300, 200, 1025), (640, 384, 96),
                                   (130, 70, 4000), (16, 20, 16400)])
def test_residue_path_agrees_with_digit_gemm_at_full_size(sdpg, exact, m, n, k):
    """At sizes the exact oracle cannot reach in seconds, the tensor-core residue path
    and the digit GEMM (both checked against exact arithmetic above) must agree within
    twice the normwise bound, entry by entry.  K above 1024 runs the tensor GEMM in
    chunks whose residues are added modulo each prime; K = 16400 exceeds the residue
    path's range and falls back to the digit GEMM (identical results)."""
    import numpy as np
    rng = random.Random(m * 7 + n * 3 + k)
    A = exact.random_ml(m * k, 8, rng, -20, 20, zero_frac=0.02)
    B = exact.random_ml(k * n, 8, rng, -20, 20, zero_frac=0.02)
    C = exact.random_ml(m * n, 8, rng, -5, 5)
    alpha = sdpg.ml_parse(["-1.25"], 8)
    beta = sdpg.ml_parse(["0.5"], 8)
    out = {}
    for method in (1, 0):
        old = sdpg.set_gemm_method(method)
        try:
            out[method] = sdpg.rgemm("N", "N", m, n, k, alpha, A, m, B, k, beta, C, m)
        finally:
            sdpg.set_gemm_method(old)
    if k > 16384:
        assert (out[0] == out[1]).all()
        return
    # normwise scale per entry: |alpha| K max_t|a_it| max_t|b_tj| + |beta c_ij|, in doubles
    a = sdpg.ml_to_double(A).reshape(k, m).T
    b = sdpg.ml_to_double(B).reshape(n, k).T
    c = sdpg.ml_to_double(C).reshape(n, m).T
    scale = 1.25 * k * np.abs(a).max(axis=1)[:, None] * np.abs(b).max(axis=0)[None, :] + 0.5 * np.abs(c)
    d = sdpg.ml_to_double(sdpg.ml_host_op(sdpg.OP_SUB, out[0], out[1])).reshape(n, m).T
    assert np.all(np.abs(d) <= 2.0 ** -(256 - 17) * scale), float(np.max(np.abs(d) / scale))
