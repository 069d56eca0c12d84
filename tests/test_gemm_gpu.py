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
def test_rgemm_matches_exact(sdpg, exact, limbs, ta, tb, m, n, k):
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


def test_rgemm_wide_dynamic_range(sdpg, exact):
    """Rows whose entries span 2^-200..2^200 (late-iteration Z^-1 shapes)."""
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
