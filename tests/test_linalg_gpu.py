"""Kernel-level parity of the dense multi-limb routines against exact arithmetic.

Each routine replaces one MPLAPACK call of the reference's Lal class:
  sdpg_rpotrf        Rpotrf("Lower")       Lal::choleskyFactorWithAdjust, sdpa_linear.cpp:608-616
  sdpg_inv_lower     Rtrsm on the identity  Lal::getInvLowTriangularMatrix, sdpa_linear.cpp:439-455
  sdpg_solve_systems two Rtrsv              Lal::solveSystems, sdpa_linear.cpp:683-695
  sdpg_tridiag_min   Rsteqr's smallest pair Lal::getMinEigen, sdpa_linear.cpp:65-112
  sdpg_sym_min_eigen Rsyev('N', 'L')        Lal::getMinEigenValue, sdpa_linear.cpp:126-158

Residuals are formed exactly (dyadic integers) from the GPU's outputs.  Tolerances
(p = 32 * limbs bits, normwise like GMP's truncated arithmetic in MPLAPACK):
  Cholesky   max|L L^T - A|    <= 2^-(p-20) n max|A|  (n <= 97, exact residual);
             |L L^T - A|_ij    <= 2^-(p-24) n sqrt(A_ii A_jj)  (n = 200 .. 501)
  inverse    max|L X - I|      <= 2^-(p-24) n max|L| max|X|, strict upper of X exactly 0
  solve      max|L L^T x - b|  <= 2^-(p-24) n^2 max|L|^2 max|x|
  eigen      no eigenvalue below lambda - delta, one below lambda + delta (exact inertia),
             delta = 2^-(p-40) n max|T|; last eigenvector component to 2^-100 relative.
"""
import random
from fractions import Fraction

import numpy as np
import pytest

gpu = pytest.mark.gpu


def _lower_well_conditioned(exact, n, limbs, rng, ld=None):
    """Lower-triangular L with diagonal in [1, 4) and small off-diagonal entries."""
    ld = ld or n
    vals = [(0, 0)] * (ld * n)
    for j in range(n):
        for i in range(j, n):
            if i == j:
                M = rng.getrandbits(32 * limbs) | (1 << (32 * limbs - 1))
                vals[i + j * ld] = (M, rng.randint(1, 2) - 32 * limbs)
            else:
                M = rng.getrandbits(32 * limbs) | (1 << (32 * limbs - 1))
                s = -1 if rng.random() < 0.5 else 1
                vals[i + j * ld] = (s * M, rng.randint(-7, -4) - 32 * limbs)
    return exact.ml_encode(vals, limbs)


def _spd(exact, n, limbs, rng):
    """A = G G^T / n + I, truncated into the format (its stored value is what is checked)."""
    G = exact.ml_decode(exact.random_ml(n * n, limbs, rng, -1, 0))
    Gt = [G[c + r * n] for c in range(n) for r in range(n)]  # column-major G^T
    GGt = exact.matmul(G, Gt, n, n, n, n, n)
    shift = (n - 1).bit_length()
    vals = []
    for j in range(n):
        for i in range(n):
            v = GGt[i + j * n]
            v = (v[0], v[1] - shift)
            if i == j:
                v = exact.dy_add(v, (1, 0))
            vals.append(v)
    return exact.ml_encode(vals, limbs)


@gpu
@pytest.mark.parametrize("limbs,n", [(8, 1), (8, 5), (8, 32), (8, 33), (8, 97), (16, 40), (16, 97)])
def test_rpotrf_residual(sdpg, exact, limbs, n):
    rng = random.Random(1000 * limbs + n)
    A = _spd(exact, n, limbs, rng)
    Lml, info = sdpg.rpotrf(A, n, n)
    assert info == 0
    L = exact.ml_decode(Lml)
    Lt = [L[c + r * n] if c >= r else (0, 0) for c in range(n) for r in range(n)]  # column-major L^T
    Lz = [L[i + j * n] if i >= j else (0, 0) for j in range(n) for i in range(n)]
    LLt = exact.matmul(Lz, Lt, n, n, n, n, n, a_lower=True)
    Ad = exact.ml_decode(A)
    worst = max(abs(exact.to_fraction(exact.dy_add(LLt[i + j * n], (-Ad[i + j * n][0], Ad[i + j * n][1]))))
                for j in range(n) for i in range(j, n))
    assert worst <= Fraction(n) * exact.max_abs(Ad) / (1 << (32 * limbs - 20)), float(worst)
    # diagonal of the factor is positive
    assert all(L[i + i * n][0] > 0 for i in range(n))


@gpu
@pytest.mark.parametrize("n,spread", [(200, 0), (333, 40), (501, 20)])
def test_rpotrf_residual_large(sdpg, n, spread):
    """Factors of the Schur and X / Z sizes (256 bits, the residue path with the panel
    residues cached): A = D^(1/2) (c I + S) D^(1/2) with S symmetric in [-1, 1] and the
    row scales D_i = 2^k_i, k_i uniform in [-spread, spread].  The residual L L^T - A,
    formed by the digit GEMM (normwise error 2^-240), must satisfy Cholesky's
    componentwise backward-error form |R_ij| <= 2^-(p-24) n sqrt(A_ii A_jj)."""
    rng = np.random.default_rng(n + spread)
    S = rng.uniform(-1, 1, (n, n))
    S = np.round((S + S.T) * 2.0 ** 20) / 2.0 ** 21
    k = rng.integers(-spread, spread + 1, n) if spread else np.zeros(n, dtype=int)
    half = np.exp2(k / 2.0).round(6)  # exact doubles, about 2^(k/2)
    A = (S + np.eye(n) * (n / 4.0)) * np.outer(half, half)
    Aml = sdpg.ml_from_double(A.T.reshape(-1), 8)  # column-major
    Lml, info = sdpg.rpotrf(Aml, n, n)
    assert info == 0
    lower = np.tril(np.ones((n, n), dtype=bool)).T.reshape(-1)  # column-major i >= j
    Lml[~lower] = 0
    one = sdpg.ml_from_double(np.array([1.0]), 8)
    mone = sdpg.ml_from_double(np.array([-1.0]), 8)
    old = sdpg.set_gemm_method(1)
    try:
        R = sdpg.rgemm("N", "T", n, n, n, one, Lml, n, Lml, n, mone, Aml, n)
    finally:
        sdpg.set_gemm_method(old)
    Rd = np.abs(sdpg.ml_to_double(R).reshape(n, n).T)
    d = np.sqrt(np.diag(A))
    bound = 2.0 ** -(256 - 24) * n * np.outer(d, d)
    worst = float(np.max(Rd / bound))
    print(f"\nn={n} spread={spread}: max |L L^T - A| / bound = {worst:.3e}")
    assert worst <= 1.0
    assert sdpg.tensor_error(0) == 0


@gpu
@pytest.mark.parametrize("n,bad", [(40, 17), (70, 0), (70, 69), (200, 100)])
def test_rpotrf_reports_first_bad_pivot(sdpg, exact, n, bad):
    """A non-positive pivot at column `bad` gives info = bad + 1, like Rpotrf (n = 200: the
    look-ahead products and cached residues are in flight when panel 3 fails; the later
    panels leave at once)."""
    vals = [(0, 0)] * (n * n)
    for i in range(n):
        vals[i + i * n] = (-1, 0) if i == bad else (1, 0)
    A = exact.ml_encode(vals, 8)
    _, info = sdpg.rpotrf(A, n, n)
    assert info == bad + 1


@gpu
@pytest.mark.parametrize("limbs,n,ld", [(8, 1, 1), (8, 7, 9), (8, 32, 32), (8, 33, 33), (8, 65, 70),
                                        (8, 100, 100), (8, 128, 128), (16, 45, 45), (16, 64, 64)])
def test_inv_lower_residual(sdpg, exact, limbs, n, ld):
    rng = random.Random(7 * limbs + n)
    Lml = _lower_well_conditioned(exact, n, limbs, rng, ld)
    Xml = sdpg.inv_lower(Lml, n, ld)
    X = exact.ml_decode(Xml)
    assert all(X[i + j * n][0] == 0 for j in range(n) for i in range(j)), "strict upper triangle not zero"
    L = exact.ml_decode(Lml)
    LX = exact.matmul(L, X, n, n, n, ld, n, a_lower=True, b_lower=True)
    worst = Fraction(0)
    for j in range(n):
        for i in range(n):
            v = LX[i + j * n]
            if i == j:
                v = exact.dy_add(v, (-1, 0))
            worst = max(worst, abs(exact.to_fraction(v)))
    Lmax = exact.max_abs(L)
    Xmax = exact.max_abs(X)
    assert worst <= Fraction(n) * Lmax * Xmax / (1 << (32 * limbs - 24)), float(worst)


@gpu
@pytest.mark.parametrize("limbs,n", [(8, 1), (8, 31), (8, 64), (8, 90), (16, 50)])
def test_solve_systems_residual(sdpg, exact, limbs, n):
    rng = random.Random(31 * limbs + n)
    Lml = _lower_well_conditioned(exact, n, limbs, rng)
    b = exact.random_ml(n, limbs, rng, -2, 2)
    xml = sdpg.solve_systems(Lml, n, n, b)
    L = exact.ml_decode(Lml)
    x = exact.ml_decode(xml)
    Lt = [L[c + r * n] if c >= r else (0, 0) for c in range(n) for r in range(n)]  # column-major L^T
    y = exact.matmul(Lt, x, n, 1, n, n, n)
    r = exact.matmul(L, y, n, 1, n, n, n, a_lower=True)
    bd = exact.ml_decode(b)
    worst = max(abs(exact.to_fraction(exact.dy_add(r[i], (-bd[i][0], bd[i][1])))) for i in range(n))
    Lmax = exact.max_abs(L)
    assert worst <= Fraction(n * n) * Lmax * Lmax * exact.max_abs(x) / (1 << (32 * limbs - 24)), float(worst)


def _check_min_eig(exact, lam, limbs, scale, count_below):
    delta = scale / (1 << (32 * limbs - 40))
    assert count_below(lam - delta) == 0
    assert count_below(lam + delta) >= 1


@gpu
@pytest.mark.parametrize("limbs,k", [(8, 1), (8, 2), (8, 7), (8, 40), (8, 130), (16, 25)])
def test_tridiag_min(sdpg, exact, limbs, k):
    rng = random.Random(5 * limbs + k)
    d = exact.random_ml(k, limbs, rng, -1, 1)
    e = exact.random_ml(max(k - 1, 0), limbs, rng, -1, 1) if k > 1 else exact.random_ml(0, limbs, rng)
    out = sdpg.tridiag_min(d, e)
    res = exact.ml_decode(out)
    lam = exact.to_fraction(res[0])
    dd, ee = exact.ml_decode(d), exact.ml_decode(e) if k > 1 else []
    scale = Fraction(k) * max(exact.max_abs(dd), exact.max_abs(ee) if ee else Fraction(0))
    _check_min_eig(exact, lam, limbs, scale, lambda s: exact.count_below_tridiag(dd, ee, s))
    z2 = exact.tridiag_last_component_sq(dd, ee, lam)
    got = exact.to_fraction(res[1]) ** 2
    assert abs(got - z2) <= z2 / (1 << 100) + Fraction(1, 1 << 200), (float(got), float(z2))


@gpu
@pytest.mark.parametrize("limbs,n", [(8, 1), (8, 2), (8, 10), (8, 33), (8, 64), (16, 20)])
def test_sym_min_eigen(sdpg, exact, limbs, n):
    rng = random.Random(11 * limbs + n)
    half = exact.ml_decode(exact.random_ml(n * n, limbs, rng, -2, 1))
    vals = [half[max(i, j) + min(i, j) * n] for j in range(n) for i in range(n)]
    A = exact.ml_encode(vals, limbs)
    out = sdpg.sym_min_eigen(A, n)
    lam = exact.to_fraction(exact.ml_decode(out)[0])
    scale = Fraction(n) * exact.max_abs(vals)
    _check_min_eig(exact, lam, limbs, scale, lambda s: exact.count_below_dense(vals, n, s))


def test_argument_errors_need_no_gpu(sdpg):
    """Bad sizes are rejected on the host before any device work."""
    a = sdpg.ml_empty(4, 8)
    with pytest.raises(sdpg.SdpgError):
        sdpg.sym_min_eigen(sdpg.ml_empty(65 * 65, 8), 65)
    with pytest.raises(sdpg.SdpgError):
        sdpg.inv_lower(a, 0, 1)
    with pytest.raises(sdpg.SdpgError):
        sdpg.check(sdpg.lib().sdpg_tridiag_min(8, 0, a.ctypes.data, a.ctypes.data, a.ctypes.data))
    with pytest.raises(sdpg.SdpgError):
        sdpg.solve_systems(a, 2, 1, a)
