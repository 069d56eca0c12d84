"""Exact-arithmetic CPU restatement of the reference's dense kernels.

TEST INFRASTRUCTURE ONLY: imported by tests/ and __graft_entry__.smoke() as
the checker; never part of the product path.

Values are dyadic rationals ``v * 2**x`` held as Python integer pairs, so
sums and products are exact; square roots and quotients are computed to a
requested number of bits (far beyond the 256/512-bit formats under test).
Each function names the reference routine whose mathematics it restates.
The multi-limb element layout matches include/sdpg.h:
``[e, s, m[0..limbs-1]]`` (uint32), value = (-1)^s * M * 2^(e - 32*limbs).
"""
from __future__ import annotations

import random
from fractions import Fraction

import numpy as np

# ---------------------------------------------------------------- encoding


def ml_decode(arr: np.ndarray) -> list[tuple[int, int]]:
    """ml array -> list of (signed integer v, exponent x) with value v * 2**x."""
    arr = np.asarray(arr, dtype=np.uint32)
    limbs = arr.shape[1] - 2
    out = []
    for row in arr:
        e = int(np.int32(row[0]))
        s = int(row[1])
        M = 0
        for k in range(limbs - 1, -1, -1):
            M = (M << 32) | int(row[2 + k])
        if M == 0:
            out.append((0, 0))
        else:
            out.append((-M if s else M, e - 32 * limbs))
    return out


def ml_encode(vals, limbs: int) -> np.ndarray:
    """(v, x) pairs or Fractions -> ml array, truncating toward zero."""
    out = np.zeros((len(vals), limbs + 2), dtype=np.uint32)
    for i, val in enumerate(vals):
        if isinstance(val, Fraction):
            num, den = val.numerator, val.denominator
            if num == 0:
                continue
            s = 1 if num < 0 else 0
            num = abs(num)
            # find M = floor(num/den * 2^k) with bit length exactly 32*limbs
            k = 32 * limbs - (num.bit_length() - den.bit_length())
            while True:
                M = (num << k) // den if k >= 0 else num // (den << -k)
                bl = M.bit_length()
                if bl > 32 * limbs:
                    k -= 1
                elif bl < 32 * limbs:
                    k += 1
                else:
                    break
            e = 32 * limbs - k
        else:
            v, x = val
            if v == 0:
                continue
            s = 1 if v < 0 else 0
            M = abs(v)
            bl = M.bit_length()
            if bl > 32 * limbs:
                M >>= bl - 32 * limbs
            else:
                M <<= 32 * limbs - bl
            e = x + bl
        out[i, 0] = np.uint32(e & 0xFFFFFFFF)
        out[i, 1] = s
        for k in range(limbs):
            out[i, 2 + k] = (M >> (32 * k)) & 0xFFFFFFFF
    return out


def to_fraction(p: tuple[int, int]) -> Fraction:
    v, x = p
    return Fraction(v * (1 << x)) if x >= 0 else Fraction(v, 1 << -x)


def dy_add(a: tuple[int, int], b: tuple[int, int]) -> tuple[int, int]:
    if a[0] == 0:
        return b
    if b[0] == 0:
        return a
    x = min(a[1], b[1])
    return ((a[0] << (a[1] - x)) + (b[0] << (b[1] - x)), x)


def dy_mul(a: tuple[int, int], b: tuple[int, int]) -> tuple[int, int]:
    return (a[0] * b[0], a[1] + b[1])


def dy_abs(a):
    return (abs(a[0]), a[1])


def dy_sum(vals) -> tuple[int, int]:
    vals = [v for v in vals if v[0] != 0]
    if not vals:
        return (0, 0)
    x = min(v[1] for v in vals)
    return (sum(v[0] << (v[1] - x) for v in vals), x)


def dy_cmp_abs_le(a, b, tol_bits: int, scale) -> bool:
    """|a| <= 2**-tol_bits * |scale| ?"""
    lhs = to_fraction(dy_abs(a))
    rhs = to_fraction(dy_abs(scale)) / (1 << tol_bits)
    return lhs <= rhs


# ---------------------------------------------------------------- random inputs


def random_ml(count: int, limbs: int, rng: random.Random, emin: int = -8, emax: int = 8,
              zero_frac: float = 0.0) -> np.ndarray:
    """Random full-precision values with exponents in [emin, emax]."""
    vals = []
    for _ in range(count):
        if zero_frac and rng.random() < zero_frac:
            vals.append((0, 0))
            continue
        M = rng.getrandbits(32 * limbs) | (1 << (32 * limbs - 1))
        e = rng.randint(emin, emax)
        s = -1 if rng.random() < 0.5 else 1
        vals.append((s * M, e - 32 * limbs))
    return ml_encode(vals, limbs)


# ---------------------------------------------------------------- kernels


def gemm(transa: str, transb: str, m: int, n: int, k: int, alpha, A, lda: int, B, ldb: int, beta, C,
         ldc: int):
    """Exact C = alpha*op(A)*op(B) + beta*C (Rgemm, mplapack/Rgemm_omp.cpp:41-127).

    A, B, C are lists of (v, x) pairs in column-major order; returns the exact
    result list and, per entry, the normwise scale K * max|a_i.| * max|b_.j| *
    |alpha| + |beta c_ij| used by the tolerance check."""
    def a_el(i, l):
        return A[i + l * lda] if transa.upper() == "N" else A[l + i * lda]

    def b_el(l, j):
        return B[l + j * ldb] if transb.upper() == "N" else B[j + l * ldb]

    out = list(C)
    scale = [(0, 0)] * len(C)
    rowmax = []
    for i in range(m):
        mx = Fraction(0)
        for l in range(k):
            mx = max(mx, abs(to_fraction(a_el(i, l))))
        rowmax.append(mx)
    colmax = []
    for j in range(n):
        mx = Fraction(0)
        for l in range(k):
            mx = max(mx, abs(to_fraction(b_el(l, j))))
        colmax.append(mx)
    fa = abs(to_fraction(alpha))
    fb = abs(to_fraction(beta))
    for j in range(n):
        bcol = [b_el(l, j) for l in range(k)]
        for i in range(m):
            s = dy_sum(dy_mul(a_el(i, l), bcol[l]) for l in range(k))
            r = dy_add(dy_mul(alpha, s), dy_mul(beta, C[i + j * ldc]) if beta[0] else (0, 0))
            out[i + j * ldc] = r
            sc = fa * k * rowmax[i] * colmax[j] + fb * abs(to_fraction(C[i + j * ldc]))
            scale[i + j * ldc] = sc
    return out, scale


def max_rel_err(got: np.ndarray, exact, scale) -> float:
    """max_i |got_i - exact_i| / scale_i, as a float (log2-safe)."""
    g = ml_decode(got)
    worst = Fraction(0)
    for gi, ei, si in zip(g, exact, scale):
        d = abs(to_fraction(dy_add(gi, (-ei[0], ei[1]))))
        s = si if isinstance(si, Fraction) else abs(to_fraction(si))
        if s == 0:
            if d != 0:
                return float("inf")
            continue
        worst = max(worst, d / s)
    return float(worst)


# ---------------------------------------------------------------- factorisations and eigenvalues


def matmul(A, B, m: int, n: int, k: int, lda: int, ldb: int, a_lower: bool = False,
           b_lower: bool = False) -> list[tuple[int, int]]:
    """Exact column-major m x n product of (m x k) A and (k x n) B; a triangular flag
    skips the structural zeros (used to form L L^T, L X and L (L^T x) residuals of
    Rpotrf, Rtrsm and Rtrsv, mplapack/Rpotrf.cpp, Rtrsm.cpp, Rtrsv.cpp)."""
    out = []
    for j in range(n):
        for i in range(m):
            lo, hi = 0, k
            if a_lower:
                hi = min(hi, i + 1)
            if b_lower:
                lo = max(lo, j)
            out.append(dy_sum(dy_mul(A[i + t * lda], B[t + j * ldb]) for t in range(lo, hi)))
    return out


def max_abs(vals) -> Fraction:
    return max((abs(to_fraction(v)) for v in vals), default=Fraction(0))


def _to_int_scale(vals):
    """Common exponent x and integers v_i with vals_i = v_i * 2**x."""
    nz = [v for v in vals if v[0] != 0]
    x = min((v[1] for v in nz), default=0)
    return [(v[0] << (v[1] - x)) if v[0] else 0 for v in vals], x


def count_below_tridiag(d, e, sigma: Fraction) -> int:
    """Number of eigenvalues of tridiag(e, d, e) below sigma: sign changes of the
    leading principal minors of T - sigma I (Sturm sequence), exact in rationals.
    Restates the bisection count behind Rsteqr's ordering, mplapack/Rsteqr.cpp."""
    p_prev, p = Fraction(1), to_fraction(d[0]) - sigma
    changes = 1 if p < 0 else 0
    if p == 0:
        raise ValueError("sigma is an eigenvalue of a leading block")
    for i in range(1, len(d)):
        ei = to_fraction(e[i - 1])
        p_prev, p = p, (to_fraction(d[i]) - sigma) * p - ei * ei * p_prev
        if p == 0:
            raise ValueError("sigma is an eigenvalue of a leading block")
        if (p < 0) != (p_prev < 0):
            changes += 1
    return changes


def tridiag_last_component_sq(d, e, lam: Fraction) -> Fraction:
    """z_k^2 = p_{k-1}(lam) / p_k'(lam) for the unit eigenvector of tridiag(e, d, e)
    belonging to the simple eigenvalue lam (p_i the leading minors of lam I - T)."""
    k = len(d)
    p_prev, p = Fraction(1), lam - to_fraction(d[0])
    dp_prev, dp = Fraction(0), Fraction(1)
    for i in range(1, k):
        ei2 = to_fraction(e[i - 1]) ** 2
        a = lam - to_fraction(d[i])
        p_new = a * p - ei2 * p_prev
        dp_new = p + a * dp - ei2 * dp_prev
        p_prev, p, dp_prev, dp = p, p_new, dp, dp_new
    return p_prev / dp


def count_below_dense(A, n: int, sigma: Fraction) -> int:
    """Number of eigenvalues of the symmetric n x n A (column-major, full storage)
    below sigma, from the signs of the leading principal minors of A - sigma I
    computed by fraction-free (Bareiss) elimination.  The reference obtains the
    eigenvalues from Rsyev (mplapack/Rsyev.cpp); inertia pins the smallest one."""
    num, den = sigma.numerator, sigma.denominator
    if den & (den - 1):
        raise ValueError("sigma must be dyadic")
    vals, x = _to_int_scale(list(A))
    sh = den.bit_length() - 1
    t = max(-x, sh)  # M = (A - sigma I) * 2^t is integral
    M = [[vals[i + j * n] << (x + t) for j in range(n)] for i in range(n)]
    s_int = num << (t - sh)
    for i in range(n):
        M[i][i] -= s_int
    prev = 1
    changes = 0
    sign_prev = 1
    for k in range(n):
        piv = M[k][k]
        if piv == 0:
            raise ValueError("zero leading minor")
        sgn = 1 if piv > 0 else -1
        if sgn != sign_prev:
            changes += 1
        sign_prev = sgn
        for i in range(k + 1, n):
            for j in range(k + 1, n):
                M[i][j] = (M[i][j] * piv - M[i][k] * M[k][j]) // prev
        prev = piv
    return changes
