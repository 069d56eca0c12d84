// Multi-limb binary floating point ("mlf"): the number format that stands in
// for the reference's GMP mpf_class values on the GPU and in host control code.
//
//   value = (-1)^s * M * 2^(e - 32N),   M = sum_k m[k] * 2^(32k)   (m[0] least significant)
//
// M is normalised (top bit of m[N-1] set), so |value| lies in [2^(e-1), 2^e).
// Zero has M == 0 (m[N-1] == 0), e == 0, s == 0.  Results are truncated
// toward zero like GMP's mpf operations (mpf/mul.c, mpf/add.c truncate);
// add/sub keep two guard limbs and the product keeps the columns from N-2 up,
// so each operation is accurate to a few units in the last place.
//
// N = 8 gives a 256-bit mantissa, N = 16 a 512-bit one.  GMP at precision P
// carries ((P+127)/64) 64-bit limbs (gmp-impl.h __GMPF_BITS_TO_PREC), i.e. 257-320
// bits for P = 200 or 256: the 256-bit format is at most 64 bits shorter.
//
// Everything here is __host__ __device__: the same code computes kernels on the
// GPU and the IPM's scalar control logic (step lengths, centering, gaps) on the host.
// All limb indices are compile-time after unrolling, so on the GPU the arrays
// stay in registers; variable shifts use a logarithmic barrel shifter.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define MLHD __host__ __device__ __forceinline__
#define ML_ALIGN __align__(8)
#else
#define MLHD inline
#define ML_ALIGN alignas(8)
#endif

#if defined(__CUDA_ARCH__)
#define ML_UNROLL _Pragma("unroll")
#else
#define ML_UNROLL
#endif

namespace sdpg {

template <int N>
struct ML_ALIGN mlf {
    int32_t e;
    uint32_t s;
    uint32_t m[N];
};

MLHD int ml_clz32(uint32_t x) {
#if defined(__CUDA_ARCH__)
    return __clz(x);
#else
    return x ? __builtin_clz(x) : 32;
#endif
}

// Low 32 bits of (hi:lo) >> r and high 32 bits of (hi:lo) << r, 0 <= r < 32, without a
// branch on r (SIMT lanes with different shift counts stay converged).
MLHD uint32_t ml_fshr(uint32_t lo, uint32_t hi, int r) {
#if defined(__CUDA_ARCH__)
    return __funnelshift_r(lo, hi, (unsigned)r);
#else
    return (uint32_t)((((uint64_t)hi << 32) | lo) >> r);
#endif
}
MLHD uint32_t ml_fshl(uint32_t lo, uint32_t hi, int r) {
#if defined(__CUDA_ARCH__)
    return __funnelshift_l(lo, hi, (unsigned)r);
#else
    return (uint32_t)(((((uint64_t)hi << 32) | lo) << r) >> 32);
#endif
}

template <int N>
MLHD mlf<N> ml_zero() {
    mlf<N> r;
    r.e = 0;
    r.s = 0;
    ML_UNROLL
    for (int k = 0; k < N; ++k) r.m[k] = 0;
    return r;
}

template <int N>
MLHD bool ml_is_zero(const mlf<N> &a) { return a.m[N - 1] == 0; }

template <int N>
MLHD mlf<N> ml_neg(mlf<N> a) {
    if (!ml_is_zero(a)) a.s ^= 1u;
    return a;
}

template <int N>
MLHD mlf<N> ml_abs(mlf<N> a) {
    a.s = 0;
    return a;
}

// value * 2^k (exact)
template <int N>
MLHD mlf<N> ml_ldexp(mlf<N> a, int k) {
    if (!ml_is_zero(a)) a.e += k;
    return a;
}

// --- limb-array helpers (compile-time length L) ---------------------------------

// r = a >> (32*q) for a dynamic limb count q in [0, L]; logarithmic barrel shifter.
template <int L>
MLHD void ml_limb_shr(uint32_t (&a)[L], int q) {
    ML_UNROLL
    for (int step = 1; step < 2 * L; step <<= 1) {
        if (step > L) break;
        const bool take = (q & step) != 0;
        ML_UNROLL
        for (int k = 0; k < L; ++k) {
            const uint32_t v = (k + step < L) ? a[k + step] : 0u;
            a[k] = take ? v : a[k];
        }
    }
}

// a <<= 32*q (limbs), q in [0, L]
template <int L>
MLHD void ml_limb_shl(uint32_t (&a)[L], int q) {
    ML_UNROLL
    for (int step = 1; step < 2 * L; step <<= 1) {
        if (step > L) break;
        const bool take = (q & step) != 0;
        ML_UNROLL
        for (int k = L - 1; k >= 0; --k) {
            const uint32_t v = (k - step >= 0) ? a[k - step] : 0u;
            a[k] = take ? v : a[k];
        }
    }
}

// a >>= r bits, 0 <= r < 32
template <int L>
MLHD void ml_bit_shr(uint32_t (&a)[L], int r) {
    ML_UNROLL
    for (int k = 0; k < L; ++k) a[k] = ml_fshr(a[k], (k + 1 < L) ? a[k + 1] : 0u, r);
}

// a <<= r bits, 0 <= r < 32
template <int L>
MLHD void ml_bit_shl(uint32_t (&a)[L], int r) {
    ML_UNROLL
    for (int k = L - 1; k >= 0; --k) a[k] = ml_fshl((k >= 1) ? a[k - 1] : 0u, a[k], r);
}

// Number of leading zero bits of the L-limb number a (32*L if zero).
template <int L>
MLHD int ml_clz_limbs(const uint32_t (&a)[L]) {
    int lz = 0;
    bool found = false;
    ML_UNROLL
    for (int k = L - 1; k >= 0; --k) {
        lz += found ? 0 : ml_clz32(a[k]);
        found = found || a[k] != 0;
    }
    return lz;
}

// Normalise an L-limb magnitude (L >= N) into an mlf<N> whose exponent is
// `e_top` when the top bit of a[L-1] is set.  Truncates the low limbs.
template <int N, int L>
MLHD mlf<N> ml_pack(uint32_t (&a)[L], int e_top, uint32_t sign) {
    const int lz = ml_clz_limbs<L>(a);
    const bool zero = lz >= 32 * L;
    ml_limb_shl<L>(a, zero ? 0 : (lz >> 5));
    ml_bit_shl<L>(a, lz & 31);
    mlf<N> r;
    r.e = zero ? 0 : e_top - lz;
    r.s = zero ? 0u : sign;
    ML_UNROLL
    for (int k = 0; k < N; ++k) r.m[k] = zero ? 0u : a[L - N + k];
    return r;
}

// Compare magnitudes of mantissas: -1, 0, 1
template <int N>
MLHD int ml_cmp_mant(const uint32_t (&a)[N], const uint32_t (&b)[N]) {
    int r = 0;
    ML_UNROLL
    for (int k = N - 1; k >= 0; --k) {
        if (r == 0) r = (a[k] > b[k]) ? 1 : ((a[k] < b[k]) ? -1 : 0);
    }
    return r;
}

// |a| vs |b|
template <int N>
MLHD int ml_cmp_abs(const mlf<N> &a, const mlf<N> &b) {
    const bool za = ml_is_zero(a), zb = ml_is_zero(b);
    const int cm = ml_cmp_mant<N>(a.m, b.m);
    const int c = (a.e > b.e) ? 1 : ((a.e < b.e) ? -1 : cm);
    return za ? (zb ? 0 : -1) : (zb ? 1 : c);
}

template <int N>
MLHD int ml_sign(const mlf<N> &a) { return ml_is_zero(a) ? 0 : (a.s ? -1 : 1); }

template <int N>
MLHD int ml_cmp(const mlf<N> &a, const mlf<N> &b) {
    const int sa = ml_sign(a), sb = ml_sign(b);
    if (sa != sb) return sa > sb ? 1 : -1;
    if (sa == 0) return 0;
    const int c = ml_cmp_abs(a, b);
    return sa > 0 ? c : -c;
}

// --- addition -------------------------------------------------------------------

// Straight-line code (selects, no data-dependent branches), so SIMT lanes adding
// operands of different signs and exponents stay converged: the smaller operand is
// aligned, added in two's complement (negated when the signs differ), a carry out of
// a same-sign sum renormalises by one bit, and cancellation is normalised by ml_pack.
template <int N>
MLHD mlf<N> ml_add(const mlf<N> &a, const mlf<N> &b) {
    constexpr int L = N + 2;
    const bool swap = ml_cmp_abs(b, a) > 0;
    mlf<N> x, y;  // |x| >= |y|
    x.e = swap ? b.e : a.e;
    x.s = swap ? b.s : a.s;
    y.e = swap ? a.e : b.e;
    y.s = swap ? a.s : b.s;
    ML_UNROLL
    for (int k = 0; k < N; ++k) {
        x.m[k] = swap ? b.m[k] : a.m[k];
        y.m[k] = swap ? a.m[k] : b.m[k];
    }
    int d = x.e - y.e;
    d = (ml_is_zero(y) || d > 32 * L) ? 32 * L : d;
    uint32_t xx[L], yy[L];
    xx[0] = 0;
    xx[1] = 0;
    yy[0] = 0;
    yy[1] = 0;
    ML_UNROLL
    for (int k = 0; k < N; ++k) {
        xx[k + 2] = x.m[k];
        yy[k + 2] = y.m[k];
    }
    ml_limb_shr<L>(yy, d >> 5);
    ml_bit_shr<L>(yy, d & 31);
    const bool sub = x.s != y.s;
    uint64_t c = sub ? 1u : 0u;
    ML_UNROLL
    for (int k = 0; k < L; ++k) {
        c += (uint64_t)xx[k] + (sub ? ~yy[k] : yy[k]);
        xx[k] = (uint32_t)c;
        c >>= 32;
    }
    const bool ovf = !sub && c != 0;  // same-sign sum one bit wider than x
    ML_UNROLL
    for (int k = 0; k < L; ++k) {
        const uint32_t hi = (k + 1 < L) ? xx[k + 1] : 1u;
        xx[k] = ovf ? ml_fshr(xx[k], hi, 1) : xx[k];
    }
    return ml_pack<N, L>(xx, x.e + (ovf ? 1 : 0), x.s);
}

template <int N>
MLHD mlf<N> ml_sub(const mlf<N> &a, const mlf<N> &b) { return ml_add(a, ml_neg(b)); }

// --- multiplication -------------------------------------------------------------------
//
// Each mantissa is split into D radix-2^28 digits; a digit product is < 2^56, so
// a column of <= D of them fits an unsigned 64-bit accumulator without carry
// handling.  Every column is an independent chain of 32x32->64 multiply-adds
// (short dependence chains, high instruction-level parallelism), followed by one
// carry pass.  Columns below D-2 are dropped (their sum is below 2^-(32N-1) of the
// product), then the top 32N bits are taken: the result is truncated like GMP's.

template <int N>
struct MulDigits {
    static constexpr int D = (32 * N + 27) / 28;  // N=8 -> 10, N=16 -> 19
    static constexpr int CK = D - 2;              // lowest kept product column
    static constexpr int NCOL = 2 * D - 1 - CK;   // kept columns CK .. 2D-2
    static constexpr int B0 = 28 * CK;            // bit weight of column CK
    static constexpr int TOPREL = 64 * N - 1 - B0;  // product's top possible bit, relative to B0
    static constexpr int LW = (28 * (NCOL + 1) + 31) / 32 + 2;
};

template <int N>
MLHD void ml_digits28(const uint32_t (&m)[N], uint32_t (&d)[MulDigits<N>::D]) {
    ML_UNROLL
    for (int t = 0; t < MulDigits<N>::D; ++t) {
        const int bit = 28 * t;
        const int w = bit >> 5, r = bit & 31;
        const uint32_t lo = (w < N) ? (m[w] >> r) : 0u;
        const uint32_t hi = (r > 4 && w + 1 < N) ? (m[w + 1] << (32 - r)) : 0u;
        d[t] = (lo | hi) & 0x0FFFFFFFu;
    }
}

// 32 bits of W starting at compile-time bit offset `off`
template <int L>
MLHD uint32_t ml_bits32(const uint32_t (&W)[L], int off) {
    const int w = off >> 5, r = off & 31;
    const uint32_t lo = (w < L) ? (W[w] >> r) : 0u;
    const uint32_t hi = (r != 0 && w + 1 < L) ? (W[w + 1] << (32 - r)) : 0u;
    return lo | hi;
}

template <int N>
MLHD mlf<N> ml_mul(const mlf<N> &a, const mlf<N> &b) {
    const bool zero = ml_is_zero(a) || ml_is_zero(b);
    using G = MulDigits<N>;
    uint32_t da[G::D], db[G::D];
    ml_digits28<N>(a.m, da);
    ml_digits28<N>(b.m, db);
    uint64_t acc[G::NCOL + 1];
    ML_UNROLL
    for (int c = 0; c <= G::NCOL; ++c) acc[c] = 0;
    ML_UNROLL
    for (int c = G::CK; c <= 2 * G::D - 2; ++c) {
        ML_UNROLL
        for (int p = 0; p < G::D; ++p) {
            const int q = c - p;
            if (q >= 0 && q < G::D) acc[c - G::CK] += (uint64_t)da[p] * db[q];
        }
    }
    ML_UNROLL
    for (int c = 0; c < G::NCOL; ++c) {
        acc[c + 1] += acc[c] >> 28;
        acc[c] &= 0x0FFFFFFFull;
    }
    uint32_t W[G::LW];
    ML_UNROLL
    for (int w = 0; w < G::LW; ++w) W[w] = 0;
    ML_UNROLL
    for (int c = 0; c <= G::NCOL; ++c) {
        const int bit = 28 * c;
        const int w = bit >> 5, r = bit & 31;
        W[w] |= (uint32_t)(acc[c] << r);
        if (w + 1 < G::LW) W[w + 1] |= (uint32_t)(acc[c] >> (32 - r));
    }
    const bool top = (W[G::TOPREL >> 5] >> (G::TOPREL & 31)) & 1u;
    constexpr int off = G::TOPREL + 1 - 32 * N;  // lowest mantissa bit when the top bit is set
    mlf<N> o;
    o.s = zero ? 0u : (a.s ^ b.s);
    o.e = zero ? 0 : a.e + b.e - (top ? 0 : 1);
    ML_UNROLL
    for (int k = 0; k < N; ++k) {
        const uint32_t hi = ml_bits32<G::LW>(W, off + 32 * k), lo = ml_bits32<G::LW>(W, off - 1 + 32 * k);
        o.m[k] = zero ? 0u : (top ? hi : lo);
    }
    return o;
}

// a*b + c (product rounded, then the sum)
template <int N>
MLHD mlf<N> ml_fma(const mlf<N> &a, const mlf<N> &b, const mlf<N> &c) { return ml_add(ml_mul(a, b), c); }

// --- conversions ----------------------------------------------------------------

MLHD uint64_t ml_dbits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, 8);
    return u;
#endif
}

MLHD double ml_bitsd(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, 8);
    return x;
#endif
}

// Exact conversion from an IEEE double (finite values).
template <int N>
MLHD mlf<N> ml_from_double(double x) {
    const uint64_t u = ml_dbits(x);
    const uint32_t sign = (uint32_t)(u >> 63);
    const int ex = (int)((u >> 52) & 0x7ff);
    uint64_t frac = u & 0xfffffffffffffull;
    int e2;  // value = frac * 2^e2 with frac an integer
    if (ex == 0) {
        if (frac == 0) return ml_zero<N>();
        e2 = -1074;
    } else {
        frac |= 1ull << 52;
        e2 = ex - 1075;
    }
    // normalise frac to 64 bits with top bit set
    int lz = 0;
    while (!(frac & 0x8000000000000000ull)) {
        frac <<= 1;
        ++lz;
    }
    mlf<N> r = ml_zero<N>();
    r.s = sign;
    r.m[N - 1] = (uint32_t)(frac >> 32);
    r.m[N - 2] = (uint32_t)frac;
    // value = frac64 * 2^(e2 - lz), frac64 in [2^63, 2^64) -> |value| in [2^(e-1), 2^e) with
    r.e = e2 - lz + 64;
    return r;
}

template <int N>
MLHD mlf<N> ml_from_int(int64_t v) {
    if (v == 0) return ml_zero<N>();
    const uint32_t sign = v < 0 ? 1u : 0u;
    uint64_t a = v < 0 ? (uint64_t)(-(v + 1)) + 1u : (uint64_t)v;
    int lz = 0;
    while (!(a & 0x8000000000000000ull)) {
        a <<= 1;
        ++lz;
    }
    mlf<N> r = ml_zero<N>();
    r.s = sign;
    r.m[N - 1] = (uint32_t)(a >> 32);
    r.m[N - 2] = (uint32_t)a;
    r.e = 64 - lz;
    return r;
}

// Truncating conversion to double (exponents outside double range give 0 or inf).
template <int N>
MLHD double ml_to_double(const mlf<N> &a) {
    if (ml_is_zero(a)) return 0.0;
    const uint64_t top = ((uint64_t)a.m[N - 1] << 32) | a.m[N - 2];
    const double v = ldexp((double)(top >> 11), a.e - 53);
    return a.s ? -v : v;
}

template <int N>
MLHD mlf<N> ml_one() { return ml_from_int<N>(1); }

// --- division and square root (Newton-Raphson on the mantissa) -------------------

// Precision conversions: keep the top M limbs (truncating) / extend with zero limbs.
template <int M, int N>
MLHD mlf<M> ml_narrow(const mlf<N> &a) {
    mlf<M> r;
    r.e = a.e;
    r.s = a.s;
    ML_UNROLL
    for (int k = 0; k < M; ++k) r.m[k] = (N - M + k >= 0) ? a.m[N - M + k] : 0u;
    return r;
}
template <int M, int N>
MLHD mlf<M> ml_widen(const mlf<N> &a) {
    mlf<M> r;
    r.e = a.e;
    r.s = a.s;
    ML_UNROLL
    for (int k = 0; k < M; ++k) r.m[k] = (k - (M - N) >= 0) ? a.m[k - (M - N)] : 0u;
    return r;
}

// Single-precision seeds.  The FP32 units give a 22-24 bit start in a few dozen
// cycles (FP64 is far slower on this part), and Newton steps carried out in the
// multi-limb format at rising precision take it from there.
template <int N>
MLHD mlf<N> ml_from_float_pos(float x) {  // x > 0, finite and normal
    uint32_t u;
    memcpy(&u, &x, 4);
    mlf<N> r = ml_zero<N>();
    r.m[N - 1] = ((u & 0x7fffffu) | 0x800000u) << 8;
    r.e = (int)((u >> 23) & 0xff) - 126;
    return r;
}

template <int N>
MLHD mlf<N> ml_from_float(float x) {  // finite x; subnormals become zero
    if (!(fabsf(x) >= 1.17549435e-38f)) return ml_zero<N>();
    mlf<N> r = ml_from_float_pos<N>(fabsf(x));
    r.s = x < 0.0f ? 1u : 0u;
    return r;
}

// top 24 bits of the mantissa scaled by 2^e, as a float (e is 0 or 1 here)
template <int N>
MLHD float ml_mant_float(const mlf<N> &a) {
    const float f = (float)(a.m[N - 1] >> 8) * 5.9604644775390625e-8f;  // 2^-24
    return a.e > 0 ? 2.0f * f : f;
}

MLHD float ml_rsqrt_float(float f) {
#ifdef __CUDA_ARCH__
    return rsqrtf(f);
#else
    return 1.0f / sqrtf(f);
#endif
}

// 1/bn for a mantissa bn in [1/2, 1): Newton steps at rising precision (N/2 first,
// then one step at N doubles the correct bits), so only the last steps pay full cost.
template <int N>
MLHD mlf<N> ml_recip_mant(const mlf<N> &bn) {
    const mlf<N> one = ml_one<N>();
    mlf<N> x;
    if constexpr (N <= 2) {
        x = ml_from_float_pos<N>(1.0f / ml_mant_float(bn));  // ~23 bits
        x = ml_add(x, ml_mul(x, ml_sub(one, ml_mul(bn, x))));
    } else {
        x = ml_widen<N, N / 2>(ml_recip_mant<N / 2>(ml_narrow<N / 2, N>(bn)));
    }
    x = ml_add(x, ml_mul(x, ml_sub(one, ml_mul(bn, x))));
    return x;
}

// 1/b.  The mantissa reciprocal at half precision seeds one cubic (Halley) step at
// full precision: with t = 1 - bn x, x' = x (1 + t + t^2) has error O(t^3).
template <int N>
MLHD mlf<N> ml_recip(const mlf<N> &b) {
    if (ml_is_zero(b)) return ml_zero<N>();  // caller guards; no IEEE infinities in this format
    mlf<N> bn = b;  // bn = mantissa in [1/2, 1)
    bn.e = 0;
    bn.s = 0;
    const mlf<N> one = ml_one<N>();
    mlf<N> x;
    if constexpr (N <= 2) {
        x = ml_recip_mant<N>(bn);
        x = ml_add(x, ml_mul(x, ml_sub(one, ml_mul(bn, x))));
    } else {
        // N/2 limbs seed: about 62 bits at N/2 = 2, 124 at 4, 248 at 8
        x = ml_widen<N, N / 2>(ml_recip_mant<N / 2>(ml_narrow<N / 2, N>(bn)));
        const mlf<N> t = ml_sub(one, ml_mul(bn, x));
        constexpr int H = N / 2 + 1;
        const mlf<H> th = ml_narrow<H, N>(t);
        const mlf<H> corr = ml_mul(ml_narrow<H, N>(x), ml_add(th, ml_mul(th, th)));
        x = ml_add(x, ml_widen<N, H>(corr));
    }
    x.e -= b.e;
    x.s = b.s;
    return x;
}

// a/b with one residual correction
template <int N>
MLHD mlf<N> ml_div(const mlf<N> &a, const mlf<N> &b) {
    if (ml_is_zero(a)) return ml_zero<N>();
    const mlf<N> x = ml_recip(b);
    mlf<N> q = ml_mul(a, x);
    const mlf<N> r = ml_sub(a, ml_mul(b, q));
    q = ml_add(q, ml_mul(r, x));
    return q;
}

// 1/sqrt(an) for an in [1/4, 1): Newton steps y += y (1 - an y^2) / 2 at rising precision
template <int N>
MLHD mlf<N> ml_rsqrt_mant(const mlf<N> &an) {
    const mlf<N> one = ml_one<N>();
    mlf<N> y;
    if constexpr (N <= 2) {
        y = ml_from_float_pos<N>(ml_rsqrt_float(ml_mant_float(an)));  // ~22 bits
        const mlf<N> t = ml_sub(one, ml_mul(an, ml_mul(y, y)));
        y = ml_add(y, ml_ldexp(ml_mul(y, t), -1));
    } else {
        y = ml_widen<N, N / 2>(ml_rsqrt_mant<N / 2>(ml_narrow<N / 2, N>(an)));
    }
    const mlf<N> t = ml_sub(one, ml_mul(an, ml_mul(y, y)));
    return ml_add(y, ml_ldexp(ml_mul(y, t), -1));
}

// 1/sqrt(a), a > 0.  Half-precision seed, then one cubic (Halley) step at full
// precision: t = 1 - an y^2, y' = y (1 + t/2 + 3t^2/8), error O(t^3).
template <int N>
MLHD mlf<N> ml_rsqrt(const mlf<N> &a) {
    if (ml_is_zero(a) || a.s) return ml_zero<N>();
    // a = an * 2^(2k) with an in [1/4, 1)
    const int k = a.e >> 1;  // floor(e/2)
    mlf<N> an = a;
    an.e = a.e - 2 * k;  // 0 or 1
    const mlf<N> one = ml_one<N>();
    mlf<N> y;
    if constexpr (N <= 2) {
        y = ml_rsqrt_mant<N>(an);
        const mlf<N> t = ml_sub(one, ml_mul(an, ml_mul(y, y)));
        y = ml_add(y, ml_ldexp(ml_mul(y, t), -1));
    } else {
        // N/2 limbs seed: about 62 bits at N/2 = 2, 124 at 4, 248 at 8
        y = ml_widen<N, N / 2>(ml_rsqrt_mant<N / 2>(ml_narrow<N / 2, N>(an)));
        const mlf<N> t = ml_sub(one, ml_mul(an, ml_mul(y, y)));
        constexpr int H = N / 2 + 1;
        const mlf<H> th = ml_narrow<H, N>(t);
        const mlf<H> t2 = ml_mul(th, th);
        // t/2 + 3t^2/8 = t/2 + (t^2 + t^2/2)/4
        const mlf<H> poly = ml_add(ml_ldexp(th, -1), ml_ldexp(ml_add(t2, ml_ldexp(t2, -1)), -2));
        y = ml_add(y, ml_widen<N, H>(ml_mul(ml_narrow<H, N>(y), poly)));
    }
    y.e -= k;
    return y;
}

template <int N>
MLHD mlf<N> ml_sqrt(const mlf<N> &a) {
    if (ml_is_zero(a) || a.s) return ml_zero<N>();
    const mlf<N> y = ml_rsqrt(a);
    mlf<N> s = ml_mul(a, y);
    // s += y * (a - s^2) / 2
    s = ml_add(s, ml_ldexp(ml_mul(y, ml_sub(a, ml_mul(s, s))), -1));
    return s;
}

template <int N>
MLHD mlf<N> ml_max(const mlf<N> &a, const mlf<N> &b) { return ml_cmp(a, b) >= 0 ? a : b; }
template <int N>
MLHD mlf<N> ml_min(const mlf<N> &a, const mlf<N> &b) { return ml_cmp(a, b) <= 0 ? a : b; }

}  // namespace sdpg
