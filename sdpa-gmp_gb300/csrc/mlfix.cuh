// Exact sums of multi-limb values in integer arithmetic (host and device).
//
// Signed fixed point (ml_to_fix / ml_fix_add / ml_from_fix): a group of values is summed
// as two's-complement integers relative to the group's largest exponent and rounded once;
// the warp and block reductions of mlwarp.cuh are built on it.
//
// Block floating point (bfp_*): values as signed fractions x 2^-E (E the largest exponent
// of their row) held as D digits of 28 bits, so a product of two is about D^2 / 2 digit
// products accumulated exactly in 64-bit columns, with no per-term normalisation; the
// columns below the top D + 1 are dropped and a whole dot product is rounded to N limbs
// once.  The Cholesky panel update (chol.cu) uses it.
#pragma once
#include "ml.cuh"

namespace sdpg {

// ---- exact sums in signed fixed point ----
// A group of values is summed as two's-complement integers of W = N + 2 words relative to
// the group's largest exponent E (a value of exponent E has its mantissa in words 1..N,
// the top word is headroom and sign), so the tree needs only word-wise integer adds and
// the sum is rounded to N limbs once.  Each value loses the bits below 2^-32 of the
// frame's last mantissa word, about 2^-(32N+32) of the largest value.
constexpr int kFixNone = -(1 << 30);  // exponent of a group with no nonzero value

template <int N>
MLHD void ml_to_fix(const mlf<N> &v, int E, uint32_t (&a)[N + 2]) {
    constexpr int W = N + 2;
    a[0] = 0u;
    ML_UNROLL
    for (int k = 0; k < N; ++k) a[k + 1] = v.m[k];
    a[N + 1] = 0u;
    const int delta = E - v.e;
    const bool zero = v.m[N - 1] == 0u || delta >= 32 * W || delta < 0;
    ml_limb_shr<W>(a, zero ? 0 : (delta >> 5));
    ml_bit_shr<W>(a, zero ? 0 : (delta & 31));
    uint32_t carry = v.s ? 1u : 0u;  // negative: ~a + 1
    ML_UNROLL
    for (int k = 0; k < W; ++k) {
        const uint32_t x = zero ? 0u : (v.s ? ~a[k] : a[k]);
        const uint64_t t = (uint64_t)x + (zero ? 0u : carry);
        a[k] = (uint32_t)t;
        carry = (uint32_t)(t >> 32);
    }
}

template <int W>
MLHD void ml_fix_add(uint32_t (&a)[W], const uint32_t (&b)[W]) {
    uint32_t carry = 0u;
    ML_UNROLL
    for (int k = 0; k < W; ++k) {
        const uint64_t t = (uint64_t)a[k] + b[k] + carry;
        a[k] = (uint32_t)t;
        carry = (uint32_t)(t >> 32);
    }
}

// the fixed-point sum of a group with largest exponent E, rounded to N limbs
template <int N>
MLHD mlf<N> ml_from_fix(uint32_t (&a)[N + 2], int E) {
    constexpr int W = N + 2;
    if (E == kFixNone) return ml_zero<N>();
    const bool neg = (a[W - 1] >> 31) != 0u;
    uint32_t carry = 1u;
    ML_UNROLL
    for (int k = 0; k < W; ++k) {  // |a|
        const uint64_t t = (uint64_t)(neg ? ~a[k] : a[k]) + (neg ? carry : 0u);
        a[k] = (uint32_t)t;
        carry = (uint32_t)(t >> 32);
    }
    return ml_pack<N, W>(a, E + 32, neg ? 1u : 0u);
}

template <int N>
struct BfpShape {
    using G = MulDigits<N>;
    static constexpr int D = G::D;              // digits per value
    static constexpr int CK = G::CK;            // lowest product column kept
    static constexpr int NC = 2 * D - 1 - CK + 2;  // kept columns plus two for carries
    static constexpr int LW = (28 * NC + 31) / 32;
    static constexpr int EVERY = N <= 8 ? 8 : 4;   // terms between carry passes (no int64 overflow)
};
// between carry passes a column gains at most EVERY * D products below 2^56 each
static_assert(BfpShape<8>::EVERY * BfpShape<8>::D < 120 && BfpShape<16>::EVERY * BfpShape<16>::D < 120,
              "column sums stay below 2^63");

// x 2^-E as D signed digits of 28 bits (x's sign on every digit); E >= x.e
template <int N>
MLHD void bfp_digits(const mlf<N> &x, int E, int32_t (&d)[BfpShape<N>::D]) {
    constexpr int D = BfpShape<N>::D, L = N + 1;
    constexpr int up = 28 * D - 32 * N;  // the mantissa's place in the 28 D-bit fraction
    static_assert(up > 0 && up < 32, "digit frame");
    uint32_t a[L];
    a[0] = x.m[0] << up;
ML_UNROLL
    for (int k = 1; k < N; ++k) a[k] = (x.m[k] << up) | (x.m[k - 1] >> (32 - up));
    a[N] = x.m[N - 1] >> (32 - up);
    const int delta = E - x.e;
    const bool zero = x.m[N - 1] == 0u || delta >= 32 * L;
    ml_limb_shr<L>(a, zero ? 0 : (delta >> 5));
    ml_bit_shr<L>(a, zero ? 0 : (delta & 31));
ML_UNROLL
    for (int p = 0; p < D; ++p) {
        const int bit = 28 * p, w = bit >> 5, r = bit & 31;
        const uint32_t lo = a[w] >> r;
        const uint32_t hi = (r > 4 && w + 1 < L) ? (a[w + 1] << (32 - r)) : 0u;
        const int32_t v = zero ? 0 : (int32_t)((lo | hi) & 0x0FFFFFFFu);
        d[p] = x.s ? -v : v;
    }
}

// signed carry pass: columns 0 .. NC-2 into [0, 2^28), the top one keeps the sign
template <int NC>
MLHD void bfp_carry(long long (&acc)[NC]) {
ML_UNROLL
    for (int c = 0; c + 1 < NC; ++c) {
        const long long carry = acc[c] >> 28;
        acc[c] -= carry << 28;
        acc[c + 1] += carry;
    }
}

// acc (columns CK .. of the products) += a b, digits of two fixed-point fractions
template <int N>
MLHD void bfp_term(long long (&acc)[BfpShape<N>::NC], const int32_t (&a)[BfpShape<N>::D],
                   const int32_t (&b)[BfpShape<N>::D]) {
    constexpr int D = BfpShape<N>::D, CK = BfpShape<N>::CK;
    ML_UNROLL
    for (int c = CK; c <= 2 * D - 2; ++c) {
    ML_UNROLL
        for (int p = 0; p < D; ++p) {
            const int q = c - p;
            if (q >= 0 && q < D) acc[c - CK] += (long long)a[p] * b[q];
        }
    }
}

// the sum held in acc (fractions x 2^-Er and y 2^-Ey) rounded to N limbs; kNone exponents
// mean an all-zero row
constexpr int kBfpNone = -(1 << 30);
template <int N>
MLHD mlf<N> bfp_result(long long (&acc)[BfpShape<N>::NC], int Er, int Ey) {
    using B = BfpShape<N>;
    constexpr int D = B::D, CK = B::CK, NC = B::NC;
    bfp_carry<NC>(acc);
    const bool neg = acc[NC - 1] < 0;
    if (neg) {
        for (int c = 0; c < NC; ++c) acc[c] = -acc[c];
        bfp_carry<NC>(acc);
    }
    uint32_t W[B::LW];
    for (int w = 0; w < B::LW; ++w) W[w] = 0;
    for (int c = 0; c < NC; ++c) {  // every column is below 2^28 here
        const int bit = 28 * c, w = bit >> 5, r = bit & 31;
        const unsigned long long v = (unsigned long long)acc[c] << r;
        W[w] |= (uint32_t)v;
        if (w + 1 < B::LW) W[w + 1] |= (uint32_t)(v >> 32);
    }
    // the sum is W 2^(28 CK - 56 D) 2^(Er + Ey)
    const long long e_top = (long long)Er + Ey + 28 * CK - 56 * D + 32 * B::LW;
    if (Er == kBfpNone || Ey == kBfpNone) return ml_zero<N>();
    return ml_pack<N, B::LW>(W, (int)e_top, neg ? 1u : 0u);
}

}  // namespace sdpg
