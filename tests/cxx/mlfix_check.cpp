// Host check of the integer summation helpers of mlfix.cuh against sums in a wider format
// (16 limbs, so the reference's own rounding is far below the bounds checked):
//   * fixed-point group sums (the warp / block reductions): |sum - exact| <= 2^(E - 250)
//     with E the group's largest exponent, for groups of 32, 256 and 1024 values;
//   * block-floating-point dots of 32 terms (the Cholesky panel update):
//     |dot - exact| <= 2^(Ex + Ey - 250) with Ex, Ey the rows' largest exponents;
//   * the same at 16 limbs against the 16-limb sums, within 2^-500.
// Values are random mantissas with exponents spread over up to 300 binades, zeros, and
// groups with exact cancellation.  Prints one line per case; exit status 0 if all pass.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "mlfix.cuh"

using namespace sdpg;

template <int N>
static mlf<N> rnd(std::mt19937_64 &g, int emin, int emax) {
    if (g() % 7 == 0) return ml_zero<N>();
    mlf<N> x{};
    for (int k = 0; k < N; ++k) x.m[k] = (uint32_t)g();
    x.m[N - 1] |= 0x80000000u;
    x.e = emin + (int)(g() % (uint64_t)(emax - emin + 1));
    x.s = (uint32_t)(g() & 1);
    return x;
}

// worst log2 |fixed-point sum - reference| - E over `reps` groups of `cnt` values
template <int N, int M>
static double fix_sum_worst(int cnt, int spread, int reps, unsigned seed) {
    std::mt19937_64 g(seed);
    double worst = -1e9;
    for (int rep = 0; rep < reps; ++rep) {
        std::vector<mlf<N>> v(cnt);
        for (auto &x : v) x = rnd<N>(g, -spread, 4);
        if (rep % 10 == 0)
            for (int i = 0; i + 1 < cnt; i += 2) v[i + 1] = ml_neg(v[i]);
        int E = kFixNone;
        for (const auto &x : v)
            if (x.m[N - 1]) E = std::max(E, x.e);
        uint32_t acc[N + 2] = {};
        for (const auto &x : v) {
            uint32_t a[N + 2];
            ml_to_fix<N>(x, E, a);
            ml_fix_add<N + 2>(acc, a);
        }
        const mlf<N> got = ml_from_fix<N>(acc, E);
        if (E == kFixNone) {
            if (!ml_is_zero(got)) return 1e9;
            continue;
        }
        mlf<M> ref = ml_zero<M>();
        for (const auto &x : v) ref = ml_add(ref, ml_widen<M, N>(x));
        const mlf<M> d = ml_sub(ml_widen<M, N>(got), ref);
        if (!ml_is_zero(d)) worst = std::max(worst, (double)d.e - (double)E);
    }
    return worst;
}

// worst log2 |bfp dot - reference| - (Ex + Ey) over `reps` pairs of 32-term rows
template <int N, int M>
static double bfp_dot_worst(int spread, int reps, unsigned seed) {
    using B = BfpShape<N>;
    std::mt19937_64 g(seed);
    double worst = -1e9;
    for (int rep = 0; rep < reps; ++rep) {
        mlf<N> x[32], y[32];
        for (int m = 0; m < 32; ++m) {
            x[m] = rnd<N>(g, -spread, 3);
            y[m] = rnd<N>(g, -spread, 5);
        }
        if (rep % 10 == 0)
            for (int m = 0; m < 32; ++m) y[m] = (m & 1) ? ml_neg(x[m]) : x[m];
        int Ex = kBfpNone, Ey = kBfpNone;
        for (int m = 0; m < 32; ++m) {
            if (x[m].m[N - 1]) Ex = std::max(Ex, x[m].e);
            if (y[m].m[N - 1]) Ey = std::max(Ey, y[m].e);
        }
        long long acc[B::NC] = {};
        for (int m = 0; m < 32; ++m) {
            int32_t a[B::D], b[B::D];
            bfp_digits<N>(x[m], Ex, a);
            bfp_digits<N>(y[m], Ey, b);
            bfp_term<N>(acc, a, b);
            if (m % B::EVERY == B::EVERY - 1) bfp_carry<B::NC>(acc);
        }
        const mlf<N> got = bfp_result<N>(acc, Ex, Ey);
        if (Ex == kBfpNone || Ey == kBfpNone) {
            if (!ml_is_zero(got)) return 1e9;
            continue;
        }
        mlf<M> ref = ml_zero<M>();
        for (int m = 0; m < 32; ++m) ref = ml_add(ref, ml_mul(ml_widen<M, N>(x[m]), ml_widen<M, N>(y[m])));
        const mlf<M> d = ml_sub(ml_widen<M, N>(got), ref);
        if (!ml_is_zero(d)) worst = std::max(worst, (double)d.e - (double)(Ex + Ey));
    }
    return worst;
}

int main() {
    struct Case {
        const char *name;
        double worst, bound;
    } cases[] = {
        {"fixed-point sum, 32 values, 256 bits", fix_sum_worst<8, 16>(32, 3, 2000, 1), -250},
        {"fixed-point sum, 256 values, 256 bits", fix_sum_worst<8, 16>(256, 60, 1000, 2), -250},
        {"fixed-point sum, 1024 values, 256 bits", fix_sum_worst<8, 16>(1024, 300, 200, 3), -250},
        {"fixed-point sum, 32 values, 512 bits", fix_sum_worst<16, 16>(32, 3, 500, 4), -500},
        {"bfp dot, 32 terms, 256 bits", bfp_dot_worst<8, 16>(2, 1000, 5), -250},
        {"bfp dot, 32 terms, spread 300, 256 bits", bfp_dot_worst<8, 16>(300, 1000, 6), -250},
        {"bfp dot, 32 terms, 512 bits", bfp_dot_worst<16, 16>(100, 300, 7), -500},
    };
    int bad = 0;
    for (const Case &c : cases) {
        const bool ok = c.worst <= c.bound;
        bad += !ok;
        printf("%-42s worst log2 error %.1f (bound %.0f) %s\n", c.name, c.worst, c.bound, ok ? "ok" : "FAIL");
    }
    return bad ? 1 : 0;
}
