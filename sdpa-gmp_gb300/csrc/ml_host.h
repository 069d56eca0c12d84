// Host-only conversions for the multi-limb float format: decimal text
// (the .dat-s / param.sdpa reader and the result printer) and GMP's public
// mpf layout (the drop-in boundary for callers that hold mpf_class arrays).
#pragma once
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "ml.cuh"

namespace sdpg {

// Little-endian arbitrary-length unsigned integer helpers (base 2^32).
struct BigU {
    std::vector<uint32_t> w;
    bool zero() const {
        for (uint32_t x : w)
            if (x) return false;
        return true;
    }
    void trim() {
        while (!w.empty() && w.back() == 0) w.pop_back();
    }
    void mul_small(uint32_t f, uint32_t add = 0) {
        uint64_t c = add;
        for (auto &x : w) {
            c += (uint64_t)x * f;
            x = (uint32_t)c;
            c >>= 32;
        }
        if (c) w.push_back((uint32_t)c);
    }
    uint32_t div_small(uint32_t d) {  // floor division in place, returns remainder
        uint64_t r = 0;
        for (size_t i = w.size(); i-- > 0;) {
            r = (r << 32) | w[i];
            w[i] = (uint32_t)(r / d);
            r %= d;
        }
        trim();
        return (uint32_t)r;
    }
    void shl(int bits) {
        if (bits <= 0) return;
        int q = bits / 32, r = bits % 32;
        std::vector<uint32_t> o(w.size() + q + 1, 0);
        for (size_t i = 0; i < w.size(); ++i) {
            uint64_t v = (uint64_t)w[i] << r;
            o[i + q] |= (uint32_t)v;
            o[i + q + 1] |= (uint32_t)(v >> 32);
        }
        w.swap(o);
        trim();
    }
    int bitlen() const {
        for (size_t i = w.size(); i-- > 0;)
            if (w[i]) return (int)(32 * i + 32 - __builtin_clz(w[i]));
        return 0;
    }
};

// Pack a big integer times 2^exp2 into mlf<N> (truncating).
template <int N>
inline mlf<N> ml_from_bigu(const BigU &b, long exp2, uint32_t sign) {
    const int bl = b.bitlen();
    if (bl == 0) return ml_zero<N>();
    mlf<N> r = ml_zero<N>();
    // take the top 32N bits
    for (int k = 0; k < 32 * N; ++k) {
        const int bit = bl - 1 - k;
        if (bit < 0) break;
        const uint32_t v = (b.w[bit >> 5] >> (bit & 31)) & 1u;
        if (v) r.m[N - 1 - (k >> 5)] |= 1u << (31 - (k & 31));
    }
    r.e = (int32_t)(bl + exp2);
    r.s = sign;
    return r;
}

// Parse a decimal floating-point literal ("-12.5e-3", "+7", "0.25").
// Returns false on a malformed number; *end receives the first unparsed char.
template <int N>
inline bool ml_parse(const char *s, mlf<N> *out, const char **end = nullptr) {
    const char *p = s;
    while (*p == ' ' || *p == '\t') ++p;
    uint32_t sign = 0;
    if (*p == '+' || *p == '-') {
        sign = (*p == '-');
        ++p;
    }
    BigU M;
    long e10 = 0;
    bool any = false;
    while (*p >= '0' && *p <= '9') {
        M.mul_small(10, (uint32_t)(*p - '0'));
        any = true;
        ++p;
    }
    if (*p == '.') {
        ++p;
        while (*p >= '0' && *p <= '9') {
            M.mul_small(10, (uint32_t)(*p - '0'));
            --e10;
            any = true;
            ++p;
        }
    }
    if (!any) {
        if (end) *end = s;
        return false;
    }
    if (*p == 'e' || *p == 'E') {
        const char *q = p + 1;
        int es = 1;
        if (*q == '+' || *q == '-') {
            es = (*q == '-') ? -1 : 1;
            ++q;
        }
        if (*q >= '0' && *q <= '9') {
            long ev = 0;
            while (*q >= '0' && *q <= '9') {
                ev = ev * 10 + (*q - '0');
                ++q;
            }
            e10 += es * ev;
            p = q;
        }
    }
    if (end) *end = p;
    M.trim();
    if (M.zero()) {
        *out = ml_zero<N>();
        return true;
    }
    if (e10 >= 0) {
        for (long i = 0; i < e10; ++i) M.mul_small(10);
        *out = ml_from_bigu<N>(M, 0, sign);
        return true;
    }
    // M * 10^e10 with e10 < 0: floor((M << k) / 10^-e10) * 2^-k
    const long neg = -e10;
    const int k = 32 * N + 64 + (int)(neg * 3.33) + 8 - M.bitlen();
    BigU Q = M;
    long shift = k > 0 ? k : 0;
    Q.shl((int)shift);
    for (long i = 0; i < neg; ++i) Q.div_small(10);
    mlf<N> r = ml_from_bigu<N>(Q, -shift, sign);
    *out = r;
    return true;
}

// Decimal significand digits of |a| (ndig digits, truncated) and the decimal exponent.
template <int N>
inline void ml_decimal_digits(const mlf<N> &a, int ndig, std::string *digits, long *e10) {
    // |a| = M * 2^(e - 32N)
    BigU M;
    M.w.assign(a.m, a.m + N);
    M.trim();
    const long e2 = (long)a.e - 32 * N;
    // estimate decimal exponent
    const double l10 = log10((double)((((uint64_t)a.m[N - 1] << 32) | a.m[N - 2]) >> 11) * 0x1p-53) + (double)a.e * 0.30102999566398119521;
    long E = (long)floor(l10);
    for (int attempt = 0; attempt < 4; ++attempt) {
        // R = floor(|a| * 10^(ndig-1-E))
        const long s10 = ndig - 1 - E;
        BigU R = M;
        long s2 = e2;
        if (s10 >= 0) {
            for (long i = 0; i < s10; ++i) R.mul_small(10);
        }
        // apply 2^s2
        if (s2 >= 0) {
            R.shl((int)s2);
            s2 = 0;
        }
        if (s10 < 0) {
            // divide by 10^-s10, keeping enough fractional bits
            R.shl(64);
            s2 -= 64;
            for (long i = 0; i < -s10; ++i) R.div_small(10);
        }
        // now value*10^s10 = R * 2^s2 with s2 <= 0 : floor
        if (s2 < 0) {
            const long sh = -s2;
            BigU T;
            const long q = sh / 32, r = sh % 32;
            T.w.assign(R.w.size() > (size_t)q ? R.w.size() - q : 0, 0);
            for (size_t i = 0; i < T.w.size(); ++i) {
                uint64_t lo = R.w[i + q];
                uint64_t hi = (i + q + 1 < R.w.size()) ? R.w[i + q + 1] : 0;
                T.w[i] = (uint32_t)(((hi << 32) | lo) >> r);
            }
            T.trim();
            R = T;
        }
        // to decimal string
        std::string d;
        BigU t = R;
        while (!t.zero()) d.push_back((char)('0' + t.div_small(10)));
        if (d.empty()) d = "0";
        std::string dd(d.rbegin(), d.rend());
        if ((int)dd.size() > ndig) {
            ++E;
            continue;
        }
        if ((int)dd.size() < ndig) {
            --E;
            continue;
        }
        *digits = dd;
        *e10 = E;
        return;
    }
    *digits = std::string(ndig, '0');
    *e10 = E;
}

// ndig significant digits of |a| rounded half up, as GMP's mpf_get_str rounds (one
// further digit decides; that digit is exact because the digits are truncated).
template <int N>
inline void ml_decimal_rounded(const mlf<N> &a, int ndig, std::string *digits, long *e10) {
    std::string d;
    long e = 0;
    ml_decimal_digits(a, ndig + 1, &d, &e);
    const bool up = d[ndig] >= '5';
    d.resize(ndig);
    if (up) {
        int i = ndig - 1;
        while (i >= 0 && d[i] == '9') d[i--] = '0';
        if (i >= 0) {
            ++d[i];
        } else {  // 99..9 rounded up to 100..0
            d = "1" + std::string(ndig - 1, '0');
            ++e;
        }
    }
    *digits = d;
    *e10 = e;
}

// printf-like "%[+]W.Pe" rendering of an mlf, rounded half up in the last digit.
template <int N>
inline std::string ml_format_e(const mlf<N> &a, int prec, bool plus = false, int width = 0) {
    std::string out;
    if (ml_is_zero(a)) {
        out = std::string(plus ? "+" : "") + "0." + std::string(prec, '0') + "e+00";
    } else {
        std::string dg;
        long e10;
        ml_decimal_rounded(a, prec + 1, &dg, &e10);
        out = a.s ? "-" : (plus ? "+" : "");
        out += dg.substr(0, 1);
        if (prec > 0) out += "." + dg.substr(1);
        char eb[32];
        snprintf(eb, sizeof eb, "e%c%02ld", e10 < 0 ? '-' : '+', e10 < 0 ? -e10 : e10);
        out += eb;
    }
    if ((int)out.size() < width) out = std::string(width - out.size(), ' ') + out;
    return out;
}

// One value rendered through a GMP-style printf format for mpf operands, as the
// reference's result file does (gmp_fprintf with xPrint / XPrint / YPrint, e.g.
// "%+50.40Fe"): text around a single conversion "%[flags][width][.prec][F](e|E|f|g|G)"
// with flags from "-+ 0#", rounded half up in the last printed digit.
template <int N>
inline std::string ml_format_gmp(const std::string &fmt, const mlf<N> &a) {
    const size_t pc = fmt.find('%');
    if (pc == std::string::npos) return fmt;
    size_t i = pc + 1;
    bool left = false, plus = false, space = false, zero = false, alt = false;
    for (; i < fmt.size(); ++i) {
        const char c = fmt[i];
        if (c == '-') left = true;
        else if (c == '+') plus = true;
        else if (c == ' ') space = true;
        else if (c == '0') zero = true;
        else if (c == '#') alt = true;
        else break;
    }
    int width = 0, prec = 6;
    while (i < fmt.size() && fmt[i] >= '0' && fmt[i] <= '9') width = 10 * width + (fmt[i++] - '0');
    if (i < fmt.size() && fmt[i] == '.') {
        prec = 0;
        ++i;
        while (i < fmt.size() && fmt[i] >= '0' && fmt[i] <= '9') prec = 10 * prec + (fmt[i++] - '0');
    }
    if (i < fmt.size() && fmt[i] == 'F') ++i;
    if (i >= fmt.size()) return fmt;
    const char conv = fmt[i];
    const std::string tail = fmt.substr(i + 1);
    const bool neg = !ml_is_zero(a) && a.s;
    std::string body;  // digits without sign
    auto exp_form = [&](int p, bool upper) {
        std::string dg;
        long e10 = 0;
        if (ml_is_zero(a)) {
            dg = std::string(p + 1, '0');
        } else {
            ml_decimal_rounded(a, p + 1, &dg, &e10);
        }
        std::string r = dg.substr(0, 1);
        if (p > 0 || alt) r += ".";
        r += dg.substr(1);
        char eb[32];
        snprintf(eb, sizeof eb, "%c%c%02ld", upper ? 'E' : 'e', e10 < 0 ? '-' : '+', e10 < 0 ? -e10 : e10);
        return r + eb;
    };
    auto fixed_form = [&](int p) {
        if (ml_is_zero(a)) return std::string("0") + (p > 0 || alt ? "." + std::string(p, '0') : "");
        std::string dg;
        long e10 = 0;
        ml_decimal_digits(a, 1, &dg, &e10);
        long nd = e10 + 1 + p;  // significant digits printed
        std::string intpart, frac;
        if (nd == 0) {  // below the last printed place: rounds to 0 or to one unit there
            const bool up = dg[0] >= '5';
            intpart = p == 0 && up ? "1" : "0";
            frac = std::string(p, '0');
            if (p > 0 && up) frac[p - 1] = '1';
        } else if (nd < 0) {
            intpart = "0";
            frac = std::string(p, '0');
        } else {
            ml_decimal_rounded(a, (int)nd, &dg, &e10);
            if ((long)dg.size() < e10 + 1 + p) dg += std::string(e10 + 1 + p - (long)dg.size(), '0');
            const long ni = e10 + 1;  // integer digits (may be <= 0)
            if (ni > 0) {
                intpart = dg.substr(0, ni);
                frac = dg.substr(ni);
            } else {
                intpart = "0";
                frac = std::string(-ni, '0') + dg;
            }
            frac.resize(p, '0');
        }
        return intpart + (p > 0 || alt ? "." + frac : "");
    };
    switch (conv) {
        case 'e':
        case 'E': body = exp_form(prec, conv == 'E'); break;
        case 'f': body = fixed_form(prec); break;
        case 'g':
        case 'G': {
            const int P = prec == 0 ? 1 : prec;
            long e10 = 0;
            if (!ml_is_zero(a)) {
                std::string dg;
                ml_decimal_rounded(a, P, &dg, &e10);
            }
            if (e10 < -4 || e10 >= P) body = exp_form(P - 1, conv == 'G');
            else body = fixed_form((int)(P - 1 - e10));
            if (!alt) {  // strip trailing zeros of the fraction
                const size_t epos = body.find_first_of("eE");
                std::string mant = body.substr(0, epos), ex = epos == std::string::npos ? "" : body.substr(epos);
                if (mant.find('.') != std::string::npos) {
                    while (!mant.empty() && mant.back() == '0') mant.pop_back();
                    if (!mant.empty() && mant.back() == '.') mant.pop_back();
                }
                body = mant + ex;
            }
            break;
        }
        default: return fmt;  // not a floating conversion: left as is
    }
    const std::string sign = neg ? "-" : (plus ? "+" : (space ? " " : ""));
    std::string out;
    const int pad = width - (int)(sign.size() + body.size());
    if (pad <= 0) out = sign + body;
    else if (left) out = sign + body + std::string(pad, ' ');
    else if (zero) out = sign + std::string(pad, '0') + body;
    else out = std::string(pad, ' ') + sign + body;
    return fmt.substr(0, pc) + out + tail;
}

// GMP mpf public layout (gmp.h: __mpf_struct {int _mp_prec; int _mp_size;
// mp_exp_t _mp_exp; mp_limb_t *_mp_d;}) for a 64-bit-limb LP64 build.
struct mpf_raw {
    int prec;
    int size;
    long exp;
    uint64_t *d;
};

// value = sign(size) * sum_{i<|size|} d[i] * 2^(64*(i - |size| + exp))
template <int N>
inline mlf<N> ml_from_mpf(int size, long exp, const uint64_t *d) {
    if (size == 0) return ml_zero<N>();
    const int n = size < 0 ? -size : size;
    BigU B;
    const int take = n < (N / 2 + 2) ? n : (N / 2 + 2);  // enough limbs for 32N bits
    for (int i = n - take; i < n; ++i) {
        B.w.push_back((uint32_t)d[i]);
        B.w.push_back((uint32_t)(d[i] >> 32));
    }
    B.trim();
    // B = top `take` limbs; value = B * 2^(64*(exp - take))
    return ml_from_bigu<N>(B, 64L * (exp - take), size < 0 ? 1u : 0u);
}

// Write an mlf into GMP mpf form: fills d[0..|size|) (least significant first),
// returns the signed limb count and the base-2^64 exponent via *exp.
template <int N>
inline int ml_to_mpf(const mlf<N> &a, long *exp, uint64_t *d, int dcap) {
    if (ml_is_zero(a)) {
        *exp = 0;
        return 0;
    }
    const long e = a.e;
    const long ex = (e >= -63) ? (e + 63) / 64 : -((-e) / 64);  // ceil(e / 64)
    const int s = (int)(e - 64 * ex + 64);                        // in (0, 64]
    // I = M << s occupies N/2 + 1 limbs; value = I * 2^(64*(ex - (N/2 + 1)))
    BigU B;
    B.w.assign(a.m, a.m + N);
    B.w.push_back(0);
    B.w.push_back(0);
    B.w.push_back(0);
    B.shl(s);
    const int n = N / 2 + 1;
    std::vector<uint64_t> L64(n, 0);
    for (int i = 0; i < n; ++i) {
        const uint64_t lo = (2 * i < (int)B.w.size()) ? B.w[2 * i] : 0;
        const uint64_t hi = (2 * i + 1 < (int)B.w.size()) ? B.w[2 * i + 1] : 0;
        L64[i] = lo | (hi << 32);
    }
    int start = 0;
    while (start < n && L64[start] == 0) ++start;
    int cnt = n - start;
    if (cnt > dcap) {
        start += cnt - dcap;
        cnt = dcap;
    }
    for (int i = 0; i < cnt; ++i) d[i] = L64[start + i];
    *exp = ex;
    return a.s ? -cnt : cnt;
}

}  // namespace sdpg
