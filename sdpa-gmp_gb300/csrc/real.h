// Host-side scalar wrapper over mlf<N> with arithmetic operators, so that the
// interior-point control logic (step lengths, centering, residual ratios,
// phase tests) reads like the reference's mpf_class expressions.  Constants
// written as C doubles convert exactly, as `mpf_class x = 0.95` does.
#pragma once
#include <string>

#include "ml.cuh"
#include "ml_host.h"

namespace sdpg {

template <int N>
struct Real {
    mlf<N> v;
    Real() : v(ml_zero<N>()) {}
    Real(const mlf<N> &x) : v(x) {}
    Real(double d) : v(ml_from_double<N>(d)) {}
    Real(int i) : v(ml_from_int<N>(i)) {}
    Real(long i) : v(ml_from_int<N>(i)) {}

    friend Real operator+(const Real &a, const Real &b) { return Real(ml_add(a.v, b.v)); }
    friend Real operator-(const Real &a, const Real &b) { return Real(ml_sub(a.v, b.v)); }
    friend Real operator*(const Real &a, const Real &b) { return Real(ml_mul(a.v, b.v)); }
    friend Real operator/(const Real &a, const Real &b) {
        if (ml_is_zero(b.v)) return Real(ml_zero<N>());  // callers guard; GMP would abort
        return Real(ml_div(a.v, b.v));
    }
    Real operator-() const { return Real(ml_neg(v)); }
    Real &operator+=(const Real &b) { return *this = *this + b; }
    Real &operator-=(const Real &b) { return *this = *this - b; }
    Real &operator*=(const Real &b) { return *this = *this * b; }
    Real &operator/=(const Real &b) { return *this = *this / b; }
    friend bool operator<(const Real &a, const Real &b) { return ml_cmp(a.v, b.v) < 0; }
    friend bool operator>(const Real &a, const Real &b) { return ml_cmp(a.v, b.v) > 0; }
    friend bool operator<=(const Real &a, const Real &b) { return ml_cmp(a.v, b.v) <= 0; }
    friend bool operator>=(const Real &a, const Real &b) { return ml_cmp(a.v, b.v) >= 0; }
    friend bool operator==(const Real &a, const Real &b) { return ml_cmp(a.v, b.v) == 0; }
    friend bool operator!=(const Real &a, const Real &b) { return ml_cmp(a.v, b.v) != 0; }
    double d() const { return ml_to_double(v); }
    std::string fmt(int prec, bool plus = false, int width = 0) const { return ml_format_e<N>(v, prec, plus, width); }
};

template <int N>
inline Real<N> rabs(const Real<N> &a) { return Real<N>(ml_abs(a.v)); }
template <int N>
inline Real<N> rsqrt_(const Real<N> &a) { return Real<N>(ml_sqrt(a.v)); }
template <int N>
inline Real<N> rmax(const Real<N> &a, const Real<N> &b) { return a < b ? b : a; }
template <int N>
inline Real<N> rmin(const Real<N> &a, const Real<N> &b) { return b < a ? b : a; }

}  // namespace sdpg
