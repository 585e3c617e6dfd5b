// Forward-mode dual numbers for the CPU oracle: a value and N directional derivatives, carried through the oracle's
// templated kernels, pieces, rules and blocks. TEST INFRASTRUCTURE ONLY (the derivative checker of the adjoint), as
// ForwardDiff is in the reference's own tests (test/kernels/test_kernels.jl:127-148).
//
// Comparisons look at the value only, so every decision (tier, split, wedge count, far switch) is the value's and
// the derivatives are those of the branch the value takes. Functions carry their derivative by the chain rule.
#pragma once
#include <cmath>

#include "vp_oracle.hpp"

namespace vpo {

constexpr int VPO_ND = 8;  // directions of one dual pass of the oracle

template <int N>
struct Dual {
    double v;
    double d[N];
    Dual() : v(0) {
        for (int i = 0; i < N; ++i) d[i] = 0;
    }
    Dual(double x) : v(x) {  // NOLINT: constants convert implicitly, as in the templated code
        for (int i = 0; i < N; ++i) d[i] = 0;
    }
    explicit operator double() const { return v; }
};

// f(a) with f'(a) = df
template <int N>
inline Dual<N> chain(const Dual<N>& a, double f, double df) {
    Dual<N> r(f);
    for (int i = 0; i < N; ++i) r.d[i] = df * a.d[i];
    return r;
}

template <int N> inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r(a.v + b.v);
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int N> inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r(a.v - b.v);
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int N> inline Dual<N> operator-(const Dual<N>& a) {
    Dual<N> r(-a.v);
    for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
    return r;
}
template <int N> inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r(a.v * b.v);
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <int N> inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
    const double q = a.v / b.v;
    Dual<N> r(q);
    for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - q * b.d[i]) / b.v;
    return r;
}
template <int N> inline Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N> inline Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N> inline Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, double b) { return a * Dual<N>(b); }
template <int N> inline Dual<N> operator*(double a, const Dual<N>& b) { return Dual<N>(a) * b; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, double b) { return a / Dual<N>(b); }
template <int N> inline Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> inline Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) { return a = a + b; }
template <int N> inline Dual<N>& operator-=(Dual<N>& a, const Dual<N>& b) { return a = a - b; }
template <int N> inline Dual<N>& operator*=(Dual<N>& a, const Dual<N>& b) { return a = a * b; }
template <int N> inline Dual<N>& operator/=(Dual<N>& a, const Dual<N>& b) { return a = a / b; }

#define VPO_DUAL_CMP(op)                                                                                             \
    template <int N> inline bool operator op(const Dual<N>& a, const Dual<N>& b) { return a.v op b.v; }              \
    template <int N> inline bool operator op(const Dual<N>& a, double b) { return a.v op b; }                        \
    template <int N> inline bool operator op(double a, const Dual<N>& b) { return a op b.v; }
VPO_DUAL_CMP(<)
VPO_DUAL_CMP(>)
VPO_DUAL_CMP(<=)
VPO_DUAL_CMP(>=)
VPO_DUAL_CMP(==)
VPO_DUAL_CMP(!=)
#undef VPO_DUAL_CMP

template <int N> inline Dual<N> sqrt(const Dual<N>& a) {
    const double s = std::sqrt(a.v);
    return chain(a, s, 0.5 / s);
}
template <int N> inline Dual<N> log(const Dual<N>& a) { return chain(a, std::log(a.v), 1.0 / a.v); }
template <int N> inline Dual<N> sin(const Dual<N>& a) { return chain(a, std::sin(a.v), std::cos(a.v)); }
template <int N> inline Dual<N> cos(const Dual<N>& a) { return chain(a, std::cos(a.v), -std::sin(a.v)); }
template <int N> inline Dual<N> acos(const Dual<N>& a) {
    return chain(a, std::acos(a.v), -1.0 / std::sqrt(std::fmax(1.0 - a.v * a.v, 1e-300)));
}
template <int N> inline Dual<N> atan2(const Dual<N>& y, const Dual<N>& x) {
    const double r2 = x.v * x.v + y.v * y.v;
    Dual<N> r(std::atan2(y.v, x.v));
    for (int i = 0; i < N; ++i) r.d[i] = (x.v * y.d[i] - y.v * x.d[i]) / r2;
    return r;
}
template <int N> inline Dual<N> fabs(const Dual<N>& a) { return a.v < 0 ? -a : a; }

// the in-plane branch of the solid angle: its value, with the off-plane formula's derivatives
template <int N>
struct carries_derivatives<Dual<N>> {
    static const bool value = true;
};
template <int N>
inline Dual<N> plane_limit(const Dual<N>& in_plane, const Dual<N>& off_plane) {
    Dual<N> r = off_plane;
    r.v = in_plane.v;
    return r;
}

}  // namespace vpo
