// pbf_dual.hpp — forward-mode dual numbers for the FP64 oracle twin
// (TEST INFRASTRUCTURE ONLY).
//
// Dual<K> carries a double value and K tangents.  Sim<Dual<K>> runs the same
// template as the FP32 oracle and its FP64 twin (pbf_oracle.hpp), so its
// value part is the FP64 twin's trajectory bit for bit, and its tangents are
// the exact derivatives of that floating-point program along K seeded
// directions: an independent check of the hand-written adjoint kernels
// (reverse mode) besides central finite differences.
//
// Rules: the product, quotient and chain rules per operation; fma(a, b, c)
// differentiates as a * b + c; sqrt'(0) is taken as 0 (every use of a zero
// length in the shaders is guarded, so the value never depends on it);
// comparisons and the integer cell coordinate read the value only (the sort
// permutation and the neighbour runs are piecewise constant); the wall clamp
// passes the tangent only where the result is strictly inside the walls, the
// same subgradient the adjoint kernels take.
#pragma once

#include <cmath>
#include <cstdint>

namespace pbfo {

template <int K>
struct Dual {
    double v;
    double d[K];

    Dual() : v(0.0) {
        for (int k = 0; k < K; ++k) d[k] = 0.0;
    }
    Dual(double x) : v(x) {  // NOLINT: constants convert implicitly, as for float
        for (int k = 0; k < K; ++k) d[k] = 0.0;
    }
    explicit operator double() const { return v; }
    explicit operator uint32_t() const { return (uint32_t)v; }
};

template <int K>
inline Dual<K> operator+(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v + b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <int K>
inline Dual<K> operator-(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v - b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <int K>
inline Dual<K> operator-(const Dual<K>& a) {
    Dual<K> r(-a.v);
    for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
    return r;
}
template <int K>
inline Dual<K> operator*(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v * b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <int K>
inline Dual<K> operator/(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v / b.v);
    for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
    return r;
}
template <int K>
inline Dual<K> fma(const Dual<K>& a, const Dual<K>& b, const Dual<K>& c) {
    Dual<K> r(std::fma(a.v, b.v, c.v));
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k] + c.d[k];
    return r;
}
template <int K>
inline Dual<K> sqrt(const Dual<K>& a) {
    Dual<K> r(std::sqrt(a.v));
    const double s = r.v > 0.0 ? 0.5 / r.v : 0.0;
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * s;
    return r;
}
template <int K>
inline bool operator<(const Dual<K>& a, const Dual<K>& b) { return a.v < b.v; }
template <int K>
inline bool operator>(const Dual<K>& a, const Dual<K>& b) { return a.v > b.v; }
template <int K>
inline bool operator<=(const Dual<K>& a, const Dual<K>& b) { return a.v <= b.v; }
template <int K>
inline bool operator>=(const Dual<K>& a, const Dual<K>& b) { return a.v >= b.v; }
template <int K>
inline bool operator==(const Dual<K>& a, const Dual<K>& b) { return a.v == b.v; }

// min(max(q, lo), hi) on the values (as the FP64 twin); the tangent is q's
// strictly inside the walls and zero on them (the walls are constants).
template <int K>
inline Dual<K> clamp_wall(const Dual<K>& q, const Dual<K>& lo, const Dual<K>& hi) {
    const double v = std::min(std::max(q.v, lo.v), hi.v);
    if (v == lo.v || v == hi.v) return Dual<K>(v);
    Dual<K> r = q;
    r.v = v;
    return r;
}

}  // namespace pbfo
