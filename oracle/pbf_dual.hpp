// pbf_dual.hpp — forward-mode dual numbers for the FP64 oracle twin
// (TEST INFRASTRUCTURE ONLY).
//
// DualT<V, K> carries a value of type V (double: the FP64 twin; float: the
// FP32 oracle) and K tangents in double.  Sim<DualT<V, K>> runs the same
// template as the FP32 oracle and its FP64 twin (pbf_oracle.hpp), so its
// value part is that instance's trajectory bit for bit, and its tangents are
// the exact derivatives of that floating-point program along K seeded
// directions: an independent check of the hand-written adjoint kernels
// (reverse mode) besides central finite differences.  With V = float the
// trajectory is the GPU's own (the GPU equals the FP32 oracle bit for bit),
// so the FP32 adjoint can be compared with the derivative of the very path it
// differentiates, separately from how far FP32 and FP64 trajectories drift
// apart.
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

template <typename V, int K>
struct DualT {
    V v;
    double d[K];

    DualT() : v(0) {
        for (int k = 0; k < K; ++k) d[k] = 0.0;
    }
    DualT(double x) : v((V)x) {  // NOLINT: constants convert implicitly, as for float
        for (int k = 0; k < K; ++k) d[k] = 0.0;
    }
    explicit operator double() const { return (double)v; }
    explicit operator uint32_t() const { return (uint32_t)v; }
    explicit operator int() const { return (int)v; }
};

template <typename V, int K>
inline DualT<V, K> operator+(const DualT<V, K>& a, const DualT<V, K>& b) {
    DualT<V, K> r(a.v + b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <typename V, int K>
inline DualT<V, K> operator-(const DualT<V, K>& a, const DualT<V, K>& b) {
    DualT<V, K> r(a.v - b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <typename V, int K>
inline DualT<V, K> operator-(const DualT<V, K>& a) {
    DualT<V, K> r(-a.v);
    for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
    return r;
}
template <typename V, int K>
inline DualT<V, K> operator*(const DualT<V, K>& a, const DualT<V, K>& b) {
    DualT<V, K> r(a.v * b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * (double)b.v + (double)a.v * b.d[k];
    return r;
}
template <typename V, int K>
inline DualT<V, K> operator/(const DualT<V, K>& a, const DualT<V, K>& b) {
    DualT<V, K> r(a.v / b.v);
    for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - (double)r.v * b.d[k]) / (double)b.v;
    return r;
}
template <typename V, int K>
inline DualT<V, K> fma(const DualT<V, K>& a, const DualT<V, K>& b, const DualT<V, K>& c) {
    DualT<V, K> r(std::fma(a.v, b.v, c.v));
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * (double)b.v + (double)a.v * b.d[k] + c.d[k];
    return r;
}
template <typename V, int K>
inline DualT<V, K> sqrt(const DualT<V, K>& a) {
    DualT<V, K> r(std::sqrt(a.v));
    const double s = r.v > 0 ? 0.5 / (double)r.v : 0.0;
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * s;
    return r;
}
template <typename V, int K>
inline bool operator<(const DualT<V, K>& a, const DualT<V, K>& b) { return a.v < b.v; }
template <typename V, int K>
inline bool operator>(const DualT<V, K>& a, const DualT<V, K>& b) { return a.v > b.v; }
template <typename V, int K>
inline bool operator<=(const DualT<V, K>& a, const DualT<V, K>& b) { return a.v <= b.v; }
template <typename V, int K>
inline bool operator>=(const DualT<V, K>& a, const DualT<V, K>& b) { return a.v >= b.v; }
template <typename V, int K>
inline bool operator==(const DualT<V, K>& a, const DualT<V, K>& b) { return a.v == b.v; }

// min(max(q, lo), hi) on the values (as the FP64 twin); the tangent is q's
// strictly inside the walls and zero on them (the walls are constants).
template <typename V, int K>
inline DualT<V, K> clamp_wall(const DualT<V, K>& q, const DualT<V, K>& lo, const DualT<V, K>& hi) {
    const V v = std::min(std::max(q.v, lo.v), hi.v);
    if (v == lo.v || v == hi.v) return DualT<V, K>((double)v);
    DualT<V, K> r = q;
    r.v = v;
    return r;
}

template <int K>
using Dual = DualT<double, K>;

}  // namespace pbfo
