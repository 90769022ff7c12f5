// repeat_add.h — m sequential IEEE single-precision additions of one value,
// r <- fl(r + w) repeated m times, in O(binades crossed) steps instead of m.
//
// Used where a sweep adds the same term many times in a row: a particle in a
// cell whose particles all sit at one position (the corner piles that the
// box clamp builds) adds W(0) once per such neighbour to its density sum
// (calclambda.glsl:80-82).  The result must be the bits of the sequential
// sum, so the jump below relies only on how round-to-nearest-even acts on a
// fixed grid:
//
// Inside one binade [2^e, 2^(e+1)) every float is a multiple n*u of the
// binade's spacing u.  For w = (q + f) u with 0 <= f < 1, the exact sum
// n u + w rounds to (n + q) u if f < 1/2 and to (n + q + 1) u if f > 1/2 —
// the same increment for every n — and for f = 1/2 (a tie) to whichever of
// the two is even; once n is even, the increment that keeps it even (q if q
// is even, q + 1 if not) repeats.  So after two consecutive steps inside a
// binade have added the same increment D (in units of u), every further step
// adds D as long as the result stays at least 2u below 2^(e+1): the exact sum
// is then below 2^(e+1) - u and rounds on the same grid.  The loop below
// takes single steps until it sees that, jumps as far as the binade allows,
// and repeats in the next binade.  A step that does not change r is a fixed
// point: every later step returns r as well.
//
// Host and device share the code; on the host `float` addition must be IEEE
// binary32 round-to-nearest-even (SSE / AArch64 scalar arithmetic, no
// extended precision, no contraction).
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define PBF_HD __host__ __device__ __forceinline__
#else
#define PBF_HD inline
#endif

namespace pbf {

PBF_HD float ra_add(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    volatile float s = a + b;  // one binary32 rounding, no contraction
    return s;
#endif
}

PBF_HD uint32_t ra_bits(float x) {
    uint32_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
}

PBF_HD float ra_float(uint32_t b) {
    float x;
    std::memcpy(&x, &b, sizeof x);
    return x;
}

// r <- step(r), m times, where step(r) = fl(r + w) for one fixed real w (a
// float addend, or an exact product c * g under fma).  Single steps run
// through `step` itself; the jump only uses increments it has observed: two
// consecutive steps that stay in one binade, keep the sign and change the
// magnitude by the same D units of u are followed by as many more steps of D
// as keep the magnitude in [2^23 + 2, 2^24 - 2] units (so every exact sum
// still lies inside the binade and rounds on its grid).  A step that leaves
// r unchanged is a fixed point.  Any w works: with the opposite sign of r
// the magnitude shrinks by the same rule, and crossing zero or a binade
// edge goes through single steps.
template <class Step>
PBF_HD float repeat_step(float r, uint32_t m, Step&& step) {
    int32_t last_d = 0;  // magnitude change of the last step in units of u, 0 = none
    while (m > 0) {
        const float next = step(r);
        --m;
        const uint32_t rb = ra_bits(r), nb = ra_bits(next);
        if (nb == rb) return r;  // fixed point
        const uint32_t er = (rb >> 23) & 0xFFu, en = (nb >> 23) & 0xFFu;
        int32_t d = 0;
        // same sign, same binade, both normal and finite
        if ((rb >> 23) == (nb >> 23) && er != 0u && er != 0xFFu && en != 0u)
            d = (int32_t)(nb & 0x7FFFFFu) - (int32_t)(rb & 0x7FFFFFu);
        r = next;
        if (d == 0 || d != last_d) {
            last_d = d;
            continue;
        }
        const int32_t mag = (int32_t)((nb & 0x7FFFFFu) | 0x800000u);  // |r| / u
        const int32_t room = d > 0 ? (1 << 24) - 2 - mag : mag - (1 << 23) - 2;
        uint32_t j = room > 0 ? (uint32_t)(room / (d > 0 ? d : -d)) : 0u;
        if (j > m) j = m;
        if (j > 0u) {
            r = ra_float((nb & 0xFF800000u) | ((uint32_t)(mag + (int32_t)j * d) & 0x7FFFFFu));
            m -= j;
        }
        last_d = 0;  // the next stretch starts over
    }
    return r;
}

// r <- fl(r + w), m times.
PBF_HD float repeat_add(float r, float w, uint32_t m) {
    return repeat_step(r, m, [w](float x) { return ra_add(x, w); });
}

#if defined(__CUDACC__)
// acc <- fma(s, a, acc) per component, m times (fma3 of common.cuh repeated).
__device__ __forceinline__ float3 repeat_fma3(float s, float3 a, float3 acc, uint32_t m) {
    return make_float3(repeat_step(acc.x, m, [s, a](float x) { return __fmaf_rn(s, a.x, x); }),
                       repeat_step(acc.y, m, [s, a](float x) { return __fmaf_rn(s, a.y, x); }),
                       repeat_step(acc.z, m, [s, a](float x) { return __fmaf_rn(s, a.z, x); }));
}
// acc <- acc + a per component, m times (add3 of common.cuh repeated).
__device__ __forceinline__ float3 repeat_add3(float3 a, float3 acc, uint32_t m) {
    return make_float3(repeat_add(acc.x, a.x, m), repeat_add(acc.y, a.y, m),
                       repeat_add(acc.z, a.z, m));
}
#endif

}  // namespace pbf
