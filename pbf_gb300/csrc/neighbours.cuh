// neighbours.cuh — the reference's neighbour enumeration, shared by the
// forward stage kernels (substep.cu) and the adjoint kernels (adjoint.cu).
#pragma once

#include "common.cuh"

namespace pbf {

// Sorted-index ranges of the 9 stencil rows of a cell (neighbourcells.glsl:52-90).
struct Runs {
    int32_t b[9], e[9];
};

__device__ __forceinline__ void runs_of(uint32_t key, const DevConsts& c,
                                        const int32_t* __restrict__ cstart,
                                        const int32_t* __restrict__ cend, Runs& r) {
    const uint32_t Gx = c.Gi[0], Gy = c.Gi[1], Gz = c.Gi[2];
    const uint32_t local = key - c.cell_base;
    const int cx = (int)(local % Gx);
    const uint32_t rem = local / Gx;
    const int cz = (int)(rem % Gz);
    const int cy = (int)(rem / Gz);
    const int xlo = cx > 0 ? cx - 1 : 0;
    const int xhi = cx + 1 < (int)Gx ? cx + 1 : (int)Gx - 1;
#pragma unroll
    for (int o = 0; o < 9; ++o) {
        const int ny = cy + (o / 3) - 1, nz = cz + (o % 3) - 1;
        int32_t first = -1, last = -1;
        if (ny >= 0 && ny < (int)Gy && nz >= 0 && nz < (int)Gz) {
            const uint32_t base = c.cell_base + (uint32_t)ny * c.GxGz + (uint32_t)nz * Gx;
            for (int xx = xlo; xx <= xhi; ++xx) {
                const int32_t s = __ldg(cstart + base + (uint32_t)xx);
                if (s != -1) {
                    if (first == -1) first = s;
                    last = __ldg(cend + base + (uint32_t)xx);
                }
            }
        }
        r.b[o] = first == -1 ? 0 : first;
        r.e[o] = first == -1 ? 0 : last;
    }
}


template <class F>
__device__ __forceinline__ void visit_full(uint32_t i, uint32_t key, const DevConsts& c,
                                           const int32_t* __restrict__ cstart,
                                           const int32_t* __restrict__ cend, F&& f) {
    // The 9 ranges live in a small local array: computing each row inside the
    // loop instead raises register use and lowers occupancy (measured slower).
    Runs r;
    runs_of(key, c, cstart, cend, r);
#pragma unroll 1
    for (int o = 0; o < 9; ++o)
        for (int32_t j = r.b[o]; j < r.e[o]; ++j)
            if ((uint32_t)j != i) f((uint32_t)j);
}

// Spreads the low 16 bits of x to the even bit positions.
__device__ __forceinline__ uint32_t spread_even(uint32_t x) {
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    return (x | (x << 1)) & 0x55555555u;
}

// The candidates of sorted particle i within h of it (r2 not above r2cut at
// positions X; a NaN distance counts as within, as in the pair bodies), in
// visit_full's order, in two loops per chunk of up to 32 consecutive
// candidates of a run: a scan marks the in-range candidates in register bit
// masks, then f runs on the marked ones in ascending order.  With most
// candidates out of range, a warp's lanes then scan together and evaluate
// pairs together, instead of all lanes waiting while some evaluate a pair
// inside the scan.
//
// The scan tests the candidates in pairs (2q, 2q+1) with float2 arithmetic;
// each lane is the same IEEE operation as the scalar form (pi - xj is
// fma(xj, -1, pi): exact product, one rounding; r2 is dot3's
// fma(dz, dz, fma(dy, dy, dx * dx))).  The inner loop only sets bit q of m0 /
// m1 for the even / odd candidate of pair q of the chunk; pair halves outside
// the run (an odd run start or end) and i itself are masked out once per
// chunk.  With LIST, `list(base, mask)` also receives, per chunk, the
// candidates base + t (bit t) with r2 <= c.r2list, before f runs on the chunk.
template <bool LIST, class S, class F>
__device__ __forceinline__ void visit_masked(uint32_t i, uint32_t key, const DevConsts& c,
                                             const int32_t* __restrict__ cstart,
                                             const int32_t* __restrict__ cend, const ScanPos& X,
                                             float3 pi, S&& list, F&& f) {
    Runs r;
    runs_of(key, c, cstart, cend, r);
    const float2 px = make_float2(pi.x, pi.x), py = make_float2(pi.y, pi.y),
                 pz = make_float2(pi.z, pi.z), neg = make_float2(-1.0f, -1.0f);
    const float cut = c.r2cut;
    const float4* __restrict__ xyp = X.xy;
    const float2* __restrict__ zp = X.z;
#pragma unroll 1
    for (int o = 0; o < 9; ++o) {
        const int32_t b = r.b[o], e = r.e[o];
#pragma unroll 1
        for (int32_t base = b & ~1; base < e; base += 32) {
            const uint32_t hi = (uint32_t)min(e - base, 32);  // candidates base + t, t < hi
            uint32_t q = (uint32_t)base >> 1;
            const uint32_t qe = q + ((hi + 1) >> 1);
            uint32_t m0 = 0, m1 = 0, l0 = 0, l1 = 0, bit = 1;
#pragma unroll 1
            for (; q < qe; ++q) {
                const float4 xy = __ldg(xyp + q);
                const float2 zz = __ldg(zp + q);
                const float2 dx = __ffma2_rn(make_float2(xy.x, xy.y), neg, px);
                const float2 dy = __ffma2_rn(make_float2(xy.z, xy.w), neg, py);
                const float2 dz = __ffma2_rn(zz, neg, pz);
                const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
                if (!(r2.x > cut)) m0 |= bit;
                if (!(r2.y > cut)) m1 |= bit;
                if constexpr (LIST) {
                    if (r2.x <= c.r2list) l0 |= bit;
                    if (r2.y <= c.r2list) l1 |= bit;
                }
                bit <<= 1;
            }
            const uint32_t lo = (uint32_t)max(b - base, 0);
            uint32_t valid = (hi == 32u ? 0xFFFFFFFFu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
            const uint32_t self = i - (uint32_t)base;
            if (self < 32u) valid &= ~(1u << self);
            if constexpr (LIST) list(base, (spread_even(l0) | (spread_even(l1) << 1)) & valid);
            uint32_t m = (spread_even(m0) | (spread_even(m1) << 1)) & valid;
            while (m) {
                const int t = __ffs(m) - 1;
                m &= m - 1;
                f((uint32_t)(base + t));
            }
        }
    }
}

}  // namespace pbf
