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

// The candidates of sorted particle i within h of it (r2 not above r2cut at
// positions X; a NaN distance counts as within, as in the pair bodies), in
// visit_full's order, in two loops per chunk of up to 32 consecutive
// candidates of a run: a scan marks the in-range candidates in a register bit
// mask, then f runs on the marked ones in ascending order.  With most
// candidates out of range, a warp's lanes then scan together and evaluate
// pairs together, instead of all lanes waiting while some evaluate a pair
// inside the scan.  The scan loop only computes r2 and sets a bit; i itself is
// masked out once per chunk.  With LIST, `list(base, mask)` also receives,
// per chunk, the candidates base + t (bit t) with r2 <= c.r2list, before f
// runs on the chunk.
template <bool LIST, class S, class F>
__device__ __forceinline__ void visit_masked(uint32_t i, uint32_t key, const DevConsts& c,
                                             const int32_t* __restrict__ cstart,
                                             const int32_t* __restrict__ cend,
                                             const float4* __restrict__ X, float3 pi, S&& list,
                                             F&& f) {
    Runs r;
    runs_of(key, c, cstart, cend, r);
    const float cut = c.r2cut;
#pragma unroll 1
    for (int o = 0; o < 9; ++o) {
        const int32_t e = r.e[o];
#pragma unroll 1
        for (int32_t base = r.b[o]; base < e; base += 32) {
            const float4* __restrict__ p = X + base;
            const float4* const pe = p + min(e - base, 32);
            uint32_t m = 0, l = 0, bit = 1;
#pragma unroll 1
            for (; p < pe; ++p) {
                const float4 xj = __ldg(p);
                const float3 d = sub3(pi, make_float3(xj.x, xj.y, xj.z));
                const float r2 = dot3(d, d);
                if (!(r2 > cut)) m |= bit;
                if constexpr (LIST) {
                    if (r2 <= c.r2list) l |= bit;
                }
                bit <<= 1;
            }
            const uint32_t self = i - (uint32_t)base;
            if (self < 32u) {
                m &= ~(1u << self);
                l &= ~(1u << self);
            }
            if constexpr (LIST) list(base, l);
            while (m) {
                const int t = __ffs(m) - 1;
                m &= m - 1;
                f((uint32_t)(base + t));
            }
        }
    }
}

}  // namespace pbf
