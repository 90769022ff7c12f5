// neighbours.cuh — the reference's neighbour enumeration, shared by the
// forward stage kernels (substep.cu) and the adjoint kernels (adjoint.cu).
#pragma once

#include "common.cuh"

namespace pbf {

// Sorted-index ranges of the 9 stencil rows around a centre (neighbourcells.glsl:52-90).
struct Runs {
    int32_t b[9], e[9];
};

// Stencil centre along one axis (neighbourcells.glsl:57): the predicted
// coordinate truncated toward zero, NOT clamped.  A particle predicted outside
// the grid (below the floor, say) searches around that outside cell, and the
// rows and cells outside the grid are empty (decision Q4), so it finds fewer
// neighbours or none, as in the reference.  Saturated to [-2, G + 1], which
// leaves the runs unchanged; NaN maps to 0.
__device__ __forceinline__ int stencil_coord(float x, uint32_t Gi) {
    if (!(x == x)) return 0;
    if (x <= -2.0f) return -2;
    if (x >= fadd(__uint2float_rn(Gi), 1.0f)) return (int)Gi + 1;
    return __float2int_rz(x);
}
__device__ __forceinline__ int3 stencil_centre(float3 q, const DevConsts& c) {
    return make_int3(stencil_coord(q.x, c.Gi[0]), stencil_coord(q.y, c.Gi[1]),
                     stencil_coord(q.z, c.Gi[2]));
}
__device__ __forceinline__ int3 stencil_centre(float4 q, const DevConsts& c) {
    return stencil_centre(make_float3(q.x, q.y, q.z), c);
}

__device__ __forceinline__ void runs_of(int3 ctr, const DevConsts& c,
                                        const int32_t* __restrict__ cstart,
                                        const int32_t* __restrict__ cend, Runs& r) {
    const uint32_t Gx = c.Gi[0], Gy = c.Gi[1], Gz = c.Gi[2];
    const int cx = ctr.x, cy = ctr.y, cz = ctr.z;
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
        if (!check_ok(c, first == -1 || (first >= 0 && first <= last &&
                                          (uint32_t)last <= c.n_total)))
            first = -1;
        r.b[o] = first == -1 ? 0 : first;
        r.e[o] = first == -1 ? 0 : last;
    }
}


// `ctr` returns the stencil centre (stencil_centre of the sweep's predicted
// position): the visits call it where they build the runs, so no centre stays
// live in registers across the neighbour loops.
template <class Ctr, class F>
__device__ __forceinline__ void visit_full(uint32_t i, Ctr&& ctr, const DevConsts& c,
                                           const int32_t* __restrict__ cstart,
                                           const int32_t* __restrict__ cend, F&& f) {
    // The 9 ranges live in a small local array: computing each row inside the
    // loop instead raises register use and lowers occupancy (measured slower).
    Runs r;
    runs_of(ctr(), c, cstart, cend, r);
#pragma unroll 1
    for (int o = 0; o < 9; ++o)
        for (int32_t j = r.b[o]; j < r.e[o]; ++j)
            if ((uint32_t)j != i) f((uint32_t)j);
}

// Runs of equal positions in sorted order.  Bit j of `runs` (32 per word) is
// set when sorted particle j starts a run: j == 0, its position differs
// (bitwise x, y, z) from particle j - 1's in the sweep's position set, j is a
// multiple of kRunStride (so a search for the next start reads at most
// kRunStride / 32 words) or j >= n (the terminator).  Built once per position
// set by k_run_flags / k_find_cells.
constexpr uint32_t kRunStride = 1024;

// First run start after j (a set bit > j exists: the terminator at n, and
// one at every multiple of kRunStride, so the search reads at most
// kRunStride / 32 + 1 words; the bounds-checked build enforces that).
__device__ __forceinline__ uint32_t run_end(const DevConsts& c, const uint32_t* __restrict__ runs,
                                           uint32_t j) {
    const uint32_t k = j + 1u;
    uint32_t w = k >> 5;
    uint32_t word = __ldg(runs + w) & (0xFFFFFFFFu << (k & 31u));
#ifdef PBF_CHECK
    for (uint32_t m = 0; word == 0u; ++m) {
        if (!check_ok(c, m < kRunStride / 32u && w + 1u <= (c.n_total >> 5) + 1u)) return k;
        word = __ldg(runs + ++w);
    }
#else
    while (word == 0u) word = __ldg(runs + ++w);
#endif
    return (w << 5) + (uint32_t)(__ffs((int)word) - 1);
}

// Cells of at least this many particles take the run path; runs of at least
// kRunMin candidates go to `uniform` as a whole.
constexpr int32_t kPileMin = 32;
constexpr uint32_t kRunMin = 4;

// visit_full's order, cell by cell, with runs of equal positions.  The box
// clamp stacks particles on single points (the box corners: by substep 300
// of the 2M dam break one corner cell holds 130,498 particles at one
// position).  In a cell of at least kPileMin particles, a candidate j that
// starts or continues a run of equal positions is tested first; the run
// [j, r) ends at the next run start or the cell's end, and every candidate in
// it is at the same offset d (r2) from particle i:
//  - r2 == 0: each candidate other than i gives the coincident term (len 0):
//    `coincident(j, r, m)` receives the run and the count of those;
//  - otherwise (i is not in the run), if it holds at least kRunMin
//    candidates and r2 is not NaN: `uniform(j, r, d, r2)` accumulates their
//    terms in order;
//  - otherwise f runs on each.
// The visit then resumes at r.  Every other candidate goes to f.  pos(j) is
// the position the sweep tests at (the set `runs` was built from).
template <class Ctr, class Pos, class F, class G, class U>
__device__ __forceinline__ void visit_direct_piles(uint32_t i, Ctr&& ctr, const DevConsts& c,
                                                   const int32_t* __restrict__ cstart,
                                                   const int32_t* __restrict__ cend,
                                                   const uint32_t* __restrict__ runs, Pos&& pos,
                                                   float3 pi, F&& f, G&& coincident,
                                                   U&& uniform) {
    const uint32_t Gx = c.Gi[0], Gy = c.Gi[1], Gz = c.Gi[2];
    const int3 cc = ctr();
    const int cx = cc.x, cy = cc.y, cz = cc.z;
    const int xlo = cx > 0 ? cx - 1 : 0;
    const int xhi = cx + 1 < (int)Gx ? cx + 1 : (int)Gx - 1;
#pragma unroll 1
    for (int o = 0; o < 9; ++o) {
        const int ny = cy + (o / 3) - 1, nz = cz + (o % 3) - 1;
        if (ny < 0 || ny >= (int)Gy || nz < 0 || nz >= (int)Gz) continue;
        const uint32_t base = c.cell_base + (uint32_t)ny * c.GxGz + (uint32_t)nz * Gx;
        int32_t b = -1, e = -1;  // the row's run, as visit_full merges it
#pragma unroll 1
        for (int xx = xlo; xx <= xhi; ++xx) {
            const uint32_t cell = base + (uint32_t)xx;
            const int32_t s = __ldg(cstart + cell);
            if (s == -1) continue;
            const int32_t t = __ldg(cend + cell);
            if (!check_ok(c, s >= 0 && s <= t && (uint32_t)t <= c.n_total)) continue;
            if (t - s < kPileMin) {
                if (b == -1) b = s;
                e = t;
                continue;
            }
            // a large cell: first the small cells before it, then its runs
            for (int32_t j = b; j < e; ++j)
                if ((uint32_t)j != i) f((uint32_t)j);
            b = e = -1;
            for (uint32_t j = (uint32_t)s; j < (uint32_t)t;) {
                const uint32_t k = j + 1u;
                const bool in_run = k < (uint32_t)t && !((__ldg(runs + (k >> 5)) >> (k & 31u)) & 1u);
                if (in_run) {
                    const float3 d = sub3(pi, pos(j));
                    const float r2 = dot3(d, d);
                    uint32_t r = run_end(c, runs, j);
                    if (r > (uint32_t)t) r = (uint32_t)t;
                    if (r2 == 0.0f) {
                        coincident(j, r, (r - j) - ((j <= i && i < r) ? 1u : 0u));
                        j = r;
                        continue;
                    }
                    if (r - j >= kRunMin && r2 == r2) {
                        uniform(j, r, d, r2);
                        j = r;
                        continue;
                    }
                }
                if (j != i) f(j);
                ++j;
            }
        }
        for (int32_t j = b; j < e; ++j)
            if ((uint32_t)j != i) f((uint32_t)j);
    }
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
template <bool LIST, class Ctr, class S, class F>
__device__ __forceinline__ void visit_masked(uint32_t i, Ctr&& ctr, const DevConsts& c,
                                             const int32_t* __restrict__ cstart,
                                             const int32_t* __restrict__ cend, const ScanPos& X,
                                             float3 pi, S&& list, F&& f) {
    Runs r;
    runs_of(ctr(), c, cstart, cend, r);
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
            // two candidate pairs per iteration (fewer loop and address
            // instructions; measured 1-3% faster per sweep), then the odd one
            if constexpr (!LIST) {
#pragma unroll 1
                for (; q + 1 < qe; q += 2) {
                    const float4 xa = __ldg(xyp + q), xb = __ldg(xyp + q + 1);
                    const float2 za = __ldg(zp + q), zb = __ldg(zp + q + 1);
                    const float2 dxa = __ffma2_rn(make_float2(xa.x, xa.y), neg, px);
                    const float2 dya = __ffma2_rn(make_float2(xa.z, xa.w), neg, py);
                    const float2 dza = __ffma2_rn(za, neg, pz);
                    const float2 ra = __ffma2_rn(dza, dza, __ffma2_rn(dya, dya, __fmul2_rn(dxa, dxa)));
                    const float2 dxb = __ffma2_rn(make_float2(xb.x, xb.y), neg, px);
                    const float2 dyb = __ffma2_rn(make_float2(xb.z, xb.w), neg, py);
                    const float2 dzb = __ffma2_rn(zb, neg, pz);
                    const float2 rb = __ffma2_rn(dzb, dzb, __ffma2_rn(dyb, dyb, __fmul2_rn(dxb, dxb)));
                    if (!(ra.x > cut)) m0 |= bit;
                    if (!(ra.y > cut)) m1 |= bit;
                    if (!(rb.x > cut)) m0 |= bit << 1;
                    if (!(rb.y > cut)) m1 |= bit << 1;
                    bit <<= 2;
                }
            }
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
