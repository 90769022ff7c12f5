// substep.cu — the per-substep stage kernels of the PBF path.
//
// Data layout in HBM (one handle, n particles):
//   x, v          float4[n]  id order; the drop-in state (SPH position/velocity buffers)
//   xstar         float4[n]  predicted positions, id order (predictpos output)
//   keys          u32[n]     cell key per id; sorted keys + perm after the sort
//   P0, P1        float4[n]  sorted-order Jacobi position buffers (w = 0)
//   L             float4[n]  sorted (x, y, z, lambda): one 16-byte load per neighbour in delta-p
//   VS            float4[n]  committed velocity, sorted order
//   VX, OM        float4[n]  velocity after XSPH / vorticity vector, sorted order
//   Q             float4[n]  sorted (x, y, z, |vorticity|) for the confinement pass
//   cell_start    i32[cells] first sorted index of each cell, -1 when empty
//   cell_end      i32[cells] one past the last sorted index (valid where start != -1)
//   scan copies   ScanPos    pair-interleaved copies of XP and the iterates (masked scans)
//   pair lists    u32[cap][n] in-range candidates per particle, SoA (PairLists)
//
// Every neighbour sweep visits, for sorted particle i, the 9 (dy, dz) rows of
// its 3x3x3 stencil in the reference's order (neighbourcells.glsl:37-47),
// each row's up-to-3-cell x-run in ascending sorted index, skipping i itself
// (foreachneighbour.glsl:1-10), and accumulates in that order.
#include <type_traits>

#include "substep.cuh"
#include "repeat_add.h"
#include "neighbours.cuh"

namespace pbf {

// predictpos.glsl:18-38 fused with the cell key of GetHash (counting.glsl:53-57).
template <class CP>
__global__ void __launch_bounds__(kBlock)
k_predict(const float4* __restrict__ x, const float4* __restrict__ v, float4* __restrict__ xstar,
          uint32_t* __restrict__ keys, uint32_t n, CP cp, uint32_t* status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const auto& c = cp.at(i);
    const float4 q = x[i];
    const float4 w = v[i];
    float wz = w.z;
    if (c.ext_force && q.z > c.half_gz) wz = fsub(wz, c.g2dt);  // :27-28
    const float wy = fsub(w.y, c.gdt);                             // :32
    const float3 s = make_float3(fadd(q.x, fmul(c.dt, w.x)), fadd(q.y, fmul(c.dt, wy)),
                                 fadd(q.z, fmul(c.dt, wz)));       // :34
    if (!finite3(s)) atomicOr(status, kDevNonFinite);
    xstar[i] = make_float4(s.x, s.y, s.z, 0.0f);
    keys[i] = cell_key(s, c);
}

// Cell keys of the current positions (no prediction), for diagnostics.
template <class CP>
__global__ void __launch_bounds__(kBlock)
k_keys_of(const float4* __restrict__ x, float4* __restrict__ xstar, uint32_t* __restrict__ keys,
          uint32_t n, CP cp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const auto& c = cp.at(i);
    const float4 q = x[i];
    xstar[i] = make_float4(q.x, q.y, q.z, 0.0f);
    keys[i] = cell_key(xyz(q), c);
}

// Clears the cell-start entries the previous sort set (its sorted keys are
// still in `prev_sorted`), so the dense table never needs a full memset.
__global__ void __launch_bounds__(kBlock)
k_unmark_cells(const uint32_t* __restrict__ prev_sorted, uint32_t n, uint32_t ncells,
               int32_t* __restrict__ cstart) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = prev_sorted[i];
    if (k < ncells && (i == 0 || prev_sorted[i - 1] != k)) cstart[k] = -1;
}

// The run-start bit of sorted particle j (neighbours.cuh: runs) from its
// position p and the previous particle's q, with the warp's 32 bits stored
// by its first lane.  Call with every lane of the warp.
__device__ __forceinline__ void store_run_bits(uint32_t j, uint32_t n, float3 p, float3 q,
                                               uint32_t* __restrict__ runs) {
    const bool start = j == 0u || j >= n || j % kRunStride == 0u ||
                       __float_as_uint(p.x) != __float_as_uint(q.x) ||
                       __float_as_uint(p.y) != __float_as_uint(q.y) ||
                       __float_as_uint(p.z) != __float_as_uint(q.z);
    const uint32_t word = __ballot_sync(0xFFFFFFFFu, start);
    // words 0 .. n / 32 exist (n / 32 + 2 are allocated); later warps write none
    if ((threadIdx.x & 31u) == 0u && (j >> 5) <= (n >> 5)) runs[j >> 5] = word;
}

// Run-start bits of a position set, indices 0..n (launch over n + 1 threads
// in whole warps).
__global__ void __launch_bounds__(kBlock)
k_run_flags(const float4* __restrict__ P, uint32_t n, uint32_t* __restrict__ runs) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    float3 p = make_float3(0.0f, 0.0f, 0.0f), q = p;
    if (j < n) {
        p = xyz(__ldg(P + j));
        if (j > 0) q = xyz(__ldg(P + j - 1));
    }
    store_run_bits(j, n, p, q, runs);
}

// Run-start bits over a sweep's whole per-particle input, for the direct
// sweeps' value runs: particle j starts a run when its position (A.xyz), or
// A.w (lambda or |vorticity|, with use_w), or B.xyz (the committed velocity,
// when B is given) differs bitwise from particle j - 1's, or at the stride
// and terminator marks of store_run_bits.  Inside such a run every candidate
// gives the same term, so a sweep adds it with repeat_step instead of a loop.
// Launch over n + 1 threads in whole warps.
__global__ void __launch_bounds__(kBlock)
k_run_flags_vals(const float4* __restrict__ A, const float4* __restrict__ B, int use_w,
                 uint32_t n, uint32_t* __restrict__ runs) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    bool start = j == 0u || j >= n || j % kRunStride == 0u;
    if (!start) {
        const float4 a = __ldg(A + j), a0 = __ldg(A + j - 1);
        start = __float_as_uint(a.x) != __float_as_uint(a0.x) ||
                __float_as_uint(a.y) != __float_as_uint(a0.y) ||
                __float_as_uint(a.z) != __float_as_uint(a0.z) ||
                (use_w && __float_as_uint(a.w) != __float_as_uint(a0.w));
        if (!start && B) {
            const float4 b = __ldg(B + j), b0 = __ldg(B + j - 1);
            start = __float_as_uint(b.x) != __float_as_uint(b0.x) ||
                    __float_as_uint(b.y) != __float_as_uint(b0.y) ||
                    __float_as_uint(b.z) != __float_as_uint(b0.z);
        }
    }
    const uint32_t word = __ballot_sync(0xFFFFFFFFu, start);
    if ((threadIdx.x & 31u) == 0u && (j >> 5) <= (n >> 5)) runs[j >> 5] = word;
}

// findcells.glsl:34-53 (start of cell(x_0) = 0 and end of cell(x_{n-1}) = n)
// fused with the gather of the predicted positions into sorted order.
// Keys >= ncells are skipped and reported through `status` (bad input only).
__global__ void __launch_bounds__(kBlock)
k_find_cells(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ perm,
             const float4* __restrict__ xstar, float4* __restrict__ P0, uint32_t n, uint32_t ncells,
             int32_t* __restrict__ cstart, int32_t* __restrict__ cend, uint32_t* bad,
             const uint32_t* __restrict__ sid, uint32_t* __restrict__ sid_sorted, ScanPos sx,
             uint32_t* __restrict__ runs, uint32_t* status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    if (status) {
        // neighbourcells.glsl:83 packs a 3-cell run's count into 8 bits
        // (foreachneighbour.glsl:5 drops counts >= 128).  Particles i and
        // i + 127 at most two cells apart in key order lie in one 3-cell
        // window: flag it (conservatively: the window may span a row end).
        const bool over = valid && i + 127u < n && skeys[i + 127u] - skeys[i] <= 2u;
        if (__any_sync(0xFFFFFFFFu, over) && (threadIdx.x & 31u) == 0u &&
            !(*(volatile uint32_t*)status & kDevRunOver127))
            atomicOr(status, kDevRunOver127);
    }
    float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#ifdef PBF_CHECK
    if (valid && perm[i] >= n) {  // bounds-checked build: a bad permutation entry
        atomicOr(status, kDevIndexFault);
        return;
    }
#endif
    if (valid && P0) {
        p = __ldg(xstar + perm[i]);
        P0[i] = p;
        if (sx.xy) scanpos_store(sx, i, p.x, p.y, p.z);
    }
    if (runs && P0) {
        // run-start bits of the predicted positions (launched over n + 1
        // threads); the previous particle's position is the previous lane's,
        // or a load on a warp's first lane
        float3 q = make_float3(__shfl_up_sync(0xFFFFFFFFu, p.x, 1),
                               __shfl_up_sync(0xFFFFFFFFu, p.y, 1),
                               __shfl_up_sync(0xFFFFFFFFu, p.z, 1));
        if ((threadIdx.x & 31u) == 0u && valid && i > 0) q = xyz(__ldg(xstar + perm[i - 1]));
        store_run_bits(i, n, xyz(p), q, runs);
    }
    if (!valid) return;
    const uint32_t k = skeys[i];
    if (sid_sorted) sid_sorted[i] = __ldg(sid + perm[i]);
    if (k >= ncells) {
        atomicOr(bad, 1u);
        return;
    }
    if (i == 0 || skeys[i - 1] != k) cstart[k] = (int32_t)i;
    if (i + 1 == n || skeys[i + 1] != k) cend[k] = (int32_t)(i + 1);
}

// ---- neighbour visitors ------------------------------------------------------
//
// Two ways to enumerate the candidates of sorted particle i, both in the
// reference's order:
//  full  the 9 stencil rows, each row's run in ascending index, i skipped;
//  list  the candidates that were within h + skin at the substep's predicted
//        positions, stored by the first lambda sweep in that same order.
// A candidate left out of the list was farther than h + skin apart at the
// predicted positions; while every particle has moved less than
// (skin - margin) / 2 since (the guard below), it is still farther than h
// apart in floating point, so it would have contributed nothing.  Both
// visitors therefore produce the same sums, bit for bit.

template <class F>
__device__ __forceinline__ void visit_list(uint32_t i, const DevConsts& c, int32_t cnt,
                                           const NbrLists& nl, F&& f) {
    const uint32_t* __restrict__ p = nl.idx + i;
    for (int32_t k = 0; k < cnt; ++k) {
        const uint32_t j = __ldg(p + (size_t)k * nl.n);
        if (check_ok(c, j < c.n_total)) f(j);
    }
}

// Writer of particle i's exact pair list (PairLists): appends in visit order,
// counts past the capacity, and marks an overflowed list with -1.
struct PairRecorder {
    const PairLists& pl;
    uint32_t i;
    uint32_t k;
    __device__ __forceinline__ void operator()(uint32_t j) {
        if (k < pl.cap) pl.idx[(size_t)k * pl.n + i] = j;
        ++k;
    }
    __device__ __forceinline__ void finish() const {
        if (pl.cap) pl.cnt[i] = k <= pl.cap ? (int32_t)k : -1;
    }
};

// Replays particle i's exact pair list when one was recorded and fits.
template <class F>
__device__ __forceinline__ bool visit_pairs(uint32_t i, const DevConsts& c, const PairLists& pl,
                                            F&& f) {
    if (!pl.cap) return false;
    const int32_t cnt = pl.cnt[i];
    if (cnt < 0) return false;
    const uint32_t* __restrict__ p = pl.idx + i;
    if (cnt > 0) {  // the next index is loaded one entry ahead
        uint32_t jn = __ldg(p);
#pragma unroll 1
        for (int32_t k = 0; k < cnt; ++k) {
            const uint32_t j = jn;
            if (k + 1 < cnt) jn = __ldg(p + (size_t)(k + 1) * pl.n);
            if (check_ok(c, j < c.n_total)) f(j);
        }
    }
    return true;
}

// Guard: may particle i (current position pi, predicted position xi) use
// its list in a sweep whose positions have moved at most dmax from the
// predicted ones?  NaN anywhere makes the answer false.
__device__ __forceinline__ bool list_usable(const DevConsts& c, const NbrLists& nl, int32_t cnt,
                                            float3 pi, float3 xi, int dmax_slot) {
    if (!c.use_lists || cnt < 0 || dmax_slot < -1) return false;  // -2: no lists built
    const float3 dd = make_float3(pi.x - xi.x, pi.y - xi.y, pi.z - xi.z);
    const float di = sqrtf(dd.x * dd.x + dd.y * dd.y + dd.z * dd.z) * 1.0001f;
    const float dmax = dmax_slot < 0 ? 0.0f : __uint_as_float(nl.guard[dmax_slot]) * 1.0001f;
    const float coord = fmaxf(__uint_as_float(nl.guard[0]), c.wall_abs_max);
    const float margin = c.margin_h + 16.0f * 5.9604645e-8f * coord;  // 16 ulp(coord)
    return di + dmax + margin < c.skin;
}

__device__ __forceinline__ void warp_max_to(uint32_t* slot, float v) {
    // v >= 0 or NaN; non-negative floats order like their bit patterns
    uint32_t b = __float_as_uint(v);
    for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
    if ((threadIdx.x & 31) == 0) atomicMax(slot, b);
}

// The full-stencil visit of a sweep: direct, or scan-then-evaluate by chunks.
template <bool MASKED, class Ctr, class F>
__device__ __forceinline__ void sweep_visit(uint32_t i, Ctr&& ctr, const DevConsts& c,
                                            const int32_t* __restrict__ cstart,
                                            const int32_t* __restrict__ cend, const ScanPos& X,
                                            float3 pi, F&& body) {
    if constexpr (MASKED)
        visit_masked<false>(i, ctr, c, cstart, cend, X, pi, [](int32_t, uint32_t) {}, body);
    else
        visit_full(i, ctr, c, cstart, cend, body);
}

// Masked stencil scan with the pair list recorded first and the pair bodies
// run from it afterwards: the scan writes the indices of the in-range
// candidates (visit order) to particle i's list, then `eval` runs on the list
// entries, read back by the same thread, so the bodies of a warp's lanes run
// together over their own list positions (the same shape as the replaying
// sweeps) instead of chunk by chunk.  A list longer than its capacity keeps
// its first `cap` entries (and is marked -1 for the replaying sweep); the
// candidates past them are found by a second scan and evaluated in order.
template <bool LIST, class Ctr, class S, class F>
__device__ __forceinline__ void scan_then_eval(uint32_t i, Ctr&& ctr, const DevConsts& c,
                                               const int32_t* __restrict__ cstart,
                                               const int32_t* __restrict__ cend,
                                               const ScanPos& X, float3 pi, const PairLists& pw,
                                               S&& list, F&& eval) {
    uint32_t* const out = pw.idx + i;
    const size_t stride = pw.n;
    uint32_t tot = 0;
    visit_masked<LIST>(i, ctr, c, cstart, cend, X, pi, list, [&](uint32_t j) {
        if (tot < pw.cap) out[(size_t)tot * stride] = j;
        ++tot;
    });
    pw.cnt[i] = tot <= pw.cap ? (int32_t)tot : -1;
    const uint32_t m = min(tot, pw.cap);
    if (m) {  // the next index is loaded one entry ahead
        uint32_t jn = out[0];
#pragma unroll 1
        for (uint32_t k = 0; k < m; ++k) {
            const uint32_t j = jn;
            if (k + 1 < m) jn = out[(size_t)(k + 1) * stride];
            eval(j);
        }
    }
    if (tot > pw.cap) {
        uint32_t rank = 0;
        visit_masked<false>(i, ctr, c, cstart, cend, X, pi, [](int32_t, uint32_t) {},
                            [&](uint32_t j) {
                                if (rank++ >= pw.cap) eval(j);
                            });
    }
}

// ---- pair bodies (shared by both visitors) ---------------------------------------

struct LambdaAcc {
    float rho, sumk;
    float3 gi;
};

// calclambda.glsl:75-95 for one neighbour at offset d = p_i - p_j, r2 = |d|^2.
// (call only for r2 not above r2cut: len > h gives Wpoly6 = gradWspiky = 0)
__device__ __forceinline__ void lambda_pair(const DevConsts& c, float3 d, float r2, LambdaAcc& a) {
    const float len = fsqrt(r2);
    a.rho = fadd(a.rho, w_poly6(c, len));  // :80-82
    if (len == 0.0f) return;               // gradWspiky(0) = 0 (:60)
    const float3 g = scale3(d, grad_scale(c.kg_lambda, c.h, len));  // :86-87
    a.sumk = fadd(a.sumk, dot3(g, g));     // :89
    a.gi = add3(a.gi, g);                  // :93
}

// lambda_pair for m neighbours at the same offset d (a run of equal
// positions): each of the four sums receives its term m times, as m calls
// would add it (repeat_add: the same bits).
__device__ __forceinline__ void lambda_pair_run(const DevConsts& c, float3 d, float r2,
                                                uint32_t m, LambdaAcc& a) {
    if (r2 > c.r2cut) return;
    const float len = fsqrt(r2);
    a.rho = repeat_add(a.rho, w_poly6(c, len), m);  // :80-82
    if (len == 0.0f) return;
    const float3 g = scale3(d, grad_scale(c.kg_lambda, c.h, len));  // :86-87
    a.sumk = repeat_add(a.sumk, dot3(g, g), m);                      // :89
    a.gi = make_float3(repeat_add(a.gi.x, g.x, m), repeat_add(a.gi.y, g.y, m),
                       repeat_add(a.gi.z, g.z, m));  // :93
}

// What the adjoint needs of a lambda evaluation: sum_j grad_pj C_i (the
// gradient w.r.t. p_i, calclambda.glsl:93) and the full denominator sum
// before epsilon (:89,97).
__device__ __forceinline__ float4 lambda_aux(const LambdaAcc& a) {
    return make_float4(a.gi.x, a.gi.y, a.gi.z, fadd(a.sumk, dot3(a.gi, a.gi)));
}

// calclambda.glsl:97-101
__device__ __forceinline__ float lambda_finish(const DevConsts& c, const LambdaAcc& a) {
    const float sumk = fadd(a.sumk, dot3(a.gi, a.gi));  // :97
    const float Ci = ffma(a.rho, c.oorho, -1.0f);        // :100
    return fdiv(-Ci, fadd(sumk, c.eps));                 // :101
}

// ---- solver kernels --------------------------------------------------------------

// Resident 256-thread blocks per SM the sweep kernels are compiled for (caps
// them at 32 registers: full occupancy hides the gather and sqrt/div latency;
// 6 or 4 blocks with more registers measured slower).  One thread per sorted
// particle.
constexpr int kSweepBlocksPerSM = 8;
// The first vorticity pass carries more state than the other sweeps (the
// XSPH and vorticity sums, the velocity, the run path's repeated steps): 6
// blocks per SM (40 registers) keep it from spilling; measured 10% faster
// than 8 blocks with spills on the 2M window.
constexpr int kVortBlocksPerSM = 6;

// Instantiations of the sweep kernels (pbf_tuning): MODE is the stencil scan
// (kDirect: the reference's loop shape; kMasked: masked scans; kPairs: masked
// scans recording the exact pair lists the next sweep replays), LISTS whether
// the skin-radius neighbour lists are compiled in.  Every instantiation gives
// the same bits.
constexpr int kDirect = 0, kMasked = 1, kPairs = 2;

// First lambda sweep of a substep (calclambda.glsl:66-102) at the predicted
// positions XP: a full stencil scan that also records, in visit order, every
// candidate within h + skin (the neighbour list of the later sweeps) and the
// largest coordinate magnitude (for the guard's rounding margin).
template <class CP, int MODE, bool LISTS>
__global__ void __launch_bounds__(kBlock, kSweepBlocksPerSM)
k_lambda_build(const float4* __restrict__ XP, const uint32_t* __restrict__ skeys,
               const int32_t* __restrict__ cstart, const int32_t* __restrict__ cend,
               float4* __restrict__ L, float4* __restrict__ aux, NbrLists nl, PairLists pw,
               ScanPos sx, uint32_t n, CP cp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n && !(pw.heavy && pw.heavy[i]);
    float3 pi = make_float3(0.0f, 0.0f, 0.0f);
    if (live) {
        const auto& c = cp.at(i);
        pi = xyz(XP[i]);
        auto ctr = [&] { return stencil_centre(pi, c); };  // neighbourcells.glsl:57
        LambdaAcc a{0.0f, 0.0f, make_float3(0.0f, 0.0f, 0.0f)};
        int32_t cnt = 0;
        const uint32_t cap = (LISTS && c.use_lists) ? nl.cap : 0u;
        auto list_rec = [&](int32_t base, uint32_t lm) {
            while (lm) {
                const int t = __ffs(lm) - 1;
                lm &= lm - 1;
                if ((uint32_t)cnt < cap) nl.idx[(size_t)cnt * n + i] = (uint32_t)(base + t);
                ++cnt;
            }
        };
        auto eval = [&](uint32_t j) {
            const float3 d = sub3(pi, xyz(__ldg(XP + j)));
            lambda_pair(c, d, dot3(d, d), a);
        };
        if constexpr (MODE == kPairs) {
            if (LISTS && cap)
                scan_then_eval<true>(i, ctr, c, cstart, cend, sx, pi, pw, list_rec, eval);
            else
                scan_then_eval<false>(i, ctr, c, cstart, cend, sx, pi, pw,
                                      [](int32_t, uint32_t) {}, eval);
        } else if constexpr (MODE == kMasked) {
            if (LISTS && cap)
                visit_masked<true>(i, ctr, c, cstart, cend, sx, pi, list_rec, eval);
            else
                visit_masked<false>(i, ctr, c, cstart, cend, sx, pi,
                                    [](int32_t, uint32_t) {}, eval);
        } else {
            bool piles = false;
            if constexpr (!LISTS) {
                if (pw.runs) {
                    // a coincident neighbour adds W(0) to the density (:80-82)
                    visit_direct_piles(
                        i, ctr, c, cstart, cend, pw.runs,
                        [&](uint32_t j) { return xyz(__ldg(XP + j)); }, pi,
                        [&](uint32_t j) {
                            const float3 d = sub3(pi, xyz(__ldg(XP + j)));
                            const float r2 = dot3(d, d);
                            if (r2 > c.r2cut) return;
                            lambda_pair(c, d, r2, a);
                        },
                        [&](uint32_t, uint32_t, uint32_t m) { a.rho = repeat_add(a.rho, w_poly6(c, 0.0f), m); },
                        [&](uint32_t j0, uint32_t r, float3 d, float r2) {
                            lambda_pair_run(c, d, r2, r - j0, a);
                        });
                    piles = true;
                }
            }
            if (!piles)
                visit_full(i, ctr, c, cstart, cend, [&](uint32_t j) {
                    const float3 d = sub3(pi, xyz(__ldg(XP + j)));
                    const float r2 = dot3(d, d);
                    if (LISTS && r2 <= c.r2list) {
                        if ((uint32_t)cnt < cap) nl.idx[(size_t)cnt * n + i] = j;
                        ++cnt;
                    }
                    if (r2 > c.r2cut) return;
                    lambda_pair(c, d, r2, a);
                });
        }
        if (LISTS) nl.cnt[i] = (uint32_t)cnt <= cap ? cnt : -1;
        L[i] = make_float4(pi.x, pi.y, pi.z, lambda_finish(c, a));
        if (aux) aux[i] = lambda_aux(a);
    }
    if (LISTS) {
        const float m = fmaxf(fmaxf(fabsf(pi.x), fabsf(pi.y)), fabsf(pi.z));
        warp_max_to(nl.guard, m);
    }
}

// calclambda.glsl:66-102 at positions P (iterations after the first).
// dmax_slot: guard slot holding the largest displacement of P from XP.
template <class CP, int MODE, bool LISTS>
__global__ void __launch_bounds__(kBlock, kSweepBlocksPerSM)
k_lambda(const float4* __restrict__ P, const float4* __restrict__ XP,
         const uint32_t* __restrict__ skeys, const int32_t* __restrict__ cstart,
         const int32_t* __restrict__ cend, float4* __restrict__ L, float4* __restrict__ aux,
         NbrLists nl, PairLists pw, ScanPos sx, int dmax_slot, uint32_t n, CP cp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (pw.heavy && pw.heavy[i])) return;
    const auto& c = cp.at(i);
    const float3 pi = xyz(P[i]);
    auto ctr = [&] { return stencil_centre(XP[i], c); };  // neighbourcells.glsl:57
    LambdaAcc a{0.0f, 0.0f, make_float3(0.0f, 0.0f, 0.0f)};
    // in_range: the candidate is known to pass the in-range test (the
    // masked scans computed the same r2 bit for bit), so the test is skipped
    auto eval_in = [&](uint32_t j) {
        const float3 d = sub3(pi, xyz(__ldg(P + j)));
        lambda_pair(c, d, dot3(d, d), a);
    };
    auto eval = [&](uint32_t j) {
        const float3 d = sub3(pi, xyz(__ldg(P + j)));
        const float r2 = dot3(d, d);
        if (r2 > c.r2cut) return;
        lambda_pair(c, d, r2, a);
    };
    bool listed = false;
    if constexpr (LISTS) {
        const int32_t cnt = nl.cnt[i];
        if (list_usable(c, nl, cnt, pi, xyz(XP[i]), dmax_slot)) {
            listed = true;
            if constexpr (MODE == kPairs) {
                PairRecorder rec{pw, i, 0u};
                visit_list(i, c, cnt, nl, [&](uint32_t j) {
                    const float3 d = sub3(pi, xyz(__ldg(P + j)));
                    if (!(dot3(d, d) > c.r2cut)) rec(j);
                    eval(j);
                });
                rec.finish();
            } else {
                visit_list(i, c, cnt, nl, eval);
            }
        }
    }
    if (!listed) {
        if constexpr (MODE == kPairs)
            scan_then_eval<false>(i, ctr, c, cstart, cend, sx, pi, pw, [](int32_t, uint32_t) {},
                                  eval_in);
        else if constexpr (MODE == kMasked)
            sweep_visit<true>(i, ctr, c, cstart, cend, sx, pi, eval_in);
        else if (!LISTS && pw.runs)
            visit_direct_piles(
                i, ctr, c, cstart, cend, pw.runs,
                [&](uint32_t j) { return xyz(__ldg(P + j)); }, pi, eval,
                [&](uint32_t, uint32_t, uint32_t m) { a.rho = repeat_add(a.rho, w_poly6(c, 0.0f), m); },
                [&](uint32_t j0, uint32_t r, float3 d, float r2) {
                    lambda_pair_run(c, d, r2, r - j0, a);
                });
        else
            sweep_visit<false>(i, ctr, c, cstart, cend, sx, pi, eval);
    }
    L[i] = make_float4(pi.x, pi.y, pi.z, lambda_finish(c, a));
    if (aux) aux[i] = lambda_aux(a);
}

// updatepos.glsl:42-104.  Reads L = (p, lambda), writes clamped positions Pn
// and the largest displacement of Pn from XP into guard slot `out_slot`.
template <class CP, int MODE, bool LISTS>
__global__ void __launch_bounds__(kBlock, kSweepBlocksPerSM)
k_delta_p(const float4* __restrict__ L, const float4* __restrict__ XP,
          const uint32_t* __restrict__ skeys, const int32_t* __restrict__ cstart,
          const int32_t* __restrict__ cend, float4* __restrict__ Pn, NbrLists nl, PairLists pr,
          ScanPos sx, ScanPos sx_out, int dmax_slot, int out_slot, uint32_t n, CP cp,
          uint32_t* status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n && !(pr.heavy && pr.heavy[i]);
    float disp = 0.0f;
    if (live) {
        const auto& c = cp.at(i);
        const float4 Li = L[i];
        const float3 pi = xyz(Li);
        const float li = Li.w;
        float3 dp = make_float3(0.0f, 0.0f, 0.0f);
        auto body = [&](uint32_t j) {
            const float4 Lj = __ldg(L + j);
            const float3 d = sub3(pi, xyz(Lj));
            const float r2 = dot3(d, d);
            if (r2 > c.r2cut) return;
            const float len = fsqrt(r2);
            if (len == 0.0f) return;
            float sc = fmul(c.scale, w_poly6(c, len));  // :57
            sc = fmul(sc, sc);                           // :58
            sc = fmul(sc, sc);                           // :59
            sc = fmul(c.negk, sc);                       // :60
            const float coef = fadd(fadd(li, Lj.w), sc); // :65
            const float3 g = scale3(d, grad_scale(c.kg, c.h, len));
            dp = fma3(coef, g, dp);                      // :65
        };
        const float3 xi = xyz(XP[i]);
        auto ctr = [&] { return stencil_centre(XP[i], c); };  // neighbourcells.glsl:57
        bool done = false;
        if constexpr (MODE == kPairs) done = visit_pairs(i, c, pr, body);
        if (!done) {
            bool listed = false;
            if constexpr (LISTS) {
                const int32_t cnt = nl.cnt[i];
                if (list_usable(c, nl, cnt, pi, xi, dmax_slot)) {
                    visit_list(i, c, cnt, nl, body);
                    listed = true;
                }
            }
            if (!listed) {
                if (MODE == kDirect && !LISTS && pr.runs)  // coincident: no term (:56)
                    visit_direct_piles(
                        i, ctr, c, cstart, cend, pr.runs,
                        [&](uint32_t j) { return xyz(__ldg(L + j)); }, pi, body, [](uint32_t, uint32_t, uint32_t) {},
                        [&](uint32_t j0, uint32_t r, float3 d, float r2) {
                            // one offset and, the run bits being over (p, lambda),
                            // one lambda_j: r - j0 equal terms in a row
                            if (r2 > c.r2cut) return;
                            const float len = fsqrt(r2);
                            float sc = fmul(c.scale, w_poly6(c, len));  // :57
                            sc = fmul(sc, sc);                           // :58
                            sc = fmul(sc, sc);                           // :59
                            sc = fmul(c.negk, sc);                       // :60
                            const float3 g = scale3(d, grad_scale(c.kg, c.h, len));
                            const float coef = fadd(fadd(li, __ldg(&L[j0].w)), sc);  // :65
                            dp = repeat_fma3(coef, g, dp, r - j0);
                        });
                else
                    sweep_visit<MODE != kDirect>(i, ctr, c, cstart, cend, sx, pi, body);
            }
        }
        float3 q = fma3(c.oorho, dp, pi);  // :85
        // clamp (:100) as min(max(q, lo), hi) with explicit selects, so signed
        // zeros and NaN behave like the oracle's std::min/std::max
        q.x = (q.x < c.lo[0]) ? c.lo[0] : q.x;
        q.x = (c.hi[0] < q.x) ? c.hi[0] : q.x;
        q.y = (q.y < c.lo[1]) ? c.lo[1] : q.y;
        q.y = (c.hi[1] < q.y) ? c.hi[1] : q.y;
        q.z = (q.z < c.lo[2]) ? c.lo[2] : q.z;
        q.z = (c.hi[2] < q.z) ? c.hi[2] : q.z;
        if (!finite3(q)) atomicOr(status, kDevNonFinite);
        Pn[i] = make_float4(q.x, q.y, q.z, 0.0f);
        if (sx_out.xy) scanpos_store(sx_out, i, q.x, q.y, q.z);
        if (LISTS) {
            const float3 dd = make_float3(q.x - xi.x, q.y - xi.y, q.z - xi.z);
            disp = sqrtf(dd.x * dd.x + dd.y * dd.y + dd.z * dd.z);
        }
    }
    if (LISTS) warp_max_to(nl.guard + out_slot, disp);
}

// ---- warp-cooperative sweeps (sweep_mode PBF_SWEEP_COOP) ---------------------------
//
// One warp per sorted particle i, for scenes too small to fill the GPU with a
// thread per particle (and for clumped states, where each particle has
// thousands of neighbours): the lanes test 32 consecutive candidates of a run
// at once (coalesced loads), each in-range lane computes its pair term, and
// every lane then folds the terms into the particle's sums in ascending
// candidate order, reading them from the owning lanes by shuffles.  The terms
// are the same functions and the folding order the same visit order as the
// one-thread sweeps, so the bits are the same.
constexpr int kCoop = 3;
constexpr uint32_t kFull = 0xFFFFFFFFu;

__device__ __forceinline__ float shf(float v, int src) { return __shfl_sync(kFull, v, src); }
__device__ __forceinline__ float3 shf3(float3 v, int src) {
    return make_float3(shf(v.x, src), shf(v.y, src), shf(v.z, src));
}

// Calls term(j, d, r2) on every in-range candidate's own lane (returning
// whether the candidate has a term), then fold(src_lane) on all lanes for
// each in-range candidate with a term, in visit order.
template <class Ctr, class T, class Fo>
__device__ __forceinline__ void coop_visit(uint32_t i, Ctr&& ctr, const DevConsts& c,
                                           const int32_t* __restrict__ cstart,
                                           const int32_t* __restrict__ cend,
                                           const float4* __restrict__ X, float3 pi, T&& term,
                                           Fo&& fold) {
    const uint32_t lane = threadIdx.x & 31u;
    Runs r;
    runs_of(ctr(), c, cstart, cend, r);
#pragma unroll 1
    for (int o = 0; o < 9; ++o) {
        const int32_t e = r.e[o];
#pragma unroll 1
        for (int32_t base = r.b[o]; base < e; base += 32) {
            const uint32_t j = (uint32_t)base + lane;
            bool has = false;
            if ((int32_t)j < e && j != i) {
                const float3 d = sub3(pi, xyz(__ldg(X + j)));
                const float r2 = dot3(d, d);
                if (!(r2 > c.r2cut)) has = term(j, d, r2);
            }
            uint32_t m = __ballot_sync(kFull, has);
            while (m) {
                const int src = __ffs(m) - 1;
                m &= m - 1;
                fold(src);
            }
        }
    }
}

// Particles a cooperative kernel processes: all n (list == nullptr, one warp
// per particle), or the `*count` entries of `list` (the heavy particles of a
// mixed sweep), taken by the grid's warps in turn.
struct CoopWork {
    const uint32_t* list;
    const uint32_t* count;
};

#define PBF_COOP_FOR_EACH(i)                                                                  \
    const uint32_t warp0_ = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;                     \
    const uint32_t nwarps_ = (gridDim.x * blockDim.x) >> 5;                                    \
    const uint32_t total_ = wk.list ? *wk.count : n;                                           \
    for (uint32_t w_ = warp0_; w_ < total_; w_ += nwarps_)                                     \
        if (const uint32_t i = wk.list ? wk.list[w_] : w_; true)

template <class CP>
__global__ void __launch_bounds__(kBlock)
k_lambda_coop(const float4* __restrict__ P, const float4* __restrict__ XP,
              const int32_t* __restrict__ cstart, const int32_t* __restrict__ cend,
              float4* __restrict__ L, float4* __restrict__ aux, uint32_t n, CP cp, CoopWork wk) {
    PBF_COOP_FOR_EACH(i) {
        const auto& c = cp.at(i);
        const float3 pi = xyz(P[i]);
        auto ctr = [&] { return stencil_centre(XP[i], c); };  // neighbourcells.glsl:57
        LambdaAcc a{0.0f, 0.0f, make_float3(0.0f, 0.0f, 0.0f)};
        float tw = 0.0f, tgg = 0.0f;
        float3 tg = make_float3(0.0f, 0.0f, 0.0f);
        bool tgrad = false;
        coop_visit(i, ctr, c, cstart, cend, P, pi,
                   [&](uint32_t, float3 d, float r2) {
                       const float len = fsqrt(r2);
                       tw = w_poly6(c, len);
                       tgrad = len != 0.0f;
                       if (tgrad) {
                           tg = scale3(d, grad_scale(c.kg_lambda, c.h, len));
                           tgg = dot3(tg, tg);
                       }
                       return true;
                   },
                   [&](int src) {
                       a.rho = fadd(a.rho, shf(tw, src));  // calclambda.glsl:80-82
                       const bool g = __shfl_sync(kFull, tgrad, src);
                       const float gg = shf(tgg, src);
                       const float3 gv = shf3(tg, src);
                       if (g) {
                           a.sumk = fadd(a.sumk, gg);  // :89
                           a.gi = add3(a.gi, gv);       // :93
                       }
                   });
        if ((threadIdx.x & 31u) == 0u) {
            L[i] = make_float4(pi.x, pi.y, pi.z, lambda_finish(c, a));
            if (aux) aux[i] = lambda_aux(a);
        }
    }
}

template <class CP>
__global__ void __launch_bounds__(kBlock)
k_delta_p_coop(const float4* __restrict__ L, const float4* __restrict__ XP,
               const int32_t* __restrict__ cstart, const int32_t* __restrict__ cend,
               float4* __restrict__ Pn, ScanPos sx_out, uint32_t n, CP cp, uint32_t* status,
               CoopWork wk) {
    PBF_COOP_FOR_EACH(i) {
        const auto& c = cp.at(i);
        const float4 Li = L[i];
        const float3 pi = xyz(Li);
        const float li = Li.w;
        auto ctr = [&] { return stencil_centre(XP[i], c); };  // neighbourcells.glsl:57
        float3 dp = make_float3(0.0f, 0.0f, 0.0f);
        float tcoef = 0.0f;
        float3 tg = make_float3(0.0f, 0.0f, 0.0f);
        coop_visit(i, ctr, c, cstart, cend, L, pi,
                   [&](uint32_t j, float3 d, float r2) {
                       const float len = fsqrt(r2);
                       if (len == 0.0f) return false;
                       float sc = fmul(c.scale, w_poly6(c, len));  // updatepos.glsl:57
                       sc = fmul(sc, sc);                           // :58
                       sc = fmul(sc, sc);                           // :59
                       sc = fmul(c.negk, sc);                       // :60
                       tcoef = fadd(fadd(li, __ldg(L + j).w), sc);  // :65
                       tg = scale3(d, grad_scale(c.kg, c.h, len));
                       return true;
                   },
                   [&](int src) { dp = fma3(shf(tcoef, src), shf3(tg, src), dp); });  // :65
        if ((threadIdx.x & 31u) == 0u) {
            float3 q = fma3(c.oorho, dp, pi);  // :85
            q.x = (q.x < c.lo[0]) ? c.lo[0] : q.x;
            q.x = (c.hi[0] < q.x) ? c.hi[0] : q.x;
            q.y = (q.y < c.lo[1]) ? c.lo[1] : q.y;
            q.y = (c.hi[1] < q.y) ? c.hi[1] : q.y;
            q.z = (q.z < c.lo[2]) ? c.lo[2] : q.z;
            q.z = (c.hi[2] < q.z) ? c.hi[2] : q.z;
            if (!finite3(q)) atomicOr(status, kDevNonFinite);
            Pn[i] = make_float4(q.x, q.y, q.z, 0.0f);
            if (sx_out.xy) scanpos_store(sx_out, i, q.x, q.y, q.z);
        }
    }
}

template <class CP>
__global__ void __launch_bounds__(kBlock)
k_vorticity_a_coop(const float4* __restrict__ P, const float4* __restrict__ VS,
                   const float4* __restrict__ XP, const int32_t* __restrict__ cstart,
                   const int32_t* __restrict__ cend, float4* __restrict__ VX,
                   float4* __restrict__ OM, float4* __restrict__ Q, uint32_t n, CP cp,
                   CoopWork wk) {
    PBF_COOP_FOR_EACH(i) {
        const auto& c = cp.at(i);
        const float3 pi = xyz(P[i]);
        const float3 vi = xyz(VS[i]);
        auto ctr = [&] { return stencil_centre(XP[i], c); };  // neighbourcells.glsl:57
        float3 acc = make_float3(0.0f, 0.0f, 0.0f), w = make_float3(0.0f, 0.0f, 0.0f);
        float tw = 0.0f;
        float3 tv = make_float3(0.0f, 0.0f, 0.0f), tc = make_float3(0.0f, 0.0f, 0.0f);
        bool tgrad = false;
        coop_visit(i, ctr, c, cstart, cend, P, pi,
                   [&](uint32_t j, float3 d, float r2) {
                       const float len = fsqrt(r2);
                       tv = sub3(xyz(__ldg(VS + j)), vi);  // vorticity.glsl:50
                       tw = w_poly6(c, len);
                       tgrad = len != 0.0f;
                       if (tgrad) tc = cross3(tv, scale3(d, grad_scale(c.kg, c.h, len)));  // :55
                       return true;
                   },
                   [&](int src) {
                       acc = fma3(shf(tw, src), shf3(tv, src), acc);  // :52-54
                       const bool g = __shfl_sync(kFull, tgrad, src);
                       const float3 cv = shf3(tc, src);
                       if (g) w = add3(w, cv);  // :55
                   });
        if ((threadIdx.x & 31u) == 0u) {
            const float3 vx = fma3(c.cx, acc, vi);  // :58
            VX[i] = make_float4(vx.x, vx.y, vx.z, 0.0f);
            OM[i] = make_float4(w.x, w.y, w.z, 0.0f);
            Q[i] = make_float4(pi.x, pi.y, pi.z, fsqrt(dot3(w, w)));  // :60
        }
    }
}

template <class CP>
__global__ void __launch_bounds__(kBlock)
k_vorticity_b_coop(const float4* __restrict__ Q, const float4* __restrict__ VX,
                   const float4* __restrict__ OM, const float4* __restrict__ XP,
                   const uint32_t* __restrict__ perm, const int32_t* __restrict__ cstart,
                   const int32_t* __restrict__ cend, float4* __restrict__ v,
                   float4* __restrict__ eta_out, uint32_t n, CP cp, CoopWork wk) {
    PBF_COOP_FOR_EACH(i) {
        const auto& c = cp.at(i);
        const float3 pi = xyz(Q[i]);
        auto ctr = [&] { return stencil_centre(XP[i], c); };  // neighbourcells.glsl:57
        float3 eta = make_float3(0.0f, 0.0f, 0.0f);
        float tq = 0.0f;
        float3 tg = make_float3(0.0f, 0.0f, 0.0f);
        coop_visit(i, ctr, c, cstart, cend, Q, pi,
                   [&](uint32_t j, float3 d, float r2) {
                       const float len = fsqrt(r2);
                       if (len == 0.0f) return false;
                       tq = __ldg(Q + j).w;
                       tg = scale3(d, grad_scale(c.kg, c.h, len));
                       return true;
                   },
                   [&](int src) { eta = fma3(shf(tq, src), shf3(tg, src), eta); });  // vorticity.glsl:72
        if ((threadIdx.x & 31u) == 0u) {
            if (eta_out) eta_out[i] = make_float4(eta.x, eta.y, eta.z, 0.0f);
            const float l = fsqrt(dot3(eta, eta));  // :76
            if (l > 0.0f) eta = make_float3(fdiv(eta.x, l), fdiv(eta.y, l), fdiv(eta.z, l));  // :77-78
            const float3 vf = fma3(c.dteps, cross3(eta, xyz(OM[i])), xyz(VX[i]));  // :82
            v[perm[i]] = make_float4(vf.x, vf.y, vf.z, 0.0f);                     // :85
        }
    }
}

// Mixed sweeps: the heavy particles (more than `threshold` stencil
// candidates) go to the cooperative kernels, listed once per substep after
// the cell pass (the set depends on the cell tables only, so every sweep of
// the substep agrees on it); the one-thread kernels skip them.  A block
// appends its heavy particles in ascending order (one atomic per block), so
// consecutive warps of a cooperative launch work on neighbouring particles.
template <class CP>
__global__ void __launch_bounds__(kBlock)
k_heavy_scan(const float4* __restrict__ XP, const int32_t* __restrict__ cstart,
             const int32_t* __restrict__ cend, uint32_t threshold, uint32_t n, CP cp,
             uint8_t* __restrict__ heavy, uint32_t* __restrict__ list, uint32_t* __restrict__ count) {
    __shared__ uint32_t warp_off[kBlock / 32];
    __shared__ uint32_t base;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    bool h = false;
    if (i < n) {
        Runs r;
        runs_of(stencil_centre(XP[i], cp.at(i)), cp.at(i), cstart, cend, r);
        uint32_t cand = 0;
#pragma unroll
        for (int o = 0; o < 9; ++o) cand += (uint32_t)(r.e[o] - r.b[o]);
        h = cand > threshold;
        heavy[i] = h ? 1 : 0;
    }
    const uint32_t m = __ballot_sync(0xffffffffu, h);
    if (lane == 0) warp_off[wid] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (uint32_t w = 0; w < blockDim.x / 32; ++w) {
            const uint32_t c = warp_off[w];
            warp_off[w] = t;
            t += c;
        }
        base = t ? atomicAdd(count, t) : 0u;
    }
    __syncthreads();
    if (h) list[base + warp_off[wid] + __popc(m & ((1u << lane) - 1u))] = i;
}

// Grid of the cooperative kernels of a mixed sweep (the heavy list's length is
// only known on the device): 8 blocks of 8 warps per SM.
constexpr unsigned kHeavyGrid = 152 * 8;

// Grid of warps, one per particle.
inline unsigned coop_grid(uint32_t n) { return (unsigned)(((size_t)n * 32 + kBlock - 1) / kBlock); }

// update.glsl:16-28: v = (x* - x_old) / dt, x = x*, scattered back to id order.
// VS receives the committed velocity in sorted order; when `v_out` is set the
// velocity is also stored in id order (vorticity confinement disabled).
template <class CP>
__global__ void __launch_bounds__(kBlock)
k_commit(const float4* __restrict__ P, const uint32_t* __restrict__ perm, float4* __restrict__ x,
         float4* __restrict__ VS, float4* __restrict__ v_out, uint32_t n, CP cp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const auto& c = cp.at(i);
    const uint32_t id = perm[i];
    if (!check_ok(c, id < c.n_total)) return;
    const float4 q = P[i];
    const float4 xo = x[id];
    const float4 w = make_float4(fdiv(fsub(q.x, xo.x), c.dt), fdiv(fsub(q.y, xo.y), c.dt),
                                 fdiv(fsub(q.z, xo.z), c.dt), 0.0f);  // :23
    VS[i] = w;
    x[id] = make_float4(q.x, q.y, q.z, 0.0f);  // :26
    if (v_out) v_out[id] = w;                  // :27
}

// vorticity.glsl:34-60: XSPH velocity and the vorticity vector, Jacobi
// (every read sees the committed velocities).
template <class CP, int MODE, bool LISTS>
__global__ void __launch_bounds__(kBlock, kVortBlocksPerSM)
k_vorticity_a(const float4* __restrict__ P, const float4* __restrict__ XP,
              const float4* __restrict__ VS, const uint32_t* __restrict__ skeys,
              const int32_t* __restrict__ cstart, const int32_t* __restrict__ cend,
              float4* __restrict__ VX, float4* __restrict__ OM, float4* __restrict__ Q,
              NbrLists nl, PairLists pw, ScanPos sx, int dmax_slot, uint32_t n, CP cp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (pw.heavy && pw.heavy[i])) return;
    const auto& c = cp.at(i);
    const float3 pi = xyz(P[i]);
    const float3 vi = xyz(VS[i]);
    auto ctr = [&] { return stencil_centre(XP[i], c); };  // neighbourcells.glsl:57
    float3 acc = make_float3(0.0f, 0.0f, 0.0f), w = make_float3(0.0f, 0.0f, 0.0f);
    // body of one candidate; IN: already known to pass the in-range test (the
    // masked scans computed the same r2 bit for bit)
    auto body = [&](uint32_t j, auto in) {
        const float3 d = sub3(pi, xyz(__ldg(P + j)));  // :51
        const float r2 = dot3(d, d);
        if (!decltype(in)::value && r2 > c.r2cut) return;
        const float len = fsqrt(r2);
        const float3 vij = sub3(xyz(__ldg(VS + j)), vi);  // :50
        acc = fma3(w_poly6(c, len), vij, acc);            // :52-54
        if (len == 0.0f) return;
        const float3 g = scale3(d, grad_scale(c.kg, c.h, len));
        w = add3(w, cross3(vij, g));  // :55
    };
    auto eval = [&](uint32_t j) { body(j, std::false_type{}); };
    auto eval_in = [&](uint32_t j) { body(j, std::true_type{}); };
    bool listed = false;
    if constexpr (LISTS) {
        const int32_t cnt = nl.cnt[i];
        if (list_usable(c, nl, cnt, pi, xyz(XP[i]), dmax_slot)) {
            listed = true;
            if constexpr (MODE == kPairs) {
                PairRecorder rec{pw, i, 0u};
                visit_list(i, c, cnt, nl, [&](uint32_t j) {
                    const float3 d = sub3(pi, xyz(__ldg(P + j)));
                    if (!(dot3(d, d) > c.r2cut)) rec(j);
                    eval(j);
                });
                rec.finish();
            } else {
                visit_list(i, c, cnt, nl, eval);
            }
        }
    }
    if (!listed) {
        if constexpr (MODE == kPairs)
            scan_then_eval<false>(i, ctr, c, cstart, cend, sx, pi, pw, [](int32_t, uint32_t) {},
                                  eval_in);
        else if constexpr (MODE == kMasked)
            sweep_visit<true>(i, ctr, c, cstart, cend, sx, pi, eval_in);
        else if (!LISTS && pw.runs)
            visit_direct_piles(
                i, ctr, c, cstart, cend, pw.runs,
                [&](uint32_t j) { return xyz(__ldg(P + j)); }, pi, eval,
                // the run bits are over (p, committed v): a run holds one
                // position and one velocity, so its terms are all equal
                [&](uint32_t j0, uint32_t, uint32_t m) {  // len 0: W(0) (v_j - v_i), no curl
                    acc = repeat_fma3(w_poly6(c, 0.0f), sub3(xyz(__ldg(VS + j0)), vi), acc, m);
                },
                [&](uint32_t j0, uint32_t r, float3 d, float r2) {
                    if (r2 > c.r2cut) return;
                    const float len = fsqrt(r2);
                    const float3 g = scale3(d, grad_scale(c.kg, c.h, len));
                    const float3 vij = sub3(xyz(__ldg(VS + j0)), vi);  // :50
                    acc = repeat_fma3(w_poly6(c, len), vij, acc, r - j0);  // :52-54
                    w = repeat_add3(cross3(vij, g), w, r - j0);            // :55
                });
        else
            sweep_visit<false>(i, ctr, c, cstart, cend, sx, pi, eval);
    }
    const float3 vx = fma3(c.cx, acc, vi);  // :58
    VX[i] = make_float4(vx.x, vx.y, vx.z, 0.0f);
    OM[i] = make_float4(w.x, w.y, w.z, 0.0f);
    Q[i] = make_float4(pi.x, pi.y, pi.z, fsqrt(dot3(w, w)));  // :60
}

// vorticity.glsl:65-85: confinement from the gradient of |vorticity|; writes
// the final velocity in id order.
template <class CP, int MODE, bool LISTS>
__global__ void __launch_bounds__(kBlock, kSweepBlocksPerSM)
k_vorticity_b(const float4* __restrict__ Q, const float4* __restrict__ XP,
              const float4* __restrict__ VX, const float4* __restrict__ OM,
              const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ perm,
              const int32_t* __restrict__ cstart, const int32_t* __restrict__ cend,
              float4* __restrict__ v, float4* __restrict__ eta_out, NbrLists nl, PairLists pr,
              ScanPos sx, int dmax_slot, uint32_t n, CP cp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (pr.heavy && pr.heavy[i])) return;
    const auto& c = cp.at(i);
    const float3 pi = xyz(Q[i]);
    auto ctr = [&] { return stencil_centre(XP[i], c); };  // neighbourcells.glsl:57
    float3 eta = make_float3(0.0f, 0.0f, 0.0f);
    auto body = [&](uint32_t j) {
        const float4 Qj = __ldg(Q + j);
        const float3 d = sub3(pi, xyz(Qj));  // :69
        const float r2 = dot3(d, d);
        if (r2 > c.r2cut) return;
        const float len = fsqrt(r2);
        if (len == 0.0f) return;
        eta = fma3(Qj.w, scale3(d, grad_scale(c.kg, c.h, len)), eta);  // :72
    };
    bool done = false;
    if constexpr (MODE == kPairs) done = visit_pairs(i, c, pr, body);
    if (!done) {
        bool listed = false;
        if constexpr (LISTS) {
            const int32_t cnt = nl.cnt[i];
            if (list_usable(c, nl, cnt, pi, xyz(XP[i]), dmax_slot)) {
                visit_list(i, c, cnt, nl, body);
                listed = true;
            }
        }
        if (!listed) {
            if (MODE == kDirect && !LISTS && pr.runs)  // coincident: no term (:71)
                visit_direct_piles(
                    i, ctr, c, cstart, cend, pr.runs,
                    [&](uint32_t j) { return xyz(__ldg(Q + j)); }, pi, body, [](uint32_t, uint32_t, uint32_t) {},
                    [&](uint32_t j0, uint32_t r, float3 d, float r2) {
                        // one offset and, the run bits being over (p, |omega|),
                        // one |omega_j|: r - j0 equal terms in a row
                        if (r2 > c.r2cut) return;
                        const float3 g = scale3(d, grad_scale(c.kg, c.h, fsqrt(r2)));
                        eta = repeat_fma3(__ldg(&Q[j0].w), g, eta, r - j0);  // :72
                    });
            else
                sweep_visit<MODE != kDirect>(i, ctr, c, cstart, cend, sx, pi, body);
        }
    }
    if (eta_out) eta_out[i] = make_float4(eta.x, eta.y, eta.z, 0.0f);
    const float l = fsqrt(dot3(eta, eta));  // :76
    if (l > 0.0f) eta = make_float3(fdiv(eta.x, l), fdiv(eta.y, l), fdiv(eta.z, l));  // :77-78
    const float3 vf = fma3(c.dteps, cross3(eta, xyz(OM[i])), xyz(VX[i]));  // :82
    if (check_ok(c, perm[i] < c.n_total)) v[perm[i]] = make_float4(vf.x, vf.y, vf.z, 0.0f);  // :85
}

// Per-particle density error |rho/rho0 - 1| (self excluded) and kinetic
// energy of the state sorted into P (positions) with velocities v (id order).
template <class CP>
__global__ void __launch_bounds__(kBlock)
k_diagnostics(const float4* __restrict__ P, const float4* __restrict__ v,
              const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ perm,
              const int32_t* __restrict__ cstart, const int32_t* __restrict__ cend,
              float4* __restrict__ out, uint32_t n, CP cp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const auto& c = cp.at(i);
    const float3 pi = xyz(P[i]);
    Runs r;
    runs_of(stencil_centre(pi, c), c, cstart, cend, r);
    float rho = 0.0f;
    int32_t cand = -1;
    for (int o = 0; o < 9; ++o) {
        cand += r.e[o] - r.b[o];
        for (int32_t j = r.b[o]; j < r.e[o]; ++j) {
            if ((uint32_t)j == i) continue;
            const float3 d = sub3(pi, xyz(__ldg(P + j)));
            const float r2 = dot3(d, d);
            if (r2 > c.r2cut) continue;
            rho = fadd(rho, w_poly6(c, fsqrt(r2)));
        }
    }
    const float4 w = v[perm[i]];
    out[i] = make_float4(fabsf(ffma(rho, c.oorho, -1.0f)),
                         0.5f * (w.x * w.x + w.y * w.y + w.z * w.z), (float)cand, 0.0f);
}

// highlight.glsl:16-30 after clearhighlight.glsl: bit 1 of every particle is
// cleared, then set on all stencil candidates (not distance-filtered, as the
// reference's FOR_EACH_NEIGHBOUR) of each particle whose bit 0 is set.
// flags are in id order; the candidates come from the last substep's sort.
template <class CP>
__global__ void __launch_bounds__(kBlock)
k_highlight(const float4* __restrict__ XP, const uint32_t* __restrict__ perm,
            const int32_t* __restrict__ cstart, const int32_t* __restrict__ cend,
            uint32_t* flags, uint32_t n, CP cp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = perm[i];
    if (id >= n || (flags[id] & 1u) == 0u) return;
    const auto& c = cp.at(i);
    visit_full(i, [&] { return stencil_centre(XP[i], c); }, c, cstart, cend, [&](uint32_t j) {
        const uint32_t pj = perm[j];
        if (pj < n) atomicOr(flags + pj, 2u);
    });
}

__global__ void __launch_bounds__(kBlock) k_clear_highlight(uint32_t* flags, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] &= 1u;  // clearhighlight.glsl:7
}

template <class CP>
void launch_highlight(unsigned g, cudaStream_t st, const float4* XP, const uint32_t* perm,
                      const int32_t* cstart, const int32_t* cend, uint32_t* flags, uint32_t n,
                      CP cp) {
    k_clear_highlight<<<g, kBlock, 0, st>>>(flags, n);
    k_highlight<CP><<<g, kBlock, 0, st>>>(XP, perm, cstart, cend, flags, n, cp);
}
template void launch_highlight<OneScene>(unsigned, cudaStream_t, const float4*, const uint32_t*,
                                         const int32_t*, const int32_t*, uint32_t*, uint32_t,
                                         OneScene);
template void launch_highlight<ManyScenes>(unsigned, cudaStream_t, const float4*,
                                           const uint32_t*, const int32_t*, const int32_t*,
                                           uint32_t*, uint32_t, ManyScenes);

// Host-side launchers: the template kernels are launched from this file
// (their host stubs are not visible to other translation units).
template <class CP>
void launch_predict(unsigned g, cudaStream_t st, const float4* x, const float4* v, float4* xstar,
                    uint32_t* keys, uint32_t n, CP cp, uint32_t* status) {
    k_predict<CP><<<g, kBlock, 0, st>>>(x, v, xstar, keys, n, cp, status);
}
template <class CP>
void launch_keys_of(unsigned g, cudaStream_t st, const float4* x, float4* xstar, uint32_t* keys,
                    uint32_t n, CP cp) {
    k_keys_of<CP><<<g, kBlock, 0, st>>>(x, xstar, keys, n, cp);
}
// Launches KERNEL<CP, MODE, LISTS> for the tuning in `sw`.
#define PBF_SWEEP_LAUNCH(KERNEL, ...)                                                        \
    do {                                                                                     \
        const unsigned g_ = grid_for(n, (int)sw.block);                                      \
        switch (sw.mode * 2 + (sw.lists ? 1 : 0)) {                                          \
            case 0: KERNEL<CP, kDirect, false><<<g_, sw.block, 0, st>>>(__VA_ARGS__); break; \
            case 1: KERNEL<CP, kDirect, true><<<g_, sw.block, 0, st>>>(__VA_ARGS__); break;  \
            case 2: KERNEL<CP, kMasked, false><<<g_, sw.block, 0, st>>>(__VA_ARGS__); break; \
            case 3: KERNEL<CP, kMasked, true><<<g_, sw.block, 0, st>>>(__VA_ARGS__); break;  \
            case 4: KERNEL<CP, kPairs, false><<<g_, sw.block, 0, st>>>(__VA_ARGS__); break;  \
            default: KERNEL<CP, kPairs, true><<<g_, sw.block, 0, st>>>(__VA_ARGS__); break;  \
        }                                                                                    \
    } while (0)

template <class CP>
void launch_lambda_build(SweepCfg sw, cudaStream_t st, const float4* XP, const uint32_t* skeys,
                         const int32_t* cstart, const int32_t* cend, float4* L, float4* aux,
                         NbrLists nl, PairLists pw, ScanPos sx, uint32_t n, CP cp) {
    if (sw.mode == kCoop) {
        k_lambda_coop<CP><<<coop_grid(n), kBlock, 0, st>>>(XP, XP, cstart, cend, L, aux, n, cp,
                                                           CoopWork{nullptr, nullptr});
        return;
    }
    PBF_SWEEP_LAUNCH(k_lambda_build, XP, skeys, cstart, cend, L, aux, nl, pw, sx, n, cp);
    if (pw.heavy)
        k_lambda_coop<CP><<<kHeavyGrid, kBlock, 0, st>>>(XP, XP, cstart, cend, L, aux, n, cp,
                                                         CoopWork{pw.heavy_list, pw.heavy_count});
}
template <class CP>
void launch_lambda(SweepCfg sw, cudaStream_t st, const float4* P, const float4* XP,
                   const uint32_t* skeys, const int32_t* cstart, const int32_t* cend, float4* L,
                   float4* aux, NbrLists nl, PairLists pw, ScanPos sx, int dmax_slot, uint32_t n,
                   CP cp) {
    if (sw.mode == kCoop) {
        k_lambda_coop<CP><<<coop_grid(n), kBlock, 0, st>>>(P, XP, cstart, cend, L, aux, n, cp,
                                                           CoopWork{nullptr, nullptr});
        return;
    }
    PBF_SWEEP_LAUNCH(k_lambda, P, XP, skeys, cstart, cend, L, aux, nl, pw, sx, dmax_slot, n, cp);
    if (pw.heavy)
        k_lambda_coop<CP><<<kHeavyGrid, kBlock, 0, st>>>(P, XP, cstart, cend, L, aux, n, cp,
                                                         CoopWork{pw.heavy_list, pw.heavy_count});
}
template <class CP>
void launch_delta_p(SweepCfg sw, cudaStream_t st, const float4* L, const float4* XP,
                    const uint32_t* skeys, const int32_t* cstart, const int32_t* cend, float4* Pn,
                    NbrLists nl, PairLists pr, ScanPos sx, ScanPos sx_out, int dmax_slot,
                    int out_slot, uint32_t n, CP cp, uint32_t* status) {
    if (sw.mode == kCoop) {
        k_delta_p_coop<CP><<<coop_grid(n), kBlock, 0, st>>>(L, XP, cstart, cend, Pn,
                                                            ScanPos{nullptr, nullptr}, n, cp, status,
                                                            CoopWork{nullptr, nullptr});
        return;
    }
    PBF_SWEEP_LAUNCH(k_delta_p, L, XP, skeys, cstart, cend, Pn, nl, pr, sx, sx_out, dmax_slot,
                     out_slot, n, cp, status);
    if (pr.heavy)
        k_delta_p_coop<CP><<<kHeavyGrid, kBlock, 0, st>>>(L, XP, cstart, cend, Pn, sx_out, n, cp,
                                                          status,
                                                          CoopWork{pr.heavy_list, pr.heavy_count});
}
template <class CP>
void launch_heavy_scan(unsigned g, cudaStream_t st, const float4* XP, const int32_t* cstart,
                       const int32_t* cend, uint32_t threshold, uint32_t n, CP cp, uint8_t* heavy,
                       uint32_t* list, uint32_t* count) {
    k_heavy_scan<CP><<<g, kBlock, 0, st>>>(XP, cstart, cend, threshold, n, cp, heavy, list, count);
}
template <class CP>
void launch_commit(unsigned g, cudaStream_t st, const float4* P, const uint32_t* perm, float4* x,
                   float4* VS, float4* v_out, uint32_t n, CP cp) {
    k_commit<CP><<<g, kBlock, 0, st>>>(P, perm, x, VS, v_out, n, cp);
}
template <class CP>
void launch_vorticity_a(SweepCfg sw, cudaStream_t st, const float4* P, const float4* XP,
                        const float4* VS, const uint32_t* skeys, const int32_t* cstart,
                        const int32_t* cend, float4* VX, float4* OM, float4* Q, NbrLists nl,
                        PairLists pw, ScanPos sx, int dmax_slot, uint32_t n, CP cp) {
    if (sw.mode == kCoop) {
        k_vorticity_a_coop<CP><<<coop_grid(n), kBlock, 0, st>>>(P, VS, XP, cstart, cend, VX, OM, Q,
                                                               n, cp, CoopWork{nullptr, nullptr});
        return;
    }
    PBF_SWEEP_LAUNCH(k_vorticity_a, P, XP, VS, skeys, cstart, cend, VX, OM, Q, nl, pw, sx, dmax_slot,
                     n, cp);
    if (pw.heavy)
        k_vorticity_a_coop<CP><<<kHeavyGrid, kBlock, 0, st>>>(
            P, VS, XP, cstart, cend, VX, OM, Q, n, cp, CoopWork{pw.heavy_list, pw.heavy_count});
}
template <class CP>
void launch_vorticity_b(SweepCfg sw, cudaStream_t st, const float4* Q, const float4* XP,
                        const float4* VX, const float4* OM, const uint32_t* skeys,
                        const uint32_t* perm, const int32_t* cstart, const int32_t* cend,
                        float4* v, float4* eta_out, NbrLists nl, PairLists pr, ScanPos sx,
                        int dmax_slot, uint32_t n, CP cp) {
    if (sw.mode == kCoop) {
        k_vorticity_b_coop<CP><<<coop_grid(n), kBlock, 0, st>>>(Q, VX, OM, XP, perm, cstart, cend, v,
                                                               eta_out, n, cp, CoopWork{nullptr, nullptr});
        return;
    }
    PBF_SWEEP_LAUNCH(k_vorticity_b, Q, XP, VX, OM, skeys, perm, cstart, cend, v, eta_out, nl, pr, sx,
                     dmax_slot, n, cp);
    if (pr.heavy)
        k_vorticity_b_coop<CP><<<kHeavyGrid, kBlock, 0, st>>>(
            Q, VX, OM, XP, perm, cstart, cend, v, eta_out, n, cp,
            CoopWork{pr.heavy_list, pr.heavy_count});
}
template <class CP>
void launch_diagnostics(unsigned g, cudaStream_t st, const float4* P, const float4* v,
                        const uint32_t* skeys, const uint32_t* perm, const int32_t* cstart,
                        const int32_t* cend, float4* out, uint32_t n, CP cp) {
    k_diagnostics<CP><<<g, kBlock, 0, st>>>(P, v, skeys, perm, cstart, cend, out, n, cp);
}

#define PBF_INSTANTIATE(CP)                                                                     \
    template void launch_predict<CP>(unsigned, cudaStream_t, const float4*, const float4*,      \
                                     float4*, uint32_t*, uint32_t, CP, uint32_t*);              \
    template void launch_keys_of<CP>(unsigned, cudaStream_t, const float4*, float4*, uint32_t*, \
                                     uint32_t, CP);                                             \
    template void launch_lambda_build<CP>(SweepCfg, cudaStream_t, const float4*, const uint32_t*, \
                                          const int32_t*, const int32_t*, float4*, float4*,     \
                                          NbrLists, PairLists, ScanPos, uint32_t, CP);          \
    template void launch_lambda<CP>(SweepCfg, cudaStream_t, const float4*, const float4*,       \
                                    const uint32_t*, const int32_t*, const int32_t*, float4*,   \
                                    float4*, NbrLists, PairLists, ScanPos, int, uint32_t, CP);  \
    template void launch_delta_p<CP>(SweepCfg, cudaStream_t, const float4*, const float4*,      \
                                     const uint32_t*, const int32_t*, const int32_t*, float4*,  \
                                     NbrLists, PairLists, ScanPos, ScanPos, int, int, uint32_t, \
                                     CP, uint32_t*);                                            \
    template void launch_heavy_scan<CP>(unsigned, cudaStream_t, const float4*, const int32_t*,    \
                                        const int32_t*, uint32_t, uint32_t, CP, uint8_t*,          \
                                        uint32_t*, uint32_t*);                                     \
    template void launch_commit<CP>(unsigned, cudaStream_t, const float4*, const uint32_t*,     \
                                    float4*, float4*, float4*, uint32_t, CP);                   \
    template void launch_vorticity_a<CP>(SweepCfg, cudaStream_t, const float4*, const float4*,  \
                                         const float4*, const uint32_t*, const int32_t*,        \
                                         const int32_t*, float4*, float4*, float4*, NbrLists,   \
                                         PairLists, ScanPos, int, uint32_t, CP);                \
    template void launch_vorticity_b<CP>(SweepCfg, cudaStream_t, const float4*, const float4*,  \
                                         const float4*, const float4*, const uint32_t*,         \
                                         const uint32_t*, const int32_t*, const int32_t*,       \
                                         float4*, float4*, NbrLists, PairLists, ScanPos, int,   \
                                         uint32_t, CP);                                         \
    template void launch_diagnostics<CP>(unsigned, cudaStream_t, const float4*, const float4*,  \
                                         const uint32_t*, const uint32_t*, const int32_t*,      \
                                         const int32_t*, float4*, uint32_t, CP);

PBF_INSTANTIATE(OneScene)
PBF_INSTANTIATE(ManyScenes)

// Loads every sweep kernel the automatic configuration may launch (the
// runtime loads a kernel on its first use otherwise, a few hundred
// microseconds each, which would land in the first trial's substeps).
template <class CP>
cudaError_t preload_sweeps() {
    cudaFuncAttributes a;
    cudaError_t e = cudaSuccess;
    auto load = [&](const void* f) {
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, f);
    };
    load((const void*)k_lambda_build<CP, kDirect, false>);
    load((const void*)k_lambda_build<CP, kMasked, false>);
    load((const void*)k_lambda_build<CP, kPairs, false>);
    load((const void*)k_lambda<CP, kDirect, false>);
    load((const void*)k_lambda<CP, kMasked, false>);
    load((const void*)k_lambda<CP, kPairs, false>);
    load((const void*)k_delta_p<CP, kDirect, false>);
    load((const void*)k_delta_p<CP, kMasked, false>);
    load((const void*)k_delta_p<CP, kPairs, false>);
    load((const void*)k_vorticity_a<CP, kDirect, false>);
    load((const void*)k_vorticity_a<CP, kMasked, false>);
    load((const void*)k_vorticity_a<CP, kPairs, false>);
    load((const void*)k_vorticity_b<CP, kDirect, false>);
    load((const void*)k_vorticity_b<CP, kMasked, false>);
    load((const void*)k_vorticity_b<CP, kPairs, false>);
    load((const void*)k_lambda_coop<CP>);
    load((const void*)k_delta_p_coop<CP>);
    load((const void*)k_vorticity_a_coop<CP>);
    load((const void*)k_vorticity_b_coop<CP>);
    load((const void*)k_run_flags);
    load((const void*)k_run_flags_vals);
    return e;
}
template cudaError_t preload_sweeps<OneScene>();
template cudaError_t preload_sweeps<ManyScenes>();

}  // namespace pbf
