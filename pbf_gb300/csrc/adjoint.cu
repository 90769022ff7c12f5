// adjoint.cu — reverse-mode gradients of whole substeps (no reference
// counterpart: the reference has no differentiation).
//
// The sort permutation, the cell tables and therefore every particle's
// neighbour candidates are frozen from the forward pass: they are piecewise
// constant in the positions, and the pair terms vanish with zero slope at
// r = h, so freezing them gives the exact derivative almost everywhere.  The
// wall clamp contributes its subgradient (zero along a clamped component).
//
// Every reverse sweep is written as a gather, not a scatter: the pair
// functions obey G(-d) = -G(d), H(-d) = H(d), W(-d) = W(d), so each particle
// sums the contributions of its own equation and of its neighbours'
// equations from per-particle adjoint quantities.  No atomic adds into any
// sum (the only atomics set a flag and append to a list whose order no result
// depends on): results are deterministic.  The candidate relation is
// symmetric except around particles
// predicted outside the grid: the forward centres a stencil on the unclamped
// predicted cell (neighbourcells.glsl:57) while the sort files the particle
// under its clamped cell, so such a particle i may be a candidate of j without
// j being one of i's.  The reverse sweeps therefore visit the stencil around
// the clamped (key) cell, which holds both directions, and, in a substep with
// such particles, weigh each pair's terms by two flags: `own` (j is i's
// candidate: the terms of i's equation) and `trans` (i is j's candidate: the
// terms of j's equation).
//
// Notation (sorted particle i, neighbour j, d = p_i - p_j, r = |d|):
//   W(r)  = k6 (h^2 - r^2)^3                 poly6 (calclambda.glsl:41-47)
//   What  = dW/dp_i = -6 k6 (h^2 - r^2)^2 d
//   G(d)  = f(r) d, f = kg (h - r)^2 / r     spiky gradient (calclambda.glsl:57-64)
//   H u   = dG/dd u = f u + (f'/r)(d.u) d,   f' = -kg (h - r)(h + r) / r^2
// Forward solver iteration (lambda then delta-p, Jacobi):
//   lambda_i = -C_i / (S_i + eps),  C_i = rho_i/rho0 - 1,  rho_i = sum W,
//   S_i = sum |g_ij|^2 + |g_i|^2,   g_ij = G_ij / rho0,  g_i = sum_j g_ij
//   q_i = p_i + sum_j a_ij G_ij,    a_ij = (lambda_i + lambda_j + s_ij) / rho0,
//   s_ij = -k (scale W_ij)^4,       p'_i = clamp(q_i)
// Reverse (q-bar = p'-bar with clamped components zeroed):
//   lambda-bar_i = (1/rho0) sum_j (qb_i - qb_j).G_ij
//   p-bar_i     += qb_i + sum_j [a_ij H_ij (qb_i - qb_j) + (s'_ij/(r rho0)) ((qb_i - qb_j).G_ij) d]
//   rho-bar_i = -lambda-bar_i / (rho0 D_i),  S-bar_i = -lambda-bar_i lambda_i / D_i,  D = S + eps
//   p-bar_i     += sum_j [(rhob_i + rhob_j) What_ij + (2/rho0) H_ij (Sb_i (g_ij + g_i) + Sb_j (g_ij - g_j))]
// Velocity update (update.glsl) and XSPH + vorticity (vorticity.glsl):
//   v_i = (p_i - x_i)/dt;  vs_i = v_i + c sum_j W_ij (v_j - v_i);  w_i = sum_j (v_j - v_i) x G_ij
//   eta_i = sum_j |w_j| G_ij;  N_i = eta_i/|eta_i|;  vf_i = vs_i + dt eps_v (N_i x w_i)
#include "neighbours.cuh"
#include "internal.h"
#include "sim.h"

#include <algorithm>
#include <cstring>

namespace pbf {

constexpr int kAdjBlock = 256;
constexpr int kParams = 4;  // epsilon, tensile k, XSPH c, vorticity epsilon

struct Tape {
    uint32_t substeps = 0, every = 0, iters = 0, nslots = 0;
    bool vort = false;
    std::vector<float4*> ckpt_x, ckpt_v;  // states at substeps 0, every, 2 every, ... (id order)
    float4 *final_x = nullptr, *final_v = nullptr;
    struct Slot {
        uint32_t* perm = nullptr;
        int32_t *cstart = nullptr, *cend = nullptr;
        std::vector<float4*> L, AUX;
        float4 *PF = nullptr, *VS = nullptr, *OM = nullptr, *Q = nullptr, *ETA = nullptr;
        float4* X0 = nullptr;  // positions at the start of the substep (id order)
    };
    std::vector<Slot> slots;
    // adjoint work buffers
    float4 *XB = nullptr, *VB = nullptr;    // x-bar, v-bar at a substep boundary (id order)
    float4 *XB2 = nullptr, *VB2 = nullptr;  // the next boundary
    float4 *QB = nullptr, *PDB = nullptr, *RS = nullptr, *PA = nullptr;  // sorted
    float4 *VSB = nullptr, *ETB = nullptr, *OMB = nullptr, *VCB = nullptr;  // sorted
    float4 *XSB = nullptr, *XOB = nullptr;  // x*-bar and x_old-bar (id order)
    double* acc = nullptr;                  // [kParams][n] per-particle parameter gradients (id order)
    uint8_t* irr = nullptr;                 // [n] stencil centre != key cell (sorted), per substep
    uint32_t* words = nullptr;              // [2]: any particle irregular; flagged particles
    uint8_t* heavy = nullptr;               // [n] swept by a warp (sorted), per substep
    uint32_t* heavy_list = nullptr;         // [n] those particles
    uint32_t warp_above = 0;                // candidates above which a particle gets a warp
    std::vector<void*> owned;
};

namespace {

// ---- pair geometry ------------------------------------------------------------

struct Pair {
    float3 d;
    float r2, r;
};

__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float dotf(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 crossf(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Spiky-gradient pieces at r > 0: G = f d and
// H u = f u + (f'/r)(d.u) d = f u + f' r (rhat.u) rhat.
// The spiky gradient turns direction at r = 0, so H grows like 1/r; pairs
// closer than 1e-6 h (only in collapsed clumps) keep their first-order terms
// and drop H, which would otherwise overflow FP32.
struct Spiky {
    float f, fpr, inv_r;  // f(r), f'(r) r, 1/r
    bool near;
    __device__ __forceinline__ Spiky(const DevConsts& c, float r) {
        const float u = c.h - r;
        inv_r = 1.0f / r;
        f = c.kg * u * u * inv_r;
        fpr = -c.kg * u * (c.h + r) * inv_r;
        near = r < 1e-6f * c.h;
    }
    __device__ __forceinline__ float3 G(float3 d) const { return f * d; }
    __device__ __forceinline__ float3 H(float3 d, float3 v) const {
        if (near) return make_float3(0.0f, 0.0f, 0.0f);
        const float3 rh = inv_r * d;
        return f * v + (fpr * dotf(rh, v)) * rh;
    }
};

__device__ __forceinline__ float w6(const DevConsts& c, float r2) {
    const float t = c.h2 - r2;
    return c.k6 * t * t * t;
}
// dW/dp_i = -6 k6 (h^2 - r^2)^2 d
__device__ __forceinline__ float3 w6_grad(const DevConsts& c, float3 d, float r2) {
    const float t = c.h2 - r2;
    return (-6.0f * c.k6 * t * t) * d;
}

__device__ __forceinline__ float3 clamp_mask(float3 g, float3 p, const DevConsts& c) {
    // subgradient of clamp(): zero where the component sits on a wall
    if (p.x == c.lo[0] || p.x == c.hi[0]) g.x = 0.0f;
    if (p.y == c.lo[1] || p.y == c.hi[1]) g.y = 0.0f;
    if (p.z == c.lo[2] || p.z == c.hi[2]) g.z = 0.0f;
    return g;
}

// ---- candidate directions ---------------------------------------------------------

// The key (sorted) cell of a predicted position, the clamped counterpart of
// stencil_centre (counting.glsl:55 with the cap at G - 1).
__device__ __forceinline__ int3 key_cell(float4 q, const DevConsts& c) {
    return make_int3((int)cell_coord(q.x, c.G[0], c.Gi[0]), (int)cell_coord(q.y, c.G[1], c.Gi[1]),
                     (int)cell_coord(q.z, c.G[2], c.Gi[2]));
}

// Whether each direction of pair (i, j) is a forward candidate (see the top
// of this file).  `on` (the substep has irregular particles) is uniform.
struct PairDirs {
    const uint8_t* irr;
    const float4* XPc;
    const uint32_t* any;  // nonzero when the substep has irregular particles
    __device__ __forceinline__ void of(const DevConsts& c, uint32_t i, uint32_t j, float& own,
                                       float& trans) const {
        own = trans = 1.0f;
        if (!__ldg(any) || !(__ldg(irr + i) | __ldg(irr + j))) return;
        const float4 qi = __ldg(XPc + i), qj = __ldg(XPc + j);
        auto inside = [](int3 cell, int3 ctr) {
            return abs(cell.x - ctr.x) <= 1 && abs(cell.y - ctr.y) <= 1 && abs(cell.z - ctr.z) <= 1;
        };
        own = inside(key_cell(qj, c), stencil_centre(qi, c)) ? 1.0f : 0.0f;
        trans = inside(key_cell(qi, c), stencil_centre(qj, c)) ? 1.0f : 0.0f;
    }
};

// ---- neighbour visits of the reverse sweeps -----------------------------------
//
// Two reverse sweeps read each position set (delta-p then lambda at an
// iterate, vorticity pass B then pass A at the final positions), so the first
// scans the stencil once, writing each particle's in-range candidates (visit
// order) to a list in the handle's pair-list buffer, and runs its pair terms
// from that list; the second replays the list.  The lanes of a warp then run
// their (heavy) pair terms together instead of each at its own point of the
// stencil.  A particle whose list would overflow, or a handle without pair
// lists, uses the direct stencil visit; results are the same either way (the
// pair terms test r2 themselves, in the same order).
struct AdjLists {
    uint32_t* idx;
    int32_t* cnt;
    uint32_t cap, n;
};

template <class F>
__device__ __forceinline__ void adj_replay(uint32_t i, const DevConsts& c, const AdjLists& al,
                                           F&& f) {
    const int32_t cnt = al.cnt[i];
    const uint32_t* p = al.idx + i;
    if (cnt > 0) {  // the next index is loaded one entry ahead
        uint32_t jn = p[0];
#pragma unroll 1
        for (int32_t k = 0; k < cnt; ++k) {
            const uint32_t j = jn;
            if (k + 1 < cnt) jn = p[(size_t)(k + 1) * al.n];
            if (check_ok(c, j < c.n_total)) f(j);
        }
    }
}

template <class Ctr, class F>
__device__ __forceinline__ void adj_scan_eval(uint32_t i, Ctr&& ctr, const DevConsts& c,
                                              const int32_t* __restrict__ cstart,
                                              const int32_t* __restrict__ cend,
                                              const float4* __restrict__ X, float3 pi,
                                              const AdjLists& al, F&& f) {
    if (!al.cap) {
        visit_full(i, ctr, c, cstart, cend, f);
        return;
    }
    Runs r;
    runs_of(ctr(), c, cstart, cend, r);
    uint32_t tot = 0;
    uint32_t* const out = al.idx + i;
#pragma unroll 1
    for (int o = 0; o < 9; ++o) {
        const int32_t e = r.e[o];
#pragma unroll 1
        for (int32_t base = r.b[o]; base < e; base += 32) {
            const float4* __restrict__ p = X + base;
            const float4* const pe = p + min(e - base, 32);
            uint32_t m = 0, bit = 1;
#pragma unroll 1
            for (; p < pe; ++p) {
                const float4 xj = __ldg(p);
                const float3 d = make_float3(pi.x - xj.x, pi.y - xj.y, pi.z - xj.z);
                if (!(d.x * d.x + d.y * d.y + d.z * d.z > c.r2cut)) m |= bit;
                bit <<= 1;
            }
            const uint32_t self = i - (uint32_t)base;
            if (self < 32u) m &= ~(1u << self);
            while (m) {
                const int t = __ffs(m) - 1;
                m &= m - 1;
                if (tot < al.cap) out[(size_t)tot * al.n] = (uint32_t)(base + t);
                ++tot;
            }
        }
    }
    if (tot <= al.cap) {
        al.cnt[i] = (int32_t)tot;
        adj_replay(i, c, al, f);
    } else {
        al.cnt[i] = -1;
        visit_full(i, ctr, c, cstart, cend, f);
    }
}

template <class Ctr, class F>
__device__ __forceinline__ void adj_visit_again(uint32_t i, Ctr&& ctr, const DevConsts& c,
                                                const int32_t* __restrict__ cstart,
                                                const int32_t* __restrict__ cend,
                                                const AdjLists& al, F&& f) {
    if (al.cap && al.cnt[i] >= 0)
        adj_replay(i, c, al, f);
    else
        visit_full(i, ctr, c, cstart, cend, f);
}

// ---- a warp per particle for dense stencils ---------------------------------------
//
// A thread per particle leaves a dense stencil to one thread's serial loop
// over thousands of candidates (collapsed states: the 32,768-particle
// epsilon = 0.01 run holds piles of up to ~11,000 particles by substep 40),
// and with few particles per SM the slowest such thread sets the launch time.
// Particles whose key-cell stencil holds more than `warp_above` candidates
// are flagged by k_adj_flags and swept by a warp each: lane l takes the
// candidates b + l, b + l + 32, ... of each stencil row, in order, and the
// lanes' partial sums are folded by a fixed butterfly; lane 0 writes.  The
// thread sweeps skip flagged particles.  The sums run in another order than
// the thread's, so the two agree to rounding, not bitwise; both are
// deterministic.

template <class Ctr, class F>
__device__ __forceinline__ void warp_visit(uint32_t i, Ctr&& ctr, const DevConsts& c,
                                           const int32_t* __restrict__ cstart,
                                           const int32_t* __restrict__ cend, uint32_t lane,
                                           F&& f) {
    Runs r;
    runs_of(ctr(), c, cstart, cend, r);
#pragma unroll 1
    for (int o = 0; o < 9; ++o)
#pragma unroll 1
        for (int32_t j = r.b[o] + (int32_t)lane; j < r.e[o]; j += 32)
            if ((uint32_t)j != i) f((uint32_t)j);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}
__device__ __forceinline__ float3 warp_sum(float3 v) {
    return make_float3(warp_sum(v.x), warp_sum(v.y), warp_sum(v.z));
}

// The particles of one substep swept by warps (flag == nullptr: none).
struct Heavy {
    const uint8_t* flag;    // [n] 1: flagged (sorted index)
    const uint32_t* list;   // the flagged particles, in no fixed order
    const uint32_t* count;  // how many
};

// Warps per launch of the warp sweeps (4 blocks of 8 warps on each of 152 SMs);
// each takes flagged particles in turn.
constexpr unsigned kAdjWarpBlocks = 608;
constexpr uint32_t kAdjNoWarps = 0xFFFFFFFFu;  // warp_above: no particle gets a warp
constexpr uint32_t kAdjWarpAbove = 512;        // warp_above when the tuning gives 0

// Constants of particle `id` (scene lookup by id for batches).
template <class CP>
__device__ __forceinline__ const DevConsts& consts_of(const CP& cp, uint32_t id) {
    return cp.at(id);
}

// ---- reverse kernels --------------------------------------------------------------

// Per substep: irr[i] = 1 when particle i's stencil centre is not its key
// cell (predicted outside the grid), and word[0] set when some particle is;
// with `above` != kAdjNoWarps, heavy[i] = 1 when i's key-cell stencil holds
// more than `above` candidates, those particles listed (in no fixed order:
// each one's result does not depend on it) and counted in word[1].
template <class CP>
__global__ void __launch_bounds__(kAdjBlock)
k_adj_flags(const uint32_t* __restrict__ perm, const float4* __restrict__ XPc,
            const int32_t* __restrict__ cstart, const int32_t* __restrict__ cend,
            uint32_t above, uint8_t* __restrict__ irr, uint8_t* __restrict__ heavy,
            uint32_t* __restrict__ list, uint32_t* __restrict__ word, uint32_t n, CP cp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevConsts& c = consts_of(cp, perm[i]);
    const float4 q = XPc[i];
    const int3 a = stencil_centre(q, c), b = key_cell(q, c);
    const bool odd = a.x != b.x || a.y != b.y || a.z != b.z;
    irr[i] = odd ? 1 : 0;
    if (odd) atomicOr(word, 1u);
    if (above == kAdjNoWarps) return;
    Runs r;
    runs_of(b, c, cstart, cend, r);
    uint32_t cand = 0;
#pragma unroll
    for (int o = 0; o < 9; ++o) cand += (uint32_t)(r.e[o] - r.b[o]);
    const bool h = cand > above;
    heavy[i] = h ? 1 : 0;
    if (h) {
        const uint32_t k = atomicAdd(word + 1, 1u);
        if (check_ok(c, k < n)) list[k] = i;
    }
}

// One neighbour reversal (Body::run<W>): blocks below `tblocks` take a
// thread per unflagged particle, the blocks after them a warp per flagged
// particle (in turn, from the list).
template <class Body>
__global__ void __launch_bounds__(kAdjBlock) k_adj_sweep(Body b, Heavy hv, uint32_t n,
                                                         uint32_t tblocks) {
    if (blockIdx.x < tblocks) {
        const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n || (hv.flag && hv.flag[i])) return;
        b.template run<false>(i, 0u);
        return;
    }
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t w = ((blockIdx.x - tblocks) * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = ((gridDim.x - tblocks) * blockDim.x) >> 5;
    const uint32_t cnt = min(*hv.count, n);
#pragma unroll 1
    for (uint32_t k = w; k < cnt; k += nw) b.template run<true>(hv.list[k], lane);
}

// vorticity.glsl:76-85 reversed, pointwise: from vf-bar to vs-bar, eta-bar and
// the direct part of w-bar; accumulates d/d(eps_v).
template <class CP>
__global__ void __launch_bounds__(kAdjBlock)
k_adj_vort_b1(const uint32_t* __restrict__ perm, const float4* __restrict__ VB,
              const float4* __restrict__ OM, const float4* __restrict__ ETA,
              float4* __restrict__ VSB, float4* __restrict__ ETB, float4* __restrict__ OMB,
              double* __restrict__ acc_epsv, uint32_t n, CP cp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = perm[i];
    const DevConsts& c = consts_of(cp, id);
    const float3 vfb = f3(VB[id]);
    const float3 w = f3(OM[i]);
    const float3 eta = f3(ETA[i]);
    const float le = sqrtf(dotf(eta, eta));
    const float3 N = le > 0.0f ? (1.0f / le) * eta : eta;
    const float3 u = c.dteps * vfb;
    const float3 Nb = crossf(w, u);
    const float3 wb = crossf(u, N);
    acc_epsv[id] += (double)(c.dt * dotf(crossf(N, w), vfb));
    // d(eta/|eta|)/d(eta) grows like 1/|eta|; below 1e-20 (a particle with no
    // vorticity gradient) the normalisation's derivative is dropped
    const float3 eb = le > 1e-20f ? (1.0f / le) * (Nb - dotf(N, Nb) * N)
                                  : (le > 0.0f ? make_float3(0.0f, 0.0f, 0.0f) : Nb);
    VSB[i] = make_float4(vfb.x, vfb.y, vfb.z, 0.0f);
    ETB[i] = make_float4(eb.x, eb.y, eb.z, 0.0f);
    OMB[i] = make_float4(wb.x, wb.y, wb.z, 0.0f);
}

// vorticity.glsl:65-74 reversed: eta_i = sum_j |w_j| G_ij.  Gathers |w|-bar
// and the position adjoint, then folds |w|-bar into w-bar.
template <class CP>
struct AdjVortB2 {
    const uint32_t* __restrict__ perm;
    const float4* __restrict__ XPc;
    const int32_t* __restrict__ cstart;
    const int32_t* __restrict__ cend;
    const float4* __restrict__ Q;
    const float4* __restrict__ OM;
    const float4* __restrict__ ETB;
    float4* __restrict__ OMB;
    float4* __restrict__ PA;
    AdjLists al;
    PairDirs dirs;
    CP cp;
    template <bool W>
    __device__ __forceinline__ void run(uint32_t i, uint32_t lane) const {
        const uint32_t id = perm[i];
        const DevConsts& c = consts_of(cp, id);
        const float4 Qi = Q[i];
        const float3 pi = f3(Qi);
        const float mi = Qi.w;
        const float3 ebi = f3(ETB[i]);
        float mb = 0.0f;
        float3 pb = make_float3(0.0f, 0.0f, 0.0f);
        auto ctr = [&] { return key_cell(XPc[i], c); };
        auto pair = [&](uint32_t j) {
            const float4 Qj = __ldg(Q + j);
            const float3 d = pi - f3(Qj);
            const float r2 = dotf(d, d);
            if (r2 > c.r2cut || r2 == 0.0f) return;
            const Spiky sp(c, sqrtf(r2));
            float own, trans;
            dirs.of(c, i, j, own, trans);
            const float3 ebj = trans * f3(__ldg(ETB + j));
            mb -= dotf(ebj, sp.G(d));
            pb = pb + sp.H(d, (own * Qj.w) * ebi - mi * ebj);
        };
        if constexpr (W) {
            warp_visit(i, ctr, c, cstart, cend, lane, pair);
            mb = warp_sum(mb);
            pb = warp_sum(pb);
            if (lane) return;
        } else {
            adj_scan_eval(i, ctr, c, cstart, cend, Q, pi, al, pair);
        }
        float3 wb = f3(OMB[i]);
        if (mi > 0.0f) wb = wb + (mb / mi) * f3(OM[i]);
        OMB[i] = make_float4(wb.x, wb.y, wb.z, 0.0f);
        PA[i] = make_float4(pb.x, pb.y, pb.z, 0.0f);
    }
};

// vorticity.glsl:47-58 reversed (XSPH and the vorticity vector): gathers the
// committed-velocity adjoint and adds the position adjoint; accumulates d/dc.
template <class CP>
struct AdjVortA {
    const uint32_t* __restrict__ perm;
    const float4* __restrict__ XPc;
    const int32_t* __restrict__ cstart;
    const int32_t* __restrict__ cend;
    const float4* __restrict__ PF;
    const float4* __restrict__ VS;
    const float4* __restrict__ VSB;
    const float4* __restrict__ OMB;
    float4* __restrict__ VCB;
    float4* __restrict__ PA;
    double* __restrict__ acc_c;
    AdjLists al;
    PairDirs dirs;
    CP cp;
    template <bool W>
    __device__ __forceinline__ void run(uint32_t i, uint32_t lane) const {
        const uint32_t id = perm[i];
        const DevConsts& c = consts_of(cp, id);
        const float3 pi = f3(PF[i]);
        const float3 vi = f3(VS[i]);
        const float3 sbi = f3(VSB[i]);
        const float3 wbi = f3(OMB[i]);
        const float3 zero = make_float3(0.0f, 0.0f, 0.0f);
        float3 vb = W ? zero : sbi;
        float3 pb = W ? zero : f3(PA[i]);
        float3 wsum = zero;
        auto ctr = [&] { return key_cell(XPc[i], c); };
        auto pair = [&](uint32_t j) {
            const float3 d = pi - f3(__ldg(PF + j));
            const float r2 = dotf(d, d);
            if (r2 > c.r2cut) return;
            float own, trans;
            dirs.of(c, i, j, own, trans);
            const float3 vji = f3(__ldg(VS + j)) - vi;
            const float3 sbj = trans * f3(__ldg(VSB + j));
            const float3 sbo = own * sbi;
            const float W6 = w6(c, r2);
            vb = vb + (c.cx * W6) * (sbj - sbo);
            wsum = wsum + (own * W6) * vji;
            pb = pb + (c.cx * dotf(sbo - sbj, vji)) * w6_grad(c, d, r2);
            if (r2 == 0.0f) return;
            const Spiky sp(c, sqrtf(r2));
            const float3 wbs = own * wbi + trans * f3(__ldg(OMB + j));
            vb = vb - crossf(sp.G(d), wbs);
            pb = pb + sp.H(d, crossf(wbs, vji));
        };
        if constexpr (W) {
            warp_visit(i, ctr, c, cstart, cend, lane, pair);
            vb = sbi + warp_sum(vb);
            pb = f3(PA[i]) + warp_sum(pb);
            wsum = warp_sum(wsum);
            if (lane) return;
        } else {
            adj_visit_again(i, ctr, c, cstart, cend, al, pair);
        }
        acc_c[id] += (double)dotf(sbi, wsum);
        VCB[i] = make_float4(vb.x, vb.y, vb.z, 0.0f);
        PA[i] = make_float4(pb.x, pb.y, pb.z, 0.0f);
    }
};

// update.glsl:23-27 reversed: p-bar of the final positions, x_old-bar, and
// the clamp mask of the last solver iteration.
template <class CP>
__global__ void __launch_bounds__(kAdjBlock)
k_adj_commit(const uint32_t* __restrict__ perm, const float4* __restrict__ XB,
             const float4* __restrict__ VB, const float4* __restrict__ VCB,
             const float4* __restrict__ PA, const float4* __restrict__ PF, float4* __restrict__ QB,
             float4* __restrict__ XOB, float4* __restrict__ XSB, int vort, int iters, uint32_t n,
             CP cp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = perm[i];
    const DevConsts& c = consts_of(cp, id);
    const float3 vc = vort ? f3(VCB[i]) : f3(VB[id]);
    const float inv_dt = 1.0f / c.dt;
    float3 pb = f3(XB[id]) + inv_dt * vc;
    if (vort) pb = pb + f3(PA[i]);
    const float3 xo = (-inv_dt) * vc;
    XOB[id] = make_float4(xo.x, xo.y, xo.z, 0.0f);
    if (iters > 0) {
        pb = clamp_mask(pb, f3(PF[i]), c);
        QB[i] = make_float4(pb.x, pb.y, pb.z, 0.0f);
    } else {
        XSB[id] = make_float4(pb.x, pb.y, pb.z, 0.0f);
    }
}

// updatepos.glsl:42-104 reversed (one iteration), plus the pointwise part of
// calclambda's reverse: writes p-bar of the delta-p terms and (rho-bar, S-bar);
// accumulates d/d(eps) and d/dk.
template <class CP>
struct AdjDeltaP {
    const uint32_t* __restrict__ perm;
    const float4* __restrict__ XPc;
    const int32_t* __restrict__ cstart;
    const int32_t* __restrict__ cend;
    const float4* __restrict__ L;
    const float4* __restrict__ AUX;
    const float4* __restrict__ QB;
    float4* __restrict__ PDB;
    float4* __restrict__ RS;
    double* __restrict__ acc_eps;
    double* __restrict__ acc_k;
    AdjLists al;
    PairDirs dirs;
    CP cp;
    template <bool W>
    __device__ __forceinline__ void run(uint32_t i, uint32_t lane) const {
        const uint32_t id = perm[i];
        const DevConsts& c = consts_of(cp, id);
        const float4 Li = L[i];
        const float3 pi = f3(Li);
        const float li = Li.w;
        const float3 qbi = f3(QB[i]);
        float lb = 0.0f, kb = 0.0f;
        float3 pb = W ? make_float3(0.0f, 0.0f, 0.0f) : qbi;
        const float sc4 = c.scale * c.scale * c.scale * c.scale;
        auto ctr = [&] { return key_cell(XPc[i], c); };
        auto pair = [&](uint32_t j) {
            const float4 Lj = __ldg(L + j);
            const float3 d = pi - f3(Lj);
            const float r2 = dotf(d, d);
            if (r2 > c.r2cut || r2 == 0.0f) return;
            const Spiky sp(c, sqrtf(r2));
            const float t = c.h2 - r2;
            const float W6 = c.k6 * t * t * t;
            const float W3 = W6 * W6 * W6;
            const float s = c.negk * sc4 * W3 * W6;
            const float a = (li + Lj.w + s) * c.oorho;
            const float3 G = sp.G(d);
            float own, trans;
            dirs.of(c, i, j, own, trans);
            const float3 dq = own * qbi - trans * f3(__ldg(QB + j));
            const float dqG = dotf(dq, G);
            lb += c.oorho * dqG;
            // (ds/dr)/r = 4 negk scale^4 W^3 (-6 k6 (h^2 - r^2)^2)
            const float sr = 4.0f * c.negk * sc4 * W3 * (-6.0f * c.k6 * t * t);
            pb = pb + sp.H(d, a * dq) + (c.oorho * sr * dqG) * d;
            kb -= own * c.oorho * dotf(qbi, G) * sc4 * W3 * W6;
        };
        if constexpr (W) {
            warp_visit(i, ctr, c, cstart, cend, lane, pair);
            lb = warp_sum(lb);
            kb = warp_sum(kb);
            pb = qbi + warp_sum(pb);
            if (lane) return;
        } else {
            adj_scan_eval(i, ctr, c, cstart, cend, L, pi, al, pair);
        }
        const float4 aux = AUX[i];
        const float D = aux.w + c.eps;
        const float rb = -lb * c.oorho / D;
        const float Sb = -lb * li / D;
        acc_eps[id] += (double)Sb;
        acc_k[id] += (double)kb;
        PDB[i] = make_float4(pb.x, pb.y, pb.z, 0.0f);
        RS[i] = make_float4(rb, Sb, 0.0f, 0.0f);
    }
};

// calclambda.glsl:75-101 reversed (one iteration): gathers the density and
// denominator terms; masks the previous iteration's clamp, or un-sorts into
// the predicted-position adjoint after the first iteration.
template <class CP>
struct AdjLambda {
    const uint32_t* __restrict__ perm;
    const float4* __restrict__ XPc;
    const int32_t* __restrict__ cstart;
    const int32_t* __restrict__ cend;
    const float4* __restrict__ L;
    const float4* __restrict__ AUX;
    const float4* __restrict__ RS;
    const float4* __restrict__ PDB;
    float4* __restrict__ QB;
    float4* __restrict__ XSB;
    int first;
    AdjLists al;
    PairDirs dirs;
    CP cp;
    template <bool W>
    __device__ __forceinline__ void run(uint32_t i, uint32_t lane) const {
        const uint32_t id = perm[i];
        const DevConsts& c = consts_of(cp, id);
        const float3 pi = f3(L[i]);
        const float4 RSi = RS[i];
        const float3 gi = f3(AUX[i]);
        float3 pb = W ? make_float3(0.0f, 0.0f, 0.0f) : f3(PDB[i]);
        auto ctr = [&] { return key_cell(XPc[i], c); };
        auto pair = [&](uint32_t j) {
            const float3 d = pi - f3(__ldg(L + j));
            const float r2 = dotf(d, d);
            if (r2 > c.r2cut) return;
            float own, trans;
            dirs.of(c, i, j, own, trans);
            const float4 RSj = __ldg(RS + j);
            pb = pb + (own * RSi.x + trans * RSj.x) * w6_grad(c, d, r2);
            if (r2 == 0.0f) return;
            const Spiky sp(c, sqrtf(r2));
            const float3 gij = c.oorho * sp.G(d);
            const float3 gj = f3(__ldg(AUX + j));
            const float3 u = (own * RSi.y) * (gij + gi) + (trans * RSj.y) * (gij - gj);
            pb = pb + (2.0f * c.oorho) * sp.H(d, u);
        };
        if constexpr (W) {
            warp_visit(i, ctr, c, cstart, cend, lane, pair);
            pb = f3(PDB[i]) + warp_sum(pb);
            if (lane) return;
        } else {
            adj_visit_again(i, ctr, c, cstart, cend, al, pair);
        }
        if (first) {
            XSB[id] = make_float4(pb.x, pb.y, pb.z, 0.0f);
        } else {
            pb = clamp_mask(pb, pi, c);
            QB[i] = make_float4(pb.x, pb.y, pb.z, 0.0f);
        }
    }
};

// predictpos.glsl:32-34 reversed: x* = x + dt v'; plus the commit's x_old.
template <class CP>
__global__ void __launch_bounds__(kAdjBlock)
k_adj_predict(const float4* __restrict__ XSB, const float4* __restrict__ XOB,
              float4* __restrict__ XB, float4* __restrict__ VB, uint32_t n, CP cp) {
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const DevConsts& c = consts_of(cp, id);
    const float3 xs = f3(XSB[id]);
    const float3 xb = xs + f3(XOB[id]);
    const float3 vb = c.dt * xs;
    XB[id] = make_float4(xb.x, xb.y, xb.z, 0.0f);
    VB[id] = make_float4(vb.x, vb.y, vb.z, 0.0f);
}

// ---- host side ------------------------------------------------------------------

template <class T>
cudaError_t talloc(Tape* t, T** p, size_t count) {
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess) t->owned.push_back(*p);
    return e;
}

cudaError_t alloc_tape(pbf_sim* s, Tape* t) {
    const size_t n = s->n;
    const uint32_t nck = (t->substeps + t->every - 1) / t->every;
    cudaError_t e = cudaSuccess;
    t->ckpt_x.assign(nck, nullptr);
    t->ckpt_v.assign(nck, nullptr);
    for (uint32_t k = 0; k < nck && e == cudaSuccess; ++k) {
        e = talloc(t, &t->ckpt_x[k], n);
        if (e == cudaSuccess) e = talloc(t, &t->ckpt_v[k], n);
    }
    if (e == cudaSuccess) e = talloc(t, &t->final_x, n);
    if (e == cudaSuccess) e = talloc(t, &t->final_v, n);
    t->slots.resize(t->nslots);
    for (auto& sl : t->slots) {
        if (e == cudaSuccess) e = talloc(t, &sl.perm, n);
        if (e == cudaSuccess) e = talloc(t, &sl.cstart, s->ncells);
        if (e == cudaSuccess) e = talloc(t, &sl.cend, s->ncells);
        sl.L.assign(t->iters, nullptr);
        sl.AUX.assign(t->iters, nullptr);
        for (uint32_t k = 0; k < t->iters && e == cudaSuccess; ++k) {
            e = talloc(t, &sl.L[k], n);
            if (e == cudaSuccess) e = talloc(t, &sl.AUX[k], n);
        }
        if (e == cudaSuccess) e = talloc(t, &sl.PF, n);
        if (e == cudaSuccess) e = talloc(t, &sl.VS, n);
        if (e == cudaSuccess) e = talloc(t, &sl.OM, n);
        if (e == cudaSuccess) e = talloc(t, &sl.Q, n);
        if (e == cudaSuccess) e = talloc(t, &sl.ETA, n);
        if (e == cudaSuccess) e = talloc(t, &sl.X0, n);
    }
    float4** work[] = {&t->XB, &t->VB, &t->XB2, &t->VB2, &t->QB, &t->PDB, &t->RS, &t->PA,
                       &t->VSB, &t->ETB, &t->OMB, &t->VCB, &t->XSB, &t->XOB};
    for (float4** w : work)
        if (e == cudaSuccess) e = talloc(t, w, n);
    if (e == cudaSuccess) e = talloc(t, &t->acc, (size_t)kParams * n);
    if (e == cudaSuccess) e = talloc(t, &t->irr, n);
    if (e == cudaSuccess) e = talloc(t, &t->words, 2);
    if (e == cudaSuccess) e = talloc(t, &t->heavy, n);
    if (e == cudaSuccess) e = talloc(t, &t->heavy_list, n);
    return e;
}

template <class CP>
cudaError_t reverse_substep(pbf_sim* s, Tape* t, const Tape::Slot& sl, const CP& cp) {
    const uint32_t n = s->n;
    const unsigned g = grid_for(n, kAdjBlock);
    cudaStream_t st = s->stream;
    const int iters = (int)t->iters;
    double* acc_eps = t->acc;
    double* acc_k = t->acc + n;
    double* acc_c = t->acc + 2 * (size_t)n;
    double* acc_ev = t->acc + 3 * (size_t)n;
    const AdjLists al{s->pair_idx, s->pair_cnt, s->pair_cap, n};
    // the substep's predicted positions (sorted), where every stencil is
    // centred (neighbourcells.glsl:57): the first lambda sweep's L holds them,
    // and PF does when there is no solver iteration
    const float4* XPc = iters > 0 ? sl.L[0] : sl.PF;
    cudaError_t fe = cudaMemsetAsync(t->words, 0, 2 * sizeof(uint32_t), st);
    if (fe != cudaSuccess) return fe;
    k_adj_flags<<<g, kAdjBlock, 0, st>>>(sl.perm, XPc, sl.cstart, sl.cend, t->warp_above, t->irr,
                                         t->heavy, t->heavy_list, t->words, n, cp);
    const PairDirs dirs{t->irr, XPc, t->words};
    // the particles with dense stencils get a warp each
    const bool warps = t->warp_above != kAdjNoWarps;
    const Heavy hv{warps ? t->heavy : nullptr, t->heavy_list, t->words + 1};
    auto sweep = [&](const auto& body) {
        k_adj_sweep<<<g + (warps ? kAdjWarpBlocks : 0u), kAdjBlock, 0, st>>>(body, hv, n, g);
    };
    if (t->vort) {
        k_adj_vort_b1<<<g, kAdjBlock, 0, st>>>(sl.perm, t->VB, sl.OM, sl.ETA, t->VSB, t->ETB,
                                               t->OMB, acc_ev, n, cp);
        sweep(AdjVortB2<CP>{sl.perm, XPc, sl.cstart, sl.cend, sl.Q, sl.OM, t->ETB, t->OMB, t->PA,
                            al, dirs, cp});
        sweep(AdjVortA<CP>{sl.perm, XPc, sl.cstart, sl.cend, sl.PF, sl.VS, t->VSB, t->OMB,
                           t->VCB, t->PA, acc_c, al, dirs, cp});
    }
    k_adj_commit<<<g, kAdjBlock, 0, st>>>(sl.perm, t->XB, t->VB, t->VCB, t->PA, sl.PF, t->QB,
                                          t->XOB, t->XSB, t->vort ? 1 : 0, iters, n, cp);
    for (int k = iters - 1; k >= 0; --k) {
        sweep(AdjDeltaP<CP>{sl.perm, XPc, sl.cstart, sl.cend, sl.L[k], sl.AUX[k], t->QB, t->PDB,
                            t->RS, acc_eps, acc_k, al, dirs, cp});
        sweep(AdjLambda<CP>{sl.perm, XPc, sl.cstart, sl.cend, sl.L[k], sl.AUX[k], t->RS, t->PDB,
                            t->QB, t->XSB, k == 0 ? 1 : 0, al, dirs, cp});
    }
    k_adj_predict<<<g, kAdjBlock, 0, st>>>(t->XSB, t->XOB, t->XB2, t->VB2, n, cp);
    std::swap(t->XB, t->XB2);
    std::swap(t->VB, t->VB2);
    return cudaGetLastError();
}

cudaError_t reverse_dispatch(pbf_sim* s, Tape* t, const Tape::Slot& sl) {
    if (s->nscenes == 1) return reverse_substep(s, t, sl, OneScene{s->dc});
    return reverse_substep(s, t, sl, ManyScenes{s->d_consts, s->sid});
}

// Runs `count` substeps from the current state, recording each into a slot.
cudaError_t record_segment(pbf_sim* s, Tape* t, uint32_t count) {
    cudaStream_t st = s->stream;
    const size_t n = s->n;
    for (uint32_t k = 0; k < count; ++k) {
        Tape::Slot& sl = t->slots[k];
        cudaError_t e = cudaMemcpyAsync(sl.X0, s->x, sizeof(float4) * n, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return e;
        Recording rec;
        rec.L = sl.L.data();
        rec.AUX = sl.AUX.data();
        rec.PF = sl.PF;
        rec.VS = sl.VS;
        rec.OM = sl.OM;
        rec.Q = sl.Q;
        rec.ETA = sl.ETA;
        e = enqueue_substep(s, nullptr, &rec);
        if (e != cudaSuccess) return e;
        e = cudaMemcpyAsync(sl.perm, s->perm, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sl.cstart, s->cstart, sizeof(int32_t) * s->ncells,
                                cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sl.cend, s->cend, sizeof(int32_t) * s->ncells,
                                cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace

void free_tape(pbf_sim* s) {
    if (!s->tape) return;
    for (void* p : s->tape->owned) cudaFree(p);
    delete s->tape;
    s->tape = nullptr;
}

}  // namespace pbf

using namespace pbf;

extern "C" {

pbf_status pbf_forward_record(pbf_sim* s, uint32_t substeps, uint32_t checkpoint_every) {
    NvtxRange nvtx_("pbf_forward_record");
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (substeps == 0 || checkpoint_every == 0)
        return fail(s, PBF_ERR_INVALID_ARGUMENT, "substeps and checkpoint_every must be positive");
    DeviceGuard dg(s->device);
    PBF_CUDA(s, cudaStreamSynchronize(s->stream));
    free_tape(s);
    Tape* t = new Tape();
    s->tape = t;
    t->substeps = substeps;
    t->every = std::min(checkpoint_every, substeps);
    t->iters = s->params.num_solver_iterations;
    t->nslots = t->every;
    t->vort = s->params.vorticity_confinement != 0;
    cudaError_t e = alloc_tape(s, t);
    if (e != cudaSuccess) {
        free_tape(s);
        return cuda_fail(s, e, "tape allocation");
    }
    const size_t b = sizeof(float4) * s->n;
    for (uint32_t k = 0; k < substeps; ++k) {
        if (k % t->every == 0) {
            PBF_CUDA(s, cudaMemcpyAsync(t->ckpt_x[k / t->every], s->x, b, cudaMemcpyDeviceToDevice, s->stream));
            PBF_CUDA(s, cudaMemcpyAsync(t->ckpt_v[k / t->every], s->v, b, cudaMemcpyDeviceToDevice, s->stream));
        }
        pbf_status r = pbf_step(s, 1);
        if (r != PBF_OK) return r;
    }
    PBF_CUDA(s, cudaMemcpyAsync(t->final_x, s->x, b, cudaMemcpyDeviceToDevice, s->stream));
    PBF_CUDA(s, cudaMemcpyAsync(t->final_v, s->v, b, cudaMemcpyDeviceToDevice, s->stream));
    return check_status(s);
}

pbf_status pbf_backward(pbf_sim* s, const float* dL_dx4, const float* dL_dv4, int where,
                        float* dL_dx0_4, float* dL_dv0_4, pbf_param_grads* grads) {
    NvtxRange nvtx_("pbf_backward");
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (!s->tape) return fail(s, PBF_ERR_INVALID_ARGUMENT, "no recorded forward run (pbf_forward_record)");
    if (where != PBF_HOST && where != PBF_DEVICE) return fail(s, PBF_ERR_INVALID_ARGUMENT, "bad where");
    Tape* t = s->tape;
    if (t->iters != s->params.num_solver_iterations ||
        t->vort != (s->params.vorticity_confinement != 0))
        return fail(s, PBF_ERR_INVALID_ARGUMENT, "parameters changed since the recorded run");
    DeviceGuard dg(s->device);
    cudaStream_t st = s->stream;
    const size_t n = s->n;
    const size_t b = sizeof(float4) * n;
    const cudaMemcpyKind in = where == PBF_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    const cudaMemcpyKind out = where == PBF_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (dL_dx4)
        PBF_CUDA(s, cudaMemcpyAsync(t->XB, dL_dx4, b, in, st));
    else
        PBF_CUDA(s, cudaMemsetAsync(t->XB, 0, b, st));
    if (dL_dv4)
        PBF_CUDA(s, cudaMemcpyAsync(t->VB, dL_dv4, b, in, st));
    else
        PBF_CUDA(s, cudaMemsetAsync(t->VB, 0, b, st));
    PBF_CUDA(s, cudaMemsetAsync(t->acc, 0, sizeof(double) * kParams * n, st));
    PBF_CUDA(s, cudaMemsetAsync(t->VCB, 0, b, st));
    PBF_CUDA(s, cudaMemsetAsync(t->PA, 0, b, st));
    t->warp_above = s->tuning.adjoint_warp_candidates ? s->tuning.adjoint_warp_candidates
                                                      : kAdjWarpAbove;
    const uint32_t nseg = (t->substeps + t->every - 1) / t->every;
    for (int seg = (int)nseg - 1; seg >= 0; --seg) {
        const uint32_t t0 = (uint32_t)seg * t->every;
        const uint32_t cnt = std::min(t->every, t->substeps - t0);
        PBF_CUDA(s, cudaMemcpyAsync(s->x, t->ckpt_x[seg], b, cudaMemcpyDeviceToDevice, st));
        PBF_CUDA(s, cudaMemcpyAsync(s->v, t->ckpt_v[seg], b, cudaMemcpyDeviceToDevice, st));
        PBF_CUDA(s, record_segment(s, t, cnt));
        for (int k = (int)cnt - 1; k >= 0; --k) PBF_CUDA(s, reverse_dispatch(s, t, t->slots[k]));
    }
    // the handle's state returns to the end of the recorded run
    PBF_CUDA(s, cudaMemcpyAsync(s->x, t->final_x, b, cudaMemcpyDeviceToDevice, st));
    PBF_CUDA(s, cudaMemcpyAsync(s->v, t->final_v, b, cudaMemcpyDeviceToDevice, st));
    if (dL_dx0_4) PBF_CUDA(s, cudaMemcpyAsync(dL_dx0_4, t->XB, b, out, st));
    if (dL_dv0_4) PBF_CUDA(s, cudaMemcpyAsync(dL_dv0_4, t->VB, b, out, st));
    pbf_status r = check_status(s);
    if (r != PBF_OK) return r;
    if (grads) {
        std::vector<double> acc((size_t)kParams * n);
        PBF_CUDA(s, cudaMemcpy(acc.data(), t->acc, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost));
        for (uint32_t sc = 0; sc < s->nscenes; ++sc) {
            double sum[kParams] = {0, 0, 0, 0};
            for (int p = 0; p < kParams; ++p)
                for (uint32_t i = s->offsets[sc]; i < s->offsets[sc + 1]; ++i) sum[p] += acc[p * n + i];
            grads[sc].epsilon = sum[0];
            grads[sc].tensile_instability_k = sum[1];
            grads[sc].xsph_viscosity_c = sum[2];
            grads[sc].vorticity_epsilon = sum[3];
        }
    }
    return PBF_OK;
}

pbf_status pbf_release_record(pbf_sim* s) {
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    DeviceGuard dg(s->device);
    PBF_CUDA(s, cudaStreamSynchronize(s->stream));
    free_tape(s);
    return PBF_OK;
}

}  // extern "C"
