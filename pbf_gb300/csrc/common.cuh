// common.cuh — shared device definitions of the GB300 PBF substep library.
//
// Every floating-point operation on the physics path goes through the
// explicitly rounded intrinsics below (one IEEE-754 binary32 rounding per
// operation, fused multiply-add only where written).  Together with a
// neighbour visit order equal to the reference's FOR_EACH_NEIGHBOUR
// (shaders/sph/foreachneighbour.glsl:1-10) this makes every substep
// reproducible bit for bit on any IEEE-754 machine that evaluates the same
// sequence.  The library is built with -fmad=false as a second guard.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pbf {

constexpr int kBlock = 256;

// Device status word bits (mirrors PBF_DEV_* in include/pbf.h).
constexpr uint32_t kDevNonFinite = 0x1u;
constexpr uint32_t kDevSortTimeout = 0x2u;
constexpr uint32_t kDevRunOver127 = 0x4u;
constexpr uint32_t kDevIndexFault = 0x8u;  // a bounds check of the -DPBF_CHECK build failed

// Per-handle constants, folded on the host from pbf_params.
struct DevConsts {
    float h, h2;
    float r2cut;      // largest float r2 with sqrtf(r2) <= h: (r2 > r2cut) == (sqrtf(r2) > h)
    float k6;         // 1.56668147106 / h^9            (calclambda.glsl:41-47)
    float kg;         // -3 * 4.774648292756860 / h^6   (calclambda.glsl:57-64)
    float kg_lambda;  // kg * one_over_rho_0           (calclambda.glsl:86-87)
    float oorho, eps, scale, negk, cx, dt, gdt, g2dt, dteps;
    float lo[3], hi[3];
    float G[3];       // GRID_SIZE as floats (the clamp bound of GetHash)
    float half_gz;    // GRID_SIZE.z / 2 (predictpos.glsl:27)
    uint32_t Gi[3];
    uint32_t GxGz;    // hash weight of y (src/SPH.cpp:31)
    uint32_t ncells;
    uint32_t cell_base;  // first global cell index of this scene (0 for a single scene)
    uint32_t ext_force;
    // neighbour lists (a tuning choice: results are identical with or without)
    uint32_t use_lists;
    float skin;          // list radius is h + skin
    float r2list;        // inclusion threshold on |d|^2 at the predicted positions
    float margin_h;      // fixed part of the guard's rounding margin
    float wall_abs_max;  // largest |wall| coordinate (positions are clamped inside)
    // bounds checks of the -DPBF_CHECK build: the handle's status word and
    // its particle count (all scenes)
    uint32_t* check_status;
    uint32_t n_total;
};

// Index check of the bounds-checked build (-DPBF_CHECK): a failed check sets
// kDevIndexFault in the handle's status word and the caller skips the access
// (the next synchronising call reports PBF_ERR_DEVICE_FAULT).  In the normal
// build the check is compiled out.
#ifdef PBF_CHECK
__device__ __forceinline__ bool check_ok(const DevConsts& c, bool ok) {
    if (!ok) atomicOr(c.check_status, kDevIndexFault);
    return ok;
}
#else
__device__ __forceinline__ constexpr bool check_ok(const DevConsts&, bool) { return true; }
#endif

// Order-preserving neighbour lists of one substep.  idx is [cap][n] (entry k
// of particle i at idx[k * n + i], coalesced across a warp); cnt[i] = -1
// marks a particle whose list overflowed (it always scans its full stencil).
// guard[0] holds the largest coordinate magnitude of the predicted positions,
// guard[1 + k] the largest displacement from them after delta-p iteration k
// (both as float bits).
struct NbrLists {
    uint32_t* idx;
    int32_t* cnt;
    uint32_t* guard;
    uint32_t cap;
    uint32_t n;
};

// Exact pair lists: the candidates within h of each particle (r2 not above
// r2cut, NaN included) at one set of positions, in visit order, recorded by
// the sweep that first reads those positions (lambda, vorticity pass A) and
// replayed by the next sweep over the same positions (delta-p, vorticity
// pass B).  SoA [cap][n]; cnt -1 when a list overflowed; cap 0 = off.
struct PairLists {
    uint32_t* idx;
    int32_t* cnt;
    uint32_t cap;
    uint32_t n;
    const uint8_t* heavy = nullptr;  // mixed sweeps: particles the cooperative kernels take
    const uint32_t* heavy_list = nullptr;   // their sorted indices
    const uint32_t* heavy_count = nullptr;  // and how many there are
    // run-start bits of the sweep's position set (neighbours.cuh: runs), read
    // by the direct sweeps' coincident runs; NULL: no run path
    const uint32_t* runs = nullptr;
};

// Scan copy of a sorted position array, read by the masked stencil scans two
// candidates at a time with packed (float2) arithmetic: x and y of the
// particle pair (2q, 2q+1) interleaved in xy[q] = (x0, x1, y0, y1), z as a
// plain array read as the float2 z[q] = (z0, z1).  (n + 1) / 2 entries each.
struct ScanPos {
    float4* xy;
    float2* z;
};

__device__ __forceinline__ void scanpos_store(const ScanPos& sp, uint32_t i, float x, float y,
                                              float z) {
    float* xy = reinterpret_cast<float*>(sp.xy) + 4 * (size_t)(i >> 1) + (i & 1u);
    xy[0] = x;
    xy[2] = y;
    reinterpret_cast<float*>(sp.z)[i] = z;
}

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

__device__ __forceinline__ float3 sub3(float3 a, float3 b) {
    return make_float3(fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z));
}
__device__ __forceinline__ float3 add3(float3 a, float3 b) {
    return make_float3(fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z));
}
__device__ __forceinline__ float3 scale3(float3 a, float s) {
    return make_float3(fmul(a.x, s), fmul(a.y, s), fmul(a.z, s));
}
// dot(a, b) = fma(az, bz, fma(ay, by, ax * bx))
__device__ __forceinline__ float dot3(float3 a, float3 b) {
    return ffma(a.z, b.z, ffma(a.y, b.y, fmul(a.x, b.x)));
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(ffma(a.y, b.z, -fmul(a.z, b.y)), ffma(a.z, b.x, -fmul(a.x, b.z)),
                       ffma(a.x, b.y, -fmul(a.y, b.x)));
}
// acc + s * a, fused per component
__device__ __forceinline__ float3 fma3(float s, float3 a, float3 acc) {
    return make_float3(ffma(s, a.x, acc.x), ffma(s, a.y, acc.y), ffma(s, a.z, acc.z));
}
__device__ __forceinline__ float3 xyz(float4 a) { return make_float3(a.x, a.y, a.z); }

// Wpoly6 for len <= h: k6 * (h^2 - len^2)^3, t = fma(-len, len, h^2).
__device__ __forceinline__ float w_poly6(const DevConsts& c, float len) {
    float t = ffma(-len, len, c.h2);
    return fmul(fmul(fmul(t, t), t), c.k6);
}
// gradWspiky(d) = d * s for 0 < len <= h, s = ((k * u) * u) / len, u = h - len.
__device__ __forceinline__ float grad_scale(float k, float h, float len) {
    float u = fsub(h, len);
    return fdiv(fmul(fmul(k, u), u), len);
}

// int(clamp(x, 0, G)) as GetHash computes it (shaders/radixsort/counting.glsl:55),
// capped at G - 1 so every position owns a valid cell; NaN maps to 0.
__device__ __forceinline__ uint32_t cell_coord(float x, float G, uint32_t Gi) {
    float c = (x >= 0.0f) ? x : 0.0f;
    c = (c <= G) ? c : G;
    uint32_t ic = __float2uint_rz(c);
    return ic < Gi ? ic : Gi - 1u;
}
// key = cx + cy * Gx*Gz + cz * Gx (GRID_HASHWEIGHTS, src/SPH.cpp:31)
__device__ __forceinline__ uint32_t cell_key(float3 q, const DevConsts& c) {
    uint32_t cx = cell_coord(q.x, c.G[0], c.Gi[0]);
    uint32_t cy = cell_coord(q.y, c.G[1], c.Gi[1]);
    uint32_t cz = cell_coord(q.z, c.G[2], c.Gi[2]);
    return c.cell_base + cx + cy * c.GxGz + cz * c.Gi[0];
}

// Where a kernel finds the constants of particle i.  One scene: the kernel
// parameter itself (constant bank, no load).  Several scenes: the particle's
// scene id indexes a device table of per-scene constants.
struct OneScene {
    DevConsts c;
    __device__ __forceinline__ const DevConsts& at(uint32_t) const { return c; }
};
struct ManyScenes {
    const DevConsts* __restrict__ cs;
    const uint32_t* __restrict__ sid;  // scene of each particle (id or sorted order)
    __device__ __forceinline__ const DevConsts& at(uint32_t i) const { return cs[__ldg(sid + i)]; }
};

__device__ __forceinline__ bool finite3(float3 a) {
    return isfinite(a.x) && isfinite(a.y) && isfinite(a.z);
}

inline unsigned grid_for(uint32_t n, int block = kBlock) {
    return (unsigned)((n + (uint32_t)block - 1u) / (uint32_t)block);
}

}  // namespace pbf
