// pbf_oracle.hpp — CPU restatement of pbf's per-substep simulation path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA library is
// checked against and the timed CPU baseline; nothing in the product
// (pbf_gb300/) includes, links or calls it.
//
// It transcribes the reference's GLSL compute shaders stage by stage:
//   predict            shaders/sph/predictpos.glsl:18-38
//   cell key           shaders/radixsort/counting.glsl:53-57 (GetHash)
//   stable sort        src/RadixSort.cpp:24-30,44,124-133 (LSD, ties in id order)
//   cell ranges        shaders/neighbourcellfinder/findcells.glsl:34-53
//   neighbour runs     shaders/neighbourcellfinder/neighbourcells.glsl:37-90
//   neighbour loop     shaders/sph/foreachneighbour.glsl:1-10 (order, self skip)
//   lambda             shaders/sph/calclambda.glsl:41-102
//   delta-p + walls    shaders/sph/updatepos.glsl:17-104
//   commit             shaders/sph/update.glsl:16-28
//   XSPH + vorticity   shaders/sph/vorticity.glsl:17-85
//   constants          src/SPH.cpp:28-60,136-144,159-164
// in FP32 (T = float) and as an FP64 twin (T = double) from one template.
//
// Decisions on the reference's undefined or buggy behaviour:
//   Q1  h is a parameter; the stencil is the 27 cells around the particle's
//       cell as in the reference, so h <= 1 makes it complete.
//   Q2  key cell coordinate = min(int(clamp(x, 0, G)), G - 1) per axis, so
//       every position has a valid cell; the stencil centre is the reference's
//       unclamped int(x) (neighbourcells.glsl:57), see stencil_coord.
//   Q3  start[cell(x_0)] = 0 and end[cell(x_{N-1})] = N; empty cells -1.
//   Q4  stencil cells outside the grid are empty.
//   Q5  Jacobi everywhere: each stage reads only the previous stage's output.
//   Q6  XSPH runs together with vorticity confinement, under the same flag.
//   Q7  neighbour runs keep full 32-bit start/count (no 8-bit packing).
//   Q8  any particle count.
//   Q9  the self term stays excluded from rho.
//   Q10 one IEEE-754 rounding per operation, in the order written below,
//       with std::fma exactly where the code says fma (GLSL lets a compiler
//       contract a*b+c; the choice is pinned here so that a CUDA build can
//       reproduce it bit for bit).  Constant factors that depend only on the
//       parameters are folded in double on the host and rounded once.
//
// Compile with -ffp-contract=off and without -ffast-math.
#pragma once

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace pbfo {

// Unqualified fma / sqrt below resolve to these for float and double, and by
// argument-dependent lookup to the dual-number overloads of pbf_dual.hpp.
using std::fma;
using std::sqrt;

// Same layout as pbf_params in include/pbf.h (checked by the tests).
struct Params {
    float one_over_rho_0;
    float epsilon;
    float gravity;
    float timestep;
    float tensile_instability_k;
    float tensile_instability_scale;
    float xsph_viscosity_c;
    float vorticity_epsilon;
    float h;
    uint32_t num_solver_iterations;
    uint32_t vorticity_confinement;
    uint32_t external_force;
    uint32_t grid[3];
    float wall_lo[3];
    float wall_hi[3];
};

template <typename T>
struct V3 {
    T x, y, z;
};

template <typename T>
static inline V3<T> sub3(V3<T> a, V3<T> b) {
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename T>
static inline V3<T> add3(V3<T> a, V3<T> b) {
    return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename T>
static inline V3<T> scale3(V3<T> a, T s) {
    return {a.x * s, a.y * s, a.z * s};
}
// dot(a, b) = fma(az, bz, fma(ay, by, ax * bx))
template <typename T>
static inline T dot3(V3<T> a, V3<T> b) {
    return fma(a.z, b.z, fma(a.y, b.y, a.x * b.x));
}
// cross(a, b) with one fused multiply-add per component
template <typename T>
static inline V3<T> cross3(V3<T> a, V3<T> b) {
    return {fma(a.y, b.z, -(a.z * b.y)), fma(a.z, b.x, -(a.x * b.z)),
            fma(a.x, b.y, -(a.y * b.x))};
}
// acc + s * a, fused per component
template <typename T>
static inline V3<T> fma3(T s, V3<T> a, V3<T> acc) {
    return {fma(s, a.x, acc.x), fma(s, a.y, acc.y), fma(s, a.z, acc.z)};
}

// Poly6 normalisation 315/(64 pi) and spiky normalisation 15/pi as the
// shaders write them (calclambda.glsl:46,54).
static constexpr double kPoly6 = 1.56668147106;
static constexpr double kSpiky = 4.774648292756860;

template <typename T>
struct Consts {
    T h, h2;
    T k6;         // 1.56668147106 / h^9        (Wpoly6, calclambda.glsl:41-47)
    T kg;         // -3 * 4.774648292756860 / h^6  (gradWspiky, calclambda.glsl:57-64)
    T kg_lambda;  // kg * one_over_rho_0           (calclambda.glsl:86-87)
    T oorho, eps, scale, negk, cx, dt, gdt, g2dt, dteps;
    T lo[3], hi[3];
    T G[3];       // grid extents as reals (the clamp bound GRID_SIZE)
    T half_gz;    // GRID_SIZE.z / 2 (predictpos.glsl:27)
};

template <typename T>
static Consts<T> make_consts(const Params& p) {
    Consts<T> c{};
    const double hd = (double)p.h;
    double h6 = 1.0, h9 = 1.0;
    for (int i = 0; i < 6; ++i) h6 *= hd;
    for (int i = 0; i < 9; ++i) h9 *= hd;
    c.h = (T)p.h;
    c.h2 = (T)(hd * hd);
    c.k6 = (T)(kPoly6 / h9);
    c.kg = (T)(-3.0 * kSpiky / h6);
    c.kg_lambda = (T)((-3.0 * kSpiky / h6) * (double)p.one_over_rho_0);
    c.oorho = (T)p.one_over_rho_0;
    c.eps = (T)p.epsilon;
    c.scale = (T)p.tensile_instability_scale;
    c.negk = -(T)p.tensile_instability_k;
    c.cx = (T)p.xsph_viscosity_c;
    c.dt = (T)p.timestep;
    c.gdt = (T)p.gravity * (T)p.timestep;               // gravity * timestep
    c.g2dt = ((T)2 * (T)p.gravity) * (T)p.timestep;      // 2 * gravity * timestep
    c.dteps = (T)p.timestep * (T)p.vorticity_epsilon;   // timestep * vorticity_epsilon
    for (int a = 0; a < 3; ++a) {
        c.lo[a] = (T)p.wall_lo[a];
        c.hi[a] = (T)p.wall_hi[a];
        c.G[a] = (T)p.grid[a];
    }
    c.half_gz = (T)p.grid[2] / (T)2;
    return c;
}

// Cell coordinate along one axis: int(clamp(x, 0, G)) as GetHash computes it
// (counting.glsl:55), capped at G - 1 (decision Q2).  NaN maps to 0.
template <typename T>
static inline uint32_t cell_coord(T x, T G, uint32_t Gi) {
    T c = (x >= (T)0) ? x : (T)0;
    c = (c <= G) ? c : G;
    uint32_t ic = (uint32_t)c;
    return ic < Gi ? ic : Gi - 1;
}

// Stencil centre along one axis: ivec3(particlekeys[i].xyz) of
// neighbourcells.glsl:57, the predicted coordinate truncated toward zero with
// no clamp, so a particle predicted outside the grid looks for neighbours
// around that outside cell (rows and cells outside the grid are empty,
// decision Q4).  Saturated to [-2, G + 1], which leaves the runs unchanged
// (every row of a centre beyond that lies outside the grid); NaN maps to 0.
template <typename T>
static inline int stencil_coord(T x, uint32_t Gi) {
    if (!(x == x)) return 0;
    if (x <= (T)-2) return -2;
    if (x >= (T)Gi + (T)1) return (int)Gi + 1;
    return (int)x;
}

// min(max(q, lo), hi) (updatepos.glsl:100)
static inline float clamp_wall(float q, float lo, float hi) { return std::min(std::max(q, lo), hi); }
static inline double clamp_wall(double q, double lo, double hi) { return std::min(std::max(q, lo), hi); }

// Wpoly6 for len <= h: k6 * ((h^2 - len^2)^3)  with t = fma(-len, len, h^2).
template <typename T>
static inline T w_poly6(const Consts<T>& c, T len) {
    T t = fma(-len, len, c.h2);
    return ((t * t) * t) * c.k6;
}

// Scalar s with gradWspiky(d) = d * s for 0 < len <= h:
// s = ((k * u) * u) / len, u = h - len.
template <typename T>
static inline T grad_scale(T k, T h, T len) {
    T u = h - len;
    return ((k * u) * u) / len;
}

template <typename T>
struct Sim {
    Params p{};
    Consts<T> c{};
    uint32_t n = 0;
    uint32_t ncells = 0;
    int nthreads = 0;

    // state, id order
    std::vector<V3<T>> x, v;

    // intermediates of the last substep
    std::vector<V3<T>> xstar;           // predicted positions, id order
    std::vector<uint32_t> key_by_id;    // cell key, id order
    std::vector<uint32_t> sorted_keys;  // sorted keys
    std::vector<uint32_t> perm;         // perm[i] = id of sorted particle i
    std::vector<int32_t> cstart, cend;  // dense cell tables
    std::vector<V3<T>> xpred;           // predicted positions, sorted order
    std::vector<V3<T>> pa, pb;          // Jacobi position buffers, sorted order
    std::vector<T> lambda;              // sorted order
    std::vector<V3<T>> vs;              // committed velocity, sorted order
    std::vector<V3<T>> vx;              // after XSPH, sorted order
    std::vector<V3<T>> om;              // vorticity vector, sorted order
    std::vector<T> omag;                // |vorticity|, sorted order
    double candidate_pairs = 0;

    std::vector<uint32_t> tmpk, tmpv;

    void init(const Params& prm, uint32_t count) {
        p = prm;
        c = make_consts<T>(p);
        n = count;
        ncells = p.grid[0] * p.grid[1] * p.grid[2];
        x.assign(n, V3<T>{0, 0, 0});
        v.assign(n, V3<T>{0, 0, 0});
        xstar.resize(n);
        key_by_id.resize(n);
        sorted_keys.resize(n);
        perm.resize(n);
        cstart.assign(ncells, -1);
        cend.assign(ncells, -1);
        xpred.resize(n);
        pa.resize(n);
        pb.resize(n);
        lambda.resize(n);
        vs.resize(n);
        vx.resize(n);
        om.resize(n);
        omag.resize(n);
        tmpk.resize(n);
        tmpv.resize(n);
    }

    void set_params(const Params& prm) {
        p = prm;
        c = make_consts<T>(p);
    }

    int threads() const {
#ifdef _OPENMP
        return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
        return 1;
#endif
    }

    uint32_t key_of(V3<T> q) const {
        uint32_t cx = cell_coord<T>(q.x, c.G[0], p.grid[0]);
        uint32_t cy = cell_coord<T>(q.y, c.G[1], p.grid[1]);
        uint32_t cz = cell_coord<T>(q.z, c.G[2], p.grid[2]);
        // GRID_HASHWEIGHTS = (1, Gx*Gz, Gx)  (src/SPH.cpp:31)
        return cx + cy * (p.grid[0] * p.grid[2]) + cz * p.grid[0];
    }

    // predictpos.glsl:18-38 + GetHash (counting.glsl:53-57)
    void predict() {
        const int nt = threads();
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t id = 0; id < (int64_t)n; ++id) {
            V3<T> q = x[id];
            V3<T> w = v[id];
            if (p.external_force && q.z > c.half_gz) w.z = w.z - c.g2dt;  // :27-28
            w.y = w.y - c.gdt;                                              // :32
            q = {q.x + c.dt * w.x, q.y + c.dt * w.y, q.z + c.dt * w.z};    // :34
            xstar[id] = q;
            key_by_id[id] = key_of(q);
        }
    }

    // Stable LSD radix sort of (key, id), 8-bit digits, per-thread histograms.
    // RadixSort sorts 2 bits per pass over ceil(numbits/2) passes
    // (src/RadixSort.cpp:124-133); any stable LSD sort over the same bits
    // gives the same order: ascending key, ties in id order.
    void sort() {
        uint64_t span = (uint64_t)ncells - 1;
        unsigned numbits = 1;
        while (span >>= 1) numbits++;  // count_sortbits (src/RadixSort.cpp:24-30)
        const unsigned passes = (numbits + 7) / 8;
        std::vector<uint32_t>& k0 = sorted_keys;
        std::vector<uint32_t>& v0 = perm;
        for (uint32_t i = 0; i < n; ++i) {
            k0[i] = key_by_id[i];
            v0[i] = i;
        }
        uint32_t* ks = k0.data();
        uint32_t* vsrc = v0.data();
        uint32_t* kd = tmpk.data();
        uint32_t* vd = tmpv.data();
        const int nt = threads();
        std::vector<uint32_t> hist((size_t)nt * 256);
        for (unsigned pass = 0; pass < passes; ++pass) {
            const unsigned shift = 8 * pass;
            std::fill(hist.begin(), hist.end(), 0u);
#pragma omp parallel num_threads(nt)
            {
#ifdef _OPENMP
                const int t = omp_get_thread_num();
#else
                const int t = 0;
#endif
                const uint64_t lo = (uint64_t)n * t / nt, hi = (uint64_t)n * (t + 1) / nt;
                uint32_t* hst = &hist[(size_t)t * 256];
                for (uint64_t i = lo; i < hi; ++i) hst[(ks[i] >> shift) & 255u]++;
#pragma omp barrier
#pragma omp single
                {
                    uint32_t run = 0;
                    for (unsigned d = 0; d < 256; ++d)
                        for (int tt = 0; tt < nt; ++tt) {
                            uint32_t cnt = hist[(size_t)tt * 256 + d];
                            hist[(size_t)tt * 256 + d] = run;
                            run += cnt;
                        }
                }
                for (uint64_t i = lo; i < hi; ++i) {
                    uint32_t d = (ks[i] >> shift) & 255u;
                    uint32_t o = hst[d]++;
                    kd[o] = ks[i];
                    vd[o] = vsrc[i];
                }
            }
            std::swap(ks, kd);
            std::swap(vsrc, vd);
        }
        if (ks != k0.data()) {
            std::memcpy(k0.data(), ks, sizeof(uint32_t) * n);
            std::memcpy(v0.data(), vsrc, sizeof(uint32_t) * n);
        }
    }

    // findcells.glsl:34-53 with decision Q3, then the sorted positions.
    void find_cells() {
        std::fill(cstart.begin(), cstart.end(), -1);
        std::fill(cend.begin(), cend.end(), -1);
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t k = sorted_keys[i];
            if (i == 0 || sorted_keys[i - 1] != k) cstart[k] = (int32_t)i;
            if (i + 1 == n || sorted_keys[i + 1] != k) cend[k] = (int32_t)(i + 1);
        }
        const int nt = threads();
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t i = 0; i < (int64_t)n; ++i) xpred[i] = xstar[perm[i]];
    }

    // neighbourcells.glsl:52-90: the 9 (y, z) rows in the order of
    // gridoffsets (:37-47), each an x-run of up to 3 cells.  run_begin/end
    // receive sorted-index ranges; returns the number of runs (always 9,
    // empty runs have begin == end).
    void runs_of(uint32_t i, int32_t rb[9], int32_t re[9]) const {
        const uint32_t Gx = p.grid[0], Gy = p.grid[1], Gz = p.grid[2];
        const int cx = stencil_coord<T>(xpred[i].x, Gx);
        const int cy = stencil_coord<T>(xpred[i].y, Gy);
        const int cz = stencil_coord<T>(xpred[i].z, Gz);
        int o = 0;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz, ++o) {
                rb[o] = 0;
                re[o] = 0;
                const int ny = cy + dy, nz = cz + dz;
                if (ny < 0 || ny >= (int)Gy || nz < 0 || nz >= (int)Gz) continue;  // Q4
                const uint32_t base = (uint32_t)ny * (Gx * Gz) + (uint32_t)nz * Gx;
                const int xlo = cx > 0 ? cx - 1 : 0;
                const int xhi = cx + 1 < (int)Gx ? cx + 1 : (int)Gx - 1;
                int32_t first = -1, last = -1;
                for (int xx = xlo; xx <= xhi; ++xx) {
                    int32_t s = cstart[base + (uint32_t)xx];
                    if (s != -1) {
                        if (first == -1) first = s;
                        last = cend[base + (uint32_t)xx];
                    }
                }
                if (first != -1) {
                    rb[o] = first;
                    re[o] = last;
                }
            }
    }

    // FOR_EACH_NEIGHBOUR (foreachneighbour.glsl:1-10): runs in order, j
    // ascending inside a run, j == i skipped.
    template <class F>
    inline void for_each_neighbour(uint32_t i, F&& f) const {
        int32_t rb[9], re[9];
        runs_of(i, rb, re);
        for (int o = 0; o < 9; ++o)
            for (int32_t j = rb[o]; j < re[o]; ++j)
                if ((uint32_t)j != i) f((uint32_t)j);
    }

    // calclambda.glsl:66-102, reading positions `P`, for sorted [lo, hi).
    void calc_lambda(const std::vector<V3<T>>& P, int64_t lo = 0, int64_t hi = -1) {
        const int nt = threads();
        if (hi < 0) hi = n;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
        for (int64_t ii = lo; ii < hi; ++ii) {
            const uint32_t i = (uint32_t)ii;
            const V3<T> pi = P[i];
            T rho = 0, sumk = 0;
            V3<T> gi{0, 0, 0};
            for_each_neighbour(i, [&](uint32_t j) {
                const V3<T> d = sub3(pi, P[j]);
                const T len = sqrt(dot3(d, d));
                if (len > c.h) return;           // Wpoly6 and gradWspiky are 0
                rho = rho + w_poly6(c, len);     // :80-82
                if (len == (T)0) return;         // gradWspiky(0) = 0 (:60)
                const V3<T> g = scale3(d, grad_scale(c.kg_lambda, c.h, len));  // :86-87
                sumk = sumk + dot3(g, g);        // :89
                gi = add3(gi, g);                // :93
            });
            sumk = sumk + dot3(gi, gi);                  // :97
            const T Ci = fma(rho, c.oorho, (T)-1);  // :100
            lambda[i] = -Ci / (sumk + c.eps);            // :101
        }
    }

    // updatepos.glsl:42-104, reading `P` and lambda, writing `Q`, for sorted [lo, hi).
    void update_pos(const std::vector<V3<T>>& P, std::vector<V3<T>>& Q, int64_t lo = 0,
                    int64_t hi = -1) {
        const int nt = threads();
        if (hi < 0) hi = n;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
        for (int64_t ii = lo; ii < hi; ++ii) {
            const uint32_t i = (uint32_t)ii;
            const V3<T> pi = P[i];
            const T li = lambda[i];
            V3<T> dp{0, 0, 0};
            for_each_neighbour(i, [&](uint32_t j) {
                const V3<T> d = sub3(pi, P[j]);
                const T len = sqrt(dot3(d, d));
                if (len > c.h || len == (T)0) return;  // gradWspiky = 0
                T sc = c.scale * w_poly6(c, len);      // :57
                sc = sc * sc;                          // :58
                sc = sc * sc;                          // :59
                sc = c.negk * sc;                      // :60
                const T coef = (li + lambda[j]) + sc;  // :65
                const V3<T> g = scale3(d, grad_scale(c.kg, c.h, len));
                dp = fma3(coef, g, dp);                // :65
            });
            V3<T> q = fma3(c.oorho, dp, pi);  // :85
            // clamp (:100)
            q.x = clamp_wall(q.x, c.lo[0], c.hi[0]);
            q.y = clamp_wall(q.y, c.lo[1], c.hi[1]);
            q.z = clamp_wall(q.z, c.lo[2], c.hi[2]);
            Q[i] = q;
        }
    }

    // update.glsl:16-28: velocity from the displacement, back to id order.
    void commit(const std::vector<V3<T>>& P, int64_t lo = 0, int64_t hi = -1) {
        const int nt = threads();
        if (hi < 0) hi = n;
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t ii = lo; ii < hi; ++ii) {
            const uint32_t id = perm[ii];
            const V3<T> q = P[ii];
            const V3<T> xo = x[id];
            vs[ii] = {(q.x - xo.x) / c.dt, (q.y - xo.y) / c.dt, (q.z - xo.z) / c.dt};  // :23
            x[id] = q;                                                                // :26
        }
    }

    // vorticity.glsl:34-60 (pass A, XSPH + vorticity vector) and :65-85
    // (pass B, confinement), Jacobi between and within the passes.
    void vorticity(const std::vector<V3<T>>& P, int64_t lo = 0, int64_t hi = -1) {
        const int nt = threads();
        if (hi < 0) hi = n;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
        for (int64_t ii = lo; ii < hi; ++ii) {
            const uint32_t i = (uint32_t)ii;
            const V3<T> pi = P[i];
            const V3<T> vi = vs[i];
            V3<T> acc{0, 0, 0}, w{0, 0, 0};
            for_each_neighbour(i, [&](uint32_t j) {
                const V3<T> vij = sub3(vs[j], vi);  // :50
                const V3<T> d = sub3(pi, P[j]);     // :51
                const T len = sqrt(dot3(d, d));
                if (len > c.h) return;
                const T wp = w_poly6(c, len);  // :52
                acc = fma3(wp, vij, acc);      // :54
                if (len == (T)0) return;
                const V3<T> g = scale3(d, grad_scale(c.kg, c.h, len));
                w = add3(w, cross3(vij, g));  // :55
            });
            vx[i] = fma3(c.cx, acc, vi);         // :58
            om[i] = w;
            omag[i] = sqrt(dot3(w, w));     // :60
        }
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
        for (int64_t ii = lo; ii < hi; ++ii) {
            const uint32_t i = (uint32_t)ii;
            const V3<T> pi = P[i];
            V3<T> eta{0, 0, 0};
            for_each_neighbour(i, [&](uint32_t j) {
                const V3<T> d = sub3(pi, P[j]);  // :69
                const T len = sqrt(dot3(d, d));
                if (len > c.h || len == (T)0) return;
                const V3<T> g = scale3(d, grad_scale(c.kg, c.h, len));
                eta = fma3(omag[j], g, eta);  // :72
            });
            const T l = sqrt(dot3(eta, eta));  // :76
            if (l > (T)0) eta = {eta.x / l, eta.y / l, eta.z / l};  // :77-78
            v[perm[i]] = fma3(c.dteps, cross3(eta, om[i]), vx[i]);  // :82,85
        }
    }

    void count_candidates() {
        double total = 0;
        const int nt = threads();
#pragma omp parallel for schedule(static) reduction(+ : total) num_threads(nt)
        for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
            int32_t rb[9], re[9];
            runs_of((uint32_t)ii, rb, re);
            int64_t s = 0;
            for (int o = 0; o < 9; ++o) s += re[o] - rb[o];
            total += (double)(s - 1);
        }
        candidate_pairs = total;
    }

    // SPH::Run (src/SPH.cpp:246-334).
    void substep() {
        if (n == 0) return;
        predict();
        sort();
        find_cells();
        pa = xpred;
        std::vector<V3<T>>* cur = &pa;
        std::vector<V3<T>>* nxt = &pb;
        for (uint32_t it = 0; it < p.num_solver_iterations; ++it) {
            calc_lambda(*cur);
            update_pos(*cur, *nxt);
            std::swap(cur, nxt);
        }
        commit(*cur);
        if (p.vorticity_confinement) {
            vorticity(*cur);
        } else {
            const int nt = threads();
#pragma omp parallel for schedule(static) num_threads(nt)
            for (int64_t ii = 0; ii < (int64_t)n; ++ii) v[perm[ii]] = vs[ii];
        }
        if (cur != &pa) pa = *cur;  // pa holds the final sorted positions
    }

    // A bounded timing sample of one substep: predict, sort and cell ranges
    // over all n particles, then the solver, commit and vorticity stages over
    // the sorted slice [lo, hi) only.  Returns the seconds of the two parts.
    // For timing only: particles outside the slice keep stale solver data.
    void sample_substep(int64_t lo, int64_t hi, double* t_full, double* t_slice) {
        auto t0 = std::chrono::steady_clock::now();
        predict();
        sort();
        find_cells();
        auto t1 = std::chrono::steady_clock::now();
        std::copy(xpred.begin() + lo, xpred.begin() + hi, pa.begin() + lo);
        std::vector<V3<T>>* cur = &pa;
        std::vector<V3<T>>* nxt = &pb;
        for (uint32_t it = 0; it < p.num_solver_iterations; ++it) {
            calc_lambda(*cur, lo, hi);
            update_pos(*cur, *nxt, lo, hi);
            std::swap(cur, nxt);
        }
        commit(*cur, lo, hi);
        if (p.vorticity_confinement) vorticity(*cur, lo, hi);
        auto t2 = std::chrono::steady_clock::now();
        *t_full = std::chrono::duration<double>(t1 - t0).count();
        *t_slice = std::chrono::duration<double>(t2 - t1).count();
    }

    // Density error and kinetic energy of the current state, with a fresh
    // key sort of the current positions.
    void diagnostics(double* mean_err, double* max_err, double* ke, double* cand) {
        if (n == 0) {
            *mean_err = *max_err = *ke = *cand = 0;
            return;
        }
        // keys from current positions
        const int nt = threads();
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t id = 0; id < (int64_t)n; ++id) {
            xstar[id] = x[id];
            key_by_id[id] = key_of(x[id]);
        }
        sort();
        find_cells();
        count_candidates();
        double se = 0, me = 0, k = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : se, k) reduction(max : me) num_threads(nt)
        for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
            const uint32_t i = (uint32_t)ii;
            const V3<T> pi = xpred[i];
            T rho = 0;
            for_each_neighbour(i, [&](uint32_t j) {
                const V3<T> d = sub3(pi, xpred[j]);
                const T len = sqrt(dot3(d, d));
                if (len > c.h) return;
                rho = rho + w_poly6(c, len);
            });
            double e = std::fabs((double)rho * (double)c.oorho - 1.0);
            se += e;
            me = std::max(me, e);
            const V3<T> w = v[perm[i]];
            k += 0.5 * ((double)w.x * w.x + (double)w.y * w.y + (double)w.z * w.z);
        }
        *mean_err = se / n;
        *max_err = me;
        *ke = k;
        *cand = candidate_pairs;
    }
};

}  // namespace pbfo
