// pbf_oracle.cpp — C entry points of the CPU oracle (test infrastructure).
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py, never by the product library.  The FP32
// instance follows the reference shaders as restated in pbf_oracle.hpp; the
// FP64 instance is the same template in double precision.
#include "pbf_oracle.hpp"

#include <chrono>

using pbfo::Params;
using pbfo::Sim;
using pbfo::V3;

namespace {

struct Handle {
    int fp64 = 0;
    Sim<float> f;
    Sim<double> d;
};

template <typename T>
void set_state(Sim<T>& s, const float* x4, const float* v4) {
    for (uint32_t i = 0; i < s.n; ++i) {
        s.x[i] = {(T)x4[4 * i], (T)x4[4 * i + 1], (T)x4[4 * i + 2]};
        s.v[i] = {(T)v4[4 * i], (T)v4[4 * i + 1], (T)v4[4 * i + 2]};
    }
}

template <typename T, typename O>
void get3(const std::vector<V3<T>>& a, O* out4, uint32_t n) {
    for (uint32_t i = 0; i < n; ++i) {
        out4[4 * i] = (O)a[i].x;
        out4[4 * i + 1] = (O)a[i].y;
        out4[4 * i + 2] = (O)a[i].z;
        out4[4 * i + 3] = 0;
    }
}

}  // namespace

extern "C" {

int pbfo_params_size(void) { return (int)sizeof(Params); }

void* pbfo_create(const Params* p, uint32_t n, int fp64, int nthreads) {
    Handle* h = new Handle();
    h->fp64 = fp64;
    if (fp64) {
        h->d.init(*p, n);
        h->d.nthreads = nthreads;
    } else {
        h->f.init(*p, n);
        h->f.nthreads = nthreads;
    }
    return h;
}

void pbfo_destroy(void* hp) { delete (Handle*)hp; }

void pbfo_set_params(void* hp, const Params* p) {
    Handle* h = (Handle*)hp;
    if (h->fp64)
        h->d.set_params(*p);
    else
        h->f.set_params(*p);
}

void pbfo_set_state(void* hp, const float* x4, const float* v4) {
    Handle* h = (Handle*)hp;
    if (h->fp64)
        set_state(h->d, x4, v4);
    else
        set_state(h->f, x4, v4);
}

// Copies x, v (id order) as float4 (fp32 handle) or double4 (fp64 handle).
void pbfo_get_state(void* hp, void* x4, void* v4) {
    Handle* h = (Handle*)hp;
    if (h->fp64) {
        if (x4) get3(h->d.x, (double*)x4, h->d.n);
        if (v4) get3(h->d.v, (double*)v4, h->d.n);
    } else {
        if (x4) get3(h->f.x, (float*)x4, h->f.n);
        if (v4) get3(h->f.v, (float*)v4, h->f.n);
    }
}

// Runs `substeps` substeps; returns the wall time in seconds.
double pbfo_step(void* hp, uint32_t substeps) {
    Handle* h = (Handle*)hp;
    auto t0 = std::chrono::steady_clock::now();
    for (uint32_t s = 0; s < substeps; ++s) {
        if (h->fp64)
            h->d.substep();
        else
            h->f.substep();
    }
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

// Intermediates of the last substep.  Any pointer may be NULL.  Real-valued
// outputs are float (fp32 handle) or double (fp64 handle).
void pbfo_get_sort(void* hp, uint32_t* keys_by_id, uint32_t* sorted_keys, uint32_t* perm) {
    Handle* h = (Handle*)hp;
    const uint32_t n = h->fp64 ? h->d.n : h->f.n;
    const std::vector<uint32_t>& kb = h->fp64 ? h->d.key_by_id : h->f.key_by_id;
    const std::vector<uint32_t>& sk = h->fp64 ? h->d.sorted_keys : h->f.sorted_keys;
    const std::vector<uint32_t>& pm = h->fp64 ? h->d.perm : h->f.perm;
    if (keys_by_id) std::memcpy(keys_by_id, kb.data(), 4ull * n);
    if (sorted_keys) std::memcpy(sorted_keys, sk.data(), 4ull * n);
    if (perm) std::memcpy(perm, pm.data(), 4ull * n);
}

void pbfo_get_cells(void* hp, int32_t* start, int32_t* end) {
    Handle* h = (Handle*)hp;
    const std::vector<int32_t>& cs = h->fp64 ? h->d.cstart : h->f.cstart;
    const std::vector<int32_t>& ce = h->fp64 ? h->d.cend : h->f.cend;
    if (start) std::memcpy(start, cs.data(), 4ull * cs.size());
    if (end) std::memcpy(end, ce.data(), 4ull * ce.size());
}

void pbfo_get_solver(void* hp, void* lambda_sorted, void* xpred4_sorted) {
    Handle* h = (Handle*)hp;
    if (h->fp64) {
        if (lambda_sorted) std::memcpy(lambda_sorted, h->d.lambda.data(), 8ull * h->d.n);
        if (xpred4_sorted) get3(h->d.xpred, (double*)xpred4_sorted, h->d.n);
    } else {
        if (lambda_sorted) std::memcpy(lambda_sorted, h->f.lambda.data(), 4ull * h->f.n);
        if (xpred4_sorted) get3(h->f.xpred, (float*)xpred4_sorted, h->f.n);
    }
}

// Runs of sorted particle i: 9 (begin, end) pairs into runs[18].
void pbfo_get_runs(void* hp, uint32_t i, int32_t* runs) {
    Handle* h = (Handle*)hp;
    int32_t rb[9], re[9];
    if (h->fp64)
        h->d.runs_of(i, rb, re);
    else
        h->f.runs_of(i, rb, re);
    for (int o = 0; o < 9; ++o) {
        runs[2 * o] = rb[o];
        runs[2 * o + 1] = re[o];
    }
}

// clearhighlight.glsl:7 then highlight.glsl:16-30 over the last substep's
// runs: bit 1 cleared, then set on every stencil candidate (j != i) of a
// particle whose bit 0 is set.  flags[n] in id order.
void pbfo_highlight(void* hp, uint32_t* flags) {
    Handle* h = (Handle*)hp;
    auto run = [&](auto& s) {
        for (uint32_t i = 0; i < s.n; ++i) flags[i] &= 1u;
        for (uint32_t i = 0; i < s.n; ++i)
            if (flags[s.perm[i]] & 1u) s.for_each_neighbour(i, [&](uint32_t j) { flags[s.perm[j]] |= 2u; });
    };
    if (h->fp64)
        run(h->d);
    else
        run(h->f);
}

// The folded constants (k6, kg, kg_lambda, h2) as doubles, for tests.
void pbfo_get_consts(void* hp, double* out4) {
    Handle* h = (Handle*)hp;
    if (h->fp64) {
        out4[0] = h->d.c.k6;
        out4[1] = h->d.c.kg;
        out4[2] = h->d.c.kg_lambda;
        out4[3] = h->d.c.h2;
    } else {
        out4[0] = h->f.c.k6;
        out4[1] = h->f.c.kg;
        out4[2] = h->f.c.kg_lambda;
        out4[3] = h->f.c.h2;
    }
}

// mean |C|, max |C|, kinetic energy, candidate pairs of the current state.
void pbfo_diagnostics(void* hp, double* out4) {
    Handle* h = (Handle*)hp;
    if (h->fp64)
        h->d.diagnostics(&out4[0], &out4[1], &out4[2], &out4[3]);
    else
        h->f.diagnostics(&out4[0], &out4[1], &out4[2], &out4[3]);
}

// Standalone stable sort of arbitrary keys on their low numbits bits
// (same LSD order as the substep's sort), for sort edge-case tests.
void pbfo_radix_sort(const uint32_t* keys, uint32_t n, uint32_t numbits, uint32_t* keys_out,
                     uint32_t* perm_out) {
    const uint32_t mask = numbits >= 32 ? 0xFFFFFFFFu : ((1u << numbits) - 1u);
    std::vector<uint32_t> idx(n);
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(),
                     [&](uint32_t a, uint32_t b) { return (keys[a] & mask) < (keys[b] & mask); });
    for (uint32_t i = 0; i < n; ++i) {
        perm_out[i] = idx[i];
        if (keys_out) keys_out[i] = keys[idx[i]];
    }
}

// Timing sample (see Sim::sample_substep): returns the extrapolated seconds
// of one full substep, t_full + t_slice * n / (hi - lo).
double pbfo_sample_substep(void* hp, uint32_t lo, uint32_t hi, double* t_full, double* t_slice) {
    Handle* h = (Handle*)hp;
    const uint32_t n = h->fp64 ? h->d.n : h->f.n;
    if (hi > n) hi = n;
    if (lo >= hi) return 0.0;
    if (h->fp64)
        h->d.sample_substep(lo, hi, t_full, t_slice);
    else
        h->f.sample_substep(lo, hi, t_full, t_slice);
    return *t_full + *t_slice * (double)n / (double)(hi - lo);
}

int pbfo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
