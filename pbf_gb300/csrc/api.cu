// api.cu — the C ABI of include/pbf.h: the pbf_sim handle (the reference's SPH
// class, src/SPH.h / src/SPH.cpp), its substep pipeline, CUDA-graph replay,
// debug reads and the standalone sort / cell-finder entry points.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pbf.h"
#include "common.cuh"
#include "internal.h"
#include "sim.h"
#include "sort.cuh"
#include "substep.cuh"

using namespace pbf;

namespace {

thread_local std::string g_error;  // last error of calls without a handle

}  // namespace

void pbf::set_last_error(const char* msg) { g_error = msg ? msg : ""; }

pbf_status pbf::fail(pbf_sim* s, pbf_status st, const std::string& msg) {
    if (s)
        s->err = msg;
    else
        g_error = msg;
    return st;
}

pbf_status pbf::cuda_fail(pbf_sim* s, cudaError_t e, const char* what) {
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(s, e == cudaErrorMemoryAllocation ? PBF_ERR_OUT_OF_MEMORY : PBF_ERR_CUDA, msg);
}



namespace {


pbf_status validate_params(const pbf_params* p, std::string& why) {
    if (!p) {
        why = "params is NULL";
        return PBF_ERR_INVALID_ARGUMENT;
    }
    if (!(p->h > 0.0f) || !std::isfinite(p->h)) {
        why = "h must be positive and finite";
        return PBF_ERR_INVALID_ARGUMENT;
    }
    if (!(p->timestep > 0.0f) || !std::isfinite(p->timestep)) {
        why = "timestep must be positive and finite";
        return PBF_ERR_INVALID_ARGUMENT;
    }
    const float fs[] = {p->one_over_rho_0, p->epsilon, p->gravity, p->tensile_instability_k,
                        p->tensile_instability_scale, p->xsph_viscosity_c, p->vorticity_epsilon};
    for (float f : fs)
        if (!std::isfinite(f)) {
            why = "parameters must be finite";
            return PBF_ERR_INVALID_ARGUMENT;
        }
    uint64_t cells = 1;
    for (int a = 0; a < 3; ++a) {
        if (p->grid[a] == 0 || p->grid[a] > (1u << 24)) {
            why = "grid extents must be in [1, 2^24]";
            return PBF_ERR_INVALID_ARGUMENT;
        }
        cells *= p->grid[a];
        if (!(p->wall_lo[a] <= p->wall_hi[a]) || !std::isfinite(p->wall_lo[a]) ||
            !std::isfinite(p->wall_hi[a])) {
            why = "wall_lo must be <= wall_hi and finite";
            return PBF_ERR_INVALID_ARGUMENT;
        }
    }
    if (cells > 0x7FFFFFFFull) {
        why = "grid has more than 2^31-1 cells";
        return PBF_ERR_INVALID_ARGUMENT;
    }
    return PBF_OK;
}

// Folds pbf_params into the kernel constants.  The folding is part of the
// arithmetic contract: one double-precision evaluation, one rounding to float.
DevConsts make_consts(const pbf_params& p) {
    constexpr double kPoly6 = 1.56668147106;
    constexpr double kSpiky = 4.774648292756860;
    DevConsts c{};
    const double hd = (double)p.h;
    double h6 = 1.0, h9 = 1.0;
    for (int i = 0; i < 6; ++i) h6 *= hd;
    for (int i = 0; i < 9; ++i) h9 *= hd;
    c.h = p.h;
    c.h2 = (float)(hd * hd);
    float r2 = c.h2;
    while (std::sqrt(r2) > c.h) r2 = std::nextafter(r2, 0.0f);
    while (std::sqrt(std::nextafter(r2, INFINITY)) <= c.h) r2 = std::nextafter(r2, INFINITY);
    c.r2cut = r2;
    c.k6 = (float)(kPoly6 / h9);
    c.kg = (float)(-3.0 * kSpiky / h6);
    c.kg_lambda = (float)((-3.0 * kSpiky / h6) * (double)p.one_over_rho_0);
    c.oorho = p.one_over_rho_0;
    c.eps = p.epsilon;
    c.scale = p.tensile_instability_scale;
    c.negk = -p.tensile_instability_k;
    c.cx = p.xsph_viscosity_c;
    c.dt = p.timestep;
    volatile float g = p.gravity, dt = p.timestep, ev = p.vorticity_epsilon;
    c.gdt = g * dt;
    c.g2dt = (2.0f * g) * dt;
    c.dteps = dt * ev;
    for (int a = 0; a < 3; ++a) {
        c.lo[a] = p.wall_lo[a];
        c.hi[a] = p.wall_hi[a];
        c.G[a] = (float)p.grid[a];
        c.Gi[a] = p.grid[a];
    }
    c.half_gz = (float)p.grid[2] / 2.0f;
    c.GxGz = p.grid[0] * p.grid[2];
    c.ncells = p.grid[0] * p.grid[1] * p.grid[2];
    c.ext_force = p.external_force;
    return c;
}

void apply_tuning(DevConsts& c, const pbf_params& p, const pbf_tuning& t) {
    c.use_lists = t.use_neighbour_lists ? 1u : 0u;
    c.skin = t.skin_h * p.h;
    const double rl = (double)p.h + (double)c.skin;
    c.r2list = (float)(rl * rl * (1.0 + 1e-5));
    c.margin_h = 1e-3f * p.h;
    float wm = 0.0f;
    for (int a = 0; a < 3; ++a) wm = std::fmax(wm, std::fmax(std::fabs(p.wall_lo[a]), std::fabs(p.wall_hi[a])));
    c.wall_abs_max = wm;
}

// Handles below this many particles default to the warp-cooperative sweeps: a
// thread per particle cannot fill the GPU there (measured faster at 16,384
// particles in every state of the dam break; from 32,768 up the masked sweeps
// win until the fluid clumps).
constexpr uint32_t kCoopBelow = 32768;

// The autotuner's mixed-sweep candidate: warps for particles with more than
// 256 stencil candidates (in the dam break's initial lattice, 8 particles
// per cell, an interior particle has 216).  It won while the fluid was part
// clumped (262,144 particles: 2.7 ms per substep against 4.2 cooperative and
// 5.7 masked, before the direct sweeps skipped pile runs) and loses once
// every particle is over the threshold, so it is not a default.
constexpr uint32_t kMixedCandidates = 256;

pbf_tuning default_tuning() {
    pbf_tuning t{};
    t.use_neighbour_lists = 0;
    t.list_capacity = 128;
    t.skin_h = 0.15f;
    t.block_size = 256;
    t.sweep_mode = PBF_SWEEP_AUTO;
    t.pair_list_capacity = 128;
    return t;
}

// The all-cooperative candidate is tried below this many particles only: a
// warp per particle costs ~3x the instructions and, on a GPU that a thread per
// particle already fills, a trial substep under it costs several substeps.
constexpr uint32_t kCoopTrialBelow = 262144;

// Chooses the starting configuration and the candidates, and restarts the
// trial schedule (a new state or tuning).
void reset_sweep_choice(pbf_sim* s) {
    const uint32_t m = s->tuning.sweep_mode;
    uint32_t pass = m == PBF_SWEEP_DIRECT ? PBF_PASS_DIRECT
                    : m == PBF_SWEEP_COOP ? PBF_PASS_COOP
                                          : PBF_PASS_MASKED;
    // (mixed for one large scene: the 2M dam break's window runs 2.1x faster
    // under it than masked; a batch of small scenes starts masked, where mixed
    // measured slower)
    if (m == PBF_SWEEP_AUTO)
        pass = s->n < kCoopBelow ? PBF_PASS_COOP
                                 : (s->nscenes == 1 ? PBF_PASS_MIXED : PBF_PASS_MASKED);
    s->pass_solver = s->pass_vort = pass;
    s->autop.reset(s->tuning.auto_period);
    s->auto_trial = -1;
}

// A trial's candidates (auto_policy.h).  (Direct + cooperative is not tried:
// its cooperative second sweep has no run path, so it wins while piles are
// small and then costs O(pile^2 / 32) as they grow, where the direct sweeps
// stay fast.)
void pick_trial_candidates(pbf_sim* s) {
    s->auto_cands = s->autop.candidates(s->pass_solver, s->pass_vort, s->n < kCoopTrialBelow,
                                        s->n >= kCoopBelow);
}

// SweepCfg modes (0 direct, 1 masked, 2 masked + pair lists, 3 cooperative)
// of a pass's first and second sweep.
struct PassModes {
    int first, second;
};
PassModes modes_of(const pbf_sim* s, uint32_t pass) {
    switch (pass) {
        case PBF_PASS_DIRECT: return {0, 0};
        case PBF_PASS_COOP: return {3, 3};
        case PBF_PASS_DIRECT_COOP: return {0, 3};
        default: {
            const int masked = s->pair_cap ? 2 : 1;
            return {masked, masked};
        }
    }
}
bool skin_lists_on(const pbf_sim* s) {
    return s->tuning.use_neighbour_lists != 0 && s->tuning.sweep_mode != PBF_SWEEP_AUTO;
}
// Whether a pass's one-thread sweeps leave the heavy particles to warps:
// every such pass when coop_candidates is set (the opt-in mixed sweeps), and
// the PBF_PASS_MIXED configuration (threshold coop_candidates, or 256).
bool pass_mixed(const pbf_sim* s, uint32_t pass) {
    if (skin_lists_on(s)) return false;
    if (pass == PBF_PASS_MIXED) return true;
    if (s->tuning.coop_candidates == 0) return false;
    const PassModes m = modes_of(s, pass);
    return m.first != 3 || m.second != 3;
}
bool mixed_on(const pbf_sim* s) {
    const bool vort = s->params.vorticity_confinement != 0;
    return pass_mixed(s, s->pass_solver) || (vort && pass_mixed(s, s->pass_vort));
}
uint32_t heavy_threshold(const pbf_sim* s) {
    return s->tuning.coop_candidates ? s->tuning.coop_candidates : kMixedCandidates;
}

// Host-side fault injection (pbf_debug_fail_allocation): when armed, the
// k-th device allocation through dalloc reports cudaErrorMemoryAllocation
// without touching the device.
std::atomic<int> g_fail_alloc_after{-1};

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
    int k = g_fail_alloc_after.load();
    while (k >= 0) {
        if (g_fail_alloc_after.compare_exchange_weak(k, k - 1)) {
            if (k == 0) {
                *p = nullptr;
                return cudaErrorMemoryAllocation;
            }
            break;
        }
    }
    return cudaMalloc((void**)p, sizeof(T) * (count > 0 ? count : 1));
}

// (Re)allocates the neighbour-list and guard buffers for the current
// tuning and iteration count.
cudaError_t ensure_lists(pbf_sim* s) {
    const uint32_t cap = s->tuning.use_neighbour_lists ? s->tuning.list_capacity : 0u;
    if (cap != s->nbr_cap || !s->nbr_cnt) {
        if (s->nbr_idx) cudaFree(s->nbr_idx);
        if (s->nbr_cnt) cudaFree(s->nbr_cnt);
        s->nbr_idx = nullptr;
        s->nbr_cnt = nullptr;
        s->nbr_cap = 0;
        cudaError_t e = dalloc(&s->nbr_idx, (size_t)(cap > 0 ? cap : 1) * s->n);
        if (e == cudaSuccess) e = dalloc(&s->nbr_cnt, s->n);
        if (e != cudaSuccess) return e;
        s->nbr_cap = cap;
    }
    const uint32_t pcap = s->tuning.pair_list_capacity;
    if (pcap != s->pair_cap || (pcap > 0 && !s->pair_cnt)) {
        if (s->pair_idx) cudaFree(s->pair_idx);
        if (s->pair_cnt) cudaFree(s->pair_cnt);
        s->pair_idx = nullptr;
        s->pair_cnt = nullptr;
        s->pair_cap = 0;
        if (pcap > 0) {
            cudaError_t e = dalloc(&s->pair_idx, (size_t)pcap * s->n);
            if (e == cudaSuccess) e = dalloc(&s->pair_cnt, s->n);
            if (e != cudaSuccess) return e;
            s->pair_cap = pcap;
        }
    }
    const uint32_t slots = 2 + s->params.num_solver_iterations;
    if (slots > s->guard_slots) {
        if (s->guard) cudaFree(s->guard);
        s->guard = nullptr;
        s->guard_slots = 0;
        cudaError_t e = dalloc(&s->guard, slots);
        if (e != cudaSuccess) return e;
        s->guard_slots = slots;
    }
    return cudaSuccess;
}

void free_sim(pbf_sim* s) {
    if (!s) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_tape(s);
    for (int k = 0; k < 25; ++k) {
        if (s->execs[k]) cudaGraphExecDestroy(s->execs[k]);
        if (s->graphs[k]) cudaGraphDestroy(s->graphs[k]);
    }
    for (cudaEvent_t e : s->trial_ev)
        if (e) cudaEventDestroy(e);
    void* bufs[] = {s->x,  s->v,  s->xstar, s->XP,   s->Pa,     s->Pb,   s->L,
                    s->VS, s->VX, s->OM,    s->Q,    s->keys,   s->skeys, s->perm,
                    s->cstart, s->cend, s->status, s->sort_mem, s->nbr_idx, s->nbr_cnt,
                    s->guard, s->d_consts, s->sid, s->sid_sorted, s->pair_idx, s->pair_cnt,
                    s->scan_xy, s->scan_z, s->heavy, s->heavy_list, s->heavy_count,
                    s->runs};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (s->h_status) cudaFreeHost(s->h_status);
    for (cudaEvent_t e : s->ev)
        if (e) cudaEventDestroy(e);
    s->ev.clear();
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    cudaSetDevice(prev);
    delete s;
}


// Kernel launches per substep (the sort's launches plus one per stage).
uint32_t kernels_per_substep(const pbf_sim* s) {
    const uint32_t passes = (s->numbits + 7) / 8;
    const uint32_t iters = s->params.num_solver_iterations;
    const bool vort = s->params.vorticity_confinement != 0;
    uint32_t k = 1u /*predict*/ + 1u /*unmark*/ + 2u + passes /*sort*/ + 1u /*cells*/ +
                 2u * iters + 1u /*commit*/ + (vort ? 2u : 0u);
    {  // run-start bits before each direct sweep (enqueue_impl): the positions
       // of every lambda sweep after the first, (p, lambda) of every delta-p,
       // (p, v) and (p, |vorticity|) of the vorticity passes
        const PassModes a = modes_of(s, s->pass_solver), b = modes_of(s, s->pass_vort);
        const bool lists = skin_lists_on(s);
        if (!lists && iters > 0) k += (iters - 1) * (a.first == 0 ? 1u : 0u);
        if (!lists) k += iters * (a.second == 0 ? 1u : 0u);
        if (!lists && vort) k += (b.first == 0 ? 1u : 0u) + (b.second == 0 ? 1u : 0u);
    }
    if (mixed_on(s)) {  // the flag pass and a cooperative launch after each one-thread sweep
        const PassModes a = modes_of(s, s->pass_solver), b = modes_of(s, s->pass_vort);
        k += 1u;
        if (pass_mixed(s, s->pass_solver)) k += iters * ((a.first != 3) + (a.second != 3));
        if (vort && pass_mixed(s, s->pass_vort)) k += (uint32_t)((b.first != 3) + (b.second != 3));
    }
    return k;
}

// One eager substep with stage events; accumulates the stage sums.
pbf_status timed_substep(pbf_sim* s);


// Launches `count` substeps of the captured graph of the current solver and
// vorticity configurations (captured on first use).
pbf_status launch_graph(pbf_sim* s, uint32_t count) {
    const uint32_t key = s->pass_solver * 5u + s->pass_vort;
    if (!s->execs[key]) {
        PBF_CUDA(s, cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = enqueue_substep(s, nullptr);
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
        if (e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(s, e, "substep capture");
        }
        if (e2 != cudaSuccess) return cuda_fail(s, e2, "cudaStreamEndCapture");
        s->graphs[key] = g;
        PBF_CUDA(s, cudaGraphInstantiate(&s->execs[key], g, 0));
    }
    for (uint32_t k = 0; k < count; ++k) PBF_CUDA(s, cudaGraphLaunch(s->execs[key], s->stream));
    s->launched += (uint64_t)count * kernels_per_substep(s);
    return PBF_OK;
}

// One substep of a PBF_SWEEP_AUTO trial: the next candidate configuration for
// both passes, eager, with stage events.  After the last candidate, waits for
// the trial's events and hands each candidate's solver and vorticity times
// to the policy (auto_policy.h), which keeps the choices and the schedule.
pbf_status trial_substep(pbf_sim* s) {
    NvtxRange nvtx_("sweep trial substep");
    const uint32_t iters = s->params.num_solver_iterations;
    const size_t per = 7 + 2 * (size_t)iters;
    const size_t nc = s->auto_cands.size();
    while (s->trial_ev.size() < per * nc) {
        cudaEvent_t e = nullptr;
        PBF_CUDA(s, cudaEventCreate(&e));
        s->trial_ev.push_back(e);
    }
    const uint32_t keep_s = s->pass_solver, keep_v = s->pass_vort;
    const int k = s->auto_trial;
    s->pass_solver = s->pass_vort = s->auto_cands[k];
    cudaError_t e = enqueue_substep(s, s->trial_ev.data() + per * k);
    s->launched += kernels_per_substep(s);
    s->pass_solver = keep_s;
    s->pass_vort = keep_v;
    if (e != cudaSuccess) return cuda_fail(s, e, "trial substep launch");
    if (++s->auto_trial < (int)nc) return PBF_OK;
    PBF_CUDA(s, cudaEventSynchronize(s->trial_ev[per * nc - 1]));
    auto span = [&](size_t c, size_t a, size_t b) {
        float m = 0.0f;
        cudaEventElapsedTime(&m, s->trial_ev[per * c + a], s->trial_ev[per * c + b]);
        return (double)m;
    };
    std::vector<double> solver_ms(nc), vort_ms(nc);
    for (size_t c = 0; c < nc; ++c) {
        solver_ms[c] = span(c, 3, 3 + 2 * (size_t)iters);
        vort_ms[c] = span(c, 4 + 2 * (size_t)iters, 6 + 2 * (size_t)iters);
    }
    s->autop.finish(s->auto_cands, solver_ms.data(), vort_ms.data(),
                    s->params.vorticity_confinement != 0, s->pass_solver, s->pass_vort);
    s->auto_trial = -1;
    return PBF_OK;
}

pbf_status timed_substep(pbf_sim* s) {
    NvtxRange nvtx_("timed substep");
    const uint32_t iters = s->params.num_solver_iterations;
    const size_t need = 7 + 2 * (size_t)iters;
    while (s->ev.size() < need) {
        cudaEvent_t e = nullptr;
        PBF_CUDA(s, cudaEventCreate(&e));
        s->ev.push_back(e);
    }
    cudaError_t e = enqueue_substep(s, s->ev.data());
    if (e != cudaSuccess) return cuda_fail(s, e, "substep launch");
    s->launched += kernels_per_substep(s);
    PBF_CUDA(s, cudaEventSynchronize(s->ev[need - 1]));
    auto span = [&](size_t a, size_t b) {
        float m = 0.0f;
        cudaEventElapsedTime(&m, s->ev[a], s->ev[b]);
        return (double)m;
    };
    double lam = 0.0, dp = 0.0;
    for (uint32_t it = 0; it < iters; ++it) {
        lam += span(3 + 2 * it, 4 + 2 * it);
        dp += span(4 + 2 * it, 5 + 2 * it);
    }
    const double st[8] = {span(0, 1), span(1, 2), span(2, 3), lam, dp,
                          span(3 + 2 * iters, 4 + 2 * iters), span(4 + 2 * iters, 5 + 2 * iters),
                          span(5 + 2 * iters, 6 + 2 * iters)};
    for (int i = 0; i < 8; ++i) s->stage_ms[i] += st[i];
    s->timed_substeps++;
    s->ms[0] = (float)st[0];
    s->ms[1] = (float)st[1];
    s->ms[2] = (float)st[2];
    s->ms[3] = (float)(lam + dp);
    s->ms[4] = (float)(st[5] + st[6] + st[7]);
    return PBF_OK;
}

}  // namespace

namespace pbf {

// Enqueues one substep (SPH::Run, src/SPH.cpp:246-334) on s->stream.  With
// `ev` non-null, records an event at every stage boundary: before predict,
// after predict, sort, cells, each lambda and delta-p launch, commit and the
// two vorticity passes (7 + 2 * iterations events).
template <class CPi, class CPs>
cudaError_t enqueue_impl(pbf_sim* s, cudaEvent_t* ev, const Recording* rec, const CPi& cpi,
                         const CPs& cps) {
    const uint32_t n = s->n;
    if (!s->nbr_cnt || s->guard_slots < 2 + s->params.num_solver_iterations)
        return cudaErrorInvalidValue;  // ensure_lists() runs before any capture
    const unsigned g = grid_for(n);
    const unsigned blk = s->tuning.block_size ? s->tuning.block_size : (unsigned)kBlock;
    const bool lists = skin_lists_on(s);
    const PassModes ms = modes_of(s, s->pass_solver), mv = modes_of(s, s->pass_vort);
    const SweepCfg s_lam{blk, ms.first, lists}, s_dp{blk, ms.second, lists},
        s_va{blk, mv.first, lists}, s_vb{blk, mv.second, lists};
    const bool vort = s->params.vorticity_confinement != 0;
    // delta-p writes the scan copy of its output when a sweep reading that
    // position set scans through it (masked modes; a pair-list replay falls
    // back to a scan on overflow)
    auto scans = [](int m) { return m == 1 || m == 2; };
    const bool solver_scans = scans(ms.first) || scans(ms.second);
    const bool vort_scans = vort && (scans(mv.first) || scans(mv.second));
    const uint32_t iters = s->params.num_solver_iterations;
    cudaStream_t st = s->stream;
    auto mark = [&](uint32_t idx) {
        if (ev) cudaEventRecord(ev[idx], st);
    };
    mark(0);
    // 1 predict (predictpos.glsl)
    launch_predict(g, st, s->x, s->v, s->xstar, s->keys, n, cpi, s->status);
    mark(1);
    // 2 sort (RadixSort::Run); first clear the cell starts of the previous
    // substep while its sorted keys are still there
    k_unmark_cells<<<g, kBlock, 0, st>>>(s->skeys, n, s->ncells, s->cstart);
    cudaError_t e = sort_pairs(s->sort, s->keys, s->skeys, s->perm, n, s->numbits, s->status, st);
    if (e != cudaSuccess) return e;
    mark(2);
    // 3 cell ranges (NeighbourCellFinder::FindNeighbourCells)
    const size_t half = ((size_t)n + 1) / 2;
    auto scan_set = [&](int k) { return ScanPos{s->scan_xy + k * half, s->scan_z + k * half}; };
    // (over n + 1 threads: the run-start bits end with a terminator at n)
    k_find_cells<<<grid_for(n + 1), kBlock, 0, st>>>(s->skeys, s->perm, s->xstar, s->XP, n,
                                                     s->ncells, s->cstart, s->cend, s->status + 1,
                                                     s->sid, s->sid_sorted, scan_set(0), s->runs,
                                                     s->status);
    // mixed sweeps: flag the particles with more than coop_candidates stencil
    // candidates; the cooperative kernels sweep those, the others skip them
    const bool mixed = mixed_on(s);
    if (mixed) {
        cudaError_t me = cudaMemsetAsync(s->heavy_count, 0, sizeof(uint32_t), st);
        if (me != cudaSuccess) return me;
        launch_heavy_scan(g, st, s->XP, s->cstart, s->cend, heavy_threshold(s), n, cps,
                          s->heavy, s->heavy_list, s->heavy_count);
    }
    mark(3);
    // 4 solver iterations (calclambda / updatepos).  The first lambda sweep
    // also records the neighbour lists the later sweeps replay.
    const NbrLists nl{s->nbr_idx, s->nbr_cnt, s->guard, s->nbr_cap, n};
    // the direct sweeps skip runs of coincident candidates (neighbours.cuh:
    // visit_direct_piles); run-start bits of each position set they read, and
    // for delta-p and the vorticity passes over their other inputs as well
    // (lambda, the committed velocity, |vorticity|), so that a run's terms
    // are all equal (k_run_flags_vals)
    const bool lam_direct = !lists && ms.first == 0, dp_direct = !lists && ms.second == 0;
    const bool va_direct = !lists && vort && mv.first == 0;
    const bool vb_direct = !lists && vort && mv.second == 0;
    const bool runs_solver = lam_direct || dp_direct;
    const bool runs_vort = va_direct || vb_direct;
    // the heavy list goes only to the passes that leave heavy particles to warps
    const bool mix_s = mixed && pass_mixed(s, s->pass_solver);
    const bool mix_v = mixed && pass_mixed(s, s->pass_vort);
    const PairLists pl{s->pair_idx, s->pair_cnt, s->pair_cap, n, mix_s ? s->heavy : nullptr,
                       s->heavy_list, s->heavy_count,
                       runs_solver || runs_vort ? s->runs : nullptr};
    PairLists pl_v = pl;
    pl_v.heavy = mix_v ? s->heavy : nullptr;
    cudaError_t ge = cudaMemsetAsync(s->guard, 0, sizeof(uint32_t) * (2 + iters), st);
    if (ge != cudaSuccess) return ge;
    const float4* cur = s->XP;
    int cur_set = 0;  // scan copy of `cur`
    for (uint32_t it = 0; it < iters; ++it) {
        float4* nxt = (it % 2 == 0) ? s->Pa : s->Pb;
        const int nxt_set = 1 + (int)(it % 2);
        if (rec && it + 1 == iters) nxt = rec->PF;
        float4* Lk = rec ? rec->L[it] : s->L;
        float4* aux = rec ? rec->AUX[it] : nullptr;
        const int in_slot = it == 0 ? -1 : (int)it;  // displacement of `cur` from XP
        if (it == 0)
            launch_lambda_build(s_lam, st, s->XP, s->skeys, s->cstart, s->cend, Lk, aux, nl, pl,
                                scan_set(0), n, cps);
        else
            launch_lambda(s_lam, st, cur, s->XP, s->skeys, s->cstart, s->cend, Lk, aux, nl, pl,
                          scan_set(cur_set), in_slot, n, cps);
        if (dp_direct)
            k_run_flags_vals<<<grid_for(n + 1), kBlock, 0, st>>>(Lk, nullptr, 1, n, s->runs);
        mark(4 + 2 * it);
        // delta-p replays the pair lists the lambda sweep just recorded
        const bool write_scan = it + 1 < iters ? solver_scans : vort_scans;
        launch_delta_p(s_dp, st, Lk, s->XP, s->skeys, s->cstart, s->cend, nxt, nl, pl,
                       scan_set(cur_set), write_scan ? scan_set(nxt_set) : ScanPos{nullptr, nullptr},
                       in_slot, (int)it + 1, n, cps, s->status);
        if (it + 1 < iters && lam_direct)
            k_run_flags<<<grid_for(n + 1), kBlock, 0, st>>>(nxt, n, s->runs);
        mark(5 + 2 * it);
        cur = nxt;
        cur_set = nxt_set;
    }
    if (rec && iters == 0) {
        cudaError_t ce = cudaMemcpyAsync(rec->PF, s->XP, sizeof(float4) * n,
                                         cudaMemcpyDeviceToDevice, st);
        if (ce != cudaSuccess) return ce;
        cur = rec->PF;
    }
    // 5 commit (update.glsl) and XSPH + vorticity (vorticity.glsl)
    const int fin_slot = iters == 0 ? -2 : (int)iters;  // -2: no list was built this substep
    float4* VS = rec ? rec->VS : s->VS;
    float4* OM = rec ? rec->OM : s->OM;
    float4* Q = rec ? rec->Q : s->Q;
    launch_commit(g, st, cur, s->perm, s->x, VS, vort ? nullptr : s->v, n, cps);
    if (va_direct)
        k_run_flags_vals<<<grid_for(n + 1), kBlock, 0, st>>>(cur, VS, 0, n, s->runs);
    mark(4 + 2 * iters);
    if (vort)
        launch_vorticity_a(s_va, st, cur, s->XP, VS, s->skeys, s->cstart, s->cend, s->VX, OM, Q, nl,
                           pl_v, scan_set(cur_set), fin_slot, n, cps);
    if (vb_direct)
        k_run_flags_vals<<<grid_for(n + 1), kBlock, 0, st>>>(Q, nullptr, 1, n, s->runs);
    mark(5 + 2 * iters);
    if (vort)
        launch_vorticity_b(s_vb, st, Q, s->XP, s->VX, OM, s->skeys, s->perm, s->cstart, s->cend, s->v,
                           rec ? rec->ETA : nullptr, nl, pl_v, scan_set(cur_set), fin_slot, n, cps);
    mark(6 + 2 * iters);
    return cudaGetLastError();
}

cudaError_t enqueue_substep(pbf_sim* s, cudaEvent_t* ev, const Recording* rec) {
    if (s->nscenes == 1) return enqueue_impl(s, ev, rec, OneScene{s->dc}, OneScene{s->dc});
    return enqueue_impl(s, ev, rec, ManyScenes{s->d_consts, s->sid},
                        ManyScenes{s->d_consts, s->sid_sorted});
}

void invalidate_graph(pbf_sim* s) {
    for (int k = 0; k < 25; ++k) {
        if (s->execs[k]) cudaGraphExecDestroy(s->execs[k]);
        if (s->graphs[k]) cudaGraphDestroy(s->graphs[k]);
        s->execs[k] = nullptr;
        s->graphs[k] = nullptr;
    }
}

// The bounds-checked build's fields of every scene's constants: the handle's
// status word and particle count (make_consts leaves them empty).
void bind_checks(pbf_sim* s) {
    for (auto& c : s->sdc) {
        c.check_status = s->status;
        c.n_total = s->n;
    }
    if (!s->sdc.empty()) s->dc = s->sdc[0];
}

pbf_status check_status(pbf_sim* s) {
    PBF_CUDA(s, cudaMemcpyAsync(s->h_status, s->status, 2 * sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, s->stream));
    PBF_CUDA(s, cudaStreamSynchronize(s->stream));
    const uint32_t bits = s->h_status[0];
    if (bits & (kDevNonFinite | kDevSortTimeout | kDevIndexFault)) {
        std::string m = "device status";
        if (bits & kDevNonFinite) m += ": non-finite position";
        if (bits & kDevSortTimeout) m += ": radix-sort lookback timed out";
        if (bits & kDevIndexFault) m += ": index out of bounds (bounds-checked build)";
        return fail(s, PBF_ERR_DEVICE_FAULT, m);
    }
    if (s->h_status[1]) return fail(s, PBF_ERR_DEVICE_FAULT, "device status: cell key out of range");
    return PBF_OK;
}

}  // namespace pbf

extern "C" {

pbf_status pbf_create(const pbf_params* params, uint32_t n, pbf_sim** out) {
    return pbf_create_batch(params, &n, 1, out);
}

pbf_status pbf_create_batch(const pbf_params* scene_params, const uint32_t* scene_counts,
                            uint32_t num_scenes, pbf_sim** out) {
    if (!out) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!scene_params || !scene_counts || num_scenes == 0)
        return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "scene_params, scene_counts and num_scenes are required");
    std::string why;
    uint64_t total = 0, cells = 0;
    for (uint32_t k = 0; k < num_scenes; ++k) {
        if (validate_params(&scene_params[k], why) != PBF_OK)
            return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "scene " + std::to_string(k) + ": " + why);
        if (scene_counts[k] == 0)
            return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "every scene needs at least one particle");
        if (scene_params[k].num_solver_iterations != scene_params[0].num_solver_iterations ||
            (scene_params[k].vorticity_confinement != 0) != (scene_params[0].vorticity_confinement != 0))
            return fail(nullptr, PBF_ERR_INVALID_ARGUMENT,
                        "all scenes share the iteration count and the vorticity flag");
        total += scene_counts[k];
        cells += (uint64_t)scene_params[k].grid[0] * scene_params[k].grid[1] * scene_params[k].grid[2];
    }
    if (total >= (1u << 30)) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "n must be in [1, 2^30)");
    if (cells > 0x7FFFFFFFull) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "more than 2^31-1 cells in total");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(nullptr, PBF_ERR_NO_DEVICE, "no CUDA device");
    }
    const uint32_t n = (uint32_t)total;
    pbf_sim* s = new pbf_sim();
    cudaGetDevice(&s->device);
    s->nscenes = num_scenes;
    s->sparams.assign(scene_params, scene_params + num_scenes);
    s->counts.assign(scene_counts, scene_counts + num_scenes);
    s->params = scene_params[0];
    s->tuning = default_tuning();
    s->n = n;
    s->ncells = (uint32_t)cells;
    s->numbits = sort_numbits_for_cells(s->ncells);
    s->sdc.resize(num_scenes);
    s->offsets.resize(num_scenes + 1);
    uint32_t base = 0, off = 0;
    for (uint32_t k = 0; k < num_scenes; ++k) {
        s->sdc[k] = make_consts(scene_params[k]);
        s->sdc[k].cell_base = base;
        apply_tuning(s->sdc[k], scene_params[k], s->tuning);
        base += s->sdc[k].ncells;
        s->offsets[k] = off;
        off += scene_counts[k];
    }
    s->offsets[num_scenes] = off;
    s->dc = s->sdc[0];
    cudaError_t e = cudaSuccess;
#define ALLOC(ptr, cnt)                                                  \
    if (e == cudaSuccess) e = dalloc(&s->ptr, (cnt));
    ALLOC(x, n) ALLOC(v, n) ALLOC(xstar, n) ALLOC(XP, n) ALLOC(Pa, n) ALLOC(Pb, n) ALLOC(L, n)
    ALLOC(VS, n) ALLOC(VX, n) ALLOC(OM, n) ALLOC(Q, n) ALLOC(keys, n) ALLOC(skeys, n)
    ALLOC(perm, n) ALLOC(cstart, s->ncells) ALLOC(cend, s->ncells) ALLOC(status, 2)
    ALLOC(scan_xy, 3 * (((size_t)n + 1) / 2)) ALLOC(scan_z, 3 * (((size_t)n + 1) / 2))
    ALLOC(heavy, n) ALLOC(heavy_list, n) ALLOC(heavy_count, 1) ALLOC(runs, (size_t)n / 32 + 2)
    if (num_scenes > 1) {
        ALLOC(d_consts, num_scenes) ALLOC(sid, n) ALLOC(sid_sorted, n)
    }
#undef ALLOC
    if (e == cudaSuccess) e = cudaMalloc(&s->sort_mem, SortWorkspace::bytes_for(n));
    if (e == cudaSuccess) e = ensure_lists(s);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&s->h_status, 2 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        pbf_status st = cuda_fail(nullptr, e, "pbf_create allocation");
        free_sim(s);
        return st;
    }
    s->stream = s->own_stream;
    bind_checks(s);
    reset_sweep_choice(s);
    e = num_scenes == 1 ? preload_sweeps<OneScene>() : preload_sweeps<ManyScenes>();
    if (e != cudaSuccess) {
        pbf_status st = cuda_fail(nullptr, e, "pbf_create kernel load");
        free_sim(s);
        return st;
    }
    s->sort.carve(s->sort_mem, n);
    e = cudaMemsetAsync(s->cstart, 0xFF, sizeof(int32_t) * s->ncells, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->cend, 0xFF, sizeof(int32_t) * s->ncells, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->skeys, 0, sizeof(uint32_t) * n, s->stream);
    // perm always holds ids < n, even if a sort ever fails part-way
    if (e == cudaSuccess) e = cudaMemsetAsync(s->perm, 0, sizeof(uint32_t) * n, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->x, 0, sizeof(float4) * n, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->v, 0, sizeof(float4) * n, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->status, 0, 2 * sizeof(uint32_t), s->stream);
    if (e == cudaSuccess && num_scenes > 1) {
        std::vector<uint32_t> sid(n);
        for (uint32_t k = 0; k < num_scenes; ++k)
            for (uint32_t i = s->offsets[k]; i < s->offsets[k + 1]; ++i) sid[i] = k;
        e = cudaMemcpy(s->sid, sid.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(s->d_consts, s->sdc.data(), sizeof(DevConsts) * num_scenes,
                           cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        pbf_status st = cuda_fail(nullptr, e, "pbf_create initialisation");
        free_sim(s);
        return st;
    }
    *out = s;
    return PBF_OK;
}

void pbf_destroy(pbf_sim* s) { free_sim(s); }

pbf_status pbf_set_params(pbf_sim* s, const pbf_params* p) {
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (s->nscenes != 1)
        return fail(s, PBF_ERR_INVALID_ARGUMENT, "a batch takes pbf_set_scene_params");
    return pbf_set_scene_params(s, 0, p);
}

pbf_status pbf_set_scene_params(pbf_sim* s, uint32_t scene, const pbf_params* p) {
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (scene >= s->nscenes) return fail(s, PBF_ERR_INVALID_ARGUMENT, "scene index out of range");
    std::string why;
    if (validate_params(p, why) != PBF_OK) return fail(s, PBF_ERR_INVALID_ARGUMENT, why);
    for (int a = 0; a < 3; ++a)
        if (p->grid[a] != s->sparams[scene].grid[a])
            return fail(s, PBF_ERR_INVALID_ARGUMENT, "the grid is fixed at creation");
    if (s->nscenes > 1 &&
        (p->num_solver_iterations != s->params.num_solver_iterations ||
         (p->vorticity_confinement != 0) != (s->params.vorticity_confinement != 0)))
        return fail(s, PBF_ERR_INVALID_ARGUMENT,
                    "all scenes share the iteration count and the vorticity flag");
    DeviceGuard dg(s->device);
    PBF_CUDA(s, cudaStreamSynchronize(s->stream));
    const uint32_t base = s->sdc[scene].cell_base;
    s->sparams[scene] = *p;
    s->sdc[scene] = make_consts(*p);
    s->sdc[scene].cell_base = base;
    apply_tuning(s->sdc[scene], *p, s->tuning);
    bind_checks(s);
    if (scene == 0) s->params = *p;
    if (s->nscenes > 1)
        PBF_CUDA(s, cudaMemcpy(s->d_consts + scene, &s->sdc[scene], sizeof(DevConsts),
                               cudaMemcpyHostToDevice));
    invalidate_graph(s);
    free_tape(s);  // a recorded run is only valid for the parameters it ran with
    s->auto_trial = -1;  // a running trial's events may not match the new iteration count
    PBF_CUDA(s, ensure_lists(s));
    return PBF_OK;
}

pbf_status pbf_get_scene_params(const pbf_sim* s, uint32_t scene, pbf_params* out) {
    if (!s || !out) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (scene >= s->nscenes) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "scene index out of range");
    *out = s->sparams[scene];
    return PBF_OK;
}

uint32_t pbf_num_scenes(const pbf_sim* s) { return s ? s->nscenes : 0; }
uint32_t pbf_num_cells(const pbf_sim* s) { return s ? s->ncells : 0; }

pbf_status pbf_scene_range(const pbf_sim* s, uint32_t scene, uint32_t* first, uint32_t* count) {
    if (!s || scene >= s->nscenes) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "bad scene");
    if (first) *first = s->offsets[scene];
    if (count) *count = s->counts[scene];
    return PBF_OK;
}

pbf_status pbf_set_tuning(pbf_sim* s, const pbf_tuning* t) {
    if (!s || !t) return fail(s, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (t->use_neighbour_lists && (t->list_capacity < 1 || t->list_capacity > 4096))
        return fail(s, PBF_ERR_INVALID_ARGUMENT, "list_capacity must be in [1, 4096]");
    if (!(t->skin_h >= 0.0f) || !(t->skin_h <= 1.0f))
        return fail(s, PBF_ERR_INVALID_ARGUMENT, "skin_h must be in [0, 1]");
    if (t->block_size != 0 && (t->block_size < 32 || t->block_size > (uint32_t)kBlock ||
                               t->block_size % 32 != 0))
        return fail(s, PBF_ERR_INVALID_ARGUMENT, "block_size must be 0 or a multiple of 32 in [32, 256]");
    if (t->pair_list_capacity > 4096)
        return fail(s, PBF_ERR_INVALID_ARGUMENT, "pair_list_capacity must be in [0, 4096]");
    if (t->sweep_mode != PBF_SWEEP_DIRECT && t->sweep_mode != PBF_SWEEP_MASKED &&
        t->sweep_mode != PBF_SWEEP_COOP && t->sweep_mode != PBF_SWEEP_AUTO)
        return fail(s, PBF_ERR_INVALID_ARGUMENT,
                    "sweep_mode must be PBF_SWEEP_DIRECT, PBF_SWEEP_MASKED, PBF_SWEEP_COOP or "
                    "PBF_SWEEP_AUTO");
    DeviceGuard dg(s->device);
    PBF_CUDA(s, cudaStreamSynchronize(s->stream));
    s->tuning = *t;
    for (uint32_t k = 0; k < s->nscenes; ++k) apply_tuning(s->sdc[k], s->sparams[k], s->tuning);
    s->dc = s->sdc[0];
    if (s->nscenes > 1)
        PBF_CUDA(s, cudaMemcpy(s->d_consts, s->sdc.data(), sizeof(DevConsts) * s->nscenes,
                               cudaMemcpyHostToDevice));
    invalidate_graph(s);
    PBF_CUDA(s, ensure_lists(s));
    reset_sweep_choice(s);
    return PBF_OK;
}

pbf_status pbf_autotune(pbf_sim* s, uint32_t trial_substeps, pbf_tuning* best) {
    NvtxRange nvtx_("pbf_autotune");
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (trial_substeps == 0) return fail(s, PBF_ERR_INVALID_ARGUMENT, "trial_substeps must be positive");
    DeviceGuard dg(s->device);
    const size_t b = sizeof(float4) * s->n;
    float4 *sx = nullptr, *sv = nullptr;
    PBF_CUDA(s, cudaMalloc(&sx, b));
    cudaError_t e = cudaMalloc(&sv, b);
    if (e != cudaSuccess) {
        cudaFree(sx);
        return cuda_fail(s, e, "autotune snapshot");
    }
    cudaStream_t st = s->stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto cleanup = [&]() {
        cudaFree(sx);
        cudaFree(sv);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    e = cudaMemcpyAsync(sx, s->x, b, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sv, s->v, b, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) {
        cleanup();
        return cuda_fail(s, e, "autotune snapshot");
    }
    const pbf_tuning original = s->tuning;
    std::vector<pbf_tuning> cand;
    for (uint32_t blk : {128u, 256u})
        for (uint32_t mode : {(uint32_t)PBF_SWEEP_DIRECT, (uint32_t)PBF_SWEEP_MASKED}) {
            pbf_tuning t = original;
            t.block_size = blk;
            t.sweep_mode = mode;
            t.use_neighbour_lists = 0;
            t.coop_candidates = 0;
            cand.push_back(t);
            for (float skin : {0.05f, 0.1f, 0.2f}) {
                t.use_neighbour_lists = 1;
                t.skin_h = skin;
                if (t.list_capacity == 0) t.list_capacity = 128;
                cand.push_back(t);
            }
        }
    {
        pbf_tuning t = original;  // the warp-cooperative sweeps (block size and lists unused)
        t.sweep_mode = PBF_SWEEP_COOP;
        t.use_neighbour_lists = 0;
        t.coop_candidates = 0;
        cand.push_back(t);
        t.sweep_mode = PBF_SWEEP_MASKED;  // mixed: warps for the particles in dense stencils
        t.block_size = 256;
        t.coop_candidates = kMixedCandidates;
        cand.push_back(t);
    }
    float best_ms = 1e30f;
    pbf_tuning best_t = original;
    pbf_status r = PBF_OK;
    for (const pbf_tuning& t : cand) {
        r = pbf_set_tuning(s, &t);
        if (r != PBF_OK) break;
        // one untimed substep captures the graph, then the timed trial
        for (int pass = 0; pass < 2 && r == PBF_OK; ++pass) {
            cudaMemcpyAsync(s->x, sx, b, cudaMemcpyDeviceToDevice, st);
            cudaMemcpyAsync(s->v, sv, b, cudaMemcpyDeviceToDevice, st);
            if (pass == 1) cudaEventRecord(e0, st);
            r = pbf_step(s, pass == 0 ? 1 : trial_substeps);
            if (pass == 1) cudaEventRecord(e1, st);
        }
        if (r != PBF_OK) break;
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) {
            r = cuda_fail(s, e, "autotune trial");
            break;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) {
            best_ms = ms;
            best_t = t;
        }
    }
    cudaMemcpyAsync(s->x, sx, b, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(s->v, sv, b, cudaMemcpyDeviceToDevice, st);
    cudaStreamSynchronize(st);
    cleanup();
    if (r != PBF_OK) {
        pbf_set_tuning(s, &original);
        return r;
    }
    r = pbf_set_tuning(s, &best_t);
    if (r == PBF_OK && best) *best = best_t;
    return r == PBF_OK ? check_status(s) : r;
}

pbf_status pbf_get_tuning(const pbf_sim* s, pbf_tuning* out) {
    if (!s || !out) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = s->tuning;
    return PBF_OK;
}

pbf_status pbf_get_params(const pbf_sim* s, pbf_params* out) {
    if (!s || !out) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = s->params;
    return PBF_OK;
}

uint32_t pbf_num_particles(const pbf_sim* s) { return s ? s->n : 0; }

pbf_status pbf_set_stream(pbf_sim* s, void* stream) {
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    DeviceGuard dg(s->device);
    PBF_CUDA(s, cudaStreamSynchronize(s->stream));
    cudaStream_t ns = stream ? (cudaStream_t)stream : s->own_stream;
    if (ns != s->stream) invalidate_graph(s);  // the graph is replayed on any stream, but
    s->stream = ns;                            // re-capture keeps capture and replay alike
    return PBF_OK;
}

pbf_status pbf_set_state(pbf_sim* s, const float* x4, const float* v4, int where) {
    NvtxRange nvtx_("pbf_set_state");
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (!x4 || !v4) return fail(s, PBF_ERR_INVALID_ARGUMENT, "x4 and v4 are required");
    if (where != PBF_HOST && where != PBF_DEVICE) return fail(s, PBF_ERR_INVALID_ARGUMENT, "bad where");
    DeviceGuard dg(s->device);
    const cudaMemcpyKind k = where == PBF_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    PBF_CUDA(s, cudaMemcpyAsync(s->x, x4, sizeof(float4) * s->n, k, s->stream));
    PBF_CUDA(s, cudaMemcpyAsync(s->v, v4, sizeof(float4) * s->n, k, s->stream));
    PBF_CUDA(s, cudaStreamSynchronize(s->stream));
    reset_sweep_choice(s);
    return PBF_OK;
}

pbf_status pbf_get_state(pbf_sim* s, float* x4, float* v4, int where) {
    NvtxRange nvtx_("pbf_get_state");
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (where != PBF_HOST && where != PBF_DEVICE) return fail(s, PBF_ERR_INVALID_ARGUMENT, "bad where");
    DeviceGuard dg(s->device);
    const cudaMemcpyKind k = where == PBF_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (x4) PBF_CUDA(s, cudaMemcpyAsync(x4, s->x, sizeof(float4) * s->n, k, s->stream));
    if (v4) PBF_CUDA(s, cudaMemcpyAsync(v4, s->v, sizeof(float4) * s->n, k, s->stream));
    return check_status(s);
}

pbf_status pbf_device_buffers(pbf_sim* s, float** x4, float** v4) {
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (x4) *x4 = (float*)s->x;
    if (v4) *v4 = (float*)s->v;
    return PBF_OK;
}

pbf_status pbf_step(pbf_sim* s, uint32_t substeps) {
    NvtxRange nvtx_("pbf_step");
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    DeviceGuard dg(s->device);
    if (s->timing) {
        for (uint32_t k = 0; k < substeps; ++k) {
            pbf_status r = timed_substep(s);
            if (r != PBF_OK) return r;
        }
        return PBF_OK;
    }
    const bool autom = s->tuning.sweep_mode == PBF_SWEEP_AUTO;
    uint32_t left = substeps;
    while (left > 0) {
        if (autom && s->auto_trial < 0 && s->autop.trial_due()) {
            pick_trial_candidates(s);
            s->auto_trial = 0;
        }
        if (autom && s->auto_trial >= 0) {
            pbf_status r = trial_substep(s);
            if (r != PBF_OK) return r;
            --left;
            ++s->autop.count;
            continue;
        }
        uint32_t run = left;
        if (autom) run = (uint32_t)std::min<uint64_t>(left, s->autop.next - s->autop.count);
        pbf_status r = launch_graph(s, run);
        if (r != PBF_OK) return r;
        left -= run;
        s->autop.count += run;
    }
    return PBF_OK;
}

pbf_status pbf_get_sweep_choice(const pbf_sim* s, uint32_t out[3]) {
    if (!s || !out) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    out[0] = s->pass_solver;
    out[1] = s->pass_vort;
    out[2] = s->autop.trials;
    return PBF_OK;
}

pbf_status pbf_synchronize(pbf_sim* s) {
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    DeviceGuard dg(s->device);
    return check_status(s);
}

pbf_status pbf_device_status(pbf_sim* s, uint32_t* bits) {
    if (!s || !bits) return fail(s, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    DeviceGuard dg(s->device);
    PBF_CUDA(s, cudaMemcpyAsync(s->h_status, s->status, 2 * sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, s->stream));
    PBF_CUDA(s, cudaStreamSynchronize(s->stream));
    *bits = s->h_status[0];
    return PBF_OK;
}

pbf_status pbf_enable_timing(pbf_sim* s, int enable) {
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    s->timing = enable != 0;
    for (double& m : s->stage_ms) m = 0.0;
    s->timed_substeps = 0;
    return PBF_OK;
}

pbf_status pbf_get_stage_times(pbf_sim* s, double ms_sum[8], uint32_t* substeps) {
    if (!s || !ms_sum) return fail(s, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    for (int i = 0; i < 8; ++i) ms_sum[i] = s->stage_ms[i];
    if (substeps) *substeps = s->timed_substeps;
    return PBF_OK;
}

uint32_t pbf_kernels_per_substep(const pbf_sim* s) { return s ? kernels_per_substep(s) : 0; }

uint64_t pbf_kernels_launched(const pbf_sim* s) { return s ? s->launched : 0; }

pbf_status pbf_get_timing(pbf_sim* s, float ms[5]) {
    if (!s || !ms) return fail(s, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    for (int p = 0; p < 5; ++p) ms[p] = s->ms[p];
    return PBF_OK;
}

pbf_status pbf_get_sort(pbf_sim* s, uint32_t* keys_by_id, uint32_t* sorted_keys, uint32_t* perm) {
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    DeviceGuard dg(s->device);
    const size_t b = sizeof(uint32_t) * s->n;
    if (keys_by_id) PBF_CUDA(s, cudaMemcpyAsync(keys_by_id, s->keys, b, cudaMemcpyDeviceToHost, s->stream));
    if (sorted_keys) PBF_CUDA(s, cudaMemcpyAsync(sorted_keys, s->skeys, b, cudaMemcpyDeviceToHost, s->stream));
    if (perm) PBF_CUDA(s, cudaMemcpyAsync(perm, s->perm, b, cudaMemcpyDeviceToHost, s->stream));
    return check_status(s);
}

pbf_status pbf_get_cells(pbf_sim* s, int32_t* start, int32_t* end) {
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    DeviceGuard dg(s->device);
    std::vector<int32_t> st(s->ncells), en(s->ncells);
    PBF_CUDA(s, cudaMemcpyAsync(st.data(), s->cstart, sizeof(int32_t) * s->ncells,
                                cudaMemcpyDeviceToHost, s->stream));
    PBF_CUDA(s, cudaMemcpyAsync(en.data(), s->cend, sizeof(int32_t) * s->ncells,
                                cudaMemcpyDeviceToHost, s->stream));
    pbf_status r = check_status(s);
    if (r != PBF_OK) return r;
    // cell_end is only maintained where cell_start is set
    for (uint32_t c = 0; c < s->ncells; ++c)
        if (st[c] == -1) en[c] = -1;
    if (start) std::memcpy(start, st.data(), sizeof(int32_t) * s->ncells);
    if (end) std::memcpy(end, en.data(), sizeof(int32_t) * s->ncells);
    return PBF_OK;
}

pbf_status pbf_get_solver(pbf_sim* s, float* lambda_sorted, float* xpred4_sorted) {
    if (!s) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sim is NULL");
    DeviceGuard dg(s->device);
    if (xpred4_sorted)
        PBF_CUDA(s, cudaMemcpyAsync(xpred4_sorted, s->XP, sizeof(float4) * s->n,
                                    cudaMemcpyDeviceToHost, s->stream));
    if (lambda_sorted) {
        std::vector<float4> l(s->n);
        PBF_CUDA(s, cudaMemcpyAsync(l.data(), s->L, sizeof(float4) * s->n, cudaMemcpyDeviceToHost,
                                    s->stream));
        pbf_status r = check_status(s);
        if (r != PBF_OK) return r;
        for (uint32_t i = 0; i < s->n; ++i) lambda_sorted[i] = l[i].w;
        return PBF_OK;
    }
    return check_status(s);
}

pbf_status pbf_compute_diagnostics(pbf_sim* s, pbf_diagnostics* out) {
    NvtxRange nvtx_("pbf_compute_diagnostics");
    if (!s || !out) return fail(s, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    DeviceGuard dg(s->device);
    const uint32_t n = s->n;
    const unsigned g = grid_for(n);
    cudaStream_t st = s->stream;
    k_unmark_cells<<<g, kBlock, 0, st>>>(s->skeys, n, s->ncells, s->cstart);
    if (s->nscenes == 1)
        launch_keys_of(g, st, s->x, s->xstar, s->keys, n, OneScene{s->dc});
    else
        launch_keys_of(g, st, s->x, s->xstar, s->keys, n, ManyScenes{s->d_consts, s->sid});
    cudaError_t e = sort_pairs(s->sort, s->keys, s->skeys, s->perm, n, s->numbits, s->status, st);
    if (e != cudaSuccess) return cuda_fail(s, e, "diagnostics sort");
    k_find_cells<<<g, kBlock, 0, st>>>(s->skeys, s->perm, s->xstar, s->XP, n, s->ncells, s->cstart,
                                       s->cend, s->status + 1, s->sid, s->sid_sorted,
                                       ScanPos{nullptr, nullptr}, nullptr, nullptr);
    if (s->nscenes == 1)
        launch_diagnostics(g, st, s->XP, s->v, s->skeys, s->perm, s->cstart, s->cend,
                                            s->VX, n, OneScene{s->dc});
    else
        launch_diagnostics(g, st, s->XP, s->v, s->skeys, s->perm, s->cstart, s->cend,
                                            s->VX, n, ManyScenes{s->d_consts, s->sid_sorted});
    PBF_CUDA(s, cudaGetLastError());
    std::vector<float4> h(n);
    PBF_CUDA(s, cudaMemcpyAsync(h.data(), s->VX, sizeof(float4) * n, cudaMemcpyDeviceToHost, st));
    pbf_status r = check_status(s);
    if (r != PBF_OK) return r;
    double se = 0, me = 0, ke = 0, cand = 0;
    for (uint32_t i = 0; i < n; ++i) {
        se += h[i].x;
        me = me > h[i].x ? me : h[i].x;
        ke += h[i].y;
        cand += h[i].z;
    }
    out->mean_density_error = se / n;
    out->max_density_error = me;
    out->kinetic_energy = ke;
    out->candidate_pairs = cand;
    return PBF_OK;
}

// ---- standalone stages ------------------------------------------------------

namespace {

struct CachedSortScratch {
    void* mem = nullptr;
    uint32_t capacity = 0;
    uint32_t* keys_scratch = nullptr;
    uint32_t* status = nullptr;
    SortWorkspace ws;
};
std::mutex g_scratch_mu;
std::map<int, CachedSortScratch> g_scratch;

}  // namespace

pbf_status pbf_radix_sort(const uint32_t* keys_in, uint32_t* keys_out, uint32_t* perm_out,
                          uint32_t n, uint32_t numbits, void* stream) {
    if (n == 0) return PBF_OK;
    if (!keys_in || !perm_out) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "keys_in and perm_out are required");
    if (n >= (1u << 30)) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "n must be below 2^30");
    if (numbits < 1 || numbits > 32) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "numbits must be in [1, 32]");
    // The sort reads its key buffer once per pass and writes keys and ids in
    // the same final pass: no output may alias keys_in or the other output.
    if ((const void*)perm_out == (const void*)keys_in ||
        (keys_out && (const void*)keys_out == (const void*)keys_in))
        return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "outputs must not alias keys_in");
    if (keys_out && (const void*)keys_out == (const void*)perm_out)
        return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "keys_out must not alias perm_out");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(nullptr, PBF_ERR_NO_DEVICE, "no CUDA device");
    cudaStream_t st = (cudaStream_t)stream;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    CachedSortScratch& c = g_scratch[dev];
    if (c.capacity < n) {
        if (c.mem) {
            cudaDeviceSynchronize();
            cudaFree(c.mem);
            c.mem = nullptr;
            c.capacity = 0;
        }
        const size_t wsb = (SortWorkspace::bytes_for(n) + 255) & ~size_t(255);
        const size_t bytes = wsb + sizeof(uint32_t) * (size_t)n + 256;
        cudaError_t e = cudaMalloc(&c.mem, bytes);
        if (e != cudaSuccess) return cuda_fail(nullptr, e, "sort scratch allocation");
        c.capacity = n;
        c.ws.carve(c.mem, n);
        c.keys_scratch = (uint32_t*)((uint8_t*)c.mem + wsb);
        c.status = (uint32_t*)((uint8_t*)c.keys_scratch + sizeof(uint32_t) * (size_t)n);
    }
    uint32_t* kout = keys_out ? keys_out : c.keys_scratch;
    cudaError_t e = cudaMemsetAsync(c.status, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = sort_pairs(c.ws, keys_in, kout, perm_out, n, numbits, c.status, st);
    uint32_t bits = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, c.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "pbf_radix_sort");
    if (bits & kDevSortTimeout) return fail(nullptr, PBF_ERR_DEVICE_FAULT, "radix-sort lookback timed out");
    return PBF_OK;
}

pbf_status pbf_find_cells(const uint32_t* sorted_keys, uint32_t n, uint32_t num_cells, int32_t* start,
                          int32_t* end, void* stream) {
    if (!start || !end || num_cells == 0) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "start, end and num_cells are required");
    if (n > 0 && !sorted_keys) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sorted_keys is NULL");
    if (num_cells > 0x7FFFFFFFu || n > 0x7FFFFFFFu) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "sizes above 2^31-1");
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t* bad = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&bad, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(start, 0xFF, sizeof(int32_t) * (size_t)num_cells, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(end, 0xFF, sizeof(int32_t) * (size_t)num_cells, st);
    if (e == cudaSuccess && n > 0) {
        k_find_cells<<<grid_for(n), kBlock, 0, st>>>(sorted_keys, nullptr, nullptr, nullptr, n,
                                                     num_cells, start, end, bad, nullptr, nullptr,
                                                     ScanPos{nullptr, nullptr}, nullptr, nullptr);
        e = cudaGetLastError();
    }
    uint32_t hbad = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, bad, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (bad) cudaFreeAsync(bad, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "pbf_find_cells");
    if (hbad) return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "a sorted key is >= num_cells");
    return PBF_OK;
}

pbf_status pbf_highlight_neighbours(pbf_sim* s, uint32_t* flags, int where) {
    if (!s || !flags) return fail(s, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (where != PBF_HOST && where != PBF_DEVICE) return fail(s, PBF_ERR_INVALID_ARGUMENT, "bad where");
    DeviceGuard dg(s->device);
    cudaStream_t st = s->stream;
    const size_t b = sizeof(uint32_t) * s->n;
    uint32_t* d = flags;
    if (where == PBF_HOST) {
        PBF_CUDA(s, cudaMallocAsync((void**)&d, b, st));
        PBF_CUDA(s, cudaMemcpyAsync(d, flags, b, cudaMemcpyHostToDevice, st));
    }
    const unsigned g = grid_for(s->n);
    // the sorted particle's scene for batches comes from the sorted scene ids
    if (s->nscenes == 1)
        launch_highlight(g, st, s->XP, s->perm, s->cstart, s->cend, d, s->n, OneScene{s->dc});
    else
        launch_highlight(g, st, s->XP, s->perm, s->cstart, s->cend, d, s->n,
                         ManyScenes{s->d_consts, s->sid_sorted});
    PBF_CUDA(s, cudaGetLastError());
    if (where == PBF_HOST) {
        PBF_CUDA(s, cudaMemcpyAsync(flags, d, b, cudaMemcpyDeviceToHost, st));
        PBF_CUDA(s, cudaFreeAsync(d, st));
    }
    return check_status(s);
}

// Snapshot file: "PBFSTATE" magic, u32 format version 1, u32 particle count,
// u32 scene count, u32 reserved, then x and v as float4[n] (id order),
// little-endian.
pbf_status pbf_save_state(pbf_sim* s, const char* path) {
    if (!s || !path) return fail(s, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    std::vector<float> x(4ull * s->n), v(4ull * s->n);
    pbf_status r = pbf_get_state(s, x.data(), v.data(), PBF_HOST);
    if (r != PBF_OK) return r;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(s, PBF_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    const uint32_t hdr[4] = {1u, s->n, s->nscenes, 0u};
    bool ok = std::fwrite("PBFSTATE", 1, 8, f) == 8 && std::fwrite(hdr, 4, 4, f) == 4 &&
              std::fwrite(x.data(), 4, x.size(), f) == x.size() &&
              std::fwrite(v.data(), 4, v.size(), f) == v.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? PBF_OK : fail(s, PBF_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
}

pbf_status pbf_load_state(pbf_sim* s, const char* path) {
    if (!s || !path) return fail(s, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(s, PBF_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    char magic[8];
    uint32_t hdr[4];
    std::vector<float> x(4ull * s->n), v(4ull * s->n);
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "PBFSTATE", 8) == 0 &&
              std::fread(hdr, 4, 4, f) == 4 && hdr[0] == 1u && hdr[1] == s->n &&
              std::fread(x.data(), 4, x.size(), f) == x.size() &&
              std::fread(v.data(), 4, v.size(), f) == v.size() && std::fgetc(f) == EOF;
    std::fclose(f);
    if (!ok) return fail(s, PBF_ERR_INVALID_ARGUMENT, std::string("not a snapshot of this handle: ") + path);
    return pbf_set_state(s, x.data(), v.data(), PBF_HOST);
}

void pbf_debug_fail_allocation(int after) { g_fail_alloc_after.store(after < 0 ? -1 : after); }

const char* pbf_last_error(const pbf_sim* s) {
    if (s) return s->err.c_str();
    return g_error.c_str();
}

}  // extern "C"
