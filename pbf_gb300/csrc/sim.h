// sim.h — the pbf_sim handle and the host helpers shared by api.cu and
// adjoint.cu (internal; not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/pbf.h"
#include "auto_policy.h"
#include "common.cuh"
#include "sort.cuh"

namespace pbf {
struct Tape;  // adjoint.cu
}

using pbf::DevConsts;
using pbf::SortWorkspace;

struct pbf_sim {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    pbf_params params{};  // scene 0; its iteration count and vorticity flag hold for all scenes
    DevConsts dc{};       // scene 0's constants (the kernel parameter of a single scene)
    uint32_t n = 0;
    uint32_t ncells = 0;  // all scenes
    uint32_t numbits = 0;
    // several scenes in one handle (pbf_create_batch): concatenated scene-major
    uint32_t nscenes = 1;
    std::vector<pbf_params> sparams;
    std::vector<DevConsts> sdc;
    std::vector<uint32_t> counts, offsets;
    DevConsts* d_consts = nullptr;  // [nscenes]
    uint32_t* sid = nullptr;        // scene of each particle, id order
    uint32_t* sid_sorted = nullptr; // scene of each particle, sorted order

    // id-order state and predicted positions
    float4 *x = nullptr, *v = nullptr, *xstar = nullptr;
    // sorted-order buffers
    float4 *XP = nullptr, *Pa = nullptr, *Pb = nullptr, *L = nullptr;
    float4 *VS = nullptr, *VX = nullptr, *OM = nullptr, *Q = nullptr;
    uint32_t *keys = nullptr, *skeys = nullptr, *perm = nullptr;
    int32_t *cstart = nullptr, *cend = nullptr;
    uint32_t* status = nullptr;  // device status word [0], bad-key flag [1]
    // neighbour lists (pbf_tuning)
    pbf_tuning tuning{};
    uint32_t* nbr_idx = nullptr;
    int32_t* nbr_cnt = nullptr;
    uint32_t* guard = nullptr;
    uint32_t nbr_cap = 0;       // capacity of nbr_idx in entries per particle
    uint32_t guard_slots = 0;
    // exact pair lists (PairLists), recorded and replayed within a substep
    uint32_t* pair_idx = nullptr;
    int32_t* pair_cnt = nullptr;
    uint32_t pair_cap = 0;
    // mixed sweeps (pbf_tuning::coop_candidates): per-particle flag, the
    // flagged sorted indices and their count
    uint8_t* heavy = nullptr;
    uint32_t* heavy_list = nullptr;
    uint32_t* heavy_count = nullptr;
    // run-start bits of the position set the direct sweeps read (k_find_cells,
    // k_run_flags), n / 32 + 2 words
    uint32_t* runs = nullptr;
    // scan copies (ScanPos) of the predicted positions (set 0) and of the
    // solver iterates (sets 1 and 2, alternating), (n + 1) / 2 pairs per set
    float4* scan_xy = nullptr;
    float2* scan_z = nullptr;
    uint32_t* h_status = nullptr;
    void* sort_mem = nullptr;
    SortWorkspace sort;

    // PBF_PASS_* configuration of the solver sweeps and the vorticity passes
    // the next substep runs; one captured graph per pair
    uint32_t pass_solver = 0, pass_vort = 0;
    cudaGraph_t graphs[25] = {};  // one per (solver pass, vorticity pass): 5 x 5
    cudaGraphExec_t execs[25] = {};

    // PBF_SWEEP_AUTO: the schedule and sit-outs (auto_policy.h), the
    // candidate the running trial steps next (-1: none), the trial's
    // candidates and their stage events
    pbf::AutoPolicy autop;
    int auto_trial = -1;
    std::vector<uint32_t> auto_cands;
    std::vector<cudaEvent_t> trial_ev;  // (7 + 2 * iterations) per candidate
    uint64_t launched = 0;  // kernels launched by substeps so far (pbf_kernels_launched)

    bool timing = false;
    std::vector<cudaEvent_t> ev;  // 7 + 2 * iterations stage boundaries
    float ms[5] = {};             // reference phases of the last timed substep
    double stage_ms[8] = {};      // stage sums since timing was enabled
    uint32_t timed_substeps = 0;

    pbf::Tape* tape = nullptr;  // recorded forward run for pbf_backward

    std::string err;
};

namespace pbf {

// Where a recorded substep stores what the adjoint needs (sorted order):
// L[k] = (x, y, z, lambda) and AUX[k] = (sum_j grad C_i, sum |grad C|^2 + |sum grad C|^2)
// of solver iteration k, the final positions, and the vorticity pass outputs.
struct Recording {
    float4* const* L = nullptr;    // [iterations]
    float4* const* AUX = nullptr;  // [iterations]
    float4* PF = nullptr;
    float4* VS = nullptr;
    float4* OM = nullptr;
    float4* Q = nullptr;
    float4* ETA = nullptr;
};

pbf_status fail(pbf_sim* s, pbf_status st, const std::string& msg);
pbf_status cuda_fail(pbf_sim* s, cudaError_t e, const char* what);
pbf_status check_status(pbf_sim* s);
// Enqueues one substep on s->stream; with `rec`, the stage outputs land in
// the recording's buffers.  `ev`: optional stage events (timing mode).
cudaError_t enqueue_substep(pbf_sim* s, cudaEvent_t* ev, const Recording* rec = nullptr);
void invalidate_graph(pbf_sim* s);
void free_tape(pbf_sim* s);

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev)
            cudaSetDevice(dev);
        else
            prev = -1;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

}  // namespace pbf

#define PBF_CUDA(s, call)                                                \
    do {                                                                 \
        cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) return ::pbf::cuda_fail((s), e_, #call);  \
    } while (0)
