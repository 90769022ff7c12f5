// substep.cuh — stage kernels of one PBF substep (definitions and the
// explicit instantiations for OneScene / ManyScenes in substep.cu).
#pragma once

#include "common.cuh"

namespace pbf {

__global__ void k_unmark_cells(const uint32_t* __restrict__ prev_sorted, uint32_t n,
                               uint32_t ncells, int32_t* __restrict__ cstart);
__global__ void k_run_flags(const float4* __restrict__ P, uint32_t n, uint32_t* __restrict__ runs);
__global__ void k_run_flags_vals(const float4* __restrict__ A, const float4* __restrict__ B,
                                 int use_w, uint32_t n, uint32_t* __restrict__ runs);
__global__ void k_find_cells(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ perm,
                             const float4* __restrict__ xstar, float4* __restrict__ P0, uint32_t n,
                             uint32_t ncells, int32_t* __restrict__ cstart,
                             int32_t* __restrict__ cend, uint32_t* bad,
                             const uint32_t* __restrict__ sid, uint32_t* __restrict__ sid_sorted,
                             ScanPos sx, uint32_t* __restrict__ runs, uint32_t* status);

// Host launchers of the templated stage kernels (explicitly instantiated for
// OneScene and ManyScenes in substep.cu).  The neighbour-sweep launchers take
// their block size (32..256, a multiple of 32); the others take a grid of
// kBlock-thread blocks.
// Launch shape of the neighbour sweeps: threads per block; the stencil scan
// (0: the reference's loop shape, visit_full; 1: masked scans, visit_masked;
// 2: masked scans that record the exact pair lists the next sweep replays);
// whether the skin-radius neighbour lists are used.
struct SweepCfg {
    unsigned block;
    int mode;
    bool lists;
};

template <class CP>
void launch_predict(unsigned g, cudaStream_t st, const float4* x, const float4* v, float4* xstar,
                    uint32_t* keys, uint32_t n, CP cp, uint32_t* status);
template <class CP>
void launch_keys_of(unsigned g, cudaStream_t st, const float4* x, float4* xstar, uint32_t* keys,
                    uint32_t n, CP cp);
template <class CP>
void launch_lambda_build(SweepCfg sw, cudaStream_t st, const float4* XP, const uint32_t* skeys,
                         const int32_t* cstart, const int32_t* cend, float4* L, float4* aux,
                         NbrLists nl, PairLists pw, ScanPos sx, uint32_t n, CP cp);
template <class CP>
void launch_lambda(SweepCfg sw, cudaStream_t st, const float4* P, const float4* XP,
                   const uint32_t* skeys, const int32_t* cstart, const int32_t* cend, float4* L,
                   float4* aux, NbrLists nl, PairLists pw, ScanPos sx, int dmax_slot, uint32_t n,
                   CP cp);
template <class CP>
void launch_delta_p(SweepCfg sw, cudaStream_t st, const float4* L, const float4* XP,
                    const uint32_t* skeys, const int32_t* cstart, const int32_t* cend, float4* Pn,
                    NbrLists nl, PairLists pr, ScanPos sx, ScanPos sx_out, int dmax_slot,
                    int out_slot, uint32_t n, CP cp, uint32_t* status);
// Loads the sweep kernels the automatic configuration may launch.
template <class CP>
cudaError_t preload_sweeps();
template <class CP>
void launch_heavy_scan(unsigned g, cudaStream_t st, const float4* XP, const int32_t* cstart,
                       const int32_t* cend, uint32_t threshold, uint32_t n, CP cp, uint8_t* heavy,
                       uint32_t* list, uint32_t* count);
template <class CP>
void launch_commit(unsigned g, cudaStream_t st, const float4* P, const uint32_t* perm, float4* x,
                   float4* VS, float4* v_out, uint32_t n, CP cp);
template <class CP>
void launch_vorticity_a(SweepCfg sw, cudaStream_t st, const float4* P, const float4* XP,
                        const float4* VS, const uint32_t* skeys, const int32_t* cstart,
                        const int32_t* cend, float4* VX, float4* OM, float4* Q, NbrLists nl,
                        PairLists pw, ScanPos sx, int dmax_slot, uint32_t n, CP cp);
template <class CP>
void launch_vorticity_b(SweepCfg sw, cudaStream_t st, const float4* Q, const float4* XP,
                        const float4* VX, const float4* OM, const uint32_t* skeys,
                        const uint32_t* perm, const int32_t* cstart, const int32_t* cend,
                        float4* v, float4* eta_out, NbrLists nl, PairLists pr, ScanPos sx,
                        int dmax_slot, uint32_t n, CP cp);
template <class CP>
void launch_diagnostics(unsigned g, cudaStream_t st, const float4* P, const float4* v,
                        const uint32_t* skeys, const uint32_t* perm, const int32_t* cstart,
                        const int32_t* cend, float4* out, uint32_t n, CP cp);

template <class CP>
void launch_highlight(unsigned g, cudaStream_t st, const float4* XP, const uint32_t* perm,
                      const int32_t* cstart, const int32_t* cend, uint32_t* flags, uint32_t n,
                      CP cp);

}  // namespace pbf
