// substep.cuh — stage kernels of one PBF substep (definitions in substep.cu).
#pragma once

#include "common.cuh"

namespace pbf {

__global__ void k_predict(const float4* __restrict__ x, const float4* __restrict__ v,
                          float4* __restrict__ xstar, uint32_t* __restrict__ keys, uint32_t n,
                          DevConsts c, uint32_t* status);
__global__ void k_keys_of(const float4* __restrict__ x, float4* __restrict__ xstar,
                          uint32_t* __restrict__ keys, uint32_t n, DevConsts c);
__global__ void k_unmark_cells(const uint32_t* __restrict__ prev_sorted, uint32_t n,
                               uint32_t ncells, int32_t* __restrict__ cstart);
__global__ void k_find_cells(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ perm,
                             const float4* __restrict__ xstar, float4* __restrict__ P0, uint32_t n,
                             uint32_t ncells, int32_t* __restrict__ cstart,
                             int32_t* __restrict__ cend, uint32_t* bad);
__global__ void k_lambda_build(const float4* __restrict__ XP, const uint32_t* __restrict__ skeys,
                               const int32_t* __restrict__ cstart, const int32_t* __restrict__ cend,
                               float4* __restrict__ L, NbrLists nl, uint32_t n, DevConsts c);
__global__ void k_lambda(const float4* __restrict__ P, const float4* __restrict__ XP,
                         const uint32_t* __restrict__ skeys, const int32_t* __restrict__ cstart,
                         const int32_t* __restrict__ cend, float4* __restrict__ L, NbrLists nl,
                         int dmax_slot, uint32_t n, DevConsts c);
__global__ void k_delta_p(const float4* __restrict__ L, const float4* __restrict__ XP,
                          const uint32_t* __restrict__ skeys, const int32_t* __restrict__ cstart,
                          const int32_t* __restrict__ cend, float4* __restrict__ Pn, NbrLists nl,
                          int dmax_slot, int out_slot, uint32_t n, DevConsts c, uint32_t* status);
__global__ void k_commit(const float4* __restrict__ P, const uint32_t* __restrict__ perm,
                         float4* __restrict__ x, float4* __restrict__ VS,
                         float4* __restrict__ v_out, uint32_t n, DevConsts c);
__global__ void k_vorticity_a(const float4* __restrict__ P, const float4* __restrict__ XP,
                              const float4* __restrict__ VS, const uint32_t* __restrict__ skeys,
                              const int32_t* __restrict__ cstart, const int32_t* __restrict__ cend,
                              float4* __restrict__ VX, float4* __restrict__ OM,
                              float4* __restrict__ Q, NbrLists nl, int dmax_slot, uint32_t n,
                              DevConsts c);
__global__ void k_vorticity_b(const float4* __restrict__ Q, const float4* __restrict__ XP,
                              const float4* __restrict__ VX, const float4* __restrict__ OM,
                              const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ perm,
                              const int32_t* __restrict__ cstart, const int32_t* __restrict__ cend,
                              float4* __restrict__ v, NbrLists nl, int dmax_slot, uint32_t n,
                              DevConsts c);
__global__ void k_diagnostics(const float4* __restrict__ P, const float4* __restrict__ v,
                              const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ perm,
                              const int32_t* __restrict__ cstart, const int32_t* __restrict__ cend,
                              float4* __restrict__ out, uint32_t n, DevConsts c);

}  // namespace pbf
