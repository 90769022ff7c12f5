// sort.cuh — onesweep radix sort of (32-bit key, 32-bit payload) pairs.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace pbf {

constexpr uint32_t kMaxPasses = 4;     // 8-bit digits, 32-bit keys
constexpr uint32_t kSortTile = 4096;   // keys per onesweep tile

// Bytes of the workspace SortWorkspace::carve lays out for up to n keys.
constexpr size_t sort_ws_bytes(uint32_t n) {
    const size_t tiles = ((size_t)n + kSortTile - 1) / kSortTile;
    size_t b = sizeof(uint32_t) * kMaxPasses * 256        // hist / digit base
               + sizeof(uint32_t) * kMaxPasses * 32       // tile counters (padded)
               + sizeof(uint32_t) * kMaxPasses * 256 * tiles;  // lookback status
    b = (b + 255) & ~size_t(255);
    return b + 2 * sizeof(uint32_t) * (size_t)n;          // ping-pong keys + values
}

// Device scratch of one sort: digit histograms, per-pass tile counters and
// lookback status words (reset before every sort), and ping-pong buffers.
struct SortWorkspace {
    uint32_t* hist = nullptr;         // [kMaxPasses][256]; becomes digit bases
    uint32_t* counters = nullptr;     // [kMaxPasses][32]
    uint32_t* tile_status = nullptr;  // [kMaxPasses][tiles_max][256]
    uint32_t* ktmp = nullptr;         // [capacity]
    uint32_t* vtmp = nullptr;         // [capacity]
    size_t reset_bytes = 0;           // bytes from hist that are zeroed per sort
    uint32_t capacity = 0;
    uint32_t tiles_max = 0;

    static size_t bytes_for(uint32_t n);
    void carve(void* base, uint32_t n);
};

// bitlength(ncells - 1), at least 1: RadixSort's numbits (src/RadixSort.cpp:24-30,44).
uint32_t sort_numbits_for_cells(uint64_t ncells);

// Stable sort of keys_in[0..n) on bits [0, numbits): keys_out receives the
// sorted keys, vals_out the input index of each.  keys_in is not modified;
// keys_out and vals_out must not alias keys_in or the workspace.  n < 2^30.
cudaError_t sort_pairs(const SortWorkspace& ws, const uint32_t* keys_in, uint32_t* keys_out,
                       uint32_t* vals_out, uint32_t n, uint32_t numbits, uint32_t* status,
                       cudaStream_t stream);

}  // namespace pbf
