// sort.cu — stable onesweep LSD radix sort of 32-bit cell keys with a 32-bit
// payload (the particle id), replacing the reference's 2-bit-per-pass
// RadixSort (src/RadixSort.cpp:124-200, shaders/radixsort/*.glsl).
//
// Design (GB300): 8-bit digits, so a 2^24-cell grid sorts in 3 passes where
// the reference needs 12.  One upfront kernel histograms every pass's digits;
// each pass is then a single kernel: a CTA claims a 4096-key tile from an
// atomic counter, ranks its keys stably with warp match/ballot, publishes its
// per-digit counts and resolves its global offsets by decoupled lookback over
// earlier tiles, then scatters through shared memory so each digit's keys
// leave as one contiguous run.  The lookback spin is bounded: on expiry the
// kernel latches kDevSortTimeout in the status word and finishes instead of
// hanging.
//
// Stability: inside a tile, keys are ranked in element order; across tiles,
// offsets follow tile order.  Pass 0 reads the ids implicitly (id = element
// index), so the result is the permutation that orders (key, id), exactly the
// order the reference's stable passes give on its id-ordered input.
#include "sort.cuh"
#include "common.cuh"
#include "internal.h"

#include <atomic>
#include <mutex>
#include <string>

#include "../../include/pbf.h"

#include <algorithm>

namespace pbf {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kItems = 16;
constexpr uint32_t kTile = kSortThreads * kItems;  // 4096 keys
static_assert(kTile == kSortTile, "tile size");
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
constexpr uint32_t kSpinLimit = 1u << 22;

// Test hook (pbf_debug_sort_stall): when nonzero, every onesweep pass
// launched afterwards looks back at a scratch word nothing sets, with this
// spin limit, so each tile after the first gives up and latches
// kDevSortTimeout: the timeout path runs without a real stall.
std::atomic<uint32_t> g_stall_spins{0};

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Mask of pass p's digit: only bits [0, numbits) take part in the sort.
__host__ __device__ __forceinline__ uint32_t digit_mask(uint32_t numbits, uint32_t p) {
    const uint32_t rem = numbits - 8 * p;
    return rem >= 8 ? 255u : ((1u << rem) - 1u);
}

__device__ __forceinline__ uint32_t load_volatile(const uint32_t* p) {
    return *(const volatile uint32_t*)p;
}
__device__ __forceinline__ void store_volatile(uint32_t* p, uint32_t v) {
    *(volatile uint32_t*)p = v;
}

// Digit histograms of all passes in one read of the keys.
__global__ void __launch_bounds__(kSortThreads)
k_sort_histogram(const uint32_t* __restrict__ keys, uint32_t n, uint32_t passes, uint32_t numbits,
                 uint32_t* __restrict__ hist) {
    __shared__ uint32_t s_hist[kMaxPasses][256];
    for (uint32_t i = threadIdx.x; i < kMaxPasses * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t k = keys[i];
        for (uint32_t p = 0; p < passes; ++p)
            atomicAdd(&s_hist[p][(k >> (8 * p)) & digit_mask(numbits, p)], 1u);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        uint32_t c = (&s_hist[0][0])[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// Exclusive scan of each pass's 256 digit counts; one CTA per pass.
__global__ void __launch_bounds__(256) k_sort_digit_base(uint32_t* __restrict__ hist) {
    __shared__ uint32_t s_warp[8];
    uint32_t* h = hist + blockIdx.x * 256;
    const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t v = h[t];
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (uint32_t)o) inc += y;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    uint32_t wbase = 0;
    for (uint32_t w = 0; w < warp; ++w) wbase += s_warp[w];
    h[t] = wbase + inc - v;
}

// One onesweep pass over `n` keys.  vin == nullptr means the payload is the
// element index.
__global__ void __launch_bounds__(kSortThreads)
k_onesweep(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
           uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, uint32_t n, uint32_t shift,
           uint32_t dmask, const uint32_t* __restrict__ digit_base, uint32_t* tile_status, uint32_t* tile_counter,
           uint32_t* status, const uint32_t* stall_word, uint32_t spin_limit) {
    __shared__ uint32_t s_k[kTile];
    __shared__ uint32_t s_v[kTile];
    __shared__ uint32_t s_wh[kSortWarps][256];
    __shared__ uint32_t s_dstart[256];
    __shared__ uint32_t s_goff[256];
    __shared__ uint32_t s_wsum[kSortWarps];
    __shared__ uint32_t s_tile;

    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
    for (uint32_t i = tid; i < kSortWarps * 256; i += kSortThreads) (&s_wh[0][0])[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t tile_base = (uint64_t)tile * kTile;
    const uint64_t wbase = tile_base + (uint64_t)warp * (kItems * 32);

    uint32_t key[kItems], val[kItems], rank[kItems];
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const uint64_t e = wbase + (uint64_t)k * 32 + lane;
        const bool valid = e < n;
        key[k] = valid ? kin[e] : 0u;
        val[k] = valid ? (vin ? vin[e] : (uint32_t)e) : 0u;
    }
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const uint64_t e = wbase + (uint64_t)k * 32 + lane;
        const bool valid = e < n;
        const uint32_t d = (key[k] >> shift) & dmask;
        const uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : 256u);
        const uint32_t before = valid ? s_wh[warp][d] : 0u;
        __syncwarp();
        if (valid) {
            rank[k] = before + __popc(peers & lt);
            if (lane == (uint32_t)(__ffs(peers) - 1)) s_wh[warp][d] = before + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();

    // Thread d owns digit d: warp offsets inside the tile, tile count.
    const uint32_t d = tid;
    uint32_t count = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
        uint32_t c = s_wh[w][d];
        s_wh[w][d] = count;
        count += c;
    }
    uint32_t* my_status = tile_status + (uint64_t)tile * 256 + d;
    store_volatile(my_status, (tile == 0 ? kFlagPrefix : kFlagAgg) | count);

    // Tile-local digit starts: exclusive scan of the counts over digits.
    uint32_t inc = count;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (uint32_t)o) inc += y;
    }
    if (lane == 31) s_wsum[warp] = inc;
    __syncthreads();
    uint32_t wb = 0;
    for (uint32_t w = 0; w < warp; ++w) wb += s_wsum[w];
    const uint32_t dstart = wb + inc - count;
    s_dstart[d] = dstart;

    // Decoupled lookback over earlier tiles for digit d.
    uint32_t excl = 0;
    if (tile > 0) {
        int64_t t = (int64_t)tile - 1;
        while (t >= 0) {
            const uint32_t* ps = stall_word ? stall_word : tile_status + (uint64_t)t * 256 + d;
            uint32_t s = load_volatile(ps);
            uint32_t spins = 0;
            while ((s & ~kValueMask) == 0u) {
                if (++spins > spin_limit) {
                    atomicOr(status, kDevSortTimeout);
                    s = kFlagPrefix;  // give up: results are invalid, the status says so
                    break;
                }
                if (spins > 32) __nanosleep(64);
                s = load_volatile(ps);
            }
            excl += s & kValueMask;
            if ((s & ~kValueMask) == kFlagPrefix) break;
            --t;
        }
        store_volatile(my_status, kFlagPrefix | ((excl + count) & kValueMask));
    }
    s_goff[d] = digit_base[d] + excl - dstart;
    __syncthreads();

#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const uint64_t e = wbase + (uint64_t)k * 32 + lane;
        if (e < n) {
            const uint32_t dk = (key[k] >> shift) & dmask;
            const uint32_t pos = s_dstart[dk] + s_wh[warp][dk] + rank[k];
            s_k[pos] = key[k];
            s_v[pos] = val[k];
        }
    }
    __syncthreads();

    const uint64_t left = (uint64_t)n - tile_base;
    const uint32_t cnt = left < kTile ? (uint32_t)left : kTile;
    for (uint32_t i = tid; i < cnt; i += kSortThreads) {
        const uint32_t kk = s_k[i];
        const uint32_t dst = s_goff[(kk >> shift) & dmask] + i;
        // Always true unless a lookback timed out; keeps a failed sort in bounds.
        if (dst < n) {
            kout[dst] = kk;
            vout[dst] = s_v[i];
        }
    }
}

}  // namespace

uint32_t sort_numbits_for_cells(uint64_t ncells) {
    // count_sortbits(ncells - 1) (src/RadixSort.cpp:24-30, :44)
    uint64_t v = ncells > 0 ? ncells - 1 : 0;
    uint32_t r = 1;
    while (v >>= 1) r++;
    return r;
}

size_t SortWorkspace::bytes_for(uint32_t n) { return sort_ws_bytes(n); }

void SortWorkspace::carve(void* base, uint32_t n) {
    capacity = n;
    tiles_max = (n + kTile - 1) / kTile;
    uint8_t* p = (uint8_t*)base;
    hist = (uint32_t*)p;
    p += sizeof(uint32_t) * kMaxPasses * 256;
    counters = (uint32_t*)p;
    p += sizeof(uint32_t) * kMaxPasses * 32;
    tile_status = (uint32_t*)p;
    p += sizeof(uint32_t) * kMaxPasses * 256 * (size_t)tiles_max;
    p = (uint8_t*)(((uintptr_t)p + 255) & ~uintptr_t(255));
    reset_bytes = (size_t)(p - (uint8_t*)base);
    ktmp = (uint32_t*)p;
    p += sizeof(uint32_t) * (size_t)n;
    vtmp = (uint32_t*)p;
}

cudaError_t sort_pairs(const SortWorkspace& ws, const uint32_t* keys_in, uint32_t* keys_out,
                       uint32_t* vals_out, uint32_t n, uint32_t numbits, uint32_t* status,
                       cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const uint32_t passes = std::min<uint32_t>((numbits + 7) / 8, kMaxPasses);
    const uint32_t tiles = (n + kTile - 1) / kTile;
    cudaError_t err = cudaMemsetAsync(ws.hist, 0, ws.reset_bytes, stream);
    if (err != cudaSuccess) return err;
    const unsigned hgrid = std::min<unsigned>((n + 4095) / 4096, 4u * 152u);
    k_sort_histogram<<<hgrid, kSortThreads, 0, stream>>>(keys_in, n, passes, numbits, ws.hist);
    k_sort_digit_base<<<passes, 256, 0, stream>>>(ws.hist);
    // Pass p writes to the final buffers when (passes - 1 - p) is even, so the
    // last pass always lands in keys_out / vals_out and no pass reads the
    // buffer it writes.
    const uint32_t* ksrc = keys_in;
    const uint32_t* vsrc = nullptr;
    const uint32_t stall = g_stall_spins.load();
    for (uint32_t p = 0; p < passes; ++p) {
        const bool to_final = ((passes - 1 - p) % 2) == 0;
        uint32_t* kdst = to_final ? keys_out : ws.ktmp;
        uint32_t* vdst = to_final ? vals_out : ws.vtmp;
        k_onesweep<<<tiles, kSortThreads, 0, stream>>>(
            ksrc, vsrc, kdst, vdst, n, 8 * p, digit_mask(numbits, p), ws.hist + p * 256,
            ws.tile_status + (size_t)p * 256 * ws.tiles_max, ws.counters + p * 32, status,
            // a word of the pass's counter block that stays zero (only word 0 counts tiles)
            stall ? ws.counters + p * 32 + 16 : nullptr, stall ? stall : kSpinLimit);
        ksrc = kdst;
        vsrc = vdst;
    }
    return cudaGetLastError();
}

}  // namespace pbf

extern "C" void pbf_debug_sort_stall(uint32_t spins) { pbf::g_stall_spins.store(spins); }

// ---- allocation-free variant -------------------------------------------------
//
// For callers that must not allocate device memory: a library embedded in a
// host application whose own allocator has reserved all of the GPU's memory
// (a cudaMalloc here would fail or take memory from its pool), or a
// real-time loop that may not stall on the allocator's implicit
// synchronisation.  The
// sort's scratch (digit histograms, lookback status, ping-pong buffers, a key
// buffer for callers that want no sorted keys, the status word) lives in one
// file-scope device array sized for at most kNoAllocMaxKeys keys.  Every GPU
// that loads the library holds this array (about 13.6 MB) until the process
// exits.

static constexpr uint32_t kNoAllocMaxKeys = 1u << 20;
static constexpr size_t kNoAllocWsBytes = pbf::sort_ws_bytes(kNoAllocMaxKeys);
static constexpr size_t kNoAllocBytes =
    kNoAllocWsBytes + sizeof(uint32_t) * kNoAllocMaxKeys + 256;  // + key buffer + status
static constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) uint8_t g_sort_scratch[kNoAllocBytes];

// Host code cannot use g_sort_scratch's name as a device address; the address
// is looked up once per device (with that device current) and cached for the
// life of the process, so a cudaDeviceReset after the first call on a device
// is not supported (the module would be reloaded at another address).
static std::mutex g_sort_scratch_mu;
static void* g_sort_scratch_addr[kNoAllocMaxDevices] = {};

static cudaError_t sort_scratch_address(int dev, void** out) {
    std::lock_guard<std::mutex> lock(g_sort_scratch_mu);
    if (!g_sort_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess) return e;
        g_sort_scratch_addr[dev] = p;
    }
    *out = g_sort_scratch_addr[dev];
    return cudaSuccess;
}

static pbf_status noalloc_fail(pbf_status st, const std::string& msg) {
    pbf::set_last_error(msg.c_str());
    return st;
}

extern "C" pbf_status pbf_radix_sort_noalloc(const uint32_t* keys_in, uint32_t* keys_out,
                                             uint32_t* perm_out, uint32_t n, uint32_t numbits,
                                             void* stream) {
    if (n == 0) return PBF_OK;
    if (!keys_in || !perm_out)
        return noalloc_fail(PBF_ERR_INVALID_ARGUMENT, "keys_in and perm_out are required");
    if (numbits < 1 || numbits > 32)
        return noalloc_fail(PBF_ERR_INVALID_ARGUMENT, "numbits must be in [1, 32]");
    if (n > kNoAllocMaxKeys)
        return noalloc_fail(PBF_ERR_INVALID_ARGUMENT,
                            "n = " + std::to_string(n) +
                                " exceeds the allocation-free sort's limit of " +
                                std::to_string(kNoAllocMaxKeys) + " keys");
    if ((const void*)perm_out == (const void*)keys_in ||
        (keys_out && (const void*)keys_out == (const void*)keys_in))
        return noalloc_fail(PBF_ERR_INVALID_ARGUMENT, "outputs must not alias keys_in");
    if (keys_out && (const void*)keys_out == (const void*)perm_out)
        return noalloc_fail(PBF_ERR_INVALID_ARGUMENT, "keys_out must not alias perm_out");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return noalloc_fail(PBF_ERR_NO_DEVICE, "no CUDA device");
    }
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return noalloc_fail(PBF_ERR_UNSUPPORTED, "device ordinal above 63");
    void* base = nullptr;
    cudaError_t e = sort_scratch_address(dev, &base);
    if (e != cudaSuccess)
        return noalloc_fail(PBF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    pbf::SortWorkspace ws;
    ws.carve(base, kNoAllocMaxKeys);
    uint32_t* key_buf = (uint32_t*)((uint8_t*)base + kNoAllocWsBytes);
    uint32_t* status = key_buf + kNoAllocMaxKeys;
    uint32_t* kout = keys_out ? keys_out : key_buf;
    cudaStream_t st = (cudaStream_t)stream;
    // The array keeps the previous call's contents: the status word is
    // cleared here and sort_pairs clears its histograms, tile counters and
    // lookback words before use.
    uint32_t bits = 0;
    e = cudaMemsetAsync(status, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = pbf::sort_pairs(ws, keys_in, kout, perm_out, n, numbits, status, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return noalloc_fail(PBF_ERR_CUDA, std::string("pbf_radix_sort_noalloc: ") + cudaGetErrorString(e));
    if (bits & pbf::kDevSortTimeout)
        return noalloc_fail(PBF_ERR_DEVICE_FAULT, "radix-sort lookback timed out");
    return PBF_OK;
}
