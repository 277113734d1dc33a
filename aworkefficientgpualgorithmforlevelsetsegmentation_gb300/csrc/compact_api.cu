// Kernel-level stream compaction on caller-owned device buffers: the C-ABI
// replacement of the reference's CudppCompact (code/gpuseg/code/src/cuda/
// Cuda.cpp:699-758), which wraps CUDPP 1.1's cudppCompact.
//
// Stable: dst receives src[i] for every i < n with valid[i] != 0, in index
// order.  Single pass with decoupled lookback over tiles of 4096 elements; the
// count is written to device memory (the reference copies it to the host
// after every 2^25-element chunk).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <string>

#include "common.cuh"
#include "lss.h"

namespace lss {

constexpr int kCompactThreads = 256;
constexpr int kCompactItems = 16;
constexpr int kCompactTile = kCompactThreads * kCompactItems;

struct CompactScratch {
    uint64_t* status;        // one word per tile, zero before the pass
    uint32_t* tile_counter;  // zero before the pass
    uint32_t* err;
};

__global__ void __launch_bounds__(kCompactThreads) k_compact_u32(const uint32_t* __restrict__ src,
                                                                 const uint32_t* __restrict__ valid,
                                                                 uint32_t* __restrict__ dst,
                                                                 uint64_t n,
                                                                 unsigned long long* count,
                                                                 CompactScratch sc) {
    __shared__ uint32_t s_tile;
    const uint64_t ntiles = (n + kCompactTile - 1) / kCompactTile;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(sc.tile_counter, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        __syncthreads();
        if (tile >= ntiles) break;
        const uint64_t base = (uint64_t)tile * kCompactTile + (uint64_t)threadIdx.x * kCompactItems;
        uint32_t flags = 0;
        for (int q = 0; q < kCompactItems; ++q)
            if (base + q < n && valid[base + q] != 0u) flags |= 1u << q;
        uint32_t total;
        const uint32_t off = block_exclusive_sum(__popc(flags), &total);
        const uint64_t prefix = tile_exclusive_prefix(sc.status, tile, total, sc.err);
        uint64_t o = prefix + off;
        for (int q = 0; q < kCompactItems; ++q)
            if (flags & (1u << q)) dst[o++] = src[base + q];
        if (tile == ntiles - 1 && threadIdx.x == 0) *count = prefix + total;
    }
}

// Launches the compaction with caller-provided (already zeroed) scratch.
cudaError_t launch_compact_u32(const uint32_t* src, const uint32_t* valid, uint32_t* dst, uint64_t n,
                               uint64_t* count, CompactScratch sc, cudaStream_t st) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t ntiles = (n + kCompactTile - 1) / kCompactTile;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ntiles, (uint64_t)sms * 4));
    k_compact_u32<<<grid, kCompactThreads, 0, st>>>(src, valid, dst, n, (unsigned long long*)count, sc);
    return cudaGetLastError();
}

uint64_t compact_status_words(uint64_t n) { return (n + kCompactTile - 1) / kCompactTile + 1; }

}  // namespace lss

extern "C" lss_status lss_compact_u32(const uint32_t* d_src, const uint32_t* d_valid, uint32_t* d_dst,
                                      uint64_t n, uint64_t* d_count, void* stream) {
    if (!d_src || !d_valid || !d_dst || !d_count) return LSS_ERR_INVALID_ARGUMENT;
    if (n >= (1ull << 40)) return LSS_ERR_CAPACITY;
    cudaStream_t st = (cudaStream_t)stream;
    if (n == 0) {
        return cudaMemsetAsync(d_count, 0, sizeof(uint64_t), st) == cudaSuccess ? LSS_OK : LSS_ERR_CUDA;
    }
    // Scratch: status words, tile counter and error word, stream-ordered.
    const uint64_t words = lss::compact_status_words(n);
    const size_t bytes = words * 8 + 16;
    void* scratch = nullptr;
    if (cudaMallocAsync(&scratch, bytes, st) != cudaSuccess) {
        cudaGetLastError();
        return LSS_ERR_OUT_OF_MEMORY;
    }
    lss::CompactScratch sc;
    sc.status = (uint64_t*)scratch;
    sc.tile_counter = (uint32_t*)((char*)scratch + words * 8);
    sc.err = sc.tile_counter + 1;
    lss_status s = LSS_OK;
    if (cudaMemsetAsync(scratch, 0, bytes, st) != cudaSuccess ||
        lss::launch_compact_u32(d_src, d_valid, d_dst, n, d_count, sc, st) != cudaSuccess)
        s = LSS_ERR_CUDA;
    uint32_t err = 0;
    if (s == LSS_OK && cudaMemcpyAsync(&err, sc.err, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        s = LSS_ERR_CUDA;
    cudaFreeAsync(scratch, st);
    if (s == LSS_OK && cudaStreamSynchronize(st) != cudaSuccess) s = LSS_ERR_CUDA;
    if (s == LSS_OK && err) s = LSS_ERR_TIMEOUT;
    return s;
}

// ---------------------------------------------------------------------------
// Allocation-free variant.
//
// Some callers cannot allocate device memory at the moment they need a
// compaction: real-time pipelines whose device memory is reserved once at
// start-up, or hosts whose allocator is owned by another framework (a
// cudaMalloc of their own would bypass its pool or its accounting).  For
// them lss_compact_u32_noalloc keeps its scratch in this file-scope device
// array instead of asking the stream-ordered allocator.  Every GPU that loads
// the library holds the array (a little over 128 KiB) until the process exits.
// The call reads the error word back and synchronises its stream before it
// returns.
namespace lss {

// Largest n the allocation-free call accepts.
constexpr uint64_t kNoAllocMaxElements = 1ull << 26;
constexpr uint64_t kNoAllocStatusWords = kNoAllocMaxElements / kCompactTile + 1;

// Status words, then the tile counter and the error word (one u64).
static __device__ __align__(256) uint64_t g_noalloc_scratch[kNoAllocStatusWords + 1];

// Device address of the array, looked up once per device with that device
// current (in host code the symbol is only a host-side stand-in).
static std::mutex g_noalloc_mu;
static uint64_t* g_noalloc_addr[64] = {nullptr};

static lss_status noalloc_scratch(uint64_t** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return LSS_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return LSS_ERR_CUDA;
        }
        g_noalloc_addr[dev] = (uint64_t*)p;
    }
    *out = g_noalloc_addr[dev];
    return LSS_OK;
}

}  // namespace lss

extern "C" lss_status lss_compact_u32_noalloc(const uint32_t* d_src, const uint32_t* d_valid,
                                              uint32_t* d_dst, uint64_t n, uint64_t* d_count,
                                              void* stream) {
    if (!d_src || !d_valid || !d_dst || !d_count) return LSS_ERR_INVALID_ARGUMENT;
    if (n > lss::kNoAllocMaxElements) return LSS_ERR_CAPACITY;
    cudaStream_t st = (cudaStream_t)stream;
    if (n == 0)
        return cudaMemsetAsync(d_count, 0, sizeof(uint64_t), st) == cudaSuccess ? LSS_OK : LSS_ERR_CUDA;
    uint64_t* base = nullptr;
    lss_status s = lss::noalloc_scratch(&base);
    if (s != LSS_OK) return s;
    const uint64_t words = lss::compact_status_words(n);  // <= kNoAllocStatusWords
    lss::CompactScratch sc;
    sc.status = base;
    sc.tile_counter = (uint32_t*)(base + lss::kNoAllocStatusWords);
    sc.err = sc.tile_counter + 1;
    // The array keeps the previous call's contents: clear the words this call
    // reads before writing them, plus the tile counter and the error word.
    if (cudaMemsetAsync(base, 0, words * 8, st) != cudaSuccess ||
        cudaMemsetAsync(sc.tile_counter, 0, 8, st) != cudaSuccess ||
        lss::launch_compact_u32(d_src, d_valid, d_dst, n, d_count, sc, st) != cudaSuccess) {
        cudaGetLastError();
        return LSS_ERR_CUDA;
    }
    uint32_t err = 0;
    if (cudaMemcpyAsync(&err, sc.err, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return LSS_ERR_CUDA;
    }
    return err ? LSS_ERR_TIMEOUT : LSS_OK;
}
