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
