// Kernel-level stream compaction on caller-owned device buffers: the C-ABI
// replacement of the reference's CudppCompact (code/gpuseg/code/src/cuda/
// Cuda.cpp:699-758), which wraps CUDPP 1.1's cudppCompact.
//
// Stable: dst receives src[i] for every i < n with valid[i] != 0, in index
// order.  Single pass with decoupled lookback over tiles of 16384 elements
// (16-byte coalesced loads, a warp-parallel lookback); the count is written
// to device memory (the reference copies it to the host after every
// 2^25-element chunk).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <string>

#include "common.cuh"
#include "lss.h"

namespace lss {

constexpr int kCompactThreads = 1024;
constexpr int kCompactItems = 16;
constexpr int kCompactTile = kCompactThreads * kCompactItems;
constexpr int kCompactWarps = kCompactThreads / 32;
constexpr int kCompactSeg = kCompactTile / kCompactWarps;  // 512 elements a warp: 4 chunks of 128
// 16384-element tiles (1024 threads, one block an SM): at 2^28 elements
// 1.09 ms a call against 1.20 with 8192 (512 threads) and 1.25 with 4096
// (256 threads): fewer tiles in flight for each lookback to walk past.

struct CompactScratch {
    uint64_t* status;        // one word per tile, zero before the pass
    uint32_t* tile_counter;  // zero before the pass
    uint32_t* err;
};

// Stable compaction, tiles of kCompactTile elements taken from a tile counter (so
// every lookback waits on a resident block).  Warp w of a tile takes the 512
// elements [512 w, 512 w + 512) as four chunks of 128, lane l the four
// elements 4 l .. 4 l + 3 of each chunk, read as 16-byte loads (a warp's load
// is 512 contiguous bytes; all eight loads of a thread are issued before any
// is used).  Ranks: one warp inclusive scan of the four per-chunk counts
// packed into the bytes of a word (a chunk holds at most 128), the warps'
// totals by a block scan, the tile's prefix by warp 0's lookback.  A lane's
// kept elements go to consecutive places, after those of the lanes before
// it, so the stores of a chunk are contiguous too.  n need not be a multiple
// of 4: the tail is read element by element.
__global__ void __launch_bounds__(kCompactThreads) k_compact_u32(const uint32_t* __restrict__ src,
                                                                 const uint32_t* __restrict__ valid,
                                                                 uint32_t* __restrict__ dst,
                                                                 uint64_t n,
                                                                 unsigned long long* count,
                                                                 CompactScratch sc) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp[kCompactWarps];
    __shared__ uint64_t s_prefix;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t ntiles = (n + kCompactTile - 1) / kCompactTile;
    const bool vec = ((uintptr_t)src % 16 == 0) && ((uintptr_t)valid % 16 == 0);
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(sc.tile_counter, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        const uint64_t seg = (uint64_t)tile * kCompactTile + (uint64_t)warp * kCompactSeg;
        uint4 fv[4], sv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint64_t i = seg + (uint64_t)q * 128 + (uint64_t)lane * 4;
            if (vec && i + 4 <= n) {
                fv[q] = *reinterpret_cast<const uint4*>(valid + i);
                sv[q] = *reinterpret_cast<const uint4*>(src + i);
            } else {
                fv[q] = make_uint4(i < n ? valid[i] : 0u, i + 1 < n ? valid[i + 1] : 0u,
                                   i + 2 < n ? valid[i + 2] : 0u, i + 3 < n ? valid[i + 3] : 0u);
                sv[q] = make_uint4(i < n ? src[i] : 0u, i + 1 < n ? src[i + 1] : 0u, i + 2 < n ? src[i + 2] : 0u,
                                   i + 3 < n ? src[i + 3] : 0u);
            }
        }
        // Flags (bit e of nibble q) and the packed per-chunk counts.
        uint32_t flags = 0, packed = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t f = (fv[q].x != 0u ? 1u : 0u) | (fv[q].y != 0u ? 2u : 0u) | (fv[q].z != 0u ? 4u : 0u) |
                               (fv[q].w != 0u ? 8u : 0u);
            flags |= f << (4 * q);
            packed |= (uint32_t)__popc(f) << (8 * q);
        }
        uint32_t incl = packed;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const uint32_t totals = __shfl_sync(0xffffffffu, incl, 31);  // byte q: chunk q's count
        const uint32_t excl_lane = incl - packed;
        const uint32_t t0c = totals & 0xFFu, t1c = (totals >> 8) & 0xFFu, t2c = (totals >> 16) & 0xFFu;
        const uint32_t wtotal = t0c + t1c + t2c + (totals >> 24);
        if (lane == 0) s_warp[warp] = wtotal;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = lane < kCompactWarps ? s_warp[lane] : 0u;
            uint32_t ws = w;
#pragma unroll
            for (int o = 1; o < kCompactWarps; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, ws, o);
                if (lane >= o) ws += y;
            }
            const uint32_t ttotal = __shfl_sync(0xffffffffu, ws, kCompactWarps - 1);
            if (lane < kCompactWarps) s_warp[lane] = ws - w;  // the warps' exclusive offsets
            const uint64_t prefix = warp_tile_prefix(sc.status, tile, ttotal, sc.err);
            if (lane == 0) {
                s_prefix = prefix;
                if (tile == ntiles - 1) *count = prefix + ttotal;
            }
        }
        __syncthreads();
        const uint64_t wbase = s_prefix + s_warp[warp];
        const uint32_t cbase[4] = {0u, t0c, t0c + t1c, t0c + t1c + t2c};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint64_t o = wbase + cbase[q] + ((excl_lane >> (8 * q)) & 0xFFu);
            const uint32_t f = (flags >> (4 * q)) & 0xFu;
            if (f & 1u) dst[o++] = sv[q].x;
            if (f & 2u) dst[o++] = sv[q].y;
            if (f & 4u) dst[o++] = sv[q].z;
            if (f & 8u) dst[o++] = sv[q].w;
        }
        __syncthreads();  // s_tile, s_warp and s_prefix free for the next tile
    }
}

// Launches the compaction with caller-provided (already zeroed) scratch.
cudaError_t launch_compact_u32(const uint32_t* src, const uint32_t* valid, uint32_t* dst, uint64_t n,
                               uint64_t* count, CompactScratch sc, cudaStream_t st) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t ntiles = (n + kCompactTile - 1) / kCompactTile;
    // Every block resident at once (tiles are taken in order by running
    // blocks in any case, so a lookback never waits on a block not started).
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_compact_u32, kCompactThreads, 0) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 1;
    }
    per_sm = std::max(per_sm, 1);
    const unsigned grid =
        (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ntiles, (uint64_t)sms * (uint64_t)per_sm));
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
// the library holds the array (a little over 32 KiB) until the process exits.
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
