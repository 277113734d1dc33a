// Kernel-level stream compaction on caller-owned device buffers: the C-ABI
// replacement of the reference's CudppCompact (code/gpuseg/code/src/cuda/
// Cuda.cpp:699-758), which wraps CUDPP 1.1's cudppCompact.
//
// Stable: dst receives src[i] for every i < n with valid[i] != 0, in index
// order.  Three stream-ordered kernels over tiles of 4096 elements: the
// count of each tile, which also packs the flags into one bit an element
// (the flags are read once); an exclusive scan of the tile counts
// (decoupled lookback over 8192 counts a block); and the scatter, which
// reads the packed bits and only the values they keep, and stores the kept
// values from each tile's prefix.  The count is written to device memory
// (the reference copies it to the host after every 2^25-element chunk).
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
constexpr int kCompactTile = kCompactThreads * kCompactItems;  // 4096 elements
constexpr int kCompactWarps = kCompactThreads / 32;
constexpr int kCompactSeg = kCompactTile / kCompactWarps;  // 512 elements a warp: 4 chunks of 128
static_assert(kCompactSeg == 512, "a warp's segment is four 128-element chunks");
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // tile counts a scan block takes

struct CompactScratch {
    uint64_t* counts;        // one word per tile: its count, then its exclusive prefix
    uint16_t* bits;          // 16 flag bits per thread and tile (bit 4 q + e: element e of chunk q)
    uint64_t* status;        // one word per scan block, zero before the call
    uint32_t* tile_counter;  // zero before the call
    uint32_t* err;
};

// Four elements from i: one 16-byte load when the buffer is aligned and all
// four are inside, else element by element (0 past n).
template <bool STREAM>
__device__ __forceinline__ uint4 load_quad(const uint32_t* __restrict__ p, uint64_t i, uint64_t n, bool vec) {
    if (vec && i + 4 <= n) {
        const uint4* q = reinterpret_cast<const uint4*>(p + i);
        return STREAM ? __ldcs(q) : *q;
    }
    return make_uint4(i < n ? p[i] : 0u, i + 1 < n ? p[i + 1] : 0u, i + 2 < n ? p[i + 2] : 0u,
                      i + 3 < n ? p[i + 3] : 0u);
}

// Pass 1: the number of nonzero flags of each tile, and the flags packed.
// Warp w of a tile reads the elements [512 w, 512 w + 512) as four chunks of
// 128 (lane l the four elements 4 l .. 4 l + 3 of each chunk, 16-byte loads,
// a warp's load 512 contiguous bytes); the thread's 16 flags go to one
// 16-bit word (the tile's 256 words contiguous).  The flags are streamed
// (evict first): the packed words are what the scatter reads.  Tiles i,
// i + G, ... for block i of G.
__global__ void __launch_bounds__(kCompactThreads) k_compact_count(const uint32_t* __restrict__ valid,
                                                                   uint64_t n, uint64_t* __restrict__ counts,
                                                                   uint16_t* __restrict__ bits,
                                                                   uint64_t* __restrict__ clear,
                                                                   uint64_t nclear) {
    __shared__ uint32_t s_warp[2][kCompactWarps];  // by tile parity: one barrier a tile
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t ntiles = (n + kCompactTile - 1) / kCompactTile;
    // The scan's status words, block counter and error word, zeroed here:
    // the scan is the next kernel on the stream.
    if (blockIdx.x == 0)
        for (uint64_t i = threadIdx.x; i < nclear; i += kCompactThreads) clear[i] = 0ull;
    const bool vec = (uintptr_t)valid % 16 == 0;
    int buf = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, buf ^= 1) {
        const uint64_t i0 = tile * kCompactTile + (uint64_t)warp * kCompactSeg + (uint64_t)lane * 4;
        uint4 fv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) fv[q] = load_quad<true>(valid, i0 + (uint64_t)q * 128, n, vec);
        uint32_t flags = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            flags |= ((fv[q].x != 0u ? 1u : 0u) | (fv[q].y != 0u ? 2u : 0u) | (fv[q].z != 0u ? 4u : 0u) |
                      (fv[q].w != 0u ? 8u : 0u))
                     << (4 * q);
        bits[tile * kCompactThreads + threadIdx.x] = (uint16_t)flags;
        const uint32_t c = __reduce_add_sync(0xffffffffu, (uint32_t)__popc(flags));
        if (lane == 0) s_warp[buf][warp] = c;
        __syncthreads();
        if (warp == 0) {
            const uint32_t t = __reduce_add_sync(0xffffffffu, lane < kCompactWarps ? s_warp[buf][lane] : 0u);
            if (lane == 0) counts[tile] = t;
        }
        // s_warp[buf] is written again two tiles on, after the next barrier.
    }
}

// Pass 2: the tile counts replaced in place by their exclusive prefix sums.
// Blocks take 8192 counts at a time from a counter (so a lookback only waits
// on blocks already running); the block's offset comes from the decoupled
// lookback over the status words.  The last block writes the total count.
__global__ void __launch_bounds__(kScanThreads) k_compact_scan(uint64_t ntiles, unsigned long long* total,
                                                               CompactScratch sc) {
    __shared__ uint32_t s_tile;
    const uint64_t nscan = (ntiles + kScanTile - 1) / kScanTile;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(sc.tile_counter, 1u);
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= nscan) break;
        const uint64_t i0 = (uint64_t)t * kScanTile + (uint64_t)threadIdx.x * kScanItems;
        uint64_t v[kScanItems], sum = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            v[k] = i0 + k < ntiles ? sc.counts[i0 + k] : 0ull;
            sum += v[k];
        }
        uint64_t agg = 0;
        const uint64_t ex = block_exclusive_sum64<true>(sum, &agg);
        const uint64_t prefix = tile_exclusive_prefix(sc.status, t, agg, sc.err);  // ends with a barrier
        uint64_t run = prefix + ex;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            if (i0 + k < ntiles) sc.counts[i0 + k] = run;
            run += v[k];
        }
        if (t == nscan - 1 && threadIdx.x == 0) *total = prefix + agg;
    }
}

// Pass 3: each tile's kept values, stored from the tile's prefix.  The
// elements of a thread are those of pass 1, its flags the 16 bits pass 1
// packed; a value is loaded only where one of its four flags is set (16-byte
// loads, streamed: each is read once).  Ranks inside the tile: one warp
// inclusive scan of the four per-chunk counts packed into the bytes of a
// word (a chunk holds at most 128), the warps' totals through shared memory.
// A warp's kept values are gathered in order in a shared-memory row and
// stored from there, 32 consecutive words an instruction.  The next tile's flag
// bits and prefix are loaded one tile ahead, so the value loads wait on
// nothing.
__global__ void __launch_bounds__(kCompactThreads) k_compact_scatter(const uint32_t* __restrict__ src,
                                                                     const uint16_t* __restrict__ bits,
                                                                     uint32_t* __restrict__ dst, uint64_t n,
                                                                     const uint64_t* __restrict__ prefix) {
    __shared__ uint32_t s_warp[2][kCompactWarps];  // by tile parity: one barrier a tile
    __shared__ uint32_t s_out[kCompactWarps][kCompactSeg];  // a staging row per warp
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t ntiles = (n + kCompactTile - 1) / kCompactTile;
    const bool vec = (uintptr_t)src % 16 == 0;
    int buf = 0;
    uint32_t flags_next = 0;
    uint64_t base_next = 0;
    if (blockIdx.x < ntiles) {
        flags_next = bits[(uint64_t)blockIdx.x * kCompactThreads + threadIdx.x];
        base_next = prefix[blockIdx.x];
    }
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, buf ^= 1) {
        const uint32_t flags = flags_next;
        const uint64_t base = base_next;
        const uint64_t tn = tile + gridDim.x;
        if (tn < ntiles) {
            flags_next = bits[tn * kCompactThreads + threadIdx.x];
            base_next = prefix[tn];
        }
        const uint64_t i0 = tile * kCompactTile + (uint64_t)warp * kCompactSeg + (uint64_t)lane * 4;
        uint4 sv[4];
        uint32_t packed = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t f = (flags >> (4 * q)) & 0xFu;
            sv[q] = f ? load_quad<true>(src, i0 + (uint64_t)q * 128, n, vec) : make_uint4(0u, 0u, 0u, 0u);
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
        // The warp's kept values in order in its staging row, then stored
        // from there as whole 128-byte rows of dst.
        uint32_t* row = s_out[warp];
        const uint32_t cbase[4] = {0u, t0c, t0c + t1c, t0c + t1c + t2c};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint32_t o = cbase[q] + ((excl_lane >> (8 * q)) & 0xFFu);
            const uint32_t f = (flags >> (4 * q)) & 0xFu;
            if (f & 1u) row[o++] = sv[q].x;
            if (f & 2u) row[o++] = sv[q].y;
            if (f & 4u) row[o++] = sv[q].z;
            if (f & 8u) row[o++] = sv[q].w;
        }
        if (lane == 0) s_warp[buf][warp] = wtotal;
        __syncthreads();  // also orders the staging row's writes before its reads
        // s_warp[buf] is written again two tiles on, after the next barrier.
        const uint64_t wbase =
            base + __reduce_add_sync(0xffffffffu, lane < warp ? s_warp[buf][lane] : 0u);
        for (uint32_t i = (uint32_t)lane; i < wtotal; i += 32) __stcs(dst + wbase + i, row[i]);
        __syncwarp();  // the row is rewritten by this warp for the next tile
    }
}

// Blocks of fn that fit on the device at once.
static unsigned resident_grid(const void* fn, int threads, int sms) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 1;
    }
    return (unsigned)(std::max(per_sm, 1) * sms);
}

uint64_t compact_tiles(uint64_t n) { return (n + kCompactTile - 1) / kCompactTile; }
uint64_t compact_scan_blocks(uint64_t n) { return (compact_tiles(n) + kScanTile - 1) / kScanTile; }
// Scratch of a call, in 8-byte words: the tile counts, the packed flags (512
// bytes a tile), the scan's status words, then one word for the scan's block
// counter and the error word.
constexpr uint64_t kBitsWordsPerTile = kCompactThreads * sizeof(uint16_t) / 8;
uint64_t compact_scratch_words(uint64_t n) {
    return compact_tiles(n) * (1 + kBitsWordsPerTile) + compact_scan_blocks(n) + 1 + 1;
}

// Points sc into words [0, compact_scratch_words(n)) of base.  The words from
// *clear_from on are the ones to zero before the call.
CompactScratch compact_scratch(uint64_t* base, uint64_t n, uint64_t* clear_from) {
    CompactScratch sc;
    const uint64_t nt = compact_tiles(n), ns = compact_scan_blocks(n);
    sc.counts = base;
    sc.bits = (uint16_t*)(base + nt);
    sc.status = base + nt * (1 + kBitsWordsPerTile);
    sc.tile_counter = (uint32_t*)(sc.status + ns + 1);
    sc.err = sc.tile_counter + 1;
    *clear_from = nt * (1 + kBitsWordsPerTile);
    return sc;
}

// Resident blocks of each pass on a device (every block of a pass resident
// at once), worked out once per device.
struct CompactGrids {
    unsigned count, scan, scatter;
};
static std::mutex g_grid_mu;
static CompactGrids g_grids[64] = {};

static CompactGrids compact_grids(int dev) {
    std::lock_guard<std::mutex> g(g_grid_mu);
    const bool cached = dev >= 0 && dev < 64 && g_grids[dev].count != 0;
    if (cached) return g_grids[dev];
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    sms = std::max(sms, 1);
    CompactGrids r;
    r.count = resident_grid((const void*)k_compact_count, kCompactThreads, sms);
    r.scan = resident_grid((const void*)k_compact_scan, kScanThreads, sms);
    r.scatter = resident_grid((const void*)k_compact_scatter, kCompactThreads, sms);
    if (dev >= 0 && dev < 64) g_grids[dev] = r;
    return r;
}

// Launches the three passes on scratch of compact_scratch_words(n) words at
// base (the count pass clears the words the scan needs zeroed).
cudaError_t launch_compact_u32(const uint32_t* src, const uint32_t* valid, uint32_t* dst, uint64_t n,
                               uint64_t* count, uint64_t* base, cudaStream_t st) {
    uint64_t clear_from = 0;
    const CompactScratch sc = compact_scratch(base, n, &clear_from);
    const uint64_t nclear = compact_scratch_words(n) - clear_from;
    int dev = 0;
    cudaGetDevice(&dev);
    const CompactGrids cg = compact_grids(dev);
    const uint64_t nt = compact_tiles(n);
    const unsigned g1 = (unsigned)std::min<uint64_t>(cg.count, nt);
    const unsigned g3 = (unsigned)std::min<uint64_t>(cg.scatter, nt);
    // Scan blocks take their counts in order from a counter, so a lookback
    // never waits on a block not started.
    const unsigned g2 = (unsigned)std::min<uint64_t>(cg.scan, compact_scan_blocks(n));
    k_compact_count<<<g1, kCompactThreads, 0, st>>>(valid, n, sc.counts, sc.bits, base + clear_from, nclear);
    k_compact_scan<<<g2, kScanThreads, 0, st>>>(nt, (unsigned long long*)count, sc);
    k_compact_scatter<<<g3, kCompactThreads, 0, st>>>(src, sc.bits, dst, n, sc.counts);
    return cudaGetLastError();
}

// The allocating entry point's memory pool, one per device: stream-ordered
// like the default pool, but it keeps up to kPoolKeep bytes reserved when
// streams synchronise (the default pool hands its memory back at every
// synchronisation, and mapping it again cost about 0.17 ms a call).
constexpr uint64_t kPoolKeep = 128ull << 20;
static std::mutex g_pool_mu;
static cudaMemPool_t g_pools[64] = {};

static lss_status compact_pool(cudaMemPool_t* out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return LSS_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> g(g_pool_mu);
    if (!g_pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
            cudaGetLastError();
            return LSS_ERR_CUDA;
        }
        uint64_t keep = kPoolKeep;
        if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
            cudaGetLastError();
            cudaMemPoolDestroy(pool);
            return LSS_ERR_CUDA;
        }
        g_pools[dev] = pool;
    }
    *out = g_pools[dev];
    return LSS_OK;
}

}  // namespace lss

extern "C" lss_status lss_compact_u32(const uint32_t* d_src, const uint32_t* d_valid, uint32_t* d_dst,
                                      uint64_t n, uint64_t* d_count, void* stream) {
    if (!d_src || !d_valid || !d_dst || !d_count) return LSS_ERR_INVALID_ARGUMENT;
    if (n >= (1ull << 40)) return LSS_ERR_CAPACITY;
    cudaStream_t st = (cudaStream_t)stream;
    if (n == 0) {
        return cudaMemsetAsync(d_count, 0, sizeof(uint64_t), st) == cudaSuccess ? LSS_OK : LSS_ERR_CUDA;
    }
    // Scratch: tile counts, packed flags, status words, block counter and
    // error word, stream-ordered from the library's pool.
    cudaMemPool_t pool = nullptr;
    const lss_status ps = lss::compact_pool(&pool);
    if (ps != LSS_OK) return ps;
    const uint64_t words = lss::compact_scratch_words(n);
    void* scratch = nullptr;
    if (cudaMallocFromPoolAsync(&scratch, words * 8, pool, st) != cudaSuccess) {
        cudaGetLastError();
        return LSS_ERR_OUT_OF_MEMORY;
    }
    uint64_t clear_from = 0;
    const lss::CompactScratch sc = lss::compact_scratch((uint64_t*)scratch, n, &clear_from);
    lss_status s = LSS_OK;
    if (lss::launch_compact_u32(d_src, d_valid, d_dst, n, d_count, (uint64_t*)scratch, st) != cudaSuccess)
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
// the library holds the array (a little over 8 MiB) until the process exits.
// The call reads the error word back and synchronises its stream before it
// returns.
namespace lss {

// Largest n the allocation-free call accepts.
constexpr uint64_t kNoAllocMaxElements = 1ull << 26;
constexpr uint64_t kNoAllocWords = kNoAllocMaxElements / kCompactTile * (1 + kBitsWordsPerTile) +
                                   (kNoAllocMaxElements / kCompactTile + kScanTile - 1) / kScanTile + 2;

// The scratch of compact_scratch_words(n) for every n up to the maximum.
static __device__ __align__(256) uint64_t g_noalloc_scratch[kNoAllocWords];

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
    // compact_scratch_words(n) <= kNoAllocWords.  The array keeps the
    // previous call's contents: the count pass clears the words the scan
    // reads before writing (the tile counts and packed flags are written
    // before they are read).
    uint64_t clear_from = 0;
    const lss::CompactScratch sc = lss::compact_scratch(base, n, &clear_from);
    if (lss::launch_compact_u32(d_src, d_valid, d_dst, n, d_count, base, st) != cudaSuccess) {
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
