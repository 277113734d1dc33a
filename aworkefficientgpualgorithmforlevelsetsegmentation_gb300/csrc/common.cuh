// Shared host/device helpers of the level-set engine: error type, CUDA call
// checking, device error word, bounded waits and the 16^3-tile indexing of
// the reference's int8 fields.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

#include "lss.h"

namespace lss {

// Host-side error carrying an lss_status; converted to a return code at the
// C ABI boundary (lss_api.cpp).
struct Error : std::runtime_error {
    lss_status status;
    Error(lss_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define LSS_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            throw ::lss::Error(e_ == cudaErrorMemoryAllocation ? LSS_ERR_OUT_OF_MEMORY  \
                                                               : LSS_ERR_CUDA,          \
                               std::string(#call) + ": " + cudaGetErrorString(e_));     \
    } while (0)

#define LSS_REQUIRE(cond, status, msg)                   \
    do {                                                 \
        if (!(cond)) throw ::lss::Error((status), (msg)); \
    } while (0)

// Device-side error word bits (read back after each step).
enum : uint32_t {
    ERR_BARRIER_TIMEOUT = 1u << 0,  // a grid barrier wait gave up
    ERR_LOOKBACK_TIMEOUT = 1u << 1, // a decoupled-lookback wait gave up
    ERR_TMA_TIMEOUT = 1u << 2,      // an mbarrier wait for a TMA load gave up
    ERR_BOUNDS = 1u << 3,           // an index failed its bounds check
    ERR_CAPACITY = 1u << 4,         // a list would have overflowed its buffer
};

// Every spin-wait gives up after this many nanoseconds of %globaltimer.
constexpr uint64_t kWaitLimitNs = 2000000000ull;

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint64_t ld_acquire_u64(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u64(uint64_t* p, uint64_t v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void set_error(uint32_t* err, uint32_t bit) { atomicOr(err, bit); }

// --------------------------------------------------------------------------
// Decoupled-lookback tile prefix (single pass).  status[] holds one word per
// tile: bits 63..62 = flag (0 invalid, 1 aggregate, 2 inclusive prefix),
// bits 61..0 = value.  Values may pack two 31-bit counters (hi, lo); packed
// sums add field-wise as long as no field overflows.  status[0..ntiles) must
// be zero before the pass.  Returns the exclusive prefix of `tile`.  Tiles
// must be acquired in increasing order by running blocks (a dynamic tile
// counter), so every wait is on a tile whose block is resident; each wait
// still gives up after kWaitLimitNs.
constexpr uint64_t kFlagA = 1ull << 62, kFlagP = 2ull << 62, kValMask = (1ull << 62) - 1;

// Exclusive prefix of `tile` by decoupled lookback, one warp (all 32 lanes
// call it): lane 0 publishes the tile's aggregate, then the warp reads the
// status words of the 32 tiles before a window start at once; it adds the
// values up to and including the nearest inclusive prefix, or moves the
// window back by 32 when there is none.  A tile in the window that is not
// published yet (before the nearest inclusive prefix) is read again, for
// kWaitLimitNs at most (then the error bit is set and the sum so far
// returned).  Lane 0 then publishes the tile's inclusive prefix.
__device__ __forceinline__ uint64_t warp_tile_prefix(uint64_t* status, uint32_t tile, uint64_t aggregate,
                                                     uint32_t* err) {
    const int lane = threadIdx.x & 31;
    if (tile == 0) {
        if (lane == 0) st_release_u64(&status[0], kFlagP | (aggregate & kValMask));
        return 0;
    }
    if (lane == 0) st_release_u64(&status[tile], kFlagA | (aggregate & kValMask));
    uint64_t excl = 0;
    int64_t j = (int64_t)tile - 1;  // the window is tiles j, j-1, ..., j-31 (lane order)
    uint64_t t0 = 0;
    for (;;) {
        const int64_t idx = j - lane;
        const uint64_t st = idx >= 0 ? ld_acquire_u64(&status[idx]) : kFlagP;  // before tile 0: prefix 0
        const uint32_t flag = (uint32_t)(st >> 62);
        const uint32_t pmask = __ballot_sync(0xffffffffu, flag == 2u);
        const uint32_t zmask = __ballot_sync(0xffffffffu, flag == 0u);
        const int first_p = pmask ? __ffs(pmask) - 1 : 32;
        const uint32_t need = first_p == 32 ? 0xffffffffu : ((2u << first_p) - 1u);  // lanes 0..first_p
        if (zmask & need) {
            // Lane 0 keeps the time, so the whole warp gives up together.
            int give_up = 0;
            if (lane == 0) {
                if (t0 == 0) t0 = globaltimer_ns();
                else if (globaltimer_ns() - t0 > kWaitLimitNs) give_up = 1;
            }
            if (__shfl_sync(0xffffffffu, give_up, 0)) {
                if (lane == 0) set_error(err, ERR_LOOKBACK_TIMEOUT);
                break;
            }
            continue;
        }
        uint64_t v = ((need >> lane) & 1u) ? (st & kValMask) : 0ull;
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        excl += v;
        if (first_p < 32) break;
        j -= 32;
        t0 = 0;
    }
    if (lane == 0) st_release_u64(&status[tile], kFlagP | ((excl + aggregate) & kValMask));
    return excl;
}

// The same for the whole block (every thread calls it): warp 0 looks back.
__device__ __forceinline__ uint64_t tile_exclusive_prefix(uint64_t* status, uint32_t tile,
                                                          uint64_t aggregate, uint32_t* err) {
    __shared__ uint64_t s_prefix;
    if (threadIdx.x < 32) {
        const uint64_t excl = warp_tile_prefix(status, tile, aggregate, err);
        if (threadIdx.x == 0) s_prefix = excl;
    }
    __syncthreads();
    uint64_t r = s_prefix;
    __syncthreads();
    return r;
}

// Block-wide exclusive sum of one uint32 per thread (blockDim.x a multiple of
// 32, at most 1024).  Returns the thread's exclusive prefix; *total gets the
// block sum.
// The block total lives in its own slot (s_warp[32]): with 32 warps, slot 31
// holds warp 31's exclusive prefix.
__device__ __forceinline__ uint32_t block_exclusive_sum(uint32_t v, uint32_t* total) {
    __shared__ uint32_t s_warp[33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nw ? s_warp[lane] : 0;
        uint32_t ws = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, ws, o);
            if (lane >= o) ws += y;
        }
        if (lane < nw) s_warp[lane] = ws - w;
        if (lane == nw - 1) s_warp[32] = ws;
    }
    __syncthreads();
    uint32_t r = s_warp[warp] + x - v;
    *total = s_warp[32];
    __syncthreads();
    return r;
}

// Same for 64-bit values (packed counters).
// Sync = false leaves out the closing barrier (it only guards the shared
// slots against a following call): the caller separates calls by a barrier.
template <bool Sync = true>
__device__ __forceinline__ uint64_t block_exclusive_sum64(uint64_t v, uint64_t* total) {
    __shared__ uint64_t s_warp64[33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp64[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint64_t w = lane < nw ? s_warp64[lane] : 0;
        uint64_t ws = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t y = __shfl_up_sync(0xffffffffu, ws, o);
            if (lane >= o) ws += y;
        }
        if (lane < nw) s_warp64[lane] = ws - w;
        if (lane == nw - 1) s_warp64[32] = ws;
    }
    __syncthreads();
    uint64_t r = s_warp64[warp] + x - v;
    *total = s_warp64[32];
    if (Sync) __syncthreads();
    return r;
}

// Host-side fault injection for tests: LSS_FAULT=alloc|launch|timeout makes
// the named host step fail with LSS_ERR_INJECTED (no GPU fault is made).
bool fault_injected(const char* what);

// Device address of a host buffer in pinned host memory (cudaHostAlloc or
// cudaHostRegister, mapped into the device's address space under unified
// addressing), or null for pageable memory.  Kernels read or write pinned
// buffers in place over the host link: as fast as a copy-engine transfer
// (about 200 GB/s each way on GB300), with no device staging buffer and no
// second pass.
inline void* pinned_device_ptr(const void* host) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Device address of a buffer kernels can read or write in place: pinned host
// memory (as above), device or managed memory; null for pageable memory.
inline void* device_view(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost) return a.devicePointer;
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return const_cast<void*>(p);
    return nullptr;
}

// True for device memory of the current device.
inline bool device_memory(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    int dev = -1;
    return a.type == cudaMemoryTypeDevice && cudaGetDevice(&dev) == cudaSuccess && a.device == dev;
}

}  // namespace lss
