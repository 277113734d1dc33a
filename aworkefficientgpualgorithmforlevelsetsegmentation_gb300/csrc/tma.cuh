// TMA (cp.async.bulk.tensor) and mbarrier helpers in inline PTX for sm_103a,
// plus host-side tensor-map encoding through the driver entry point (no link
// dependency on libcuda).
//
// Every load lands in shared memory and completes on an mbarrier; every wait
// is bounded (kWaitLimitNs) and reports ERR_TMA_TIMEOUT instead of hanging.
// Loads may start at negative coordinates (the out-of-bounds part is filled
// with zeros); the innermost coordinate is always a multiple of 4 floats
// (16 bytes).  Stores start at non-negative coordinates only.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace lss {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

// Waits for the phase `parity` of the barrier to complete; false on timeout.
// Each try_wait may suspend the thread in hardware for up to 20 us (it
// resumes as soon as the phase completes), so waiting threads issue few
// instructions; the clock is read once per try.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done = 0;
    uint64_t t0 = 0;
    for (;;) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity), "r"(20000u)
            : "memory");
        if (done) return true;
        if (t0 == 0) t0 = globaltimer_ns();
        else if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
    }
}

// Makes a tensor map written to global memory by the host visible to the
// tensor-map proxy of this thread.
__device__ __forceinline__ void tmap_acquire(const void* tmap) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tmap) : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const void* tmap, int x, int y, int z,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
        "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

// Shared memory written by threads, then read by the TMA engine.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tma_store_3d(const void* tmap, int x, int y, int z, const void* src) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                     tmap),
                 "r"(x), "r"(y), "r"(z), "r"(smem_addr(src))
                 : "memory");
}

__device__ __forceinline__ void tma_store_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Waits until the shared-memory sources of all committed stores were read.
__device__ __forceinline__ void tma_store_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// Waits until all committed stores are complete (visible in global memory).
__device__ __forceinline__ void tma_store_wait_all() {
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// Host: encodes a 3D fp32 tiled tensor map over a padded volume.
//   dims    = logical extent (elements), x fastest
//   pitch_x = row pitch in elements, pitch_xy = slice pitch in elements
void encode_tmap_f32_3d(CUtensorMap* out, const float* base, uint64_t nx, uint64_t ny,
                        uint64_t nz, uint64_t pitch_x, uint64_t pitch_xy, uint32_t bx,
                        uint32_t by, uint32_t bz);

}  // namespace lss
