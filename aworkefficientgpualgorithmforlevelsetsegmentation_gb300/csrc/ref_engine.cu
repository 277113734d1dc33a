// LSS_MODE_REF: the reference's solver path on sm_103a, bit for bit.
//
// Buffers and their roles follow Segmenter.cpp:110-285: two int8 level-set
// fields in 16^3 tiles (ping-pong), an int8 export volume (linear), a u8 tag
// volume (tiled), the u32 coordinate and valid volumes that double as the
// seven offset buffers B^e of the few-active path, and the compacted active
// list.  The per-iteration sequence is Segmenter.cpp:811-1019:
//
//   update -> swap -> plan -> { few:  output, clear tag, filter x7, compact(7A)
//                               many: coordinate init, scatter, compact(N)
//                               re-init: dense activity, coordinate init, compact(N) }
//
// Differences from the reference are in mechanism only:
//   * the active count never leaves the device: a one-block plan kernel picks
//     the path (Segmenter.cpp:1363-1369) and sizes the compaction, and every
//     kernel is a grid-stride loop that reads the count, so an iteration is a
//     fixed launch sequence (capturable in a CUDA graph);
//   * CUDPP's compaction is a single-pass decoupled-lookback compaction that
//     also clears the valid flags it consumed (the reference clears them with
//     a cudaMemset / sparse memset afterwards, Segmenter.cpp:977, 1018; both
//     leave every consumed flag zero);
//   * the duplicate filter's same-kernel tag reads (texture reads in the
//     reference, FilterDuplicates.cu:141) see the tag state at kernel launch:
//     segment e marks its entries with e+1 and treats only other non-zero
//     values as "already set".  Every marked voxel is in the next active list,
//     so the next update overwrites the markers with 0/1 flags.
// The translation unit is compiled with -fmad=false: every float operation
// is one IEEE-754 binary32 operation in the reference's order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.hpp"

namespace lss {
namespace {

constexpr int kTile = 4096;  // compaction elements per tile (256 threads x 16)
constexpr int kThreads = 256;

struct RefDims {
    uint32_t x, y, z;
};

// Iterations a run to convergence launches between two reads of the rule's
// state (an iteration launched after the rule stopped costs its launches).
constexpr int kRuleChunk = 16;

struct RefCtl {
    unsigned long long n;        // active count (the list length)
    unsigned long long updates;  // sum of n over updates
    uint32_t err;
    uint32_t coord_ok;           // coordinate volume holds pack(x) at tiled(x)
    uint32_t path;               // 0 few, 1 many, 2 re-init
    uint32_t A;                  // align256(n)
    uint32_t m;                  // compaction input length
    uint32_t do_coord;           // initialise the coordinate volume this iteration
    uint32_t clear;              // compaction clears consumed valid flags
    uint32_t ntiles;
    uint32_t tile_counter;
    // The stopping rule on the device (k_ref_rule_start, k_ref_rule): once
    // `halt` is set every iteration kernel returns at entry, so iterations
    // launched after the rule stopped change nothing.
    uint32_t halt;
    int32_t conv, streak, patience;
    unsigned long long done;     // iterations run since k_ref_rule_start
    unsigned long long n0, abs_thr;
    double rel;
};

__device__ __forceinline__ uint32_t d_tiled(uint32_t x, uint32_t y, uint32_t z, RefDims d) {
    uint32_t tile = (z >> 4) * ((d.y >> 4) * (d.x >> 4)) + (y >> 4) * (d.x >> 4) + (x >> 4);
    return tile * 4096u + ((z & 15u) * 16u + (y & 15u)) * 16u + (x & 15u);
}

__device__ __forceinline__ uint3 d_untile(uint32_t i, RefDims d) {
    uint32_t tile = i >> 12, r = i & 4095u;
    uint32_t TX = d.x >> 4, TY = d.y >> 4;
    uint32_t tx = tile % TX, ty = (tile / TX) % TY, tz = tile / (TX * TY);
    return make_uint3(tx * 16 + (r & 15u), ty * 16 + ((r >> 4) & 15u), tz * 16 + (r >> 8));
}

__device__ __forceinline__ uint32_t d_lin(uint32_t x, uint32_t y, uint32_t z, RefDims d) {
    return (z * d.y + y) * d.x + x;
}

__device__ __forceinline__ uint32_t d_pack(uint3 v) { return v.x | (v.y << 10) | (v.z << 20); }

// Coordinates read back from the coordinate / active buffers are checked
// before use: an entry outside the volume sets ERR_BOUNDS and is skipped.
__device__ __forceinline__ bool d_inside(uint3 v, RefDims d, uint32_t* err) {
    if (v.x < d.x && v.y < d.y && v.z < d.z) return true;
    atomicOr(err, ERR_BOUNDS);
    return false;
}
__device__ __forceinline__ uint3 d_unpack(uint32_t p) {
    return make_uint3(p & 0x3FFu, (p >> 10) & 0x3FFu, (p >> 20) & 0x3FFu);
}

// OffsetCoordinates (Coordinates.cu:132-155).
__device__ __forceinline__ uint3 d_offset(uint3 v, int dx, int dy, int dz, RefDims d) {
    int x = (int)v.x + dx, y = (int)v.y + dy, z = (int)v.z + dz;
    if (x < 0 || y < 0 || z < 0 || x >= (int)d.x || y >= (int)d.y || z >= (int)d.z) return v;
    return make_uint3(x, y, z);
}

// Normalised int8 read, c/127 floored at -1 (Textures.cu:12).
__device__ __forceinline__ float d_nread(int8_t c) {
    float f = __fdiv_rn((float)c, 127.0f);
    return f < -1.0f ? -1.0f : f;
}

__device__ __forceinline__ float d_rabs(float f) { return f > 0 ? f : -1.0f * f; }
__device__ __forceinline__ bool d_equals(float a, float b, float e) { return d_rabs(a - b) <= e; }
__device__ __forceinline__ float d_fclamp(float i, float lo, float hi) {
    if (i < lo) return lo;
    if (i > hi) return hi;
    return i;
}

// __float2int_rd(f) with saturation and NaN -> 0.
__device__ __forceinline__ int32_t d_f2i_rd(float f) { return __float2int_rd(f); }

__constant__ int c_seg_off[7][3] = {{0, 0, -1}, {0, -1, 0}, {-1, 0, 0}, {0, 0, 0},
                                    {1, 0, 0},  {0, 1, 0},  {0, 0, 1}};

__device__ __forceinline__ uint32_t align256(uint32_t v) { return v + (256u - v % 256u) % 256u; }

// ComputeActiveElementOutputs (UpdateActiveElements.cu:34-104), 6-connected.
__device__ __forceinline__ uint32_t d_outputs(uint3 v, RefDims d, const int8_t* rd,
                                              const uint8_t* tag) {
    uint32_t ti = d_tiled(v.x, v.y, v.z, d);
    if (tag[ti] != 1) return 0;
    float u4 = d_nread(rd[ti]);
    uint32_t out = 0;
    const int order[6] = {0, 1, 2, 4, 5, 6};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        int e = order[k];
        uint3 q = d_offset(v, c_seg_off[e][0], c_seg_off[e][1], c_seg_off[e][2], d);
        float un = d_nread(rd[d_tiled(q.x, q.y, q.z, d)]);
        if (!d_equals(u4, un, 0.008f)) out |= (1u << 3) | (1u << e);
    }
    return out;
}

template <typename T>
__device__ __forceinline__ int32_t d_sample(const void* src, uint32_t i) {
    return (int32_t)((const T*)src)[i];
}

// UpdateLevelSetVolumeKernelHelper (UpdateLevelSetVolume.cu:222-342).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_ref_update(
    int8_t* __restrict__ wr, uint8_t* __restrict__ ex, uint8_t* __restrict__ tag,
    const int8_t* __restrict__ rd, const uint32_t* __restrict__ active, const void* src,
    RefDims d, RefCtl* ctl, int32_t target, int32_t window, float alpha, float dt_in) {
    if (ctl->halt) return;
    const uint64_t n = ctl->n;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint3 v = d_unpack(active[i]);
        if (!d_inside(v, d, &ctl->err)) continue;
        auto R = [&](int dx, int dy, int dz) {
            uint3 q = d_offset(v, dx, dy, dz, d);
            return d_nread(rd[d_tiled(q.x, q.y, q.z, d)]);
        };
        float u4nz = R(0, 0, -1), u1 = R(0, -1, 0), u3 = R(-1, 0, 0), u4 = R(0, 0, 0),
              u5 = R(1, 0, 0), u7 = R(0, 1, 0), u4pz = R(0, 0, 1);
        int32_t s = d_sample<T>(src, d_lin(v.x, v.y, v.z, d));
        float dcx = (u5 - u3) / 2.0f, dcy = (u7 - u1) / 2.0f, dcz = (u4pz - u4nz) / 2.0f;
        float fx = u5 - u4, fy = u7 - u4, fz = u4pz - u4;
        float bx = u4 - u3, by = u4 - u1, bz = u4 - u4nz;
        float sx = fx - bx, sy = fy - by, sz = fz - bz;
        float conn = 0.0f;
        if (alpha > 0.0f) {
            if (d_equals(u4pz, u4nz, 0.1f) && d_equals(u4nz, u1, 0.1f) && d_equals(u1, u3, 0.1f) &&
                d_equals(u3, u5, 0.1f) && d_equals(u5, u7, 0.1f) && d_equals(u7, u4pz, 0.1f)) {
                float avg = (u4pz + u1 + u3 + u5 + u7 + u4nz) / 6.0f;
                conn = avg - u4;
            }
        }
        float curv = sx + sy + sz;
        int32_t diff = s - target;
        int32_t adiff = diff < 0 ? -diff : diff;
        float dens = (-1.0f / (float)(uint32_t)window) * (float)adiff + 1.0f;
        dens = -dens;
        float dt = dt_in;
        if (dt < 0) {
            dt = -dt;
            dens = -dens;
        }
        float speed = ((1.0f - alpha) * dens) + (alpha * curv);
        float glen = sqrtf(dcx * dcx + dcy * dcy + dcz * dcz);
        float delta = ((dt * speed * glen)) + conn;
        float nv = fminf(1.0f, fmaxf(-1.0f, u4 + delta));
        nv = fminf(1.0f, fmaxf(-1.0f, (((1.0f + 0.01f) * nv) + 0.01f)));
        uint32_t ti = d_tiled(v.x, v.y, v.z, d);
        wr[ti] = (int8_t)d_f2i_rd(nv * 127.0f);
        ex[d_lin(v.x, v.y, v.z, d)] = (uint8_t)d_f2i_rd(nv * 127.0f);
        float td = nv - u4;
        tag[ti] = fabsf(td) > 0.008f ? 1 : 0;
    }
}

// Path choice, compaction sizing, status reset (one block).
__global__ void k_ref_plan(RefCtl* c, uint64_t* status, uint32_t N, int reinit, int count_update) {
    if (c->halt) return;
    __shared__ uint32_t s_ntiles;
    if (threadIdx.x == 0) {
        uint32_t n = (uint32_t)c->n;
        uint32_t A = align256(n);
        bool few = !reinit && ((uint64_t)A * 7u * 4u < (uint64_t)N * 4u);
        uint32_t path = reinit ? 2u : (few ? 0u : 1u);
        uint32_t m = few ? A * 7u : N;
        c->path = path;
        c->A = A;
        c->m = m;
        c->do_coord = (path != 0u && c->coord_ok == 0u) ? 1u : 0u;
        c->coord_ok = path == 0u ? 0u : 1u;
        c->clear = path == 2u ? 0u : 1u;
        c->ntiles = (m + kTile - 1) / kTile;
        c->tile_counter = 0;
        if (count_update) c->updates += c->n;
        if (m == 0) c->n = 0;
        s_ntiles = c->ntiles;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < s_ntiles; i += blockDim.x) status[i] = 0;
}

// OutputNewActiveElementsKernel (UpdateActiveElementsVolume.cu:210-363).
__global__ void __launch_bounds__(kThreads) k_ref_output(uint32_t* coord, uint32_t* valid,
                                                        const int8_t* rd, const uint8_t* tag,
                                                        const uint32_t* active, RefDims d,
                                                        RefCtl* ctl, int quirk) {
    if (ctl->halt || ctl->path != 0u) return;
    const uint64_t n = ctl->n;
    const uint64_t A = ctl->A;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (quirk && (i & 3u) == 3u) continue;
        uint3 v = d_unpack(active[i]);
        if (!d_inside(v, d, &ctl->err)) continue;
        uint32_t out = d_outputs(v, d, rd, tag);
#pragma unroll
        for (int e = 0; e < 7; ++e)
            if (out & (1u << e)) {
                uint3 q = d_offset(v, c_seg_off[e][0], c_seg_off[e][1], c_seg_off[e][2], d);
                coord[e * A + i] = d_pack(q);
                valid[e * A + i] = 1u;
            }
    }
}

// MemSetSparseKernel<unsigned char> (MemSetFloat.cu:227-290) on the tag volume.
__global__ void __launch_bounds__(kThreads) k_ref_clear_tag(uint8_t* tag, const uint32_t* active,
                                                           RefDims d, RefCtl* ctl) {
    if (ctl->halt || ctl->path != 0u) return;
    const uint64_t n = ctl->n;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint3 v = d_unpack(active[i]);
        if (!d_inside(v, d, &ctl->err)) continue;
        tag[d_tiled(v.x, v.y, v.z, d)] = 0;
    }
}

// FilterDuplicatesInitializeKernel (FilterDuplicates.cu:87-125).
__global__ void __launch_bounds__(kThreads) k_ref_filter0(const uint32_t* coord,
                                                         const uint32_t* valid, uint8_t* tag,
                                                         RefDims d, RefCtl* ctl) {
    if (ctl->halt || ctl->path != 0u) return;
    const uint64_t n = ctl->n;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        if (valid[i] == 1u) {
            uint3 v = d_unpack(coord[i]);
            if (!d_inside(v, d, &ctl->err)) continue;
            tag[d_tiled(v.x, v.y, v.z, d)] = 1;
        }
}

// FilterDuplicatesFilterKernel (FilterDuplicates.cu:127-193) on segment e.
__global__ void __launch_bounds__(kThreads) k_ref_filter(const uint32_t* coord, uint32_t* valid,
                                                        uint8_t* tag, RefDims d, RefCtl* ctl,
                                                        int e) {
    if (ctl->halt || ctl->path != 0u) return;
    const uint64_t n = ctl->n;
    const uint64_t base = (uint64_t)ctl->A * e;
    const uint8_t mark = (uint8_t)(e + 1);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t k = base + i;
        if (valid[k] != 1u) continue;
        uint3 v = d_unpack(coord[k]);
        if (!d_inside(v, d, &ctl->err)) continue;
        uint32_t t = d_tiled(v.x, v.y, v.z, d);
        uint8_t s = *(volatile uint8_t*)&tag[t];
        if (s != 0 && s != mark) valid[k] = 0u;
        else tag[t] = mark;
    }
}

// InitializeCoordinateVolumeKernel (InitializeCoordinateVolume.cu:37-47),
// written in tiled order so that the stores coalesce.
__global__ void __launch_bounds__(kThreads) k_ref_coord_init(uint32_t* coord, RefDims d,
                                                            const RefCtl* ctl, int force) {
    if (ctl->halt || (!force && ctl->do_coord == 0u)) return;
    const uint64_t N = (uint64_t)d.x * d.y * d.z;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
         i += (uint64_t)gridDim.x * blockDim.x)
        coord[i] = d_pack(d_untile((uint32_t)i, d));
}

// UpdateActiveElementsVolumeKernel (UpdateActiveElementsVolume.cu:39-100).
__global__ void __launch_bounds__(kThreads) k_ref_scatter(uint32_t* valid, const int8_t* rd,
                                                         const uint8_t* tag,
                                                         const uint32_t* active, RefDims d,
                                                         RefCtl* ctl, int quirk) {
    if (ctl->halt || ctl->path != 1u) return;
    const uint64_t n = ctl->n;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (quirk && (i & 3u) == 3u) continue;
        uint3 v = d_unpack(active[i]);
        if (!d_inside(v, d, &ctl->err)) continue;
        uint32_t out = d_outputs(v, d, rd, tag);
#pragma unroll
        for (int e = 0; e < 7; ++e)
            if (out & (1u << e)) {
                uint3 q = d_offset(v, c_seg_off[e][0], c_seg_off[e][1], c_seg_off[e][2], d);
                valid[d_tiled(q.x, q.y, q.z, d)] = 1u;
            }
    }
}

// InitializeActiveElementsVolumeKernel (InitializeActiveElementsVolume.cu:37-72).
__global__ void __launch_bounds__(kThreads) k_ref_init_active(uint32_t* valid, const int8_t* rd,
                                                             RefDims d) {
    const uint64_t N = (uint64_t)d.x * d.y * d.z;
    const int order[6] = {0, 1, 2, 4, 5, 6};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint3 v = d_untile((uint32_t)i, d);
        float u4 = d_nread(rd[i]);
        bool flat = true;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            int e = order[k];
            uint3 q = d_offset(v, c_seg_off[e][0], c_seg_off[e][1], c_seg_off[e][2], d);
            if (!d_equals(u4, d_nread(rd[d_tiled(q.x, q.y, q.z, d)]), 0.001f)) flat = false;
        }
        valid[i] = flat ? 0u : 1u;
    }
}

// InitializeLevelSetKernel (InitializeLevelSetVolume.cu:55-98).
__global__ void __launch_bounds__(kThreads) k_ref_init_level_set(int8_t* wr, uint8_t* ex,
                                                                const int8_t* rd, RefDims d,
                                                                uint3 seed, int32_t r,
                                                                float aniso) {
    const uint64_t N = (uint64_t)d.x * d.y * d.z;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint3 v = d_untile((uint32_t)i, d);
        int32_t vx = (int32_t)(seed.x - v.x), vy = (int32_t)(seed.y - v.y);
        float vz = ((float)(int32_t)seed.z - (float)(int32_t)v.z) * aniso;
        float fx = (float)vx, fy = (float)vy;
        float d2 = fx * fx + fy * fy + vz * vz;
        float dist = sqrtf(d2);
        float smooth = 4.0f, cur = 1.0f;
        if (dist < (float)r) cur = -1.0f;
        else if (dist < (float)r + smooth) cur = -1.0f + ((dist - (float)r) / (smooth / 2.0f));
        float old = d_nread(rd[i]);
        float nv = d_fclamp(old + cur - 1.0f, -1.0f, 1.0f);
        wr[i] = (int8_t)d_f2i_rd(nv * 127.0f);
        ex[d_lin(v.x, v.y, v.z, d)] = (uint8_t)d_f2i_rd(nv * 127.0f);
    }
}

// AddLevelSetKernel (InitializeLevelSetVolume.cu:151-169).
__global__ void __launch_bounds__(kThreads) k_ref_add_level_set(uint8_t* res, const uint8_t* add,
                                                               uint64_t N) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
         i += (uint64_t)gridDim.x * blockDim.x) {
        float o = (float)(int8_t)res[i] / 127.0f;
        float a = (float)(int8_t)add[i] / 127.0f;
        float r = d_fclamp(o + a - 1.0f, -1.0f, 1.0f);
        res[i] = (uint8_t)d_f2i_rd(r * 127.0f);
    }
}

// ExportActiveElementsVolumeKernel (ExportActiveElementsVolume.cu:43-73).
__global__ void __launch_bounds__(kThreads) k_ref_export_active(uint8_t* out,
                                                               const uint32_t* active, RefDims d,
                                                               RefCtl* ctl) {
    const uint64_t n = ctl->n;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint3 v = d_unpack(active[i]);
        if (!d_inside(v, d, &ctl->err)) continue;
        out[d_tiled(v.x, v.y, v.z, d)] = 127;
    }
}

// Stable compaction of src[i] where valid[i] != 0, i < ctl->m, into dst
// (single-pass decoupled lookback; replaces CUDPP's cudppCompact,
// Cuda.cpp:699-758).  Consumed flags are cleared when ctl->clear is set.  The
// count is written to ctl->n by the last tile.
__global__ void __launch_bounds__(kThreads) k_ref_compact(const uint32_t* __restrict__ src,
                                                         uint32_t* __restrict__ valid,
                                                         uint32_t* __restrict__ dst, RefCtl* ctl,
                                                         uint64_t* status) {
    constexpr int kItems = kTile / kThreads;  // 16, contiguous per thread
    __shared__ uint32_t s_tile;
    if (ctl->halt) return;
    const uint32_t m = ctl->m, ntiles = ctl->ntiles, clear = ctl->clear;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&ctl->tile_counter, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        __syncthreads();
        if (tile >= ntiles) break;
        const uint64_t base = (uint64_t)tile * kTile + (uint64_t)threadIdx.x * kItems;
        uint32_t flags = 0, cnt = 0;
        if (base + kItems <= m) {
            const uint4* vp = reinterpret_cast<const uint4*>(valid + base);
#pragma unroll
            for (int q = 0; q < kItems / 4; ++q) {
                uint4 w = vp[q];
                flags |= (w.x != 0u ? 1u : 0u) << (4 * q);
                flags |= (w.y != 0u ? 1u : 0u) << (4 * q + 1);
                flags |= (w.z != 0u ? 1u : 0u) << (4 * q + 2);
                flags |= (w.w != 0u ? 1u : 0u) << (4 * q + 3);
            }
        } else {
            for (int q = 0; q < kItems; ++q)
                if (base + q < m && valid[base + q] != 0u) flags |= 1u << q;
        }
        cnt = __popc(flags);
        if (clear && flags) {
            for (int q = 0; q < kItems; ++q)
                if (flags & (1u << q)) valid[base + q] = 0u;
        }
        uint32_t total;
        uint32_t off = block_exclusive_sum(cnt, &total);
        uint64_t prefix = tile_exclusive_prefix(status, tile, total, &ctl->err);
        uint64_t o = prefix + off;
        for (int q = 0; q < kItems; ++q)
            if (flags & (1u << q)) dst[o++] = src[base + q];
        if (tile == ntiles - 1 && threadIdx.x == 0) ctl->n = prefix + total;
    }
}

// The stopping rule of a run to convergence, evaluated on the device after
// every iteration (the host then reads the count back once per chunk of
// launched iterations instead of once per iteration): unless halted, count
// the iteration; with the rule on, stop when n <= abs_thr, else count the
// streak of iterations with n < rel * n0 and stop when it reaches patience.
__global__ void k_ref_rule(RefCtl* c) {
    if (c->halt) return;
    c->done += 1ull;
    if (!c->conv) return;
    const unsigned long long n = c->n;
    if (n <= c->abs_thr) {
        c->halt = 1u;
        return;
    }
    c->streak = ((double)n < c->rel * (double)c->n0) ? c->streak + 1 : 0;
    if (c->streak >= c->patience) c->halt = 1u;
}

// The rule's state at the start of a step: n0 is the count the step starts
// from.
__global__ void k_ref_rule_start(RefCtl* c, int32_t conv, double rel, unsigned long long abs_thr,
                                 int32_t patience) {
    c->halt = 0u;
    c->done = 0ull;
    c->streak = 0;
    c->conv = conv;
    c->rel = rel;
    c->abs_thr = abs_thr;
    c->patience = patience;
    c->n0 = c->n;
}

// Sum and sum of squares of the source where the export volume is <= 0
// (CollectCurrentLevelSetVoxels, Segmenter.cpp:357-448), in double.
template <typename T>
__global__ void k_ref_collect(const void* src, const uint8_t* ex, uint64_t N, double mean,
                              double* acc) {
    double s = 0, q = 0, c = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
         i += (uint64_t)gridDim.x * blockDim.x)
        if ((int8_t)ex[i] <= 0) {
            double v = (double)((const T*)src)[i];
            s += v;
            q += (v - mean) * (v - mean);
            c += 1;
        }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        q += __shfl_down_sync(0xffffffffu, q, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], s);
        atomicAdd(&acc[1], q);
        atomicAdd(&acc[2], c);
    }
}

// ---------------------------------------------------------------------------

class RefEngine : public EngineBase {
   public:
    explicit RefEngine(const lss_config& c) : arena_(c.hbm_budget_bytes) { init_device(c); }
    ~RefEngine() override {
        for (auto& g : graphs_)
            if (g) cudaGraphExecDestroy(g);
    }

    void load_volume(const void* data, int nx, int ny, int nz, int dtype, float aniso) override {
        LSS_REQUIRE(data && nx > 0 && ny > 0 && nz > 0, LSS_ERR_INVALID_ARGUMENT, "bad volume");
        LSS_REQUIRE(dtype >= LSS_U8 && dtype <= LSS_S32, LSS_ERR_UNSUPPORTED,
                    "LSS_MODE_REF takes the reference's integer voxel types");
        uint32_t px = nx + (16 - nx % 16) % 16, py = ny + (16 - ny % 16) % 16,
                 pz = nz + (16 - nz % 16) % 16;
        LSS_REQUIRE(px <= 1024 && py <= 1024 && pz <= 1024, LSS_ERR_CAPACITY,
                    "LSS_MODE_REF pads to multiples of 16 and packs 10 bits per axis (<= 1024)");
        unload_volume();
        ux_ = nx; uy_ = ny; uz_ = nz;
        dtype_ = dtype;
        aniso_ = aniso;
        d_ = RefDims{px, py, pz};
        N_ = (uint64_t)px * py * pz;
        int bpv = dtype <= 1 ? 1 : dtype <= 3 ? 2 : 4;
        bool sgn = dtype == LSS_S8 || dtype == LSS_S16 || dtype == LSS_S32;
        // LoadVolumeHostPadded (Segmenter.cpp:1131-1204): byte-wise pad value.
        std::vector<uint8_t> host(N_ * bpv, 0);
        const uint8_t* in = (const uint8_t*)data;
        int pad = sgn ? -127 : 0;
        size_t pi = 0, ri = 0, rowb = (size_t)nx * bpv, padx = (size_t)(px - nx) * bpv,
               pady = (size_t)(py - ny) * px * bpv, padz = (size_t)(pz - nz) * py * px * bpv;
        for (int z = 0; z < nz; ++z) {
            for (int y = 0; y < ny; ++y) {
                std::memcpy(&host[pi], in + ri, rowb);
                pi += rowb; ri += rowb;
                std::memset(&host[pi], pad, padx);
                pi += padx;
            }
            std::memset(&host[pi], pad, pady);
            pi += pady;
        }
        std::memset(&host[pi], pad, padz);

        src_ = arena_.alloc(N_ * bpv);
        phiX_ = (int8_t*)arena_.alloc(N_);
        phiY_ = (int8_t*)arena_.alloc(N_);
        export_ = (uint8_t*)arena_.alloc(N_);
        frozen_ = (uint8_t*)arena_.alloc(N_);
        tag_ = (uint8_t*)arena_.alloc(N_);
        coord_ = (uint32_t*)arena_.alloc(N_ * 4);
        valid_ = (uint32_t*)arena_.alloc(N_ * 4);
        active_ = (uint32_t*)arena_.alloc(N_ * 4);
        status_ = (uint64_t*)arena_.alloc((N_ / kTile + 2) * 8);
        ctl_ = (RefCtl*)arena_.alloc(sizeof(RefCtl));
        acc_ = (double*)arena_.alloc(4 * sizeof(double));
        LSS_CUDA(cudaMemcpyAsync(src_, host.data(), host.size(), cudaMemcpyHostToDevice, stream));
        LSS_CUDA(cudaMemsetAsync(phiX_, 127, N_, stream));
        LSS_CUDA(cudaMemsetAsync(phiY_, 127, N_, stream));
        LSS_CUDA(cudaMemsetAsync(coord_, 0xFF, N_ * 4, stream));
        LSS_CUDA(cudaMemsetAsync(valid_, 0, N_ * 4, stream));
        LSS_CUDA(cudaMemsetAsync(tag_, 0, N_, stream));
        LSS_CUDA(cudaMemsetAsync(export_, 127, N_, stream));
        LSS_CUDA(cudaMemsetAsync(frozen_, 127, N_, stream));
        LSS_CUDA(cudaMemsetAsync(active_, 0, N_ * 4, stream));
        LSS_CUDA(cudaMemsetAsync(ctl_, 0, sizeof(RefCtl), stream));
        rd_ = phiX_;
        wr_ = phiY_;
        initialized_ = false;
        iterations_ = 0;
        Tp_ = Wp_ = Ap_ = 0.0f;
        loaded_ = true;
        sync();
    }

    void unload_volume() override {
        sync();
        for (auto& g : graphs_)
            if (g) { cudaGraphExecDestroy(g); g = nullptr; }
        arena_.release();
        loaded_ = false;
        initialized_ = false;
        scratch_ = nullptr;
    }

    void set_params(const lss_params& p) override { params = p; }

    bool params_changed() const {
        return Tp_ != params.target || Wp_ != params.window || Ap_ != params.curvature;
    }

    void swap() { std::swap(rd_, wr_); }

    int blocks() const { return num_sms * 8; }

    void initialize_seed(float cx, float cy, float cz, float r) override {
        require_loaded();
        LSS_REQUIRE(cx >= 0 && cy >= 0 && cz >= 0 && r >= 0, LSS_ERR_INVALID_ARGUMENT,
                    "seed coordinates are unsigned in the reference");
        uint3 seed = make_uint3((uint32_t)cx, (uint32_t)cy, (uint32_t)cz);
        int32_t rr = (int32_t)(uint32_t)r;
        LSS_CUDA(cudaMemsetAsync(active_, 0xFF, N_ * 4, stream));
        LSS_CUDA(cudaMemsetAsync(valid_, 0, N_ * 4, stream));
        LSS_CUDA(cudaMemsetAsync(tag_, 0, N_, stream));
        for (int k = 0; k < 2; ++k) {
            k_ref_init_level_set<<<blocks(), kThreads, 0, stream>>>(wr_, export_, rd_, d_, seed,
                                                                   rr, aniso_);
            ++launches;
            swap();
        }
        rebuild_dense();
        finish_init();
    }

    void set_phi(const float* phi) override {
        require_loaded();
        std::vector<int8_t> t(N_, 127);
        std::vector<uint8_t> ex(N_, 127);
        for (uint32_t z = 0; z < uz_; ++z)
            for (uint32_t y = 0; y < uy_; ++y)
                for (uint32_t x = 0; x < ux_; ++x) {
                    float f = phi[((size_t)z * uy_ + y) * ux_ + x];
                    f = f < -1.0f ? -1.0f : (f > 1.0f ? 1.0f : f);
                    float s = std::floor(f * 127.0f);
                    int8_t c = (int8_t)(int32_t)s;
                    t[htiled(x, y, z)] = c;
                    ex[((size_t)z * d_.y + y) * d_.x + x] = (uint8_t)c;
                }
        LSS_CUDA(cudaMemsetAsync(active_, 0xFF, N_ * 4, stream));
        LSS_CUDA(cudaMemsetAsync(valid_, 0, N_ * 4, stream));
        LSS_CUDA(cudaMemsetAsync(tag_, 0, N_, stream));
        LSS_CUDA(cudaMemcpyAsync(phiX_, t.data(), N_, cudaMemcpyHostToDevice, stream));
        LSS_CUDA(cudaMemcpyAsync(phiY_, t.data(), N_, cudaMemcpyHostToDevice, stream));
        LSS_CUDA(cudaMemcpyAsync(export_, ex.data(), N_, cudaMemcpyHostToDevice, stream));
        sync();
        rebuild_dense();
        finish_init();
    }

    void rebuild_dense() {
        k_ref_init_active<<<blocks(), kThreads, 0, stream>>>(valid_, rd_, d_);
        ++launches;
        k_ref_coord_init<<<blocks(), kThreads, 0, stream>>>(coord_, d_, ctl_, 1);
        ++launches;
        k_ref_plan<<<1, kThreads, 0, stream>>>(ctl_, status_, (uint32_t)N_, 1, 0);
        ++launches;
        k_ref_compact<<<blocks(), kThreads, 0, stream>>>(coord_, valid_, active_, ctl_, status_);
        ++launches;
        LSS_CUDA(cudaGetLastError());
    }

    void finish_init() {
        initialized_ = true;
        iterations_ = 0;
        Tp_ = params.target;
        Wp_ = params.window;
        Ap_ = params.curvature;
        check_errors();
    }

    // One iteration (Segmenter.cpp:811-1028) as a fixed launch sequence.
    void enqueue_iteration(bool reinit) {
        const int B = blocks();
        const int32_t T = (int32_t)params.target, W = (int32_t)params.window;
        switch (dtype_) {
#define LSS_REF_UPD(TY)                                                                        \
    k_ref_update<TY><<<B, kThreads, 0, stream>>>(wr_, export_, tag_, rd_, active_, src_, d_,   \
                                                 ctl_, T, W, params.curvature, params.time_step)
            case LSS_U8: LSS_REF_UPD(uint8_t); break;
            case LSS_S8: LSS_REF_UPD(int8_t); break;
            case LSS_U16: LSS_REF_UPD(uint16_t); break;
            case LSS_S16: LSS_REF_UPD(int16_t); break;
            case LSS_U32: LSS_REF_UPD(uint32_t); break;
            case LSS_S32: LSS_REF_UPD(int32_t); break;
#undef LSS_REF_UPD
        }
        ++launches;
        swap();
        k_ref_plan<<<1, kThreads, 0, stream>>>(ctl_, status_, (uint32_t)N_, reinit ? 1 : 0, 1);
        ++launches;
        if (reinit) {
            k_ref_init_active<<<B, kThreads, 0, stream>>>(valid_, rd_, d_);
            ++launches;
            k_ref_coord_init<<<B, kThreads, 0, stream>>>(coord_, d_, ctl_, 0);
            ++launches;
        } else {
            const int q = cfg.ref_quirk_i3 ? 1 : 0;
            k_ref_output<<<B, kThreads, 0, stream>>>(coord_, valid_, rd_, tag_, active_, d_, ctl_, q);
            ++launches;
            k_ref_clear_tag<<<B, kThreads, 0, stream>>>(tag_, active_, d_, ctl_);
            ++launches;
            k_ref_filter0<<<B, kThreads, 0, stream>>>(coord_, valid_, tag_, d_, ctl_);
            ++launches;
            for (int e = 1; e < 7; ++e) {
                k_ref_filter<<<B, kThreads, 0, stream>>>(coord_, valid_, tag_, d_, ctl_, e);
                ++launches;
            }
            k_ref_coord_init<<<B, kThreads, 0, stream>>>(coord_, d_, ctl_, 0);
            ++launches;
            k_ref_scatter<<<B, kThreads, 0, stream>>>(valid_, rd_, tag_, active_, d_, ctl_, q);
            ++launches;
        }
        k_ref_compact<<<B, kThreads, 0, stream>>>(coord_, valid_, active_, ctl_, status_);
        ++launches;
        k_ref_rule<<<1, 1, 0, stream>>>(ctl_);
        ++launches;
    }

    // A graph of one normal iteration for each buffer parity.
    void run_iteration(bool reinit) {
        if (reinit || !cfg.use_graph) {
            enqueue_iteration(reinit);
            LSS_CUDA(cudaGetLastError());
            return;
        }
        int parity = rd_ == phiX_ ? 0 : 1;
        GraphKey key{params.target, params.window, params.curvature, params.time_step,
                     cfg.ref_quirk_i3};
        if (!(key == gkey_)) {
            for (auto& g : graphs_)
                if (g) { cudaGraphExecDestroy(g); g = nullptr; }
            gkey_ = key;
        }
        if (!graphs_[parity]) {
            cudaGraph_t g;
            int8_t* rd0 = rd_;
            LSS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            const uint64_t l0 = launches;
            enqueue_iteration(false);
            graph_kernels_[parity] = launches - l0;  // captured, not launched
            launches = l0;
            LSS_CUDA(cudaStreamEndCapture(stream, &g));
            rd_ = rd0;
            wr_ = rd0 == phiX_ ? phiY_ : phiX_;
            LSS_CUDA(cudaGraphInstantiate(&graphs_[parity], g, 0));
            cudaGraphDestroy(g);
        }
        LSS_CUDA(cudaGraphLaunch(graphs_[parity], stream));
        launches += graph_kernels_[parity];
        swap();
    }

    uint64_t device_n() {
        unsigned long long n = 0;
        LSS_CUDA(cudaMemcpyAsync(&n, &ctl_->n, sizeof(n), cudaMemcpyDeviceToHost, stream));
        sync();
        return n;
    }

    bool finished() override {
        if (!loaded_ || !initialized_) return false;
        return (float)device_n() <= params.convergence_threshold && iterations_ > 500;
    }

    // RequestUpdateSegmentation (Segmenter.cpp:759-1051).  With a stopping
    // rule the rule runs on the device after every iteration (k_ref_rule)
    // and the host reads its state back once per kRuleChunk launched
    // iterations; iterations launched after it stopped do nothing, and the
    // buffer swaps the host made for them are undone by parity.
    int step(int k, const lss_conv* conv) override {
        require_loaded();
        if (params_changed()) iterations_ = 0;
        bool should = (initialized_ && !finished()) || params_changed();
        if (!should) return 0;
        cudaEvent_t e0, e1;
        LSS_CUDA(cudaEventCreate(&e0));
        LSS_CUDA(cudaEventCreate(&e1));
        LSS_CUDA(cudaEventRecord(e0, stream));
        k_ref_rule_start<<<1, 1, 0, stream>>>(ctl_, conv ? 1 : 0, conv ? conv->rel_threshold : 0.0,
                                              conv ? (unsigned long long)conv->abs_threshold : 0ull,
                                              conv ? conv->patience : 0);
        ++launches;
        int launched = 0;
        for (int s = 0; s < k; ++s) {
            bool reinit = params_changed();
            if (reinit) {
                Tp_ = params.target; Wp_ = params.window; Ap_ = params.curvature;
                iterations_ = 0;
            }
            run_iteration(reinit);
            ++launched;
            if (conv && launched % kRuleChunk == 0 && s + 1 < k) {
                uint32_t halt = 0;
                LSS_CUDA(cudaMemcpyAsync(&halt, &ctl_->halt, sizeof(halt), cudaMemcpyDeviceToHost, stream));
                sync();
                if (halt) break;
            }
        }
        LSS_CUDA(cudaEventRecord(e1, stream));
        unsigned long long done = 0;
        LSS_CUDA(cudaMemcpyAsync(&done, &ctl_->done, sizeof(done), cudaMemcpyDeviceToHost, stream));
        LSS_CUDA(cudaMemsetAsync(&ctl_->halt, 0, sizeof(uint32_t), stream));  // rebuilds run again
        LSS_CUDA(cudaEventSynchronize(e1));
        sync();
        LSS_REQUIRE(done <= (unsigned long long)launched, LSS_ERR_STATE, "iteration count");
        if (((unsigned long long)launched - done) & 1ull) swap();
        iterations_ += (int)done;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        last_ms_ = ms;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        check_errors();
        return (int)done;
    }

    uint64_t active_count() override { return loaded_ ? device_n() : 0; }

    uint64_t read_active(uint32_t* out, uint64_t cap, bool packed) override {
        require_loaded();
        uint64_t n = device_n();
        if (!out) return n;
        uint64_t m = std::min(n, cap);
        std::vector<uint32_t> h(m);
        if (m) LSS_CUDA(cudaMemcpyAsync(h.data(), active_, m * 4, cudaMemcpyDeviceToHost, stream));
        sync();
        for (uint64_t i = 0; i < m; ++i) {
            if (packed) { out[i] = h[i]; continue; }
            out[3 * i] = h[i] & 0x3FFu;
            out[3 * i + 1] = (h[i] >> 10) & 0x3FFu;
            out[3 * i + 2] = (h[i] >> 20) & 0x3FFu;
        }
        return n;
    }

    void read_phi(float* out) override {
        require_loaded();
        std::vector<int8_t> h(N_);
        LSS_CUDA(cudaMemcpyAsync(h.data(), rd_, N_, cudaMemcpyDeviceToHost, stream));
        sync();
        for (uint32_t z = 0; z < uz_; ++z)
            for (uint32_t y = 0; y < uy_; ++y)
                for (uint32_t x = 0; x < ux_; ++x) {
                    float f = (float)h[htiled(x, y, z)] / 127.0f;
                    out[((size_t)z * uy_ + y) * ux_ + x] = f < -1.0f ? -1.0f : f;
                }
    }

    // GetSaveableSegmentation (Segmenter.cpp:1216-1286), tag side effect included.
    void read_mask(uint8_t* out) override {
        require_loaded();
        LSS_CUDA(cudaMemcpyAsync(tag_, export_, N_, cudaMemcpyDeviceToDevice, stream));
        k_ref_add_level_set<<<blocks(), kThreads, 0, stream>>>(tag_, frozen_, N_);
        ++launches;
        std::vector<uint8_t> h(N_);
        LSS_CUDA(cudaMemcpyAsync(h.data(), tag_, N_, cudaMemcpyDeviceToHost, stream));
        LSS_CUDA(cudaMemsetAsync(tag_, 0, N_, stream));
        sync();
        for (uint32_t z = 0; z < uz_; ++z)
            for (uint32_t y = 0; y < uy_; ++y)
                for (uint32_t x = 0; x < ux_; ++x)
                    out[((size_t)z * uy_ + y) * ux_ + x] =
                        (int8_t)h[((size_t)z * d_.y + y) * d_.x + x] <= 0 ? 1 : 0;
    }

    void read_export(int8_t* out) override {
        require_loaded();
        std::vector<uint8_t> h(N_);
        LSS_CUDA(cudaMemcpyAsync(h.data(), export_, N_, cudaMemcpyDeviceToHost, stream));
        sync();
        for (uint32_t z = 0; z < uz_; ++z)
            for (uint32_t y = 0; y < uy_; ++y)
                for (uint32_t x = 0; x < ux_; ++x)
                    out[((size_t)z * uy_ + y) * ux_ + x] = (int8_t)h[((size_t)z * d_.y + y) * d_.x + x];
    }

    void read_active_volume(uint8_t* out) override {
        require_loaded();
        if (!scratch_) scratch_ = (uint8_t*)arena_.alloc(N_);
        LSS_CUDA(cudaMemsetAsync(scratch_, 0, N_, stream));
        k_ref_export_active<<<blocks(), kThreads, 0, stream>>>(scratch_, active_, d_, ctl_);
        ++launches;
        std::vector<uint8_t> h(N_);
        LSS_CUDA(cudaMemcpyAsync(h.data(), scratch_, N_, cudaMemcpyDeviceToHost, stream));
        sync();
        for (uint32_t z = 0; z < uz_; ++z)
            for (uint32_t y = 0; y < uy_; ++y)
                for (uint32_t x = 0; x < ux_; ++x)
                    out[((size_t)z * uy_ + y) * ux_ + x] = h[htiled(x, y, z)];
    }

    void freeze() override {
        require_loaded();
        k_ref_add_level_set<<<blocks(), kThreads, 0, stream>>>(frozen_, export_, N_);
        ++launches;
        sync();
    }

    void clear_current() override {
        require_loaded();
        initialized_ = false;
        iterations_ = 0;
        LSS_CUDA(cudaMemsetAsync(export_, 127, N_, stream));
        LSS_CUDA(cudaMemsetAsync(active_, 0xFF, N_ * 4, stream));
        LSS_CUDA(cudaMemsetAsync(phiX_, 127, N_, stream));
        LSS_CUDA(cudaMemsetAsync(phiY_, 127, N_, stream));
        LSS_CUDA(cudaMemsetAsync(valid_, 0, N_ * 4, stream));
        LSS_CUDA(cudaMemsetAsync(tag_, 0, N_, stream));
        LSS_CUDA(cudaMemsetAsync(&ctl_->n, 0, sizeof(unsigned long long), stream));
        sync();
    }

    void clear_all() override {
        clear_current();
        LSS_CUDA(cudaMemsetAsync(frozen_, 127, N_, stream));
        sync();
    }

    void estimate_params(float* t, float* w) override {
        require_loaded();
        double acc[3];
        double mean = 0;
        for (int pass = 0; pass < 2; ++pass) {
            LSS_CUDA(cudaMemsetAsync(acc_, 0, 3 * sizeof(double), stream));
            switch (dtype_) {
#define LSS_COL(TY) \
    k_ref_collect<TY><<<blocks(), kThreads, 0, stream>>>(src_, export_, N_, mean, acc_), ++launches
                case LSS_U8: LSS_COL(uint8_t); break;
                case LSS_S8: LSS_COL(int8_t); break;
                case LSS_U16: LSS_COL(uint16_t); break;
                case LSS_S16: LSS_COL(int16_t); break;
                case LSS_U32: LSS_COL(uint32_t); break;
                case LSS_S32: LSS_COL(int32_t); break;
#undef LSS_COL
            }
            LSS_CUDA(cudaMemcpyAsync(acc, acc_, 3 * sizeof(double), cudaMemcpyDeviceToHost, stream));
            sync();
            LSS_REQUIRE(acc[2] >= 2, LSS_ERR_STATE, "fewer than two segmented voxels");
            if (pass == 0) mean = acc[0] / acc[2];
        }
        *t = (float)mean;
        *w = (float)std::sqrt(acc[1] / (acc[2] - 1));
        params.target = *t;
        params.window = *w;
    }

    void stats(lss_stats* s) override {
        std::memset(s, 0, sizeof(*s));
        s->mode = LSS_MODE_REF;
        s->kernel_launches = launches;
        if (!loaded_) return;
        RefCtl c;
        LSS_CUDA(cudaMemcpyAsync(&c, ctl_, sizeof(c), cudaMemcpyDeviceToHost, stream));
        sync();
        s->iterations = iterations_;
        s->active_count = c.n;
        s->voxel_updates = c.updates;
        s->device_bytes = arena_.held();
        s->last_step_ms = last_ms_;
        s->padded_x = d_.x; s->padded_y = d_.y; s->padded_z = d_.z;
        s->error_flags = (int32_t)c.err;
    }

   private:
    struct GraphKey {
        float t = -1e30f, w = 0, a = 0, dt = 0;
        int q = -1;
        bool operator==(const GraphKey& o) const {
            return t == o.t && w == o.w && a == o.a && dt == o.dt && q == o.q;
        }
    };

    void require_loaded() const { LSS_REQUIRE(loaded_, LSS_ERR_STATE, "no volume loaded"); }

    uint32_t htiled(uint32_t x, uint32_t y, uint32_t z) const {
        uint32_t tile = (z >> 4) * ((d_.y >> 4) * (d_.x >> 4)) + (y >> 4) * (d_.x >> 4) + (x >> 4);
        return tile * 4096u + ((z & 15u) * 16u + (y & 15u)) * 16u + (x & 15u);
    }

    void check_errors() {
        LSS_CUDA(cudaGetLastError());
        uint32_t err = 0;
        LSS_CUDA(cudaMemcpyAsync(&err, &ctl_->err, 4, cudaMemcpyDeviceToHost, stream));
        sync();
        LSS_REQUIRE(err == 0, LSS_ERR_TIMEOUT, "device wait gave up (error word " + std::to_string(err) + ")");
    }

    DeviceArena arena_;
    RefDims d_{0, 0, 0};
    uint64_t N_ = 0;
    uint32_t ux_ = 0, uy_ = 0, uz_ = 0;
    int dtype_ = 0;
    float aniso_ = 1.0f;
    void* src_ = nullptr;
    int8_t *phiX_ = nullptr, *phiY_ = nullptr, *rd_ = nullptr, *wr_ = nullptr;
    uint8_t *export_ = nullptr, *frozen_ = nullptr, *tag_ = nullptr, *scratch_ = nullptr;
    uint32_t *coord_ = nullptr, *valid_ = nullptr, *active_ = nullptr;
    uint64_t* status_ = nullptr;
    RefCtl* ctl_ = nullptr;
    double* acc_ = nullptr;
    bool loaded_ = false, initialized_ = false;
    int iterations_ = 0;
    float Tp_ = 0, Wp_ = 0, Ap_ = 0;
    double last_ms_ = 0;
    GraphKey gkey_;
    cudaGraphExec_t graphs_[2] = {nullptr, nullptr};
    uint64_t graph_kernels_[2] = {0, 0};  // kernels of each graph
};

}  // namespace

std::unique_ptr<EngineBase> make_ref_engine(const lss_config& c) {
    return std::unique_ptr<EngineBase>(new RefEngine(c));
}

}  // namespace lss
