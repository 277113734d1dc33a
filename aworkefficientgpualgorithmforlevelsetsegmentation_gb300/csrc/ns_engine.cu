// LSS_MODE_NS host side: volume/brick bookkeeping, tensor maps, the launch
// of the persistent kernel (plain engine = one volume, batched form = many),
// initialisation, readback and the brick-shape autotuner.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "engine.hpp"
#include "ns_core.hpp"
#include "ns_kernels.cuh"

namespace lss {

// ---------------------------------------------------------------------------
// Tensor-map encoding through the driver entry point.
void encode_tmap_f32_3d(CUtensorMap* out, const float* base, uint64_t nx, uint64_t ny,
                        uint64_t nz, uint64_t pitch_x, uint64_t pitch_xy, uint32_t bx,
                        uint32_t by, uint32_t bz) {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    LSS_REQUIRE(fn, LSS_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    cuuint64_t dims[3] = {nx, ny, nz};
    cuuint64_t strides[2] = {pitch_x * 4, pitch_xy * 4};
    cuuint32_t box[3] = {bx, by, bz};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = fn(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)base, dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    LSS_REQUIRE(r == CUDA_SUCCESS, LSS_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

namespace {

// dst[i] = phi <= 0 at unpadded voxel i, or'ed with frozen[i] (may be null;
// dst may be frozen itself: each element is read and written by one thread).
// Four voxels a thread, one 4-byte store, when the rows and both byte
// arrays allow it.
__global__ void k_ns_mask(uint8_t* dst, const float* src, const uint8_t* frozen, int nx, int ny, int nz, int px,
                          int py) {
    const uint32_t rows = (uint32_t)ny * (uint32_t)nz;
    const bool vec = nx % 4 == 0 && (uintptr_t)dst % 4 == 0 && (uintptr_t)frozen % 4 == 0;
    for (uint32_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const uint32_t z = r / (uint32_t)ny, y = r - z * (uint32_t)ny;
        const float* s = src + ((size_t)z * py + y) * px;
        uint8_t* d = dst + (size_t)r * nx;
        const uint8_t* f = frozen ? frozen + (size_t)r * nx : nullptr;
        if (vec) {
            for (int x = 4 * threadIdx.x; x < nx; x += 4 * blockDim.x) {
                uint32_t m = (uint32_t)(s[x] <= 0.0f) | (uint32_t)(s[x + 1] <= 0.0f) << 8 |
                             (uint32_t)(s[x + 2] <= 0.0f) << 16 | (uint32_t)(s[x + 3] <= 0.0f) << 24;
                if (f) {
                    const uint32_t fw = *reinterpret_cast<const uint32_t*>(f + x);
                    // Nonzero frozen bytes -> 1.
                    m |= ((fw | (fw >> 1) | (fw >> 2) | (fw >> 3) | (fw >> 4) | (fw >> 5) | (fw >> 6) | (fw >> 7)) &
                          0x01010101u);
                }
                *reinterpret_cast<uint32_t*>(d + x) = m;
            }
        } else {
            for (int x = threadIdx.x; x < nx; x += blockDim.x) d[x] = (s[x] <= 0.0f || (f && f[x])) ? 1 : 0;
        }
    }
}

__global__ void k_ns_fill(float* p, uint64_t n, float v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// dst = src on the voxel box [lo, hi) of a padded volume (pitch px, py).
__global__ void k_ns_copy_box(float* dst, const float* src, int px, int py, int3 lo, int3 hi) {
    const uint64_t nx = hi.x - lo.x, ny = hi.y - lo.y, n = nx * ny * (uint64_t)(hi.z - lo.z);
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
        const int x = lo.x + (int)(t % nx), y = lo.y + (int)((t / nx) % ny), z = lo.z + (int)(t / (nx * ny));
        const size_t i = ((size_t)z * py + y) * px + x;
        dst[i] = src[i];
    }
}

// phi = min(phi, clamp(|x - c| - r)) over the box [b0, b1) of the logical
// volume (outside it the clamped distance is hi >= phi, so nothing changes).
__global__ void k_ns_sphere_union(float* phi, int nx, int ny, int nz, int px, int py, int3 b0, int3 b1,
                                  float cx, float cy, float cz, float r, float lo, float hi) {
    const int bx = b1.x - b0.x, by = b1.y - b0.y, bz = b1.z - b0.z;
    const uint64_t n = (uint64_t)bx * by * bz;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const int x = b0.x + (int)(i % bx), y = b0.y + (int)((i / bx) % by),
                  z = b0.z + (int)(i / ((uint64_t)bx * by));
        const double dx = x - (double)cx, dy = y - (double)cy, dz = z - (double)cz;
        double d = sqrt(dx * dx + dy * dy + dz * dz) - (double)r;
        d = d < lo ? lo : (d > hi ? hi : d);
        float* q = &phi[((uint64_t)z * py + y) * px + x];
        *q = fminf(*q, (float)d);
    }
}

// The speed of every voxel of a padded volume (the padding's intensities
// are 0 and never updated), four voxels a thread and round: the part of the
// update no iteration changes, with the update's own arithmetic (no bias:
// only the adjoint takes one, per call).
__global__ void k_ns_speed(const NsVol V, float* speed, uint64_t n4) {
    const float4* I4 = reinterpret_cast<const float4*>(V.img);
    float4* S4 = reinterpret_cast<float4*>(speed);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n4;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const float4 I = I4[i];
        S4[i] = make_float4(ns_speed_f32(I.x, 0.0f, V), ns_speed_f32(I.y, 0.0f, V), ns_speed_f32(I.z, 0.0f, V),
                            ns_speed_f32(I.w, 0.0f, V));
    }
}

// Dense all-voxel update with the same arithmetic as the sparse engine: the
// unconditional update the paper compares against (main.tex:523).  A block
// covers a 32 x 8 column of the volume over zc planes and marches in z
// with three planes of phi (each with a one-voxel halo, clamped to the
// volume's edge) in a shared-memory ring, so every phi value is read from
// memory about once and every neighbour from shared memory.  The descriptor
// is a kernel parameter: its scalars are constant-bank operands.
constexpr int kDenseX = 32, kDenseY = 8, kDenseZMax = 32;
constexpr int kDensePlane = (kDenseX + 2) * (kDenseY + 2);

__global__ void __launch_bounds__(256) k_ns_dense(const NsVol V, uint32_t p, int zc) {
    __shared__ float ring[3][kDensePlane];
    const int tx = threadIdx.x % kDenseX, ty = threadIdx.x / kDenseX;
    const int x0 = blockIdx.x * kDenseX, y0 = blockIdx.y * kDenseY, zb = blockIdx.z * zc;
    const float* __restrict__ src = p ? V.phi[1] : V.phi[0];
    float* __restrict__ dst = p ? V.phi[0] : V.phi[1];
    const size_t pxy = (size_t)V.px * V.py;
    // The (at most two) halo-plane elements this thread loads: in-plane
    // offsets, clamped to the volume, fixed over the march.
    size_t off[2];
    bool has[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int t = threadIdx.x + r * 256;
        has[r] = t < kDensePlane;
        const int lx = t % (kDenseX + 2), ly = t / (kDenseX + 2);
        const int gx = min(max(x0 - 1 + lx, 0), V.nx - 1), gy = min(max(y0 - 1 + ly, 0), V.ny - 1);
        off[r] = (size_t)gy * V.px + gx;
    }
    auto load_plane = [&](float* d, int z) {
        const float* s = src + (size_t)min(max(z, 0), V.nz - 1) * pxy;
#pragma unroll
        for (int r = 0; r < 2; ++r)
            if (has[r]) d[threadIdx.x + r * 256] = s[off[r]];
    };
    float* pm = ring[0];
    float* pc = ring[1];
    float* pp = ring[2];
    load_plane(pm, zb - 1);
    load_plane(pc, zb);
    const int x = x0 + tx, y = y0 + ty;
    const bool inside = x < V.nx && y < V.ny;
    const int c0 = (ty + 1) * (kDenseX + 2) + tx + 1;
    const int zend = min(zb + zc, V.nz);
    size_t k = (size_t)zb * pxy + (size_t)y * V.px + x;
    for (int z = zb; z < zend; ++z, k += pxy) {
        load_plane(pp, z + 1);  // into the ring slot freed by the barrier below
        __syncthreads();
        if (inside) {
            auto P = [&](int dx, int dy, int dz) {
                const float* pl = dz < 0 ? pm : (dz > 0 ? pp : pc);
                return pl[c0 + dy * (kDenseX + 2) + dx];
            };
            dst[k] = ns_update_speed_f32(P, V.speed[k], V);
        }
        __syncthreads();
        float* t = pm;
        pm = pc;
        pc = pp;
        pp = t;
    }
}

// Sum, sum of squares and count of the intensities where phi <= 0.
__global__ void k_ns_collect(const float* img, const float* phi, int nx, int ny, int nz, int px,
                             int py, double mean, double* acc) {
    const uint64_t n = (uint64_t)nx * ny * nz;
    double s = 0, q = 0, c = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t x = i % nx, y = (i / nx) % ny, z = i / ((uint64_t)nx * ny);
        const uint64_t k = (z * py + y) * px + x;
        if (phi[k] <= 0.0f) {
            const double v = img[k];
            s += v;
            q += (v - mean) * (v - mean);
            c += 1;
        }
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

struct KernelSet {
    void* persistent;
    void* init_active;
    void* emit;
    int words;
    int block;          // threads per block of the init / emit kernels
    int pblock;         // threads per block of the persistent kernel
    size_t smem_fixed;  // dynamic shared memory of the persistent kernel, without the stopping state
};

template <int BX, int BY, int BZ, int NT, int MINB = 1024 / NT>
KernelSet kernels_for() {
    using S = Brick<BX, BY, BZ>;
    return KernelSet{(void*)&k_ns_persistent<BX, BY, BZ, NT, MINB>, (void*)&k_ns_init_active<BX, BY, BZ, NT>,
                     (void*)&k_ns_emit<BX, BY, BZ, NT>, S::WORDS, NT, NT, 0};
}

// Brick workers: GROUPS groups of NT threads in the one block per SM.
template <int BX, int BY, int BZ, int NT, int GROUPS>
KernelSet group_kernels_for() {
    using S = Brick<BX, BY, BZ>;
    return KernelSet{(void*)&k_ns_group<BX, BY, BZ, NT, GROUPS>, (void*)&k_ns_init_active<BX, BY, BZ, NT>,
                     (void*)&k_ns_emit<BX, BY, BZ, NT>, S::WORDS, NT, NT * GROUPS,
                     group_smem_fixed<S, NT, GROUPS>()};
}

// Warp per brick, W warps in the one block per SM.
template <int BX, int BY, int BZ, int W, int NT>
KernelSet warp_kernels_for() {
    using S = Brick<BX, BY, BZ>;
    return KernelSet{(void*)&k_ns_warp<BX, BY, BZ, W>, (void*)&k_ns_init_active<BX, BY, BZ, NT>,
                     (void*)&k_ns_emit<BX, BY, BZ, NT>, S::WORDS, NT, W * 32, warp_smem_fixed<S, W>()};
}

}  // namespace

// The instantiated (brick shape, threads per brick) configurations; 32
// threads per brick = one warp per brick (k_ns_warp).
const std::vector<BrickConfig>& brick_configs() {
    static const std::vector<BrickConfig> v = {
        {8, 8, 8, 256}, {8, 8, 8, 128}, {8, 8, 8, 512}, {8, 8, 4, 128}, {8, 8, 4, 256}, {4, 4, 4, 64},
        {8, 8, 4, 32},  {8, 8, 8, 32},  {4, 4, 4, 32},  {8, 8, 8, 256, 5}, {8, 8, 8, 256, 4},
        {8, 8, 8, 256, 0, 4}};
    return v;
}

static KernelSet kernels(const BrickConfig& c) {
    if (c.groups > 1) {
        if (c.bx == 8 && c.by == 8 && c.bz == 8 && c.threads == 256 && c.groups == 4)
            return group_kernels_for<8, 8, 8, 256, 4>();
        throw Error(LSS_ERR_UNSUPPORTED, "unsupported brick-worker configuration");
    }
    if (c.bx == 8 && c.by == 8 && c.bz == 8 && c.threads == 256 && c.min_blocks == 5)
        return kernels_for<8, 8, 8, 256, 5>();
    if (c.bx == 8 && c.by == 8 && c.bz == 8 && c.threads == 256 && c.min_blocks == 4)
        return kernels_for<8, 8, 8, 256, 4>();
    // 8^3 x 256 by default three blocks per SM: 79 registers (four cap a
    // thread at 64: 3 % slower to converge at 256^3, more blocks each
    // running a rank selection every iteration).
    if (c.bx == 8 && c.by == 8 && c.bz == 8 && c.threads == 256) return kernels_for<8, 8, 8, 256, 3>();
    if (c.bx == 8 && c.by == 8 && c.bz == 8 && c.threads == 128) return kernels_for<8, 8, 8, 128>();
    if (c.bx == 8 && c.by == 8 && c.bz == 8 && c.threads == 512) return kernels_for<8, 8, 8, 512>();
    if (c.bx == 8 && c.by == 8 && c.bz == 4 && c.threads == 128) return kernels_for<8, 8, 4, 128>();
    if (c.bx == 8 && c.by == 8 && c.bz == 4 && c.threads == 256) return kernels_for<8, 8, 4, 256>();
    if (c.bx == 4 && c.by == 4 && c.bz == 4 && c.threads == 64) return kernels_for<4, 4, 4, 64>();
    if (c.bx == 8 && c.by == 8 && c.bz == 4 && c.threads == 32) return warp_kernels_for<8, 8, 4, 16, 256>();
    if (c.bx == 8 && c.by == 8 && c.bz == 8 && c.threads == 32) return warp_kernels_for<8, 8, 8, 16, 256>();
    if (c.bx == 4 && c.by == 4 && c.bz == 4 && c.threads == 32) return warp_kernels_for<4, 4, 4, 32, 64>();
    throw Error(LSS_ERR_UNSUPPORTED, "unsupported brick configuration");
}

// ---------------------------------------------------------------------------
// NsCore

NsCore::NsCore(EngineBase* owner, uint64_t budget) : owner_(owner), arena_(budget), brick_arena_(0) {}
NsCore::~NsCore() = default;

void* NsCore::workspace(uint64_t bytes) {
    if (bytes > ws_bytes_) {
        owner_->sync();  // no kernel of an earlier call still uses the old workspace
        if (ws_) arena_.free_last(ws_);
        ws_ = nullptr;
        ws_bytes_ = 0;
        adj_rec_ = AdjointRecord{};
        ws_ = arena_.alloc(bytes);
        ws_bytes_ = bytes;
    }
    return ws_;
}

// Unpadded host field -> padded device field dst of volume V.  Pageable host
// memory is copied into `stage` first (a device buffer of at least nx*ny*nz
// floats that is free during the call), or into a temporary without one.
// Returns after the host buffer was read.
void NsCore::upload_padded(float* dst, const float* host, const VolHost& V, float* stage) {
    cudaStream_t st = owner_->stream;
    const uint64_t n = (uint64_t)V.nx * V.ny * V.nz;
    const float* src = (const float*)pinned_device_ptr(host);
    float* tmp = nullptr;
    if (!src) {
        float* buf = stage ? stage : (tmp = (float*)arena_.alloc(n * 4));
        LSS_CUDA(cudaMemcpyAsync(buf, host, n * 4, cudaMemcpyHostToDevice, st));
        src = buf;
    }
    k_ns_scatter<<<owner_->num_sms * 4, 256, 0, st>>>(dst, src, V.nx, V.ny, V.nz, V.px, V.py);
    ++owner_->launches;
    LSS_CUDA(cudaGetLastError());
    owner_->sync();
    if (tmp) arena_.free_last(tmp);
}

int NsCore::add_volume(const float* data, int nx, int ny, int nz, const lss_params& p) {
    ++epoch_;
    LSS_REQUIRE(data && nx > 0 && ny > 0 && nz > 0, LSS_ERR_INVALID_ARGUMENT, "bad volume");
    LSS_REQUIRE(vols_.size() < 4096, LSS_ERR_CAPACITY, "at most 4096 volumes per batch");
    VolHost v;
    v.nx = nx; v.ny = ny; v.nz = nz;
    v.px = (nx + 7) / 8 * 8; v.py = (ny + 7) / 8 * 8; v.pz = (nz + 7) / 8 * 8;
    v.p = p;
    const uint64_t P = (uint64_t)v.px * v.py * v.pz;
    v.img = (float*)arena_.alloc(P * 4);
    v.speed = (float*)arena_.alloc(P * 4);
    v.phi[0] = (float*)arena_.alloc(P * 4);
    v.phi[1] = (float*)arena_.alloc(P * 4);
    cudaStream_t st = owner_->stream;
    LSS_CUDA(cudaMemsetAsync(v.img, 0, P * 4, st));
    upload_padded(v.img, data, v, v.phi[1]);  // phi[1] stages; it is filled below
    k_ns_fill<<<owner_->num_sms * 4, 256, 0, st>>>(v.phi[0], P, p.phi_max);
    ++owner_->launches;
    k_ns_fill<<<owner_->num_sms * 4, 256, 0, st>>>(v.phi[1], P, p.phi_max);
    ++owner_->launches;
    v.uniform = true;  // both buffers phi_max until seeded
    LSS_CUDA(cudaGetLastError());
    owner_->sync();
    vols_.push_back(v);
    configured_ = false;
    return (int)vols_.size() - 1;
}

void NsCore::configure(const BrickConfig& c) {
    ++epoch_;
    LSS_REQUIRE(!vols_.empty(), LSS_ERR_STATE, "no volume");
    owner_->sync();
    cfg_ = c;
    KernelSet ks = kernels(c);
    words_ = ks.words;
    brick_arena_.release();
    NB_ = 0;
    for (VolHost& v : vols_) {
        v.nbx = v.px / c.bx; v.nby = v.py / c.by; v.nbz = v.pz / c.bz;
        v.brick_base = (uint32_t)NB_;
        NB_ += (uint64_t)v.nbx * v.nby * v.nbz;
    }
    LSS_REQUIRE(NB_ < (1ull << 31), LSS_ERR_CAPACITY, "too many bricks");
    NW_ = (uint32_t)((NB_ + 31) / 32);
    brick_arena_.set_budget(arena_.budget_left());
    auto A = [&](size_t n) { return brick_arena_.alloc(n); };
    d_vols_ = (NsVol*)A(sizeof(NsVol) * vols_.size());
    d_vstate_ = (NsVolState*)A(sizeof(NsVolState) * vols_.size());
    d_tmaps_ = (CUtensorMap*)A(sizeof(CUtensorMap) * 5 * vols_.size());
    for (int q = 0; q < 2; ++q) d_masks_[q] = (unsigned long long*)A(NB_ * words_ * 8);
    for (int q = 0; q < 4; ++q) d_bits_[q] = (uint32_t*)A((size_t)NW_ * 4);
    for (int q = 0; q < 3; ++q) d_cnt_[q] = (unsigned long long*)A(8 * vols_.size());
    d_brick_vol_ = (uint16_t*)A(NB_ * 2);
    d_status_ = (uint64_t*)A((std::max<uint64_t>(NW_, NB_) / 32 + 16) * 8);
    d_ctl_ = (NsCtl*)A(sizeof(NsCtl));
    d_misc_ = (uint32_t*)A(64);
    std::vector<uint16_t> bv(NB_);
    for (size_t i = 0; i < vols_.size(); ++i) {
        const VolHost& v = vols_[i];
        std::fill(bv.begin() + v.brick_base, bv.begin() + v.brick_base + (size_t)v.nbx * v.nby * v.nbz,
                  (uint16_t)i);
    }
    cudaStream_t st = owner_->stream;
    LSS_CUDA(cudaMemcpyAsync(d_brick_vol_, bv.data(), NB_ * 2, cudaMemcpyHostToDevice, st));
    std::vector<CUtensorMap> maps(5 * vols_.size());
    for (size_t i = 0; i < vols_.size(); ++i) {
        const VolHost& v = vols_[i];
        const uint64_t pxy = (uint64_t)v.px * v.py;
        for (int q = 0; q < 2; ++q) {
            encode_tmap_f32_3d(&maps[5 * i + q], v.phi[q], v.nx, v.ny, v.nz, v.px, pxy, c.bx + 8,
                               c.by + 2, c.bz + 2);
            encode_tmap_f32_3d(&maps[5 * i + 2 + q], v.phi[q], v.nx, v.ny, v.nz, v.px, pxy, c.bx, c.by,
                               c.bz);
        }
        encode_tmap_f32_3d(&maps[5 * i + 4], v.speed, v.nx, v.ny, v.nz, v.px, pxy, c.bx, c.by, c.bz);
    }
    LSS_CUDA(cudaMemcpyAsync(d_tmaps_, maps.data(), maps.size() * sizeof(CUtensorMap),
                             cudaMemcpyHostToDevice, st));
    LSS_CUDA(cudaMemsetAsync(d_vstate_, 0, sizeof(NsVolState) * vols_.size(), st));
    LSS_CUDA(cudaMemsetAsync(d_ctl_, 0, sizeof(NsCtl), st));
    ctl_arrivals_ = ctl_upd_sum_[0] = ctl_upd_sum_[1] = 0;
    upload_descriptors();
    // Co-residency of the persistent grid.
    const size_t dyn = dyn_smem();
    int per_sm = 0;
    LSS_CUDA(cudaFuncSetAttribute(ks.persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    LSS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ks.persistent, ks.pblock, dyn));
    LSS_REQUIRE(per_sm > 0, LSS_ERR_CUDA, "persistent kernel does not fit on an SM");
    grid_ = owner_->num_sms * per_sm;
    block_threads_ = ks.pblock;
    configured_ = true;
    owner_->sync();
}

void NsCore::refresh_speed() {
    for (int v = 0; v < (int)vols_.size(); ++v) {
        VolHost& V = vols_[v];
        if (!V.speed_stale) continue;
        const uint64_t n4 = (uint64_t)V.px * V.py * V.pz / 4;
        k_ns_speed<<<owner_->num_sms * 4, 256, 0, owner_->stream>>>(descriptor(v), V.speed, n4);
        ++owner_->launches;
        LSS_CUDA(cudaGetLastError());
        V.speed_stale = false;
    }
}

size_t NsCore::dyn_smem() const {
    return kernels(cfg_).smem_fixed + stop_state_bytes((int)vols_.size());
}

NsVol NsCore::descriptor(int i) const {
    const VolHost& v = vols_.at(i);
    NsVol o;
    std::memset(&o, 0, sizeof(o));
    o.nx = v.nx; o.ny = v.ny; o.nz = v.nz;
    o.px = v.px; o.py = v.py; o.pz = v.pz;
    o.nbx = v.nbx; o.nby = v.nby; o.nbz = v.nbz;
    o.mnbx = 0xFFFFFFFFu / (uint32_t)v.nbx + 1u;
    o.mnbxy = 0xFFFFFFFFu / ((uint32_t)v.nbx * (uint32_t)v.nby) + 1u;
    o.brick_base = v.brick_base;
    o.phi[0] = v.phi[0]; o.phi[1] = v.phi[1];
    o.img = v.img;
    o.bias = nullptr;  // the adjoint sets its own
    o.speed = v.speed;
    o.T = v.p.target; o.eps = v.p.window; o.alpha = v.p.curvature; o.dt = v.p.time_step;
    o.lo = v.p.phi_min; o.hi = v.p.phi_max;
    o.thr_t = v.p.temporal_threshold; o.thr_s = v.p.spatial_threshold;
    o.alpha_data = v.p.alpha_role == LSS_ALPHA_CURVATURE ? 0 : 1;
    o.data_literal = v.p.data_term == LSS_DATA_LITERAL ? 1 : 0;
    o.inv_eps = o.data_literal ? 1.0f : 1.0f / v.p.window;
    o.dlo = o.data_literal ? -INFINITY : -1.0f;
    o.dhi = o.data_literal ? INFINITY : 1.0f;
    o.wc = o.alpha_data ? 1.0f - v.p.curvature : v.p.curvature;
    o.wd = 1.0f - o.wc;
    o.nbh = v.p.neighbourhood == 6 ? 6 : 26;
    o.tmap_base = (uint32_t)(5 * i);
    return o;
}

void NsCore::upload_descriptors() {
    std::vector<NsVol> d(vols_.size());
    for (size_t i = 0; i < vols_.size(); ++i) d[i] = descriptor((int)i);
    if (d_vols_)
        LSS_CUDA(cudaMemcpyAsync(d_vols_, d.data(), d.size() * sizeof(NsVol), cudaMemcpyHostToDevice,
                                 owner_->stream));
}

NsArgs NsCore::args(uint32_t k0, int max_iters, const lss_conv* conv) const {
    NsArgs a;
    std::memset(&a, 0, sizeof(a));
    a.vols = d_vols_;
    a.vstate = d_vstate_;
    a.nvol = (int32_t)vols_.size();
    a.tmaps = d_tmaps_;
    for (int q = 0; q < 2; ++q) a.masks[q] = d_masks_[q];
    for (int q = 0; q < 4; ++q) a.bits[q] = d_bits_[q];
    for (int q = 0; q < 3; ++q) a.cnt[q] = d_cnt_[q];
    a.brick_vol = d_brick_vol_;
    a.status = d_status_;
    a.ctl = d_ctl_;
    a.NB = (uint32_t)NB_;
    a.NW = NW_;
    a.k0 = k0;
    a.max_iters = max_iters;
    a.conv_mode = conv ? 1 : 0;
    a.arrivals0 = ctl_arrivals_;
    a.upd_sum0[0] = ctl_upd_sum_[0];
    a.upd_sum0[1] = ctl_upd_sum_[1];
    if (conv) {
        a.rel = conv->rel_threshold;
        a.patience = conv->patience;
        a.abs_thr = conv->abs_threshold;
    }
    return a;
}

// Rebuilds masks and membership bits of every volume from the current phi (the
// paper's initial active set, main.tex:217-231).  Both phi buffers are made
// equal first.
void NsCore::init_active() {
    LSS_REQUIRE(configured_, LSS_ERR_STATE, "not configured");
    cudaStream_t st = owner_->stream;
    // One volume whose phi is uniform outside a box (cleared, then seeded):
    // only that box can hold active voxels and differ between the buffers.
    const bool boxed = vols_.size() == 1 && vols_[0].uniform;
    int3 blo = make_int3(0, 0, 0), bn = make_int3(0, 0, 0);
    if (boxed) {
        VolHost& v = vols_[0];
        if (v.dirty_hi.x > v.dirty_lo.x && v.dirty_hi.y > v.dirty_lo.y && v.dirty_hi.z > v.dirty_lo.z) {
            // One voxel of margin for the 6-neighbour test, in whole bricks.
            blo = make_int3(std::max(0, v.dirty_lo.x - 1) / cfg_.bx, std::max(0, v.dirty_lo.y - 1) / cfg_.by,
                            std::max(0, v.dirty_lo.z - 1) / cfg_.bz);
            const int3 bhi = make_int3(std::min(v.nbx, (v.dirty_hi.x + 1 + cfg_.bx - 1) / cfg_.bx),
                                       std::min(v.nby, (v.dirty_hi.y + 1 + cfg_.by - 1) / cfg_.by),
                                       std::min(v.nbz, (v.dirty_hi.z + 1 + cfg_.bz - 1) / cfg_.bz));
            bn = make_int3(bhi.x - blo.x, bhi.y - blo.y, bhi.z - blo.z);
            k_ns_copy_box<<<owner_->num_sms * 4, 256, 0, st>>>(v.phi[parity_ ^ 1], v.phi[parity_], v.px, v.py,
                                                              v.dirty_lo, v.dirty_hi);
            ++owner_->launches;
        }
    } else {
        for (VolHost& v : vols_) {
            const uint64_t P = (uint64_t)v.px * v.py * v.pz;
            LSS_CUDA(cudaMemcpyAsync(v.phi[parity_ ^ 1], v.phi[parity_], P * 4, cudaMemcpyDeviceToDevice, st));
        }
    }
    for (int q = 0; q < 2; ++q) LSS_CUDA(cudaMemsetAsync(d_masks_[q], 0, NB_ * words_ * 8, st));
    for (int q = 0; q < 4; ++q) LSS_CUDA(cudaMemsetAsync(d_bits_[q], 0, (size_t)NW_ * 4, st));
    for (int q = 0; q < 3; ++q) LSS_CUDA(cudaMemsetAsync(d_cnt_[q], 0, 8 * vols_.size(), st));
    LSS_CUDA(cudaMemsetAsync(d_ctl_, 0, sizeof(NsCtl), st));
    ctl_arrivals_ = ctl_upd_sum_[0] = ctl_upd_sum_[1] = 0;
    // The global iteration index restarts at the phi parity: bits[k%4] holds
    // A_0 (the other three slots are empty, so A_{-1} is empty too).
    k_total_ = parity_;
    const uint32_t s0 = k_total_ % 4u;
    KernelSet ks = kernels(cfg_);
    NsArgs a = args(k_total_, 0, nullptr);
    uint32_t p = parity_, sl = s0;
    const uint64_t nbr = boxed ? (uint64_t)bn.x * bn.y * bn.z : NB_;
    if (!boxed || nbr > 0) {
        void* params[] = {&a, &p, &sl, &blo, &bn};
        const uint64_t warps = nbr * (uint64_t)(ks.words * 2);  // 32 voxels per warp
        const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((warps * 32 + ks.block - 1) / ks.block,
                                                                        (uint64_t)owner_->num_sms * 16));
        LSS_CUDA(cudaLaunchKernel(ks.init_active, dim3(grid), dim3(ks.block), params, 0, st));
        ++owner_->launches;
    }
    std::vector<unsigned long long> n0(vols_.size());
    LSS_CUDA(cudaMemcpyAsync(n0.data(), d_cnt_[0], 8 * vols_.size(), cudaMemcpyDeviceToHost, st));
    LSS_CUDA(cudaMemsetAsync(d_cnt_[0], 0, 8 * vols_.size(), st));
    owner_->sync();
    std::vector<NsVolState> vs(vols_.size());
    for (size_t i = 0; i < vols_.size(); ++i) {
        std::memset(&vs[i], 0, sizeof(NsVolState));
        vs[i].n0 = n0[i];
        vs[i].n_cur = n0[i];
        vs[i].parity = (int32_t)parity_;
        vols_[i].iterations = 0;
    }
    LSS_CUDA(cudaMemcpyAsync(d_vstate_, vs.data(), vs.size() * sizeof(NsVolState), cudaMemcpyHostToDevice,
                             st));
    owner_->sync();
    check_errors();
    initialized_ = true;
}

void NsCore::sphere_union(int v, float cx, float cy, float cz, float r) {
    ++epoch_;
    VolHost& V = vols_.at(v);
    // Voxels farther than r + phi_max from the centre keep phi (<= phi_max).
    const double reach = (double)r + std::max(0.0f, V.p.phi_max) + 1.0;
    auto lo = [&](double c, int n) { return std::max(0, std::min(n, (int)std::floor(c - reach))); };
    auto hi = [&](double c, int n) { return std::max(0, std::min(n, (int)std::ceil(c + reach) + 1)); };
    const int3 b0 = make_int3(lo(cx, V.nx), lo(cy, V.ny), lo(cz, V.nz));
    const int3 b1 = make_int3(hi(cx, V.nx), hi(cy, V.ny), hi(cz, V.nz));
    if (b1.x <= b0.x || b1.y <= b0.y || b1.z <= b0.z) return;
    if (V.uniform) {  // grow the box of voxels that may differ from the uniform value
        if (V.dirty_hi.x <= V.dirty_lo.x) {
            V.dirty_lo = b0;
            V.dirty_hi = b1;
        } else {
            V.dirty_lo = make_int3(std::min(V.dirty_lo.x, b0.x), std::min(V.dirty_lo.y, b0.y),
                                   std::min(V.dirty_lo.z, b0.z));
            V.dirty_hi = make_int3(std::max(V.dirty_hi.x, b1.x), std::max(V.dirty_hi.y, b1.y),
                                   std::max(V.dirty_hi.z, b1.z));
        }
    }
    k_ns_sphere_union<<<owner_->num_sms * 4, 256, 0, owner_->stream>>>(
        V.phi[parity_], V.nx, V.ny, V.nz, V.px, V.py, b0, b1, cx, cy, cz, r, V.p.phi_min, V.p.phi_max);
    ++owner_->launches;
    LSS_CUDA(cudaGetLastError());
}

void NsCore::set_phi(int v, const float* phi) {
    ++epoch_;
    VolHost& V = vols_.at(v);
    V.uniform = false;
    upload_padded(V.phi[parity_], phi, V, nullptr);
}

// Both buffers: phi is then uniform, which later seeding and active-set
// rebuilds exploit (only the seeded box can differ).
void NsCore::fill_phi(int v, float value) {
    ++epoch_;
    VolHost& V = vols_.at(v);
    for (int q = 0; q < 2; ++q) {
        k_ns_fill<<<owner_->num_sms * 4, 256, 0, owner_->stream>>>(V.phi[q], (uint64_t)V.px * V.py * V.pz,
                                                                  value);
        ++owner_->launches;
    }
    LSS_CUDA(cudaGetLastError());
    V.uniform = true;
    V.dirty_lo = V.dirty_hi = make_int3(0, 0, 0);
}

int NsCore::run(int max_iters, const lss_conv* conv, float* ms) {
    ++epoch_;
    LSS_REQUIRE(initialized_, LSS_ERR_STATE, "no seed / phi set");
    if (max_iters <= 0) return 0;
    refresh_speed();
    for (VolHost& v : vols_) v.uniform = false;
    cudaStream_t st = owner_->stream;
    KernelSet ks = kernels(cfg_);
    NsArgs a = args(k_total_, max_iters, conv);
    void* params[] = {&a};
    cudaEvent_t e0, e1;
    LSS_CUDA(cudaEventCreate(&e0));
    LSS_CUDA(cudaEventCreate(&e1));
    LSS_CUDA(cudaEventRecord(e0, st));
    if (fault_injected("launch")) throw Error(LSS_ERR_INJECTED, "injected launch failure");
    LSS_CUDA(cudaLaunchCooperativeKernel(ks.persistent, dim3(grid_), dim3(ks.pblock), params, dyn_smem(),
                                         st));
    ++owner_->launches;
    LSS_CUDA(cudaEventRecord(e1, st));
    LSS_CUDA(cudaEventSynchronize(e1));
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    if (ms) *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    NsCtl c;
    d2h(&c, d_ctl_, sizeof(c));
    ctl_arrivals_ = c.arrivals;
    ctl_upd_sum_[0] = c.upd_sum[0];
    ctl_upd_sum_[1] = c.upd_sum[1];
    if (fault_injected("timeout")) c.err |= ERR_BARRIER_TIMEOUT;
    LSS_REQUIRE(c.err == 0, LSS_ERR_TIMEOUT,
                "device-side wait gave up (error word " + std::to_string(c.err) + ")");
    std::vector<NsVolState> vs(vols_.size());
    d2h(vs.data(), d_vstate_, vs.size() * sizeof(NsVolState));
    k_total_ += c.iters_run;
    parity_ = k_total_ & 1u;
    last_update_ns_ = c.t_phase1_ns;
    last_barrier_ns_ = c.t_barrier_ns;
    for (size_t i = 0; i < vols_.size(); ++i) vols_[i].iterations = vs[i].iterations;
    return (int)c.iters_run;
}

void NsCore::d2h(void* dst, const void* src, size_t bytes) {
    LSS_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, owner_->stream));
    owner_->sync();
}

void NsCore::state(int v, NsVolState* out) {
    std::vector<NsVolState> vs(vols_.size());
    d2h(vs.data(), d_vstate_, vs.size() * sizeof(NsVolState));
    *out = vs.at(v);
}

uint32_t NsCore::vol_parity(int v) {
    NsVolState s;
    state(v, &s);
    return (uint32_t)s.parity;
}

void NsCore::reload_volume(int v, const float* data, const lss_params& p) {
    ++epoch_;
    LSS_REQUIRE(configured_, LSS_ERR_STATE, "not configured");
    VolHost& V = vols_.at(v);
    cudaStream_t st = owner_->stream;
    const uint64_t n = (uint64_t)V.nx * V.ny * V.nz, P = (uint64_t)V.px * V.py * V.pz;
    upload_padded(V.img, data, V, V.phi[1]);  // phi[1] stages; both are filled below
    for (int q = 0; q < 2; ++q) {
        k_ns_fill<<<owner_->num_sms * 4, 256, 0, st>>>(V.phi[q], P, p.phi_max);
        ++owner_->launches;
    }
    V.p = p;
    V.speed_stale = true;
    V.uniform = true;
    V.dirty_lo = V.dirty_hi = make_int3(0, 0, 0);
    V.iterations = 0;
    if (V.frozen) LSS_CUDA(cudaMemsetAsync(V.frozen, 0, n, st));
    LSS_CUDA(cudaMemsetAsync(d_vstate_, 0, sizeof(NsVolState) * vols_.size(), st));
    LSS_CUDA(cudaMemsetAsync(d_ctl_, 0, sizeof(NsCtl), st));
    ctl_arrivals_ = ctl_upd_sum_[0] = ctl_upd_sum_[1] = 0;
    parity_ = 0;
    k_total_ = 0;
    initialized_ = false;
    upload_descriptors();
    LSS_CUDA(cudaGetLastError());
    owner_->sync();
}

void NsCore::read_mask(int v, uint8_t* out) {
    VolHost& V = vols_.at(v);
    const uint32_t p = vols_.size() == 1 ? parity_ : vol_parity(v);
    const uint64_t n = (uint64_t)V.nx * V.ny * V.nz;
    // Pinned host memory is written in place; else through a temporary.
    uint8_t* dev = (uint8_t*)pinned_device_ptr(out);
    uint8_t* tmp = dev ? nullptr : (uint8_t*)arena_.alloc(n);
    k_ns_mask<<<owner_->num_sms * 4, 256, 0, owner_->stream>>>(dev ? dev : tmp, V.phi[p], V.frozen, V.nx, V.ny,
                                                              V.nz, V.px, V.py);
    ++owner_->launches;
    if (tmp) LSS_CUDA(cudaMemcpyAsync(out, tmp, n, cudaMemcpyDeviceToHost, owner_->stream));
    LSS_CUDA(cudaGetLastError());
    owner_->sync();
    if (tmp) arena_.free_last(tmp);
}

void NsCore::freeze(int v) {
    VolHost& V = vols_.at(v);
    const uint32_t p = vols_.size() == 1 ? parity_ : vol_parity(v);
    const uint64_t n = (uint64_t)V.nx * V.ny * V.nz;
    if (!V.frozen) {
        V.frozen = (uint8_t*)arena_.alloc(n);
        LSS_CUDA(cudaMemsetAsync(V.frozen, 0, n, owner_->stream));
    }
    k_ns_mask<<<owner_->num_sms * 4, 256, 0, owner_->stream>>>(V.frozen, V.phi[p], V.frozen, V.nx, V.ny, V.nz,
                                                              V.px, V.py);
    ++owner_->launches;
    LSS_CUDA(cudaGetLastError());
    owner_->sync();
}

void NsCore::clear_frozen(int v) {
    VolHost& V = vols_.at(v);
    if (V.frozen) LSS_CUDA(cudaMemsetAsync(V.frozen, 0, (uint64_t)V.nx * V.ny * V.nz, owner_->stream));
    owner_->sync();
}

void NsCore::read_phi(int v, float* out) {
    VolHost& V = vols_.at(v);
    const uint32_t p = vols_.size() == 1 ? parity_ : vol_parity(v);
    // Pinned host memory is written in place; else through a temporary.
    float* dev = (float*)pinned_device_ptr(out);
    float* tmp = dev ? nullptr : (float*)arena_.alloc((uint64_t)V.nx * V.ny * V.nz * 4);
    k_ns_gather<<<owner_->num_sms * 4, 256, 0, owner_->stream>>>(dev ? dev : tmp, V.phi[p], V.nx, V.ny, V.nz,
                                                                V.px, V.py);
    ++owner_->launches;
    if (tmp)
        LSS_CUDA(cudaMemcpyAsync(out, tmp, (uint64_t)V.nx * V.ny * V.nz * 4, cudaMemcpyDeviceToHost,
                                 owner_->stream));
    LSS_CUDA(cudaGetLastError());
    owner_->sync();
    if (tmp) arena_.free_last(tmp);
}

uint64_t NsCore::read_active(int v, uint64_t* out, uint64_t cap) {
    LSS_REQUIRE(vols_.size() == 1 && v == 0, LSS_ERR_UNSUPPORTED, "active list of a single volume only");
    LSS_REQUIRE(initialized_, LSS_ERR_STATE, "no seed / phi set");
    cudaStream_t st = owner_->stream;
    KernelSet ks = kernels(cfg_);
    const uint32_t s = k_total_ % 4u;
    unsigned long long* total = (unsigned long long*)d_misc_;
    auto emit = [&](uint64_t* dout) {
        // one status word per tile of block / 32 membership words
        LSS_CUDA(cudaMemsetAsync(d_status_, 0, ((uint64_t)NW_ / (ks.block / 32) + 2) * 8, st));
        LSS_CUDA(cudaMemsetAsync(d_misc_, 0, 16, st));
        LSS_CUDA(cudaMemsetAsync(&d_ctl_->emit_tile, 0, 4, st));
        NsArgs a = args(k_total_, 0, nullptr);
        uint32_t p = parity_, sl = s;
        void* params[] = {&a, &p, &sl, &dout, &total};
        LSS_CUDA(cudaLaunchKernel(ks.emit, dim3(owner_->num_sms * 2), dim3(ks.block), params, 0, st));
        ++owner_->launches;
        unsigned long long n = 0;
        LSS_CUDA(cudaMemcpyAsync(&n, total, 8, cudaMemcpyDeviceToHost, st));
        owner_->sync();
        check_errors();
        return (uint64_t)n;
    };
    const uint64_t n = emit(nullptr);
    if (!out || n == 0) return n;
    uint64_t* dout = (uint64_t*)arena_.alloc(n * 8);
    emit(dout);
    const uint64_t m = std::min(n, cap);
    LSS_CUDA(cudaMemcpyAsync(out, dout, m * 8, cudaMemcpyDeviceToHost, st));
    owner_->sync();
    arena_.free_last(dout);
    return n;
}

void NsCore::estimate(int v, float* t, float* w) {
    VolHost& V = vols_.at(v);
    double* acc = (double*)arena_.alloc(32);
    double h[3];
    double mean = 0;
    for (int pass = 0; pass < 2; ++pass) {
        LSS_CUDA(cudaMemsetAsync(acc, 0, 24, owner_->stream));
        k_ns_collect<<<owner_->num_sms * 4, 256, 0, owner_->stream>>>(V.img, V.phi[parity_], V.nx, V.ny,
                                                                     V.nz, V.px, V.py, mean, acc);
        ++owner_->launches;
        LSS_CUDA(cudaMemcpyAsync(h, acc, 24, cudaMemcpyDeviceToHost, owner_->stream));
        owner_->sync();
        LSS_REQUIRE(h[2] >= 2, LSS_ERR_STATE, "fewer than two segmented voxels");
        if (pass == 0) mean = h[0] / h[2];
    }
    arena_.free_last(acc);
    *t = (float)mean;
    *w = (float)std::sqrt(h[1] / (h[2] - 1));
}

float NsCore::dense_run(int iters) {
    ++epoch_;
    LSS_REQUIRE(initialized_, LSS_ERR_STATE, "no seed / phi set");
    refresh_speed();
    for (VolHost& v : vols_) v.uniform = false;
    cudaStream_t st = owner_->stream;
    cudaEvent_t e0, e1;
    LSS_CUDA(cudaEventCreate(&e0));
    LSS_CUDA(cudaEventCreate(&e1));
    LSS_CUDA(cudaEventRecord(e0, st));
    for (int it = 0; it < iters; ++it) {
        for (int v = 0; v < (int)vols_.size(); ++v) {
            const VolHost& V = vols_[v];
            // Planes per block: up to kDenseZMax, fewer when the volume is
            // small, so that the grid still has about four blocks per SM.
            const int gx = (V.nx + kDenseX - 1) / kDenseX, gy = (V.ny + kDenseY - 1) / kDenseY;
            const int chunks = std::max(1, (4 * owner_->num_sms + gx * gy - 1) / (gx * gy));
            const int zc = std::max(2, std::min(kDenseZMax, (V.nz + chunks - 1) / chunks));
            dim3 grid(gx, gy, (V.nz + zc - 1) / zc);
            k_ns_dense<<<grid, 256, 0, st>>>(descriptor(v), parity_, zc);
            ++owner_->launches;
        }
        parity_ ^= 1u;
    }
    LSS_CUDA(cudaEventRecord(e1, st));
    LSS_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    LSS_CUDA(cudaGetLastError());
    init_active();  // the dense pass leaves no active set: rebuild it from phi
    return ms;
}

void NsCore::check_errors() {
    LSS_CUDA(cudaGetLastError());
    NsCtl c;
    d2h(&c, d_ctl_, sizeof(c));
    LSS_REQUIRE(c.err == 0, LSS_ERR_TIMEOUT, "device-side wait gave up (error word " + std::to_string(c.err) + ")");
}

}  // namespace lss
