// ORACLE — test infrastructure only.  Nothing in the product links, imports
// or runs this file; tests, smoke() and bench.py's CPU legs use it as the
// parity reference.
//
// CPU restatement of the reference's level-set solver path in its
// reference-faithful form (LSS_MODE_REF):
//   * indexing helpers   — code/gpuseg/code/src/cuda/Coordinates.cu:42-208,
//                          Math.cu:68-71, Textures.cu:12 (normalised int8 reads)
//   * kernels (backend)  — UpdateLevelSetVolume.cu:222-342,
//                          UpdateActiveElements.cu:34-104,
//                          UpdateActiveElementsVolume.cu:39-100, 210-363,
//                          FilterDuplicates.cu:73-193, MemSetFloat.cu:227-290,
//                          InitializeLevelSetVolume.cu:55-98, 151-169,
//                          InitializeActiveElementsVolume.cu:37-72,
//                          InitializeCoordinateVolume.cu:37-47,
//                          ExportActiveElementsVolume.cu:43-73
//   * stream compaction  — CUDPP 1.1 cudppCompact (third-party, not vendored;
//                          call sites Cuda.cpp:699-758): stable compaction of
//                          src[i] where valid[i] != 0.
//   * driver             — Segmenter.cpp:110-285, 491-595, 597-679, 759-1056,
//                          1131-1204, 1216-1337, 1339-1374, 357-478
//
// The driver is a template over a kernel backend so that the same sequence
// can drive either the restated kernels below (RestatedBackend) or the
// reference's own kernel sources compiled for the CPU (oracle/ref_shim).
//
// Texture reads that race with writes of the same kernel (only the tag volume
// in FilterDuplicatesFilterKernel) are modelled as reads of the state at
// kernel launch: CUDA leaves such reads undefined, and this is the outcome
// of an incoherent texture cache.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace lssref {

struct Dims {
    uint32_t x, y, z;
    size_t n() const { return (size_t)x * y * z; }
};

// __float2int_rd with PTX cvt.rmi.s32.f32 semantics: NaN -> 0, saturating.
inline int32_t f2i_rd(float f) {
    if (f != f) return 0;
    float r = std::floor(f);
    if (r >= 2147483648.0f) return 2147483647;
    if (r < -2147483648.0f) return (-2147483647 - 1);
    return (int32_t)r;
}

// ComputeIndex3DTo1D (Coordinates.cu:42-47).
inline uint32_t lin(uint32_t x, uint32_t y, uint32_t z, Dims d) {
    return z * (d.y * d.x) + y * d.x + x;
}

// ComputeIndex3DToTiled1D (Coordinates.cu:65-96): 16^3 tiles in x-fastest tile
// order, voxels x-fastest inside a tile.
inline uint32_t tiled(uint32_t x, uint32_t y, uint32_t z, Dims d) {
    if (x >= d.x || y >= d.y || z >= d.z)
        throw std::out_of_range("coordinate outside the volume (the reference would index out of bounds)");
    uint32_t tile = (z >> 4) * ((d.y >> 4) * (d.x >> 4)) + (y >> 4) * (d.x >> 4) + (x >> 4);
    return tile * 4096u + ((z & 15u) * 16u + (y & 15u)) * 16u + (x & 15u);
}

struct U3 { uint32_t x, y, z; };

// PackCoordinates / UnpackCoordinates (Coordinates.cu:186-208): 10/10/10 bits.
inline uint32_t pack(U3 v) { return v.x | (v.y << 10) | (v.z << 20); }
inline U3 unpack(uint32_t p) { return U3{p & 0x3FFu, (p >> 10) & 0x3FFu, (p >> 20) & 0x3FFu}; }

// OffsetCoordinates (Coordinates.cu:132-155): an out-of-range neighbour is the
// voxel itself.
inline U3 offset(U3 v, int dx, int dy, int dz, Dims d) {
    int64_t x = (int64_t)v.x + dx, y = (int64_t)v.y + dy, z = (int64_t)v.z + dz;
    if (x < 0 || y < 0 || z < 0 || x >= d.x || y >= d.y || z >= d.z) return v;
    return U3{(uint32_t)x, (uint32_t)y, (uint32_t)z};
}

// Normalised-float texture read of the int8 level set (Textures.cu:12,
// cudaReadModeNormalizedFloat): c / 127, floored at -1.
inline float nread(int8_t c) {
    float f = (float)c / 127.0f;
    return f < -1.0f ? -1.0f : f;
}

// Equals (Math.cu:156-171).
inline float rabs(float f) { return f > 0 ? f : -1.0f * f; }
inline bool equals(float a, float b, float eps) { return rabs(a - b) <= eps; }

inline float fclamp(float i, float lo, float hi) {  // Math.cu:136-149
    if (i < lo) return lo;
    if (i > hi) return hi;
    return i;
}

inline uint32_t align256(uint32_t v) { return v + (256u - v % 256u) % 256u; }  // Cuda.cpp:191-200

// dtype codes, as lss_dtype.
enum { DT_U8 = 0, DT_S8 = 1, DT_U16 = 2, DT_S16 = 3, DT_U32 = 4, DT_S32 = 5, DT_F32 = 6 };

inline int bytes_of(int dt) { return dt <= 1 ? 1 : dt <= 3 ? 2 : 4; }
inline bool is_signed(int dt) { return dt == DT_S8 || dt == DT_S16 || dt == DT_S32; }

// The source sample as the int parameter of ComputeDensityTerm.
inline int32_t sample_int(const void* src, int dt, size_t i) {
    switch (dt) {
        case DT_U8: return ((const uint8_t*)src)[i];
        case DT_S8: return ((const int8_t*)src)[i];
        case DT_U16: return ((const uint16_t*)src)[i];
        case DT_S16: return ((const int16_t*)src)[i];
        case DT_U32: return (int32_t)((const uint32_t*)src)[i];
        case DT_S32: return ((const int32_t*)src)[i];
    }
    return 0;
}

// The seven output offsets in segment order (UpdateActiveElementsVolume.cu:168-182):
// -z, -y, -x, self, +x, +y, +z.
static const int kSegOff[7][3] = {{0, 0, -1}, {0, -1, 0}, {-1, 0, 0}, {0, 0, 0},
                                  {1, 0, 0},  {0, 1, 0},  {0, 0, 1}};

// ComputeActiveElementOutputs (UpdateActiveElements.cu:34-104), 6-connected
// branch with temporal culling.  out[] is indexed in segment order.
inline void active_outputs(U3 v, Dims d, const int8_t* rd, const uint8_t* tag, bool out[7]) {
    for (int e = 0; e < 7; ++e) out[e] = false;
    float u4 = nread(rd[tiled(v.x, v.y, v.z, d)]);
    if (tag[tiled(v.x, v.y, v.z, d)] != 1) return;
    const float tol = 0.008f;
    // test order -z, -y, -x, +x, +y, +z (:86-102)
    static const int order[6] = {0, 1, 2, 4, 5, 6};
    for (int k = 0; k < 6; ++k) {
        int e = order[k];
        U3 n = offset(v, kSegOff[e][0], kSegOff[e][1], kSegOff[e][2], d);
        float un = nread(rd[tiled(n.x, n.y, n.z, d)]);
        if (!equals(u4, un, tol)) { out[3] = true; out[e] = true; }
    }
}

// ---------------------------------------------------------------------------
// Restated kernels.
struct RestatedBackend {
    bool quirk_i3 = true;  // UpdateActiveElementsVolume.cu:82,329 loop `i < 3`

    bool skip(size_t i) const { return quirk_i3 && (i % 4) == 3; }

    // InitializeLevelSetKernel (InitializeLevelSetVolume.cu:55-98).
    void init_level_set(int8_t* wr, uint8_t* ex, Dims d, const int8_t* rd, U3 seed, int32_t r,
                        float aniso) {
        for (uint32_t z = 0; z < d.z; ++z)
            for (uint32_t y = 0; y < d.y; ++y)
                for (uint32_t x = 0; x < d.x; ++x) {
                    uint32_t ti = tiled(x, y, z, d), li = lin(x, y, z, d);
                    int32_t vx = (int32_t)(seed.x - x), vy = (int32_t)(seed.y - y);
                    float vz = ((float)(int32_t)seed.z - (float)(int32_t)z) * aniso;
                    float fx = (float)vx, fy = (float)vy;
                    float d2 = fx * fx + fy * fy + vz * vz;
                    float dist = std::sqrt(d2);
                    float smooth = 4.0f, cur = 1.0f;
                    if (dist < (float)r) cur = -1.0f;
                    else if (dist < (float)r + smooth) cur = -1.0f + ((dist - (float)r) / (smooth / 2.0f));
                    float old = nread(rd[ti]);
                    float nv = fclamp(old + cur - 1.0f, -1.0f, 1.0f);
                    wr[ti] = (int8_t)f2i_rd(nv * 127.0f);
                    ex[li] = (uint8_t)f2i_rd(nv * 127.0f);
                }
    }

    // InitializeActiveElementsVolumeKernel (InitializeActiveElementsVolume.cu:37-72).
    void init_active_volume(uint32_t* valid, Dims d, const int8_t* rd) {
        for (uint32_t z = 0; z < d.z; ++z)
            for (uint32_t y = 0; y < d.y; ++y)
                for (uint32_t x = 0; x < d.x; ++x) {
                    U3 v{x, y, z};
                    float u4 = nread(rd[tiled(x, y, z, d)]);
                    bool flat = true;
                    static const int order[6] = {0, 1, 2, 4, 5, 6};
                    for (int k = 0; k < 6 && flat; ++k) {
                        int e = order[k];
                        U3 n = offset(v, kSegOff[e][0], kSegOff[e][1], kSegOff[e][2], d);
                        if (!equals(u4, nread(rd[tiled(n.x, n.y, n.z, d)]), 0.001f)) flat = false;
                    }
                    valid[tiled(x, y, z, d)] = flat ? 0u : 1u;
                }
    }

    // InitializeCoordinateVolumeKernel (InitializeCoordinateVolume.cu:37-47).
    void init_coord_volume(uint32_t* coord, Dims d) {
        for (uint32_t z = 0; z < d.z; ++z)
            for (uint32_t y = 0; y < d.y; ++y)
                for (uint32_t x = 0; x < d.x; ++x) coord[tiled(x, y, z, d)] = pack(U3{x, y, z});
    }

    // UpdateLevelSetVolumeKernelHelper (UpdateLevelSetVolume.cu:222-342).
    void update(int8_t* wr, uint8_t* ex, uint8_t* tag, size_t n, Dims d, int32_t target,
                int32_t window, float alpha, float dt_in, const int8_t* rd, const uint32_t* active,
                const void* src, int dtype) {
        for (size_t i = 0; i < n; ++i) {
            U3 v = unpack(active[i]);
            auto R = [&](int dx, int dy, int dz) {
                U3 q = offset(v, dx, dy, dz, d);
                return nread(rd[tiled(q.x, q.y, q.z, d)]);
            };
            float u4nz = R(0, 0, -1), u1 = R(0, -1, 0), u3 = R(-1, 0, 0), u4 = R(0, 0, 0),
                  u5 = R(1, 0, 0), u7 = R(0, 1, 0), u4pz = R(0, 0, 1);
            int32_t s = sample_int(src, dtype, lin(v.x, v.y, v.z, d));
            float dcx = (u5 - u3) / 2.0f, dcy = (u7 - u1) / 2.0f, dcz = (u4pz - u4nz) / 2.0f;
            float fx = u5 - u4, fy = u7 - u4, fz = u4pz - u4;
            float bx = u4 - u3, by = u4 - u1, bz = u4 - u4nz;
            float sx = fx - bx, sy = fy - by, sz = fz - bz;
            float conn = 0.0f;
            if (alpha > 0.0f) {
                if (equals(u4pz, u4nz, 0.1f) && equals(u4nz, u1, 0.1f) && equals(u1, u3, 0.1f) &&
                    equals(u3, u5, 0.1f) && equals(u5, u7, 0.1f) && equals(u7, u4pz, 0.1f)) {
                    float avg = (u4pz + u1 + u3 + u5 + u7 + u4nz) / 6.0f;
                    conn = avg - u4;
                }
            }
            float curv = sx + sy + sz;
            // ComputeDensityTerm (:335-342): window arrives as unsigned int.
            int32_t diff = s - target;
            int32_t adiff = diff < 0 ? -diff : diff;
            float dens = (-1.0f / (float)(uint32_t)window) * (float)adiff + 1.0f;
            dens = -dens;
            float dt = dt_in;
            if (dt < 0) { dt = -dt; dens = -dens; }
            float speed = ((1.0f - alpha) * dens) + (alpha * curv);
            float glen = std::sqrt(dcx * dcx + dcy * dcy + dcz * dcz);
            float delta = ((dt * speed * glen)) + conn;
            float nv = std::fmin(1.0f, std::fmax(-1.0f, u4 + delta));
            nv = std::fmin(1.0f, std::fmax(-1.0f, (((1.0f + 0.01f) * nv) + 0.01f)));
            uint32_t ti = tiled(v.x, v.y, v.z, d);
            wr[ti] = (int8_t)f2i_rd(nv * 127.0f);
            ex[lin(v.x, v.y, v.z, d)] = (uint8_t)f2i_rd(nv * 127.0f);
            float td = nv - u4;
            tag[ti] = std::fabs(td) > 0.008f ? 1 : 0;
        }
    }

    // OutputNewActiveElementsKernel (UpdateActiveElementsVolume.cu:210-363).
    void output_new(uint32_t* coord, uint32_t* valid, size_t n, Dims d, const int8_t* rd,
                    const uint8_t* tag, const uint32_t* active) {
        uint32_t A = align256((uint32_t)n);
        for (size_t i = 0; i < n; ++i) {
            if (skip(i)) continue;
            U3 v = unpack(active[i]);
            bool out[7];
            active_outputs(v, d, rd, tag, out);
            for (int e = 0; e < 7; ++e)
                if (out[e]) {
                    U3 q = offset(v, kSegOff[e][0], kSegOff[e][1], kSegOff[e][2], d);
                    coord[(size_t)e * A + i] = pack(q);
                    valid[(size_t)e * A + i] = 1;
                }
        }
    }

    // MemSetSparseKernel (MemSetFloat.cu:227-290).
    template <typename T>
    void memset_sparse(T* buf, T val, size_t n, Dims d, const uint32_t* active) {
        for (size_t i = 0; i < n; ++i) {
            U3 v = unpack(active[i]);
            buf[tiled(v.x, v.y, v.z, d)] = val;
        }
    }

    // FilterDuplicates{Initialize,Filter}Kernel (FilterDuplicates.cu:16-193).
    void filter(uint32_t* coord, uint32_t* valid, uint8_t* tag, size_t n, Dims d) {
        uint32_t A = align256((uint32_t)n);
        for (size_t i = 0; i < n; ++i)
            if (valid[i] == 1) {
                U3 v = unpack(coord[i]);
                tag[tiled(v.x, v.y, v.z, d)] = 1;
            }
        std::vector<uint32_t> pending;
        for (int e = 1; e < 7; ++e) {
            pending.clear();
            for (size_t i = 0; i < n; ++i) {
                size_t k = (size_t)e * A + i;
                if (valid[k] != 1) continue;
                U3 v = unpack(coord[k]);
                uint32_t t = tiled(v.x, v.y, v.z, d);
                if (tag[t] == 1) valid[k] = 0;  // read: state at kernel launch
                else pending.push_back(t);
            }
            for (uint32_t t : pending) tag[t] = 1;
        }
    }

    // UpdateActiveElementsVolumeKernel (UpdateActiveElementsVolume.cu:39-100).
    void update_active_volume(uint32_t* valid, size_t n, Dims d, const int8_t* rd,
                              const uint8_t* tag, const uint32_t* active) {
        for (size_t i = 0; i < n; ++i) {
            if (skip(i)) continue;
            U3 v = unpack(active[i]);
            bool out[7];
            active_outputs(v, d, rd, tag, out);
            for (int e = 0; e < 7; ++e)
                if (out[e]) {
                    U3 q = offset(v, kSegOff[e][0], kSegOff[e][1], kSegOff[e][2], d);
                    valid[tiled(q.x, q.y, q.z, d)] = 1;
                }
        }
    }

    // AddLevelSetKernel (InitializeLevelSetVolume.cu:151-169).
    void add_level_set(uint8_t* res, const uint8_t* add, Dims d) {
        size_t N = d.n();
        for (size_t i = 0; i < N; ++i) {
            float o = (float)(int8_t)res[i] / 127.0f;
            float a = (float)(int8_t)add[i] / 127.0f;
            float r = fclamp(o + a - 1.0f, -1.0f, 1.0f);
            res[i] = (uint8_t)f2i_rd(r * 127.0f);
        }
    }

    // ExportActiveElementsVolumeKernel (ExportActiveElementsVolume.cu:43-73).
    void export_active(uint8_t* out, size_t n, Dims d, const uint32_t* active) {
        memset_sparse<uint8_t>(out, 127, n, d, active);
    }
};

// CUDPP 1.1 cudppCompact as called by CudppCompact (Cuda.cpp:699-758):
// stable, order preserving; returns the number of valid elements.
inline size_t compact(const uint32_t* src, const uint32_t* valid, uint32_t* dst, size_t m) {
    size_t k = 0;
    for (size_t i = 0; i < m; ++i)
        if (valid[i] != 0) dst[k++] = src[i];
    return k;
}

// ---------------------------------------------------------------------------
// The driver: Segmenter's solver-path members, headless.
template <class Backend>
class RefSegmenter {
   public:
    Backend be;
    Dims d{0, 0, 0};
    size_t N = 0;
    uint32_t ux = 0, uy = 0, uz = 0;  // unpadded dims
    int dtype = 0;
    float zaniso = 1.0f;
    std::vector<uint8_t> src;  // padded, linear, dtype-typed
    std::vector<int8_t> phiX, phiY;
    int8_t* rd = nullptr;
    int8_t* wr = nullptr;
    std::vector<uint8_t> exportv, frozen, tag;
    std::vector<uint32_t> coord, valid, active;
    size_t n = 0;
    int iterations = 0;
    bool level_set_initialized = false, coord_initialized = false;
    float T = 0, W = 0, A = 0, DT = 0, conv = 0;
    float Tp = 0, Wp = 0, Ap = 0;  // "previous" values (Segmenter.cpp:71-73 start at 0)
    std::string err;

    bool params_changed() const { return Tp != T || Wp != W || Ap != A; }

    void swap_buffers() {  // SwapLevelSetBuffers (:1339-1351)
        if (rd == phiX.data()) { rd = phiY.data(); wr = phiX.data(); }
        else { rd = phiX.data(); wr = phiY.data(); }
    }

    // LoadVolume + LoadVolumeHostPadded (:110-285, :1131-1204).
    void load(const void* data, uint32_t nx, uint32_t ny, uint32_t nz, int dt, float aniso) {
        if (dt < 0 || dt > 5) throw std::invalid_argument("REF mode takes integer voxel types");
        uint32_t px = nx + (16 - nx % 16) % 16, py = ny + (16 - ny % 16) % 16,
                 pz = nz + (16 - nz % 16) % 16;
        if (px > 1024 || py > 1024 || pz > 1024) throw std::invalid_argument("padded size > 1024");
        ux = nx; uy = ny; uz = nz; dtype = dt; zaniso = aniso;
        d = Dims{px, py, pz};
        N = d.n();
        int bpv = bytes_of(dt);
        src.assign(N * bpv, 0);
        const uint8_t* in = (const uint8_t*)data;
        int pad = is_signed(dt) ? -127 : 0;
        size_t pi = 0, ri = 0, rowb = (size_t)nx * bpv;
        size_t padx = (size_t)(px - nx) * bpv, pady = (size_t)(py - ny) * px * bpv,
               padz = (size_t)(pz - nz) * py * px * bpv;
        for (uint32_t z = 0; z < nz; ++z) {
            for (uint32_t y = 0; y < ny; ++y) {
                std::memcpy(&src[pi], in + ri, rowb);
                pi += rowb; ri += rowb;
                std::memset(&src[pi], pad, padx);
                pi += padx;
            }
            std::memset(&src[pi], pad, pady);
            pi += pady;
        }
        std::memset(&src[pi], pad, padz);
        phiX.assign(N, 127);
        phiY.assign(N, 127);
        coord.assign(N, 0xFFFFFFFFu);
        valid.assign(N, 0);
        tag.assign(N, 0);
        exportv.assign(N, 127);
        frozen.assign(N, 127);
        active.assign(N, 0);
        rd = phiX.data();
        wr = phiY.data();
        coord_initialized = false;
        level_set_initialized = false;
        n = 0;
    }

    void set_params(float t, float w, float a, float dt, float c) { T = t; W = w; A = a; DT = dt; conv = c; }

    // InitializeSeed (:491-595).
    void initialize_seed(float cx, float cy, float cz, float radius) {
        U3 seed{(uint32_t)cx, (uint32_t)cy, (uint32_t)cz};
        int32_t r = (int32_t)(uint32_t)radius;
        std::fill(active.begin(), active.end(), 0xFFFFFFFFu);
        std::fill(valid.begin(), valid.end(), 0u);
        std::fill(tag.begin(), tag.end(), 0);
        be.init_level_set(wr, exportv.data(), d, rd, seed, r, zaniso);
        swap_buffers();
        be.init_level_set(wr, exportv.data(), d, rd, seed, r, zaniso);
        swap_buffers();
        rebuild_active_dense();
        level_set_initialized = true;
        iterations = 0;
        Tp = T; Wp = W; Ap = A;
    }

    // The dense activity test + coordinate volume + full compaction
    // (:536-554).
    void rebuild_active_dense() {
        be.init_active_volume(valid.data(), d, rd);
        be.init_coord_volume(coord.data(), d);
        coord_initialized = true;
        n = compact(coord.data(), valid.data(), active.data(), N);
    }

    // Sets both int8 buffers and the export volume from floats, then the same
    // dense activity rebuild as InitializeSeed.  Not a reference operation.
    void set_phi(const float* phi) {
        std::fill(active.begin(), active.end(), 0xFFFFFFFFu);
        std::fill(valid.begin(), valid.end(), 0u);
        std::fill(tag.begin(), tag.end(), 0);
        std::fill(phiX.begin(), phiX.end(), 127);
        std::fill(phiY.begin(), phiY.end(), 127);
        std::fill(exportv.begin(), exportv.end(), 127);
        for (uint32_t z = 0; z < uz; ++z)
            for (uint32_t y = 0; y < uy; ++y)
                for (uint32_t x = 0; x < ux; ++x) {
                    float f = fclamp(phi[((size_t)z * uy + y) * ux + x], -1.0f, 1.0f);
                    int32_t c = f2i_rd(f * 127.0f);
                    phiX[tiled(x, y, z, d)] = (int8_t)c;
                    phiY[tiled(x, y, z, d)] = (int8_t)c;
                    exportv[lin(x, y, z, d)] = (uint8_t)c;
                }
        rebuild_active_dense();
        level_set_initialized = true;
        iterations = 0;
        Tp = T; Wp = W; Ap = A;
    }

    bool finished() const { return (float)n <= conv && iterations > 500; }  // :1053-1056

    bool few_active() const {  // ShouldOptimizeForFewActiveVoxels (:1363-1369)
        uint64_t aligned = (uint64_t)align256((uint32_t)n) * 7u;
        return aligned * 4u < (uint64_t)N * 4u;
    }

    // RequestUpdateSegmentation (:759-1051) with numSubSteps = k; returns the
    // number of substeps run.
    int request_update(int k) {
        if (params_changed()) iterations = 0;
        bool should = (level_set_initialized && !finished()) || params_changed();
        if (!should) return 0;
        for (int s = 0; s < k; ++s) {
            be.update(wr, exportv.data(), tag.data(), n, d, (int32_t)T, (int32_t)W, A, DT, rd,
                      active.data(), src.data(), dtype);
            swap_buffers();
            if (params_changed()) {
                Tp = T; Wp = W; Ap = A;
                iterations = 0;
                be.init_active_volume(valid.data(), d, rd);
                if (!coord_initialized) { coord_initialized = true; be.init_coord_volume(coord.data(), d); }
                n = compact(coord.data(), valid.data(), active.data(), N);
            } else if (few_active()) {
                coord_initialized = false;
                uint32_t Aal = align256((uint32_t)n);
                size_t total = (size_t)Aal * 7u;
                be.output_new(coord.data(), valid.data(), n, d, rd, tag.data(), active.data());
                be.template memset_sparse<uint8_t>(tag.data(), 0, n, d, active.data());
                be.filter(coord.data(), valid.data(), tag.data(), n, d);
                n = compact(coord.data(), valid.data(), active.data(), total);
                std::fill(valid.begin(), valid.begin() + total, 0u);
            } else {
                if (!coord_initialized) { coord_initialized = true; be.init_coord_volume(coord.data(), d); }
                be.update_active_volume(valid.data(), n, d, rd, tag.data(), active.data());
                n = compact(coord.data(), valid.data(), active.data(), N);
                be.template memset_sparse<uint32_t>(valid.data(), 0u, n, d, active.data());
            }
            ++iterations;
        }
        return k;
    }

    // GetSaveableSegmentation (:1216-1286), unpadded 0/1 mask; clears the
    // tag volume as a side effect, as the reference does.
    void read_mask(uint8_t* out) {
        std::memcpy(tag.data(), exportv.data(), N);
        be.add_level_set(tag.data(), frozen.data(), d);
        std::vector<uint8_t> host(tag);
        std::fill(tag.begin(), tag.end(), 0);
        for (uint32_t z = 0; z < uz; ++z)
            for (uint32_t y = 0; y < uy; ++y)
                for (uint32_t x = 0; x < ux; ++x)
                    out[((size_t)z * uy + y) * ux + x] = ((int8_t)host[lin(x, y, z, d)] <= 0) ? 1 : 0;
    }

    void read_phi(float* out) const {
        for (uint32_t z = 0; z < uz; ++z)
            for (uint32_t y = 0; y < uy; ++y)
                for (uint32_t x = 0; x < ux; ++x)
                    out[((size_t)z * uy + y) * ux + x] = nread(rd[tiled(x, y, z, d)]);
    }

    void read_export(int8_t* out) const {
        for (uint32_t z = 0; z < uz; ++z)
            for (uint32_t y = 0; y < uy; ++y)
                for (uint32_t x = 0; x < ux; ++x)
                    out[((size_t)z * uy + y) * ux + x] = (int8_t)exportv[lin(x, y, z, d)];
    }

    void read_active_volume(uint8_t* out) {
        std::vector<uint8_t> vol(N, 0);
        be.export_active(vol.data(), n, d, active.data());
        for (uint32_t z = 0; z < uz; ++z)
            for (uint32_t y = 0; y < uy; ++y)
                for (uint32_t x = 0; x < ux; ++x)
                    out[((size_t)z * uy + y) * ux + x] = vol[tiled(x, y, z, d)];
    }

    // FreezeCurrentSegmentation (:659-679).
    void freeze() { be.add_level_set(frozen.data(), exportv.data(), d); }

    // ClearCurrentSegmentation (:597-639).
    void clear_current() {
        level_set_initialized = false;
        n = 0;
        iterations = 0;
        std::fill(exportv.begin(), exportv.end(), 127);
        std::fill(active.begin(), active.end(), 0xFFFFFFFFu);
        std::fill(phiX.begin(), phiX.end(), 127);
        std::fill(phiY.begin(), phiY.end(), 127);
        std::fill(valid.begin(), valid.end(), 0u);
        std::fill(tag.begin(), tag.end(), 0);
    }

    void clear_all() {  // ClearAllSegmentations (:641-657)
        clear_current();
        std::fill(frozen.begin(), frozen.end(), 127);
    }

    // CollectCurrentLevelSetVoxels + CalculateSegmentationParameters
    // (:357-478): float accumulation in linear padded order.
    void estimate_params(float* t_out, float* w_out) {
        std::vector<float> vals;
        float total = 0.0f;
        for (size_t i = 0; i < N; ++i)
            if ((int8_t)exportv[i] <= 0) {
                float v;
                if (dtype == DT_U32) v = (float)((const uint32_t*)src.data())[i];
                else v = (float)sample_int(src.data(), dtype, i);
                vals.push_back(v);
                total += v;
            }
        float cnt = (float)vals.size();
        float mean = total / cnt;
        float sd = 0.0f;
        for (float v : vals) { float m = v - mean; sd += m * m; }
        sd = std::sqrt(sd / (cnt - 1));
        T = mean;
        W = sd;
        *t_out = mean;
        *w_out = sd;
    }
};

}  // namespace lssref
