// ORACLE — test infrastructure only.
//
// A minimal CUDA-runtime stand-in that lets the reference's own kernel
// sources (code/gpuseg/code/src/cuda/*.cu) compile as C++ for the CPU:
// dim3/uint3/uint4, the thread-index builtins, __umul24 and the float/int
// conversion intrinsics, 1D/3D texture references (point sampling, clamp
// addressing, normalised int8 reads as c/127 floored at -1, zero outside a
// 1D buffer), and a serial launcher that runs every block and thread of a
// grid in order.  At each launch the launcher snapshots every bound 1D
// texture, so texture reads see the state at kernel launch (the reference's
// only same-kernel read/write overlap is the tag volume in its duplicate
// filter, where CUDA leaves the outcome undefined).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __align__(n) alignas(n)

struct uint3 { unsigned int x, y, z; };
struct int3 { int x, y, z; };
struct uint4 { unsigned int x, y, z, w; };
struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
    dim3(uint3 u) : x(u.x), y(u.y), z(u.z) {}
};

namespace lss_shim {
inline uint3 g_blockIdx, g_threadIdx;
inline dim3 g_blockDim, g_gridDim;
}  // namespace lss_shim
#define blockIdx (::lss_shim::g_blockIdx)
#define threadIdx (::lss_shim::g_threadIdx)
#define blockDim (::lss_shim::g_blockDim)
#define gridDim (::lss_shim::g_gridDim)

inline unsigned int __umul24(unsigned int a, unsigned int b) { return (a & 0xFFFFFFu) * (b & 0xFFFFFFu); }
inline unsigned int __float2uint_rd(float f) {
    if (f != f || f <= 0.0f) return 0u;
    float r = std::floor(f);
    return r >= 4294967296.0f ? 0xFFFFFFFFu : (unsigned int)r;
}
inline int __float2int_rd(float f) {
    if (f != f) return 0;
    float r = std::floor(f);
    if (r >= 2147483648.0f) return 2147483647;
    if (r < -2147483648.0f) return (-2147483647 - 1);
    return (int)r;
}
inline float __int2float_rz(int i) { return (float)i; }  // exact for |i| < 2^24

inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
using std::abs;
using std::sqrt;

enum cudaTextureReadMode { cudaReadModeElementType = 0, cudaReadModeNormalizedFloat = 1 };

namespace lss_shim {

struct TexState {
    const uint8_t* base = nullptr;
    size_t bytes = 0;
    uint32_t dims[3] = {0, 0, 0};
    std::vector<uint8_t> snap;
    bool is1d = true;
};

inline std::vector<TexState*>& registry() { static std::vector<TexState*> r; return r; }

struct Region { const uint8_t* base; size_t bytes; };
inline std::vector<Region>& regions() { static std::vector<Region> r; return r; }
inline void register_region(const void* p, size_t bytes) {
    for (auto& r : regions())
        if (r.base == (const uint8_t*)p) { r.bytes = bytes; return; }
    regions().push_back(Region{(const uint8_t*)p, bytes});
}
inline size_t region_bytes_from(const void* p) {
    const uint8_t* q = (const uint8_t*)p;
    for (auto& r : regions())
        if (q >= r.base && q < r.base + r.bytes) return (size_t)(r.base + r.bytes - q);
    throw std::runtime_error("shim: texture bound to an unregistered buffer");
}

inline void refresh_snapshots() {
    for (TexState* s : registry())
        if (s->is1d && s->base) s->snap.assign(s->base, s->base + s->bytes);
}

}  // namespace lss_shim

template <typename T, int Dim, int Mode>
struct texture {
    lss_shim::TexState* st;
    texture() : st(new lss_shim::TexState()) {
        st->is1d = (Dim == 1);
        lss_shim::registry().push_back(st);
    }
};

template <typename T>
inline T tex1Dfetch(texture<T, 1, cudaReadModeElementType> t, int i) {
    T v{};
    size_t off = (size_t)i * sizeof(T);
    if (i < 0 || off + sizeof(T) > t.st->snap.size()) return v;
    std::memcpy(&v, t.st->snap.data() + off, sizeof(T));
    return v;
}

inline float tex1Dfetch(texture<signed char, 1, cudaReadModeNormalizedFloat> t, int i) {
    if (i < 0 || (size_t)i >= t.st->snap.size()) return 0.0f;
    float f = (float)(signed char)t.st->snap[i] / 127.0f;
    return f < -1.0f ? -1.0f : f;
}

template <typename T>
inline T tex3D(texture<T, 3, cudaReadModeElementType> t, float x, float y, float z) {
    auto cl = [](float c, uint32_t n) {
        long v = (long)std::floor(c);
        return (uint32_t)(v < 0 ? 0 : (v >= (long)n ? (long)n - 1 : v));
    };
    uint32_t X = cl(x, t.st->dims[0]), Y = cl(y, t.st->dims[1]), Z = cl(z, t.st->dims[2]);
    size_t idx = ((size_t)Z * t.st->dims[1] + Y) * t.st->dims[0] + X;
    T v;
    std::memcpy(&v, t.st->base + idx * sizeof(T), sizeof(T));
    return v;
}

namespace lss_shim {

template <typename... A>
struct Launch {
    dim3 g, b;
    void (*k)(A...);
    template <typename... P>
    void operator()(P&&... p) {
        refresh_snapshots();
        g_gridDim = g;
        g_blockDim = b;
        for (unsigned bz = 0; bz < g.z; ++bz)
            for (unsigned by = 0; by < g.y; ++by)
                for (unsigned bx = 0; bx < g.x; ++bx)
                    for (unsigned tz = 0; tz < b.z; ++tz)
                        for (unsigned ty = 0; ty < b.y; ++ty)
                            for (unsigned tx = 0; tx < b.x; ++tx) {
                                g_blockIdx = uint3{bx, by, bz};
                                g_threadIdx = uint3{tx, ty, tz};
                                k(p...);
                            }
    }
};

template <typename... A>
Launch<A...> launcher(dim3 g, dim3 b, void (*k)(A...)) { return Launch<A...>{g, b, k}; }

}  // namespace lss_shim

// Host-side helpers the kernel wrappers call (code/gpuseg/code/cuda/Cuda.hpp).
inline void Assert(bool c) { if (!c) throw std::runtime_error("reference Assert failed"); }
inline void CudaSynchronize() {}
inline void CudaCheckErrors() {}
inline unsigned int CudaGetWarpAlignedValue(unsigned int v) { return v + (256u - v % 256u) % 256u; }
void lss_shim_bind_by_name(const char* name, const void* ptr);  // defined after Textures.cu
template <typename A, typename B>
void CudaBindTextureToBuffer(const char* name, const A* buffer) { lss_shim_bind_by_name(name, buffer); }
template <typename A>
void CudaBindTextureToBuffer(const char* name, const A* buffer) { lss_shim_bind_by_name(name, buffer); }
