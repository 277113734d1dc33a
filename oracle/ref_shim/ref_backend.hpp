// ORACLE — test infrastructure only.
//
// A kernel backend for the RefSegmenter driver (oracle/ref_model.hpp) that
// runs the reference's own kernel sources, compiled for the CPU through
// shim_cuda.h by oracle/ref_shim/build_ref.py.  Each method binds the
// texture references the way Segmenter.cpp does before the call
// (Segmenter.cpp:157-158, 525-537, 802-806, 842) and then calls the
// reference's extern "C" entry point (code/gpuseg/code/cuda/CudaKernels.hpp).
#pragma once

#include "shim_cuda.h"

#include "Config.hpp"
#include "cuda/CudaTypes.hpp"
#include "cuda/CudaKernels.hpp"
#include "cuda/CudaTextures.hpp"

#include "gen/Textures.cu.cpp"
#include "gen/Coordinates.cu.cpp"
#include "gen/Math.cu.cpp"
#include "gen/UpdateActiveElements.cu.cpp"
#include "gen/MemSetFloat.cu.cpp"
#include "gen/InitializeCoordinateVolume.cu.cpp"
#include "gen/InitializeActiveElementsVolume.cu.cpp"
#include "gen/InitializeLevelSetVolume.cu.cpp"
#include "gen/UpdateLevelSetVolume.cu.cpp"
#include "gen/UpdateActiveElementsVolume.cu.cpp"
#include "gen/FilterDuplicates.cu.cpp"
#include "gen/ExportActiveElementsVolume.cu.cpp"

#include <string>

#include "ref_model.hpp"

inline void lss_shim_bind_by_name(const char* name, const void* ptr) {
    std::string n(name);
    lss_shim::TexState* st = nullptr;
    if (n == CUDA_TEXTURE_TAG_1D) st = CUDA_TEXTURE_REF_TAG_1D.st;
    else if (n == CUDA_TEXTURE_LEVEL_SET_1D) st = CUDA_TEXTURE_REF_LEVEL_SET_1D.st;
    else if (n == CUDA_TEXTURE_ACTIVE_ELEMENTS_1D) st = CUDA_TEXTURE_REF_ACTIVE_ELEMENTS_1D.st;
    else if (n == CUDA_TEXTURE_VALID_ELEMENTS_1D) st = CUDA_TEXTURE_REF_VALID_ELEMENTS_1D.st;
    if (!st) throw std::runtime_error("shim: unknown texture " + n);
    st->base = (const uint8_t*)ptr;
    st->bytes = lss_shim::region_bytes_from(ptr);
}

namespace lssrefshim {

using lssref::Dims;
using lssref::U3;

struct ReferenceBackend {
    static dim3 D(Dims d) { return dim3(d.x, d.y, d.z); }

    static void reg(const void* p, size_t bytes) { lss_shim::register_region(p, bytes); }

    // Forgets every binding of the previous call, so that a texture or a
    // region can never refer to a buffer of an earlier (freed) solver.
    static void begin() {
        lss_shim::regions().clear();
        for (lss_shim::TexState* st : lss_shim::registry()) {
            if (!st->is1d) continue;
            st->base = nullptr;
            st->bytes = 0;
            st->snap.clear();
        }
    }

    static void bind(const char* name, const void* p, size_t bytes) {
        reg(p, bytes);
        lss_shim_bind_by_name(name, p);
    }

    static void bind_source(const void* src, int dtype, Dims d) {
        lss_shim::TexState* st = nullptr;
        switch (dtype) {
            case 0: st = CUDA_TEXTURE_REF_SOURCE_3D_UI8.st; break;
            case 1: st = CUDA_TEXTURE_REF_SOURCE_3D_I8.st; break;
            case 2: st = CUDA_TEXTURE_REF_SOURCE_3D_UI16.st; break;
            case 3: st = CUDA_TEXTURE_REF_SOURCE_3D_I16.st; break;
            case 4: st = CUDA_TEXTURE_REF_SOURCE_3D_UI32.st; break;
            case 5: st = CUDA_TEXTURE_REF_SOURCE_3D_I32.st; break;
        }
        st->base = (const uint8_t*)src;
        st->dims[0] = d.x; st->dims[1] = d.y; st->dims[2] = d.z;
    }

    void init_level_set(int8_t* wr, uint8_t* ex, Dims d, const int8_t* rd, U3 seed, int32_t r,
                        float aniso) {
        begin();
        bind(CUDA_TEXTURE_LEVEL_SET_1D, rd, d.n());
        CudaInitializeLevelSetVolume((CudaLevelSetElement*)wr, (CudaTagElement*)ex, D(d),
                                     dim3(seed.x, seed.y, seed.z), r, aniso);
    }

    void init_active_volume(uint32_t* valid, Dims d, const int8_t* rd) {
        begin();
        bind(CUDA_TEXTURE_LEVEL_SET_1D, rd, d.n());
        CudaInitializeActiveElementsVolume(valid, D(d));
    }

    void init_coord_volume(uint32_t* coord, Dims d) {
        begin(); CudaInitializeCoordinateVolume(coord, D(d)); }

    void update(int8_t* wr, uint8_t* ex, uint8_t* tag, size_t n, Dims d, int32_t target,
                int32_t window, float alpha, float dt, const int8_t* rd, const uint32_t* active,
                const void* src, int dtype) {
        begin();
        bind_source(src, dtype, d);
        bind(CUDA_TEXTURE_LEVEL_SET_1D, rd, d.n());
        bind(CUDA_TEXTURE_ACTIVE_ELEMENTS_1D, active, d.n() * 4);
        unsigned bpv = dtype <= 1 ? 1u : dtype <= 3 ? 2u : 4u;
        bool sgn = dtype == 1 || dtype == 3 || dtype == 5;
        CudaUpdateLevelSetVolumeAsync((CudaLevelSetElement*)wr, (CudaTagElement*)ex, tag, n, D(d),
                                      target, window, alpha, dt, bpv, sgn);
    }

    void output_new(uint32_t* coord, uint32_t* valid, size_t n, Dims d, const int8_t* rd,
                    const uint8_t* tag, const uint32_t* active) {
        begin();
        reg(coord, d.n() * 4);
        reg(valid, d.n() * 4);
        bind(CUDA_TEXTURE_LEVEL_SET_1D, rd, d.n());
        bind(CUDA_TEXTURE_TAG_1D, tag, d.n());
        bind(CUDA_TEXTURE_ACTIVE_ELEMENTS_1D, active, d.n() * 4);
        CudaOutputNewActiveElements(coord, valid, n, D(d));
    }

    template <typename T>
    void memset_sparse(T* buf, T val, size_t n, Dims d, const uint32_t* active) {
        begin();
        bind(CUDA_TEXTURE_ACTIVE_ELEMENTS_1D, active, d.n() * 4);
        if constexpr (sizeof(T) == 1) CudaMemSetCharSparse((unsigned char*)buf, val, n, D(d));
        else CudaMemSetIntSparse((unsigned int*)buf, val, n, D(d));
    }

    void filter(uint32_t* coord, uint32_t* valid, uint8_t* tag, size_t n, Dims d) {
        begin();
        reg(coord, d.n() * 4);
        reg(valid, d.n() * 4);
        bind(CUDA_TEXTURE_TAG_1D, tag, d.n());
        CudaFilterDuplicates(coord, valid, tag, n, D(d));
    }

    void update_active_volume(uint32_t* valid, size_t n, Dims d, const int8_t* rd,
                              const uint8_t* tag, const uint32_t* active) {
        begin();
        bind(CUDA_TEXTURE_LEVEL_SET_1D, rd, d.n());
        bind(CUDA_TEXTURE_TAG_1D, tag, d.n());
        bind(CUDA_TEXTURE_ACTIVE_ELEMENTS_1D, active, d.n() * 4);
        CudaUpdateActiveElementsVolume(valid, n, D(d));
    }

    void add_level_set(uint8_t* res, const uint8_t* add, Dims d) {
        begin();
        CudaAddLevelSetVolume(res, (CudaTagElement*)add, D(d));
    }

    void export_active(uint8_t* out, size_t n, Dims d, const uint32_t* active) {
        begin();
        bind(CUDA_TEXTURE_ACTIVE_ELEMENTS_1D, active, d.n() * 4);
        CudaExportActiveElementsVolume(out, n, D(d));
    }
};

}  // namespace lssrefshim
