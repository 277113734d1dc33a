// The C ABI of include/lss.h over the engine objects.  Every entry point
// converts exceptions into an lss_status and keeps the message for
// lss_last_error_string; nothing aborts the process.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

#include "engine.hpp"
#include "lss.h"

namespace lss {
std::unique_ptr<EngineBase> make_batch(const lss_config& c);
int batch_add(EngineBase* b, const float* d, int nx, int ny, int nz, const lss_params& p, const float* s,
              int ns);
int batch_run(EngineBase* b, const lss_conv* c);
int batch_nvol(EngineBase* b);
void batch_read_phi(EngineBase* b, int v, float* o);
void batch_read_mask(EngineBase* b, int v, uint8_t* o);
void batch_stats(EngineBase* b, int v, lss_stats* s);
}  // namespace lss

struct lss_engine {
    std::unique_ptr<lss::EngineBase> impl;
    std::string err;
    int nx = 0, ny = 0, nz = 0;
};

struct lss_batch {
    std::unique_ptr<lss::EngineBase> impl;
    std::string err;
};

namespace {

template <class H, class F>
lss_status guard(H* h, F&& f) {
    try {
        f();
        if (h) h->err.clear();
        return LSS_OK;
    } catch (const lss::Error& e) {
        if (h) h->err = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        if (h) h->err = "host allocation failed";
        return LSS_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        if (h) h->err = e.what();
        return LSS_ERR_INVALID_ARGUMENT;
    }
}

#define CHECK_ENGINE(e) \
    if (!(e) || !(e)->impl) return LSS_ERR_INVALID_ARGUMENT

}  // namespace

extern "C" {

const char* lss_version(void) { return "lss 1.0 (sm_103a)"; }

lss_status lss_config_default(lss_config* cfg) {
    if (!cfg) return LSS_ERR_INVALID_ARGUMENT;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->mode = LSS_MODE_NS;
    cfg->device = 0;
    cfg->ref_quirk_i3 = 1;
    cfg->use_graph = 1;
    return LSS_OK;
}

lss_status lss_params_default(int32_t mode, lss_params* p) {
    if (!p) return LSS_ERR_INVALID_ARGUMENT;
    std::memset(p, 0, sizeof(*p));
    if (mode == LSS_MODE_REF) {
        p->target = 128; p->window = 64; p->curvature = 0.2f; p->time_step = 0.25f;
        p->phi_min = -1; p->phi_max = 1;
        p->temporal_threshold = 0.008f;
        p->spatial_threshold = 0.001f;
        p->convergence_threshold = 0;
        p->neighbourhood = 6;
        p->alpha_role = LSS_ALPHA_CURVATURE;
        return LSS_OK;
    }
    if (mode != LSS_MODE_NS) return LSS_ERR_INVALID_ARGUMENT;
    p->target = 0.5f; p->window = 0.1f; p->curvature = 0.5f; p->time_step = 0.5f;
    p->phi_min = -4; p->phi_max = 4;
    p->temporal_threshold = 0.01f;
    p->spatial_threshold = 0.0f;
    p->convergence_threshold = 0;
    p->neighbourhood = 26;
    p->alpha_role = LSS_ALPHA_DATA;
    p->data_term = LSS_DATA_NORMALISED;
    return LSS_OK;
}

lss_status lss_create(lss_engine** out, const lss_config* cfg) {
    if (!out) return LSS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    lss_config c;
    if (cfg) c = *cfg;
    else lss_config_default(&c);
    if (c.mode != LSS_MODE_REF && c.mode != LSS_MODE_NS) return LSS_ERR_INVALID_ARGUMENT;
    if (c.brick_workers < 0) return LSS_ERR_INVALID_ARGUMENT;
    std::unique_ptr<lss_engine> e(new lss_engine());
    lss_status s = guard(e.get(), [&] {
        if (c.mode == LSS_MODE_REF) e->impl = lss::make_ref_engine(c);
        else e->impl = lss::make_ns_engine(c);
        lss_params p;
        lss_params_default(c.mode, &p);
        e->impl->params = p;
    });
    if (s != LSS_OK) return s;
    *out = e.release();
    return LSS_OK;
}

lss_status lss_destroy(lss_engine* e) {
    if (!e) return LSS_ERR_INVALID_ARGUMENT;
    lss_status s = guard(e, [&] {
        if (e->impl) {
            e->impl->sync();
            if (e->impl->own_stream) cudaStreamDestroy(e->impl->own_stream);
            e->impl.reset();
        }
    });
    delete e;
    return s;
}

const char* lss_last_error_string(const lss_engine* e) { return e ? e->err.c_str() : "null engine"; }

lss_status lss_set_stream(lss_engine* e, void* s) {
    CHECK_ENGINE(e);
    return guard(e, [&] {
        e->impl->sync();
        e->impl->stream = s ? (cudaStream_t)s : e->impl->own_stream;
    });
}

lss_status lss_load_volume(lss_engine* e, const void* data, int32_t nx, int32_t ny, int32_t nz,
                           int32_t dtype, float aniso) {
    CHECK_ENGINE(e);
    if (!data || nx <= 0 || ny <= 0 || nz <= 0 || dtype < LSS_U8 || dtype > LSS_F32)
        return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] {
        e->impl->load_volume(data, nx, ny, nz, dtype, aniso);
        e->nx = nx; e->ny = ny; e->nz = nz;
    });
}

lss_status lss_load_volume_raw(lss_engine* e, const char* path, int32_t nx, int32_t ny, int32_t nz,
                               int32_t dtype, float aniso) {
    CHECK_ENGINE(e);
    if (!path || nx <= 0 || ny <= 0 || nz <= 0 || dtype < LSS_U8 || dtype > LSS_F32)
        return LSS_ERR_INVALID_ARGUMENT;
    // The reference reads numVoxels * numBytesPerVoxel bytes and asserts that
    // the file held them (VolumeLoader.cpp:275-303); here a missing or short
    // file, or a size whose byte count overflows, is an error status.
    std::vector<uint8_t> buf;
    const lss_status s = guard(e, [&] {
        const uint64_t bpv = dtype <= LSS_S8 ? 1 : dtype <= LSS_S16 ? 2 : 4;
        uint64_t xy = 0, vox = 0, bytes = 0;
        const bool wrap = __builtin_mul_overflow((uint64_t)nx, (uint64_t)ny, &xy) ||
                          __builtin_mul_overflow(xy, (uint64_t)nz, &vox) ||
                          __builtin_mul_overflow(vox, bpv, &bytes);
        LSS_REQUIRE(!wrap && bytes <= (uint64_t)PTRDIFF_MAX, LSS_ERR_CAPACITY, "raw volume size overflows");
        std::unique_ptr<FILE, int (*)(FILE*)> f(std::fopen(path, "rb"), &std::fclose);
        LSS_REQUIRE(f != nullptr, LSS_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
        buf.resize((size_t)bytes);
        const size_t got = std::fread(buf.data(), 1, (size_t)bytes, f.get());
        LSS_REQUIRE(got == bytes, LSS_ERR_INVALID_ARGUMENT,
                    "raw file holds " + std::to_string(got) + " bytes, expected " + std::to_string(bytes));
    });
    if (s != LSS_OK) return s;
    return lss_load_volume(e, buf.data(), nx, ny, nz, dtype, aniso);
}

lss_status lss_unload_volume(lss_engine* e) {
    CHECK_ENGINE(e);
    return guard(e, [&] { e->impl->unload_volume(); });
}

lss_status lss_set_params(lss_engine* e, const lss_params* p) {
    CHECK_ENGINE(e);
    if (!p) return LSS_ERR_INVALID_ARGUMENT;
    // A negative threshold marks every updated voxel as changed (and every
    // voxel as initially active): the dense all-voxel update.
    if (!(p->phi_min < p->phi_max) || !(p->window > 0) ||
        (p->neighbourhood != 6 && p->neighbourhood != 26) ||
        (p->data_term != LSS_DATA_NORMALISED && p->data_term != LSS_DATA_LITERAL))
        return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] { e->impl->set_params(*p); });
}

lss_status lss_get_params(const lss_engine* e, lss_params* p) {
    if (!e || !e->impl || !p) return LSS_ERR_INVALID_ARGUMENT;
    *p = e->impl->params;
    return LSS_OK;
}

lss_status lss_initialize_seed(lss_engine* e, float cx, float cy, float cz, float r) {
    CHECK_ENGINE(e);
    return guard(e, [&] { e->impl->initialize_seed(cx, cy, cz, r); });
}

lss_status lss_set_seed_spheres(lss_engine* e, const float* s, int32_t count) {
    CHECK_ENGINE(e);
    if (!s || count <= 0) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] { e->impl->initialize_seeds(s, count); });
}

lss_status lss_set_phi(lss_engine* e, const float* phi) {
    CHECK_ENGINE(e);
    if (!phi) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] { e->impl->set_phi(phi); });
}

lss_status lss_step(lss_engine* e, int32_t n, int32_t* done) {
    CHECK_ENGINE(e);
    if (n < 0) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] {
        int d = e->impl->step(n, nullptr);
        if (done) *done = d;
    });
}

lss_status lss_step_dense(lss_engine* e, int32_t n, double* ms) {
    CHECK_ENGINE(e);
    if (n < 0) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] {
        double t = e->impl->step_dense(n);
        if (ms) *ms = t;
    });
}

lss_status lss_step_until_converged(lss_engine* e, const lss_conv* c, int32_t* done) {
    CHECK_ENGINE(e);
    if (!c || c->max_iterations <= 0 || c->patience <= 0) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] {
        int d = e->impl->step(c->max_iterations, c);
        if (done) *done = d;
    });
}

lss_status lss_is_finished(lss_engine* e, int32_t* f) {
    CHECK_ENGINE(e);
    if (!f) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] { *f = e->impl->finished() ? 1 : 0; });
}

lss_status lss_active_count(lss_engine* e, uint64_t* n) {
    CHECK_ENGINE(e);
    if (!n) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] { *n = e->impl->active_count(); });
}

lss_status lss_read_active(lss_engine* e, uint32_t* xyz, uint64_t cap, uint64_t* n) {
    CHECK_ENGINE(e);
    return guard(e, [&] {
        uint64_t m = e->impl->read_active(xyz, cap, false);
        if (n) *n = m;
    });
}

lss_status lss_read_active_packed(lss_engine* e, uint32_t* packed, uint64_t cap, uint64_t* n) {
    CHECK_ENGINE(e);
    return guard(e, [&] {
        uint64_t m = e->impl->read_active(packed, cap, true);
        if (n) *n = m;
    });
}

lss_status lss_read_phi(lss_engine* e, float* out) {
    CHECK_ENGINE(e);
    if (!out) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] { e->impl->read_phi(out); });
}

lss_status lss_read_mask(lss_engine* e, uint8_t* out) {
    CHECK_ENGINE(e);
    if (!out) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] { e->impl->read_mask(out); });
}

lss_status lss_save_mask_raw(lss_engine* e, const char* path) {
    CHECK_ENGINE(e);
    if (!path || e->nx <= 0) return LSS_ERR_INVALID_ARGUMENT;
    std::vector<uint8_t> m;
    lss_status s = guard(e, [&] { m.resize((size_t)e->nx * e->ny * e->nz); });
    if (s != LSS_OK) return s;
    s = lss_read_mask(e, m.data());
    if (s != LSS_OK) return s;
    return guard(e, [&] {
        std::unique_ptr<FILE, int (*)(FILE*)> f(std::fopen(path, "wb"), &std::fclose);
        LSS_REQUIRE(f != nullptr, LSS_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
        const size_t put = std::fwrite(m.data(), 1, m.size(), f.get());
        LSS_REQUIRE(put == m.size() && std::fflush(f.get()) == 0, LSS_ERR_INVALID_ARGUMENT,
                    std::string("short write to ") + path);
    });
}

lss_status lss_read_export(lss_engine* e, int8_t* out) {
    CHECK_ENGINE(e);
    if (!out) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] { e->impl->read_export(out); });
}

lss_status lss_read_active_volume(lss_engine* e, uint8_t* out) {
    CHECK_ENGINE(e);
    if (!out) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] { e->impl->read_active_volume(out); });
}

lss_status lss_freeze_current(lss_engine* e) {
    CHECK_ENGINE(e);
    return guard(e, [&] { e->impl->freeze(); });
}

lss_status lss_clear_current(lss_engine* e) {
    CHECK_ENGINE(e);
    return guard(e, [&] { e->impl->clear_current(); });
}

lss_status lss_clear_all(lss_engine* e) {
    CHECK_ENGINE(e);
    return guard(e, [&] { e->impl->clear_all(); });
}

lss_status lss_estimate_params(lss_engine* e, float* t, float* w) {
    CHECK_ENGINE(e);
    if (!t || !w) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] { e->impl->estimate_params(t, w); });
}

lss_status lss_get_stats(lss_engine* e, lss_stats* s) {
    CHECK_ENGINE(e);
    if (!s) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] { e->impl->stats(s); });
}

lss_status lss_adjoint_run(lss_engine* e, int32_t K, int32_t every, const uint8_t* target, float scale,
                           const float* bias, float* dbias, lss_grads* out) {
    CHECK_ENGINE(e);
    if (K <= 0 || every <= 0 || !target || !out || !(scale > 0)) return LSS_ERR_INVALID_ARGUMENT;
    return guard(e, [&] { e->impl->adjoint(K, every, target, scale, bias, dbias, out); });
}

// ---- batch --------------------------------------------------------------

lss_status lss_batch_create(lss_batch** out, const lss_config* cfg) {
    if (!out) return LSS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    lss_config c;
    if (cfg) c = *cfg;
    else lss_config_default(&c);
    c.mode = LSS_MODE_NS;
    std::unique_ptr<lss_batch> b(new lss_batch());
    lss_status s = guard(b.get(), [&] { b->impl = lss::make_batch(c); });
    if (s != LSS_OK) return s;
    *out = b.release();
    return LSS_OK;
}

lss_status lss_batch_destroy(lss_batch* b) {
    if (!b) return LSS_ERR_INVALID_ARGUMENT;
    lss_status s = guard(b, [&] {
        if (b->impl) {
            b->impl->sync();
            cudaStream_t st = b->impl->own_stream;
            b->impl.reset();
            if (st) cudaStreamDestroy(st);
        }
    });
    delete b;
    return s;
}

const char* lss_batch_last_error_string(const lss_batch* b) { return b ? b->err.c_str() : "null batch"; }

lss_status lss_batch_add_volume(lss_batch* b, const float* data, int32_t nx, int32_t ny, int32_t nz,
                                const lss_params* p, const float* xyzr, int32_t nseeds, int32_t* index) {
    if (!b || !b->impl || !data || !p || nx <= 0 || ny <= 0 || nz <= 0 || nseeds < 0 ||
        (nseeds > 0 && !xyzr))
        return LSS_ERR_INVALID_ARGUMENT;
    return guard(b, [&] {
        int i = lss::batch_add(b->impl.get(), data, nx, ny, nz, *p, xyzr, nseeds);
        if (index) *index = i;
    });
}

lss_status lss_batch_run(lss_batch* b, const lss_conv* c, int32_t* iterations) {
    if (!b || !b->impl) return LSS_ERR_INVALID_ARGUMENT;
    return guard(b, [&] {
        int it = lss::batch_run(b->impl.get(), c);
        if (iterations) *iterations = it;
    });
}

lss_status lss_batch_read_phi(lss_batch* b, int32_t index, float* out) {
    if (!b || !b->impl || !out) return LSS_ERR_INVALID_ARGUMENT;
    return guard(b, [&] {
        LSS_REQUIRE(index >= 0 && index < lss::batch_nvol(b->impl.get()), LSS_ERR_INVALID_ARGUMENT, "bad index");
        lss::batch_read_phi(b->impl.get(), index, out);
    });
}

lss_status lss_batch_read_mask(lss_batch* b, int32_t index, uint8_t* out) {
    if (!b || !b->impl || !out) return LSS_ERR_INVALID_ARGUMENT;
    return guard(b, [&] {
        LSS_REQUIRE(index >= 0 && index < lss::batch_nvol(b->impl.get()), LSS_ERR_INVALID_ARGUMENT, "bad index");
        lss::batch_read_mask(b->impl.get(), index, out);
    });
}

lss_status lss_batch_get_stats(lss_batch* b, int32_t index, lss_stats* s) {
    if (!b || !b->impl || !s) return LSS_ERR_INVALID_ARGUMENT;
    return guard(b, [&] {
        LSS_REQUIRE(index >= 0 && index < lss::batch_nvol(b->impl.get()), LSS_ERR_INVALID_ARGUMENT, "bad index");
        lss::batch_stats(b->impl.get(), index, s);
    });
}

}  // extern "C"
