// Host-side engine pieces shared by both modes, the LSS_MODE_NS plain engine
// (one volume) and the batched form (many volumes, one persistent launch).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "engine.hpp"
#include "ns_core.hpp"
#include "ns_kernels.cuh"

namespace lss {

bool fault_injected(const char* what) {
    const char* f = std::getenv("LSS_FAULT");
    return f && std::strcmp(f, what) == 0;
}

void* DeviceArena::alloc(size_t bytes) {
    if (fault_injected("alloc")) throw Error(LSS_ERR_INJECTED, "injected allocation failure");
    bytes = std::max<size_t>(bytes, 16);
    if (budget_ && held_ + bytes > budget_)
        throw Error(LSS_ERR_CAPACITY, "allocation of " + std::to_string(bytes) +
                                          " bytes exceeds the HBM budget of " + std::to_string(budget_));
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(LSS_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    ptrs_.push_back({p, bytes});
    held_ += bytes;
    return p;
}

void DeviceArena::free_last(void* p) {
    for (size_t i = ptrs_.size(); i-- > 0;)
        if (ptrs_[i].first == p) {
            cudaFree(p);
            held_ -= ptrs_[i].second;
            ptrs_.erase(ptrs_.begin() + i);
            return;
        }
}

void DeviceArena::release() {
    for (auto& q : ptrs_) cudaFree(q.first);
    ptrs_.clear();
    held_ = 0;
}

void EngineBase::init_device(const lss_config& c) {
    cfg = c;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        throw Error(LSS_ERR_NO_DEVICE, "no CUDA device visible");
    }
    LSS_REQUIRE(c.device >= 0 && c.device < n, LSS_ERR_INVALID_ARGUMENT, "bad device ordinal");
    device = c.device;
    LSS_CUDA(cudaSetDevice(device));
    LSS_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device));
    LSS_CUDA(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));
    stream = own_stream;
}

void EngineBase::sync() {
    if (stream) LSS_CUDA(cudaStreamSynchronize(stream));
}

// ---------------------------------------------------------------------------
// Autotuner: times a short run of each brick configuration from the same
// initial state and keeps the fastest.  Results are voxel-exact across
// configurations (the active set is a per-voxel mask), so only the time
// differs.  Choices are cached per volume-shape bucket.
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int, int>, BrickConfig> g_tune_cache;

static bool same_config(const BrickConfig& a, const BrickConfig& b) {
    return a.bx == b.bx && a.by == b.by && a.bz == b.bz && a.threads == b.threads &&
           a.min_blocks == b.min_blocks && a.groups == b.groups;
}

static std::tuple<int, int, int, int> tune_key(NsCore& core) {
    auto& vols = core.vols();
    uint64_t vox = 0;
    for (auto& v : vols) vox += (uint64_t)v.nx * v.ny * v.nz;
    return std::make_tuple((int)vols.size(), (int)std::log2((double)vox + 1), vols[0].nx / 64, vols[0].nz / 64);
}

// The cached choice for this volume-shape bucket, if one was tuned before
// (lets an engine configure with it directly, before any state exists).
static bool cached_choice(NsCore& core, BrickConfig* out) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune_cache.find(tune_key(core));
    if (it == g_tune_cache.end()) return false;
    *out = it->second;
    return true;
}

// `iters` iterations from the seeded state, or (conv non-null) the run to
// the stopping rule: a batch spends most of its time at the widest fronts,
// which the first iterations from the seeds do not reach.
static BrickConfig autotune(NsCore& core, EngineBase* owner, int iters, const lss_conv* conv = nullptr) {
    auto& vols = core.vols();
    const auto key = tune_key(core);
    // Save the seeded phi of every volume.
    auto save = [&]() {
        std::vector<std::vector<float>> saved(vols.size());
        for (size_t i = 0; i < vols.size(); ++i) {
            saved[i].resize((size_t)vols[i].nx * vols[i].ny * vols[i].nz);
            core.read_phi((int)i, saved[i].data());
        }
        return saved;
    };
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            const BrickConfig c = it->second;
            if (!same_config(c, core.config())) {  // apply the cached choice
                auto saved = save();
                core.configure(c);
                for (size_t i = 0; i < vols.size(); ++i) core.set_phi((int)i, saved[i].data());
                core.init_active();
            }
            return c;
        }
    }
    std::vector<std::vector<float>> saved = save();
    BrickConfig best = brick_configs()[0];
    float best_ms = 1e30f;
    for (const BrickConfig& c : brick_configs()) {
        core.configure(c);
        for (size_t i = 0; i < vols.size(); ++i) core.set_phi((int)i, saved[i].data());
        core.init_active();
        float ms = 0;
        core.run(conv ? conv->max_iterations : iters, conv, &ms);
        if (ms < best_ms) { best_ms = ms; best = c; }
    }
    core.configure(best);
    for (size_t i = 0; i < vols.size(); ++i) core.set_phi((int)i, saved[i].data());
    core.init_active();
    (void)owner;
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune_cache[key] = best;
    return best;
}

// ---------------------------------------------------------------------------

namespace {

std::vector<float> to_float(const void* data, uint64_t n, int dtype) {
    std::vector<float> f(n);
    switch (dtype) {
        case LSS_U8: for (uint64_t i = 0; i < n; ++i) f[i] = ((const uint8_t*)data)[i]; break;
        case LSS_S8: for (uint64_t i = 0; i < n; ++i) f[i] = ((const int8_t*)data)[i]; break;
        case LSS_U16: for (uint64_t i = 0; i < n; ++i) f[i] = ((const uint16_t*)data)[i]; break;
        case LSS_S16: for (uint64_t i = 0; i < n; ++i) f[i] = ((const int16_t*)data)[i]; break;
        case LSS_U32: for (uint64_t i = 0; i < n; ++i) f[i] = (float)((const uint32_t*)data)[i]; break;
        case LSS_S32: for (uint64_t i = 0; i < n; ++i) f[i] = (float)((const int32_t*)data)[i]; break;
        case LSS_F32: std::memcpy(f.data(), data, n * 4); break;
        default: throw Error(LSS_ERR_INVALID_ARGUMENT, "bad dtype");
    }
    return f;
}

class NsEngine : public EngineBase {
   public:
    explicit NsEngine(const lss_config& c) { init_device(c); }

    void load_volume(const void* data, int nx, int ny, int nz, int dtype, float aniso) override {
        LSS_REQUIRE(data && nx > 0 && ny > 0 && nz > 0, LSS_ERR_INVALID_ARGUMENT, "bad volume");
        (void)aniso;
        const uint64_t n = (uint64_t)nx * ny * nz;
        std::vector<float> f;
        if (dtype != LSS_F32) f = to_float(data, n, dtype);
        const float* fp = dtype == LSS_F32 ? (const float*)data : f.data();
        if (core_ && core_->configured() && nx == nx_ && ny == ny_ && nz == nz_) {
            // Same shape: the device buffers, tensor maps and brick
            // configuration stay; only the intensities and the state change.
            core_->reload_volume(0, fp, params);
            pending_reinit_ = false;
            Tp_ = params.target; Wp_ = params.window; Ap_ = params.curvature;
            return;
        }
        unload_volume();
        core_.reset(new NsCore(this, cfg.hbm_budget_bytes));
        core_->add_volume(fp, nx, ny, nz, params);
        BrickConfig c = brick_configs()[0];
        tuned_ = cfg.brick_x > 0;
        if (cfg.brick_x > 0) c = BrickConfig{cfg.brick_x, cfg.brick_y, cfg.brick_z,
                                             cfg.threads_per_brick > 0 ? cfg.threads_per_brick : 256, 0,
                                             cfg.brick_workers > 1 ? cfg.brick_workers : 1};
        else
            tuned_ = cached_choice(*core_, &c);
        core_->configure(c);
        nx_ = nx; ny_ = ny; nz_ = nz;
        pending_reinit_ = false;
        Tp_ = params.target; Wp_ = params.window; Ap_ = params.curvature;
    }

    void unload_volume() override {
        sync();
        core_.reset();
    }

    void set_params(const lss_params& p) override {
        params = p;
        if (!core_) return;
        core_->set_params(0, p);
        if (core_->initialized() && (Tp_ != p.target || Wp_ != p.window || Ap_ != p.curvature))
            pending_reinit_ = true;
    }

    void initialize_seed(float cx, float cy, float cz, float r) override {
        require();
        core_->sphere_union(0, cx, cy, cz, r);
        core_->init_active();
        after_init();
    }

    // The active set depends on phi only, so one rebuild after the union of
    // all spheres gives the same state as one per sphere.
    void initialize_seeds(const float* xyzr, int count) override {
        require();
        for (int k = 0; k < count; ++k)
            core_->sphere_union(0, xyzr[4 * k], xyzr[4 * k + 1], xyzr[4 * k + 2], xyzr[4 * k + 3]);
        core_->init_active();
        after_init();
    }

    void set_phi(const float* phi) override {
        require();
        core_->set_phi(0, phi);
        core_->init_active();
        after_init();
    }

    void after_init() {
        pending_reinit_ = false;
        Tp_ = params.target; Wp_ = params.window; Ap_ = params.curvature;
    }

    int step(int n, const lss_conv* conv) override {
        require();
        LSS_REQUIRE(core_->initialized(), LSS_ERR_STATE, "no seed or phi set");
        if (pending_reinit_) {
            core_->init_active();
            after_init();
        }
        if (!tuned_) {
            autotune(*core_, this, 256);
            tuned_ = true;
        }
        float ms = 0;
        int it = core_->run(conv ? conv->max_iterations : n, conv, &ms);
        last_ms_ = ms;
        return it;
    }

    void adjoint(int K, int every, const uint8_t* target, float scale, const float* bias, float* dbias,
                 lss_grads* out) override {
        require();
        LSS_REQUIRE(core_->initialized(), LSS_ERR_STATE, "no seed or phi set");
        if (pending_reinit_) {
            core_->init_active();
            after_init();
        }
        ns_adjoint(*core_, K, every, target, scale, bias, dbias, out);
    }

    double step_dense(int n) override {
        require();
        LSS_REQUIRE(core_->initialized(), LSS_ERR_STATE, "no seed or phi set");
        last_ms_ = core_->dense_run(n);
        after_init();
        return last_ms_;
    }

    bool finished() override { return core_ && active_count() == 0; }

    uint64_t active_count() override {
        if (!core_ || !core_->initialized()) return 0;
        return core_->read_active(0, nullptr, 0);  // popc over the current masks
    }

    uint64_t read_active(uint32_t* out, uint64_t cap, bool packed) override {
        require();
        LSS_REQUIRE(!packed || (nx_ <= 1024 && ny_ <= 1024 && nz_ <= 1024), LSS_ERR_CAPACITY,
                    "packed coordinates need dims <= 1024");
        uint64_t n = core_->read_active(0, nullptr, 0);
        if (!out) return n;
        std::vector<uint64_t> lin(std::max<uint64_t>(n, 1));
        core_->read_active(0, lin.data(), n);
        const uint64_t m = std::min(n, cap);
        for (uint64_t i = 0; i < m; ++i) {
            uint32_t x = (uint32_t)(lin[i] % nx_), y = (uint32_t)((lin[i] / nx_) % ny_),
                     z = (uint32_t)(lin[i] / ((uint64_t)nx_ * ny_));
            if (packed) out[i] = x | (y << 10) | (z << 20);
            else { out[3 * i] = x; out[3 * i + 1] = y; out[3 * i + 2] = z; }
        }
        return n;
    }

    void read_phi(float* out) override {
        require();
        core_->read_phi(0, out);
    }

    void read_mask(uint8_t* out) override {
        require();
        core_->read_mask(0, out);
    }

    void read_export(int8_t* out) override {
        require();
        std::vector<float> phi((size_t)nx_ * ny_ * nz_);
        core_->read_phi(0, phi.data());
        const float s = 127.0f / std::max(std::fabs(params.phi_min), std::fabs(params.phi_max));
        for (size_t i = 0; i < phi.size(); ++i) {
            float v = std::floor(phi[i] * s);
            out[i] = (int8_t)std::max(-127.0f, std::min(127.0f, v));
        }
    }

    void read_active_volume(uint8_t* out) override {
        require();
        std::memset(out, 0, (size_t)nx_ * ny_ * nz_);
        uint64_t n = core_->read_active(0, nullptr, 0);
        std::vector<uint64_t> lin(std::max<uint64_t>(n, 1));
        core_->read_active(0, lin.data(), n);
        for (uint64_t i = 0; i < n; ++i) out[lin[i]] = 127;
    }

    void freeze() override {
        require();
        core_->freeze(0);
    }

    void clear_current() override {
        require();
        core_->fill_phi(0, params.phi_max);
        core_->init_active();
        after_init();
    }

    void clear_all() override {
        clear_current();
        core_->clear_frozen(0);
    }

    void estimate_params(float* t, float* w) override {
        require();
        core_->estimate(0, t, w);
        lss_params p = params;
        p.target = *t;
        p.window = *w;
        set_params(p);
    }

    void stats(lss_stats* s) override {
        std::memset(s, 0, sizeof(*s));
        s->mode = LSS_MODE_NS;
        s->kernel_launches = launches;
        if (!core_) return;
        const auto& v = core_->vols()[0];
        s->padded_x = v.px; s->padded_y = v.py; s->padded_z = v.pz;
        s->brick_x = core_->config().bx; s->brick_y = core_->config().by;
        s->brick_z = core_->config().bz; s->threads_per_brick = core_->config().threads;
        s->device_bytes = core_->held();
        s->last_step_ms = last_ms_;
        s->grid_blocks = (uint32_t)core_->grid();
        s->block_threads = (uint32_t)core_->block_threads();
        if (!core_->initialized()) return;
        NsVolState st;
        core_->state(0, &st);
        s->iterations = st.iterations;
        s->active_count = core_->read_active(0, nullptr, 0);
        s->initial_active_count = st.n0;
        s->voxel_updates = st.updates;
        s->brick_updates = st.bricks;
        s->update_ms = core_->last_update_ms();
        s->barrier_ms = core_->last_barrier_ms();
    }

    NsCore& core() { return *core_; }

   private:
    void require() const { LSS_REQUIRE(core_ != nullptr, LSS_ERR_STATE, "no volume loaded"); }

    std::unique_ptr<NsCore> core_;
    int nx_ = 0, ny_ = 0, nz_ = 0;

    bool pending_reinit_ = false, tuned_ = false;
    float Tp_ = 0, Wp_ = 0, Ap_ = 0;
    double last_ms_ = 0;
};

}  // namespace

std::unique_ptr<EngineBase> make_ns_engine(const lss_config& c) {
    return std::unique_ptr<EngineBase>(new NsEngine(c));
}

// ---------------------------------------------------------------------------
// Batched form.
class BatchEngine : public EngineBase {
   public:
    explicit BatchEngine(const lss_config& c) : core_(this, c.hbm_budget_bytes) { init_device(c); }

    // Unused EngineBase members (the batch has its own API).
    void load_volume(const void*, int, int, int, int, float) override {}
    void unload_volume() override {}
    void set_params(const lss_params&) override {}
    void initialize_seed(float, float, float, float) override {}
    void set_phi(const float*) override {}
    int step(int, const lss_conv*) override { return 0; }
    bool finished() override { return false; }
    uint64_t active_count() override { return 0; }
    uint64_t read_active(uint32_t*, uint64_t, bool) override { return 0; }
    void read_phi(float*) override {}
    void read_mask(uint8_t*) override {}
    void read_export(int8_t*) override {}
    void read_active_volume(uint8_t*) override {}
    void freeze() override {}
    void clear_current() override {}
    void clear_all() override {}
    void estimate_params(float*, float*) override {}
    void stats(lss_stats*) override {}

    int add(const float* data, int nx, int ny, int nz, const lss_params& p, const float* xyzr, int ns) {
        LSS_REQUIRE(!ran_, LSS_ERR_STATE, "volumes cannot be added after a run");
        int idx = core_.add_volume(data, nx, ny, nz, p);
        seeds_.emplace_back(xyzr, xyzr + 4 * ns);
        return idx;
    }

    int run(const lss_conv* conv) {
        LSS_REQUIRE(core_.nvol() > 0, LSS_ERR_STATE, "empty batch");
        LSS_REQUIRE(!ran_, LSS_ERR_STATE, "a batch runs once");
        BrickConfig c = brick_configs()[0];
        bool tuned = cfg.brick_x > 0;
        if (cfg.brick_x > 0)
            c = BrickConfig{cfg.brick_x, cfg.brick_y, cfg.brick_z,
                            cfg.threads_per_brick > 0 ? cfg.threads_per_brick : 256, 0,
                            cfg.brick_workers > 1 ? cfg.brick_workers : 1};
        else
            tuned = cached_choice(core_, &c);
        core_.configure(c);
        for (int v = 0; v < core_.nvol(); ++v)
            for (size_t k = 0; k + 3 < seeds_[v].size(); k += 4)
                core_.sphere_union(v, seeds_[v][k], seeds_[v][k + 1], seeds_[v][k + 2], seeds_[v][k + 3]);
        core_.init_active();
        lss_conv cv = conv ? *conv : lss_conv{0.0, 1, 1000, 0};
        if (!tuned) autotune(core_, this, 0, &cv);  // each configuration runs the whole batch once
        float ms = 0;
        int it = core_.run(cv.max_iterations, &cv, &ms);
        last_ms_ = ms;
        ran_ = true;
        return it;
    }

    void read_phi_v(int v, float* out) { core_.read_phi(v, out); }

    void read_mask_v(int v, uint8_t* out) { core_.read_mask(v, out); }

    void stats_v(int v, lss_stats* s) {
        std::memset(s, 0, sizeof(*s));
        s->mode = LSS_MODE_NS;
        s->kernel_launches = launches;
        const auto& V = core_.vols().at(v);
        s->padded_x = V.px; s->padded_y = V.py; s->padded_z = V.pz;
        s->brick_x = core_.config().bx; s->brick_y = core_.config().by; s->brick_z = core_.config().bz;
        s->threads_per_brick = core_.config().threads;
        s->device_bytes = core_.held();
        s->last_step_ms = last_ms_;
        s->grid_blocks = (uint32_t)core_.grid();
        s->block_threads = (uint32_t)core_.block_threads();
        if (!core_.initialized()) return;
        NsVolState st;
        core_.state(v, &st);
        s->iterations = st.iterations;
        s->active_count = st.n_cur;
        s->initial_active_count = st.n0;
        s->voxel_updates = st.updates;
        s->brick_updates = st.bricks;
    }

    int nvol() const { return core_.nvol(); }

   private:
    NsCore core_;
    std::vector<std::vector<float>> seeds_;
    bool ran_ = false;
    double last_ms_ = 0;
};

std::unique_ptr<BatchEngine> make_batch_engine(const lss_config& c) {
    return std::unique_ptr<BatchEngine>(new BatchEngine(c));
}

// C-ABI helpers for the batch (declared in lss_api.cpp).
int batch_add(EngineBase* b, const float* d, int nx, int ny, int nz, const lss_params& p, const float* s,
              int ns) {
    return static_cast<BatchEngine*>(b)->add(d, nx, ny, nz, p, s, ns);
}
int batch_run(EngineBase* b, const lss_conv* c) { return static_cast<BatchEngine*>(b)->run(c); }
int batch_nvol(EngineBase* b) { return static_cast<BatchEngine*>(b)->nvol(); }
void batch_read_phi(EngineBase* b, int v, float* o) { static_cast<BatchEngine*>(b)->read_phi_v(v, o); }
void batch_read_mask(EngineBase* b, int v, uint8_t* o) { static_cast<BatchEngine*>(b)->read_mask_v(v, o); }
void batch_stats(EngineBase* b, int v, lss_stats* s) { static_cast<BatchEngine*>(b)->stats_v(v, s); }
std::unique_ptr<EngineBase> make_batch(const lss_config& c) {
    return std::unique_ptr<EngineBase>(make_batch_engine(c).release());
}

}  // namespace lss
