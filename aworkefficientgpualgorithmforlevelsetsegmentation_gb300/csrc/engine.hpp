// Host-side engine objects behind the C ABI (include/lss.h).
//
// RefEngine reproduces the reference's solver path bit for bit
// (Segmenter.cpp:759-1051 over the kernels of code/gpuseg/code/src/cuda);
// NsEngine is the fp32 bricked engine with the persistent iteration kernel.
// Both keep the active count on the device and only read it back when a
// caller asks for it.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "common.cuh"
#include "lss.h"

namespace lss {

// Device allocation with an engine-wide byte budget.
class DeviceArena {
   public:
    explicit DeviceArena(uint64_t budget) : budget_(budget) {}
    ~DeviceArena() { release(); }
    DeviceArena(const DeviceArena&) = delete;
    DeviceArena& operator=(const DeviceArena&) = delete;
    void* alloc(size_t bytes);
    void free_last(void* p);  // frees one allocation (any position)
    void release();
    uint64_t held() const { return held_; }
    void set_budget(uint64_t b) { budget_ = b; }
    uint64_t budget_left() const { return budget_ == 0 ? 0 : (budget_ > held_ ? budget_ - held_ : 1); }

   private:
    uint64_t budget_ = 0, held_ = 0;
    std::vector<std::pair<void*, size_t>> ptrs_;
};

class EngineBase {
   public:
    virtual ~EngineBase() = default;
    lss_config cfg{};
    lss_params params{};
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    std::string last_error;
    int device = 0;
    int num_sms = 0;
    uint64_t launches = 0;  // kernels launched by this engine (graph launches count their kernels)

    virtual void load_volume(const void* data, int nx, int ny, int nz, int dtype, float aniso) = 0;
    virtual void unload_volume() = 0;
    virtual void set_params(const lss_params& p) = 0;
    virtual void initialize_seed(float cx, float cy, float cz, float r) = 0;
    // Several seeds (x, y, z, r) in a row; the default seeds them one by one.
    virtual void initialize_seeds(const float* xyzr, int count) {
        for (int k = 0; k < count; ++k) initialize_seed(xyzr[4 * k], xyzr[4 * k + 1], xyzr[4 * k + 2], xyzr[4 * k + 3]);
    }
    virtual void set_phi(const float* phi) = 0;
    virtual int step(int n, const lss_conv* conv) = 0;  // conv == nullptr: exactly n
    virtual bool finished() = 0;
    virtual uint64_t active_count() = 0;
    virtual uint64_t read_active(uint32_t* xyz, uint64_t cap, bool packed) = 0;
    virtual void read_phi(float* out) = 0;
    virtual void read_mask(uint8_t* out) = 0;
    virtual void read_export(int8_t* out) = 0;
    virtual void read_active_volume(uint8_t* out) = 0;
    virtual void freeze() = 0;
    virtual void clear_current() = 0;
    virtual void clear_all() = 0;
    virtual void estimate_params(float* t, float* w) = 0;
    virtual void stats(lss_stats* s) = 0;
    virtual double step_dense(int n) {
        (void)n;
        throw Error(LSS_ERR_UNSUPPORTED, "the dense update is available in LSS_MODE_NS only");
    }
    virtual void adjoint(int K, int every, const uint8_t* target, float scale, const float* bias,
                         float* dbias, lss_grads* out) {
        (void)K; (void)every; (void)target; (void)scale; (void)bias; (void)dbias; (void)out;
        throw Error(LSS_ERR_UNSUPPORTED, "adjoint is available in LSS_MODE_NS only");
    }

    void init_device(const lss_config& c);
    void sync();
};

std::unique_ptr<EngineBase> make_ref_engine(const lss_config& c);
std::unique_ptr<EngineBase> make_ns_engine(const lss_config& c);

}  // namespace lss
