// NsCore: device state of one or many LSS_MODE_NS volumes sharing one global
// brick space, one set of brick masks/membership bits and one persistent launch.
#pragma once

#include <cuda.h>
#include <vector_types.h>

#include <vector>

#include "engine.hpp"

namespace lss {

struct NsVol;
struct NsVolState;
struct NsCtl;
struct NsArgs;

struct BrickConfig {
    int bx, by, bz, threads;
    int min_blocks = 0;  // block per brick: resident blocks per SM the registers allow
                         // (0: 1024 threads; 8^3 x 256: 3)
    int groups = 1;      // > 1: one block per SM with this many brick workers of `threads` threads
};

const std::vector<BrickConfig>& brick_configs();

class NsCore;
// The differentiation form (csrc/ns_adjoint.cu).
void ns_adjoint(NsCore& core, int K, int every, const uint8_t* target, float tau, const float* bias,
                float* dbias, lss_grads* out);

class NsCore {
   public:
    NsCore(EngineBase* owner, uint64_t budget);
    ~NsCore();

    int add_volume(const float* data, int nx, int ny, int nz, const lss_params& p);
    // New intensities for volume v (same dimensions): the state after
    // add_volume + configure, the buffers and the configuration kept.
    void reload_volume(int v, const float* data, const lss_params& p);
    void set_params(int v, const lss_params& p) {
        vols_.at(v).p = p;
        vols_.at(v).speed_stale = true;
        upload_descriptors();
    }
    void configure(const BrickConfig& c);
    void init_active();
    void sphere_union(int v, float cx, float cy, float cz, float r);
    void set_phi(int v, const float* phi);
    void fill_phi(int v, float value);
    int run(int max_iters, const lss_conv* conv, float* ms);
    float dense_run(int iters);
    void read_phi(int v, float* out);
    // mask = phi <= 0, or'ed with the frozen mask; made on the device.
    void read_mask(int v, uint8_t* out);
    void freeze(int v);        // frozen |= (phi <= 0)
    void clear_frozen(int v);
    uint64_t read_active(int v, uint64_t* out, uint64_t cap);
    void estimate(int v, float* t, float* w);
    void state(int v, NsVolState* out);
    uint32_t vol_parity(int v);
    void check_errors();
    void d2h(void* dst, const void* src, size_t bytes);

    int nvol() const { return (int)vols_.size(); }
    bool configured() const { return configured_; }
    bool initialized() const { return initialized_; }
    const BrickConfig& config() const { return cfg_; }
    uint64_t held() const { return arena_.held() + brick_arena_.held(); }
    uint32_t parity() const { return parity_; }
    double last_update_ms() const { return last_update_ns_ * 1e-6; }
    double last_barrier_ms() const { return last_barrier_ns_ * 1e-6; }
    uint64_t bricks() const { return NB_; }
    int grid() const { return grid_; }
    int block_threads() const { return block_threads_; }
    int words() const { return words_; }
    uint64_t budget_left() const { return arena_.budget_left(); }
    // A device workspace of at least `bytes`, kept between calls (the
    // adjoint's checkpoints, adjoint fields and recorded sets) and freed with
    // the volume; grown when a call needs more.  Counted against the HBM
    // budget.
    void* workspace(uint64_t bytes);
    const unsigned long long* masks(uint32_t parity) const { return d_masks_[parity & 1u]; }
    NsVol descriptor(int v) const;  // host copy of the device descriptor of volume v
    EngineBase* owner() const { return owner_; }

    struct VolHost {
        int nx = 0, ny = 0, nz = 0, px = 0, py = 0, pz = 0, nbx = 0, nby = 0, nbz = 0;
        uint32_t brick_base = 0;
        float* phi[2] = {nullptr, nullptr};
        float* img = nullptr;
        float* speed = nullptr;     // ns_speed_f32 of every voxel (padded), made by refresh_speed
        bool speed_stale = true;    // the intensities or parameters changed since
        lss_params p{};
        uint8_t* frozen = nullptr;  // unpadded u8 mask of frozen segmentations (device), once frozen
        unsigned long long iterations = 0;
        // phi equal in both buffers and uniform outside the voxel box
        // [dirty_lo, dirty_hi) (after a fill, grown by seeding).
        bool uniform = false;
        int3 dirty_lo{0, 0, 0}, dirty_hi{0, 0, 0};
    };
    const std::vector<VolHost>& vols() const { return vols_; }
    // Counts the calls that may change a volume's phi or the layout
    // (add_volume, reload_volume, configure, sphere_union, set_phi,
    // fill_phi, run, dense_run; not parameters, masks or frozen masks): the
    // adjoint keeps copies of phi in its workspace between calls only while
    // this count stays the same.
    uint64_t epoch() const { return epoch_; }
    // What the adjoint left in its workspace (ns_adjoint.cu): `valid` while
    // the workspace stays in place (cleared when it is reallocated).
    struct AdjointRecord {
        bool valid = false;
        uint64_t epoch = 0;
        const void* key[4] = {nullptr, nullptr, nullptr, nullptr};
        uint32_t gen = 0;
    };
    AdjointRecord& adjoint_record() { return adj_rec_; }

   private:
    size_t dyn_smem() const;
    void upload_descriptors();
    void refresh_speed();  // the speed of every volume whose speed is stale
    void upload_padded(float* dst, const float* host, const VolHost& V, float* stage);
    NsArgs args(uint32_t k0, int max_iters, const lss_conv* conv) const;

    EngineBase* owner_;
    DeviceArena arena_;        // volumes (phi, intensities, speed)
    DeviceArena brick_arena_;  // brick-shape dependent state
    std::vector<VolHost> vols_;
    BrickConfig cfg_{8, 8, 8, 256};
    int words_ = 8;
    uint64_t NB_ = 0;
    uint32_t NW_ = 0;
    int grid_ = 0, block_threads_ = 0;
    // NsCtl's growing counters as of the last readback (the counter barrier's
    // starting points for the next launch); zero whenever NsCtl is cleared.
    unsigned long long ctl_arrivals_ = 0, ctl_upd_sum_[2] = {0, 0};
    uint32_t parity_ = 0;   // phi buffer holding the current field (= k_total_ & 1)
    uint32_t k_total_ = 0;  // global iteration index (bits slot k_total_ % 4, count slot % 3)
    unsigned long long last_update_ns_ = 0, last_barrier_ns_ = 0;
    bool configured_ = false, initialized_ = false;
    NsVol* d_vols_ = nullptr;
    NsVolState* d_vstate_ = nullptr;
    CUtensorMap* d_tmaps_ = nullptr;
    unsigned long long* d_masks_[2] = {nullptr, nullptr};
    uint32_t* d_bits_[4] = {nullptr, nullptr, nullptr, nullptr};
    unsigned long long* d_cnt_[3] = {nullptr, nullptr, nullptr};
    uint16_t* d_brick_vol_ = nullptr;
    uint64_t* d_status_ = nullptr;
    NsCtl* d_ctl_ = nullptr;
    uint32_t* d_misc_ = nullptr;
    void* ws_ = nullptr;
    uint64_t ws_bytes_ = 0;
    uint64_t epoch_ = 0;
    AdjointRecord adj_rec_;
};

}  // namespace lss
