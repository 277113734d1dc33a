/*
 * lss.h — C ABI of the GB300 sparse level-set segmentation engine.
 *
 * This header is the drop-in boundary for the reference's level-set solver
 * path.  The reference exposes that path as the C++ class `Segmenter`
 * (code/gpuseg/code/Segmenter.hpp:37-73), driven by `Engine`
 * (code/gpuseg/code/src/Engine.cpp:229,313,405,736), over an `extern "C"`
 * kernel layer (code/gpuseg/code/cuda/CudaKernels.hpp:1-107).  Every entry
 * point below cites the reference member it replaces.
 *
 * Conventions (all entry points):
 *   - every call returns an lss_status; nothing aborts the process;
 *   - the engine owns all device memory; host pointers are borrowed for the
 *     duration of the call and copied;
 *   - volumes are dense, x fastest, then y, then z, in the caller's
 *     (unpadded) dimensions;
 *   - calls on one engine are not thread-safe; separate engines are
 *     independent; all device work runs on the engine's stream.
 *
 * Two update modes share the boundary:
 *   LSS_MODE_REF  the reference's arithmetic and buffer semantics (int8 phi
 *                 in 16^3 tiles, integer intensities, 6-connected output
 *                 into seven offset buffers, tag-volume duplicate filter,
 *                 few/many-active path choice);
 *   LSS_MODE_NS   fp32 phi and intensity:
 *                   phi += dt * (wc * div(grad phi/|grad phi|) |grad phi|
 *                                - wd * D * |grad phi|_upwind),
 *                   D = clamp((eps - |I - T|) / eps, -1, 1) + bias   (default), or
 *                   D = eps - |I - T| + bias          (lss_params.data_term),
 *                 phi clamped to [phi_min, phi_max], inside = phi <= 0,
 *                 (wc, wd) = (1 - alpha, alpha) or (alpha, 1 - alpha) by
 *                 lss_params.alpha_role; bricked active set with 26-neighbour
 *                 expansion.
 */
#ifndef LSS_H
#define LSS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LSS_ABI_VERSION 2

typedef enum lss_status {
    LSS_OK                   = 0,
    LSS_ERR_INVALID_ARGUMENT = 1,  /* null pointer, bad size, bad enum            */
    LSS_ERR_STATE            = 2,  /* no volume loaded / not seeded               */
    LSS_ERR_OUT_OF_MEMORY    = 3,  /* device or host allocation failed           */
    LSS_ERR_CUDA             = 4,  /* a CUDA runtime call failed                  */
    LSS_ERR_TIMEOUT          = 5,  /* a bounded device-side wait gave up          */
    LSS_ERR_UNSUPPORTED      = 6,  /* option not available in this mode          */
    LSS_ERR_NO_DEVICE        = 7,  /* no CUDA device visible                      */
    LSS_ERR_INJECTED         = 8,  /* host-side fault injection (LSS_FAULT)       */
    LSS_ERR_CAPACITY         = 9   /* size above a stated limit or HBM budget     */
} lss_status;

/* Voxel types of the source volume.  The reference accepts the six integer
 * types (code/gpuseg/code/src/cuda/Textures.cu:4-10); LSS_F32 is added for
 * the fp32 mode. */
typedef enum lss_dtype {
    LSS_U8 = 0, LSS_S8 = 1, LSS_U16 = 2, LSS_S16 = 3,
    LSS_U32 = 4, LSS_S32 = 5, LSS_F32 = 6
} lss_dtype;

typedef enum lss_mode { LSS_MODE_REF = 0, LSS_MODE_NS = 1 } lss_mode;

/* Which term alpha weights in LSS_MODE_NS.  LSS_ALPHA_CURVATURE is the
 * reference's and the paper's speed F = alpha*C + (1-alpha)*D
 * (UpdateLevelSetVolume.cu:303; main.tex:178); LSS_ALPHA_DATA is
 * F = alpha*D + (1-alpha)*C (Lefohn et al. 2004), the default. */
typedef enum lss_alpha_role { LSS_ALPHA_CURVATURE = 0, LSS_ALPHA_DATA = 1 } lss_alpha_role;

/* The data speed D of LSS_MODE_NS.  LSS_DATA_NORMALISED (the default) is
 * the paper's eps - |I - T| (main.tex:176) divided by eps as the reference's
 * ComputeDensityTerm does (UpdateLevelSetVolume.cu:335-342) and clamped to
 * [-1, 1], which keeps dt*|F| inside the upwind scheme's stability bound;
 * LSS_DATA_LITERAL is eps - |I - T| as written, unscaled and unclamped. */
typedef enum lss_data_term { LSS_DATA_NORMALISED = 0, LSS_DATA_LITERAL = 1 } lss_data_term;

typedef struct lss_engine lss_engine;

/* Engine construction options. */
typedef struct lss_config {
    int32_t  mode;              /* lss_mode                                          */
    int32_t  device;            /* CUDA device ordinal                               */
    int32_t  brick_x, brick_y, brick_z;  /* NS brick shape: 8x8x8, 8x8x4 or 4x4x4;
                                            0,0,0 = pick by the autotuner          */
    int32_t  threads_per_brick; /* NS: 64..512, 32 = one warp; 0 = autotuner's choice */
    int32_t  ref_quirk_i3;      /* REF: 1 = the reference's three-of-four element
                                   loop (UpdateActiveElementsVolume.cu:82,329);
                                   0 = every active element emits                   */
    int32_t  use_graph;         /* REF: capture each step's iterations in a graph   */
    uint64_t hbm_budget_bytes;  /* refuse allocations above this total (0 = none)   */
    int32_t  brick_workers;     /* NS, 8x8x8 x 256: 1 = a block per brick (several
                                   blocks per SM); 4 = one block per SM whose four
                                   groups of 256 threads each work on a brick;
                                   0 = 1 (the autotuner may pick either)          */
    int32_t  pad_;              /* reserved, 0                                     */
} lss_config;

/* Solver parameters; ≈ the content::Parameter set of
 * code/gpuseg/code/src/Segmenter.cpp:34-40. */
typedef struct lss_params {
    float   target;               /* T      "growLevel"           */
    float   window;               /* eps    "growWindow"          */
    float   curvature;            /* alpha  "curvatureInfluence"  */
    float   time_step;            /* dt     "timeStep"            */
    float   phi_min, phi_max;     /* NS clamp of phi (default -4, 4)                     */
    float   temporal_threshold;   /* |dphi| above which a voxel counts as changed
                                     (REF: 0.008, Config.hpp:55; NS default 0.01)       */
    float   spatial_threshold;    /* |phi(n)-phi(x)| above which a voxel starts active
                                     (REF: 0.001, Config.hpp:56; NS default 0)          */
    float   convergence_threshold;/* REF: finished when n <= this and iterations > 500
                                     (Segmenter.cpp:1053-1056)                          */
    int32_t neighbourhood;        /* expansion neighbourhood: 6 (REF) or 26 (NS)         */
    int32_t alpha_role;           /* NS: lss_alpha_role (default LSS_ALPHA_DATA)         */
    int32_t data_term;            /* NS: lss_data_term (default LSS_DATA_NORMALISED)     */
} lss_params;

/* Stopping rule of lss_step_until_converged. */
typedef struct lss_conv {
    double   rel_threshold;  /* stop once n < rel_threshold * n0 ...          */
    int32_t  patience;       /* ... for this many consecutive iterations      */
    int32_t  max_iterations; /* hard cap                                      */
    uint64_t abs_threshold;  /* also stop when n <= abs_threshold             */
} lss_conv;

typedef struct lss_stats {
    uint64_t iterations;           /* iterations since the last seed / re-init       */
    uint64_t active_count;         /* current n                                      */
    uint64_t initial_active_count; /* n0 after seeding                               */
    uint64_t voxel_updates;        /* sum of n over all iterations (device counter)  */
    uint64_t brick_updates;        /* NS: sum of active bricks over iterations       */
    uint64_t device_bytes;         /* device memory held by the engine               */
    double   last_step_ms;         /* device time of the last step call              */
    uint32_t padded_x, padded_y, padded_z;
    uint32_t brick_x, brick_y, brick_z, threads_per_brick;
    int32_t  mode;
    int32_t  error_flags;          /* device-side error word (timeouts, bounds)      */
    double   update_ms;            /* NS: time of the last launch's block 0 in brick
                                      work (updates, flushes) ...                    */
    double   barrier_ms;           /* ... and waiting at the grid barrier            */
    uint64_t kernel_launches;      /* kernels launched by the engine so far (read
                                      before the stats call's own readback)          */
    uint32_t grid_blocks;          /* NS: blocks of the persistent launch            */
    uint32_t block_threads;        /* NS: threads per block of the persistent launch */
} lss_stats;

/* ---- construction / teardown ------------------------------------------ */

/* Fills defaults: NS, device 0, autotuned brick, quirk on, graphs on. */
lss_status lss_config_default(lss_config* cfg);

/* Fills the defaults of a mode: REF takes Config.hpp's constants; NS takes
 * T=0.5, eps=0.1, alpha=0.5, dt=0.5, clamp [-4,4], thresholds 0.01/0. */
lss_status lss_params_default(int32_t mode, lss_params* p);

/* ≈ Segmenter::Segmenter + CudaInitialize (Segmenter.cpp:42-95, Cuda.cpp:32-45). */
lss_status lss_create(lss_engine** out, const lss_config* cfg);

/* ≈ Segmenter::~Segmenter + UnloadVolume (Segmenter.cpp:97-108, 287-353). */
lss_status lss_destroy(lss_engine* e);

/* Message of the last failed call on this engine (empty if none). */
const char* lss_last_error_string(const lss_engine* e);

/* Version string of the library. */
const char* lss_version(void);

/* All later device work is issued on this cudaStream_t (NULL = the engine's
 * own stream).  The reference runs on the default stream only. */
lss_status lss_set_stream(lss_engine* e, void* cuda_stream);

/* ---- the solver path ---------------------------------------------------- */

/* ≈ Segmenter::LoadVolume (Segmenter.cpp:110-285) with
 * LoadVolumeHostPadded (:1131-1204): copies, pads (REF: to multiples of 16,
 * pad 0 or -127 for signed types, at most 1024 per axis) and uploads. */
lss_status lss_load_volume(lss_engine* e, const void* data, int32_t nx, int32_t ny,
                           int32_t nz, int32_t dtype, float z_anisotropy);

/* ≈ VolumeLoader::LoadVolumeRaw (code/gpuseg/code/src/VolumeLoader.cpp:275-457)
 * followed by lss_load_volume. */
lss_status lss_load_volume_raw(lss_engine* e, const char* path, int32_t nx, int32_t ny,
                               int32_t nz, int32_t dtype, float z_anisotropy);

/* ≈ Segmenter::UnloadVolume (Segmenter.cpp:287-353). */
lss_status lss_unload_volume(lss_engine* e);

/* ≈ setting the Parameter<float>s growLevel/growWindow/curvatureInfluence/
 * timeStep.  As in the reference (Segmenter.cpp:847-876, 1371-1374), a change
 * of T, eps or alpha re-initialises the active set on the next step. */
lss_status lss_set_params(lss_engine* e, const lss_params* p);
lss_status lss_get_params(const lss_engine* e, lss_params* p);

/* ≈ Segmenter::InitializeSeed (Segmenter.cpp:491-595): unions a seed sphere
 * into phi (InitializeLevelSetVolume.cu:55-98 in REF; min of signed
 * distances in NS), rebuilds the active set, resets the iteration count. */
lss_status lss_initialize_seed(lss_engine* e, float cx, float cy, float cz, float radius);

/* Several spheres at once (x, y, z, r per sphere); REF applies them as
 * consecutive InitializeSeed calls. */
lss_status lss_set_seed_spheres(lss_engine* e, const float* xyzr, int32_t count);

/* Sets phi directly (unpadded, x fastest) and rebuilds the active set.
 * REF quantises to the int8 field (floor(phi*127), phi clamped to [-1,1]). */
lss_status lss_set_phi(lss_engine* e, const float* phi);

/* ≈ Segmenter::RequestUpdateSegmentation (Segmenter.cpp:759-1051) with
 * numSubSteps = n_iters.  In REF mode nothing runs when the segmentation is
 * finished (IsSegmentationFinished) and no parameter changed. */
lss_status lss_step(lss_engine* e, int32_t n_iters, int32_t* iters_done);

/* NS: n iterations of the dense all-voxel update with the same arithmetic
 * (every voxel, no active set): the unconditional update the paper compares
 * the sparse algorithm against (documentation/papers/hpg2010/latex/
 * main.tex:523).  *ms (nullable) receives the device time.  The active set is
 * rebuilt from the resulting phi. */
lss_status lss_step_dense(lss_engine* e, int32_t n_iters, double* ms);

/* Steps until the stopping rule holds; one device launch in NS mode. */
lss_status lss_step_until_converged(lss_engine* e, const lss_conv* c, int32_t* iters_done);

/* ≈ Segmenter::IsSegmentationFinished (Segmenter.cpp:1053-1056). */
lss_status lss_is_finished(lss_engine* e, int32_t* finished);

/* ≈ Segmenter::GetActiveElementCount (Segmenter.cpp:1093-1096). */
lss_status lss_active_count(lss_engine* e, uint64_t* n);

/* The active list in list order as (x, y, z) triples (3*capacity uint32).
 * REF: the reference's compacted order; NS: brick-major order. */
lss_status lss_read_active(lss_engine* e, uint32_t* xyz, uint64_t capacity, uint64_t* n);

/* REF: the raw compacted list of packed coordinates x | y<<10 | z<<20
 * (Coordinates.cu:186-208).  NS: the same packing (dims must be <= 1024). */
lss_status lss_read_active_packed(lss_engine* e, uint32_t* packed, uint64_t capacity,
                                  uint64_t* n);

/* phi, unpadded, x fastest.  REF: the read buffer as c/127 floats. */
lss_status lss_read_phi(lss_engine* e, float* out);

/* ≈ Segmenter::GetSaveableSegmentation (Segmenter.cpp:1216-1286): 1 where the
 * (current ∪ frozen) level set is <= 0, else 0; unpadded.  In REF mode it
 * also clears the tag volume, as the reference does (:1239-1240). */
lss_status lss_read_mask(lss_engine* e, uint8_t* out);

/* Writes the lss_read_mask volume to a raw u8 file (≈ VolumeSaver's role). */
lss_status lss_save_mask_raw(lss_engine* e, const char* path);

/* REF: the int8 export volume written by the update kernel
 * (UpdateLevelSetVolume.cu:323-324); NS: floor(127*phi/max|clamp|). */
lss_status lss_read_export(lss_engine* e, int8_t* out);

/* ≈ ExportActiveElementsVolume (ExportActiveElementsVolume.cu:43-73): 127 at
 * every active voxel, 0 elsewhere; unpadded. */
lss_status lss_read_active_volume(lss_engine* e, uint8_t* out);

/* ≈ Segmenter::FreezeCurrentSegmentation / ClearCurrentSegmentation /
 * ClearAllSegmentations (Segmenter.cpp:659-679, 597-639, 641-657). */
lss_status lss_freeze_current(lss_engine* e);
lss_status lss_clear_current(lss_engine* e);
lss_status lss_clear_all(lss_engine* e);

/* ≈ Segmenter::CalculateSegmentationParameters (Segmenter.cpp:357-478):
 * T = mean and eps = sample std of the source inside the current
 * segmentation (a device reduction); the new values become the parameters. */
lss_status lss_estimate_params(lss_engine* e, float* target, float* window);

lss_status lss_get_stats(lss_engine* e, lss_stats* s);

/* ---- batched form (NS): many volumes, one persistent launch ------------ */

typedef struct lss_batch lss_batch;

lss_status lss_batch_create(lss_batch** out, const lss_config* cfg);
lss_status lss_batch_destroy(lss_batch* b);
/* Adds an f32 volume with its own parameters and seed spheres (x,y,z,r). */
lss_status lss_batch_add_volume(lss_batch* b, const float* data, int32_t nx, int32_t ny,
                                int32_t nz, const lss_params* p, const float* xyzr,
                                int32_t nseeds, int32_t* index);
/* Runs every volume to its own stopping rule in one persistent launch. */
lss_status lss_batch_run(lss_batch* b, const lss_conv* c, int32_t* iterations);
lss_status lss_batch_read_phi(lss_batch* b, int32_t index, float* out);
lss_status lss_batch_read_mask(lss_batch* b, int32_t index, uint8_t* out);
lss_status lss_batch_get_stats(lss_batch* b, int32_t index, lss_stats* s);
const char* lss_batch_last_error_string(const lss_batch* b);

/* ---- differentiation form (NS) ----------------------------------------- */

typedef struct lss_grads {
    double loss;         /* 1 - soft Dice after K iterations          */
    double d_target;     /* dloss/dT                                  */
    double d_window;     /* dloss/deps                                */
    double d_curvature;  /* dloss/dalpha                              */
    uint64_t active_voxel_iterations; /* sum over the K forward iterations of
                                         the active voxels updated          */
} lss_grads;

/* Runs K iterations from the current state with the active set of each
 * iteration recorded and then held fixed, and back-propagates the soft-Dice
 * loss of sigmoid(-phi/sigmoid_scale) against target_mask through them.
 * phi is checkpointed every `checkpoint_every` iterations (each checkpoint
 * holds the bricks its segment reaches; the last segment is logged brick by
 * brick instead).  bias (nullable) is a per-voxel speed bias added to D;
 * d_bias (nullable) receives its gradient.  target_mask, bias and d_bias
 * (nx*ny*nz, x fastest) may be host memory (pageable or pinned) or device
 * memory of the engine's device; device memory is used in place when
 * nx and ny are multiples of 8 and the pointer is 16-byte aligned.  The
 * engine state is restored to the starting state on return. */
lss_status lss_adjoint_run(lss_engine* e, int32_t K, int32_t checkpoint_every,
                           const uint8_t* target_mask, float sigmoid_scale,
                           const float* bias, float* d_bias, lss_grads* out);

/* ---- kernel level --------------------------------------------------------- */

/* ≈ CudppCompact (code/gpuseg/code/src/cuda/Cuda.cpp:699-758) over CUDPP's
 * cudppCompact: stable compaction of d_src[i] for every i < n with
 * d_valid[i] != 0 into d_dst (device pointers, caller-owned).  The count is
 * written to *d_count in device memory.  Its scratch (n/8 bytes of packed
 * flags and a word per 4096 elements) comes from a stream-ordered memory pool
 * of the library's own, which keeps up to 128 MiB reserved between calls, and
 * goes back to it before the call ends; the call synchronises `stream` (a cudaStream_t, NULL = the
 * legacy default stream) before returning. */
lss_status lss_compact_u32(const uint32_t* d_src, const uint32_t* d_valid, uint32_t* d_dst,
                           uint64_t n, uint64_t* d_count, void* stream);

/* Largest n accepted by lss_compact_u32_noalloc. */
#define LSS_COMPACT_NOALLOC_MAX_ELEMENTS (1ull << 26)

/* lss_compact_u32 for callers that cannot allocate device memory when they
 * compact: pipelines whose device memory is reserved once at start-up, and
 * hosts whose allocator belongs to another framework (an allocation of the
 * library's own would bypass that allocator's pool and accounting).  No
 * counterpart in the reference
 * (which allocates through CUDPP's plan).  Same arguments and result as
 * lss_compact_u32; allocates nothing: its scratch is a fixed device array of
 * the library (about 8 MiB, held by every GPU that loads the library until
 * the process exits).  n above LSS_COMPACT_NOALLOC_MAX_ELEMENTS returns
 * LSS_ERR_CAPACITY without touching the buffers.  The first call on a device
 * looks the array up on that device (with that device current); make that
 * first call before any stream capture.  All calls share the array, which
 * keeps the last call's contents (each call clears what it reads first):
 * calls that overlap on the GPU (other streams, other threads) race and must
 * be serialised by the caller.  The call reads a status word back and
 * synchronises `stream` before returning. */
lss_status lss_compact_u32_noalloc(const uint32_t* d_src, const uint32_t* d_valid, uint32_t* d_dst,
                                   uint64_t n, uint64_t* d_count, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LSS_H */
