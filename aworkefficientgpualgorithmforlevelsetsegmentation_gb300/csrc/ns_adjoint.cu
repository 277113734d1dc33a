// The differentiation form of LSS_MODE_NS (lss_adjoint_run): K unrolled
// iterations of the LSS_MODE_NS update from the engine's current state, with
// the active set of every iteration recorded in the forward pass and held
// fixed, the soft-Dice loss of sigmoid(-phi/tau) against a target mask, and
// its gradients with respect to T, eps, alpha and a per-voxel speed bias.
//
// A call is two cooperative launches, the forward (its last two phases the
// loss) and the reverse, the phases inside each separated by the
// cooperative-groups grid barrier.  Work-efficient like the forward engine:
// every iteration touches the bricks of its active set only.
//
// Forward (k_adj_forward).  Its first phase sets the call up (clears, the
// pair's copies of phi_0, the masks of A_0).  Iteration k finds the bricks of
// A_k by a scan of the flags iteration k-1 marked and records them in list_k
// beside the recorded brick masks.  It runs over a ping-pong pair in which
// both buffers stay current: iteration k writes the bricks of A_k whole
// (active voxels updated, the rest copied) and copies across the bricks of
// A_{k-1} that left the set; the changed voxels' ballot words are dilated
// into A_{k+1} exactly as in the persistent kernel, so the recorded sets are
// the sparse engine's sets.  Checkpoints are sparse: during segment s (of
// `every` iterations) a brick joins checkpoint s the first time the segment
// reaches it, copied while it still holds phi at the segment's start; the
// last segment logs, per iteration k, the bricks of A_k as they were before
// the update.  The bricks within one brick of some A_k are marked: lambda is
// read there only.
//
// Loss (the forward's last two phases).  The soft-Dice sums over the
// volume, then lambda_K on the marked bricks.
//
// States without dense copies.  phi_k and phi_{k+1} differ only inside the
// bricks of A_k, so a field that holds phi_{k+2} becomes phi_k by writing
// back the logged bricks of A_k (phi_k) and those of A_{k+1} outside A_k
// (phi_{k+1} = phi_k there).  A segment's states live in a pair of fields,
// state t in pair[(t - base) & 1], that starts with its two highest states
// and walks down two states at a time.
//
// Reverse (k_adj_reverse).  Segment by segment from the last: the last
// segment runs on the forward's pair (phi_K, phi_{K-1}) and its log.  Every
// other segment is recomputed from its sparse checkpoint (bit-identical, the
// arithmetic is deterministic) while the segment after it runs backwards:
// the checkpoint and a copy of its bricks form the pair of a forward-style
// ping-pong that logs its bricks as it goes.  lambda is kept as a base field
// plus the last reverse iteration's scatter, lambda_{k+1} = lam + Z[(k+1)&1];
// reverse iteration k folds Z into lam on the bricks it visits, moves
// lambda_{k+1} of A_k's voxels through the transposed stencil Jacobian of the
// update into the other Z (fp32 atomics) and marks the bricks it reached
// (adj_rev_phase).  The parameter gradients are summed per thread and block
// in FP64 (the gradient-check reduction) into the block's own slot, the bias
// gradient per voxel.
//
// Data other blocks wrote earlier in the same launch is read with plain
// loads after a grid barrier (its fence orders them), never through the
// read-only path: no pointer into a buffer the launch writes is __restrict__.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "ns_core.hpp"
#include "ns_kernels.cuh"

namespace lss {
namespace {

namespace cg = cooperative_groups;

// Threads of the two cooperative launches (a voxel of an 8^3 brick each) and
// their blocks per SM: one block an SM keeps the grid barrier, paid every
// phase, at one participant an SM (1.16 us measured at 152 x 512); the
// reverse spreads its few dozen bricks an iteration over every SM in brick
// parts.
constexpr int kAdjThreads = 512;
constexpr int kAdjBlocksPerSm = 1;

void count_launch(EngineBase* owner) {
    ++owner->launches;
    LSS_CUDA(cudaGetLastError());
}

__device__ __forceinline__ int clampi(int v, int n) { return v < 0 ? 0 : (v >= n ? n - 1 : v); }

// Voxel j of local brick b of a one-volume descriptor.
template <class S>
__device__ __forceinline__ int3 voxel_of(const NsVol& V, uint32_t b, int j) {
    const int3 o = brick_origin<S>(V, b + V.brick_base);
    return make_int3(o.x + j % S::X, o.y + (j / S::X) % S::Y, o.z + j / (S::X * S::Y));
}

// The soft-Dice loss, the last two grid phases of the forward kernel (a
// grid barrier between them): the sums over the volume's rows in groups of
// four voxels (px is a multiple of 8, so a group stays in its row and is
// 16-byte aligned): item i is group i mod Q of row i div Q (Q = ceil(nx /
// 4)), row r = (y, z) = (r mod ny, r div ny); the padding rows are never
// visited.  Then lambda_K on the bricks the reverse reads it at.

struct DiceArgs {
    const float* phi;  // phi_K
    const uint8_t* tgt;
    float* lam;
    double* part;      // [nparts][3]: the dice blocks' sums
    double* gsum;      // [8]: the total in 4..6
    int nx, ny, nz, px, py;
    uint32_t nparts;
    float tau;
    const uint32_t* reached;  // [nb]: the bricks whose lambda_K is needed
    float* z0;                // lambda's contribution fields, cleared there too
    float* z1;
    uint32_t nb;
    int bx, by, bz, nbx, nby;  // brick shape and grid
    uint32_t gen;              // the call's stamp in reached
};

__device__ __forceinline__ float soft_mask(float phi, float tau) { return 1.0f / (1.0f + expf(phi / tau)); }

// Group i: its first x, and its index among the padded field's groups.
__device__ __forceinline__ uint32_t dice_group(const DiceArgs& d, uint32_t q4, uint32_t i, uint64_t* g) {
    const uint32_t r = i / q4, x0 = (i - r * q4) * 4;
    const uint32_t z = r / (uint32_t)d.ny, y = r - z * (uint32_t)d.ny;
    *g = (((uint64_t)z * d.py + y) * d.px + x0) / 4;
    return x0;
}

// Four groups a thread in flight (the loads of a round before its math).
constexpr int kDiceUnroll = 4;

// Sums s = sigmoid(-phi_K / tau), t = target and s t over the volume: per
// voxel in fp32, per thread in fp32, per block in FP64 into part[3 * block].
// NTH threads a block.
template <int NTH>
__device__ void adj_dice_sums(const DiceArgs& d) {
    const uint32_t q4 = (uint32_t)(d.nx + 3) / 4, n = (uint32_t)d.ny * (uint32_t)d.nz * q4;
    const uint32_t nt = gridDim.x * blockDim.x;
    float ss = 0.0f, tt = 0.0f, st = 0.0f;
    for (uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += kDiceUnroll * nt) {
        float4 f[kDiceUnroll];
        uchar4 m[kDiceUnroll];
        uint32_t x0[kDiceUnroll];
#pragma unroll
        for (int u = 0; u < kDiceUnroll; ++u) {
            const uint32_t i = i0 + u * nt;
            x0[u] = 0xFFFFFFFFu;
            if (i < n) {
                uint64_t g;
                x0[u] = dice_group(d, q4, i, &g);
                f[u] = reinterpret_cast<const float4*>(d.phi)[g];
                m[u] = reinterpret_cast<const uchar4*>(d.tgt)[g];
            }
        }
#pragma unroll
        for (int u = 0; u < kDiceUnroll; ++u) {
            if (x0[u] == 0xFFFFFFFFu) continue;
            const float fv[4] = {f[u].x, f[u].y, f[u].z, f[u].w};
            const unsigned char mv[4] = {m[u].x, m[u].y, m[u].z, m[u].w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                if (x0[u] + e >= (uint32_t)d.nx) break;
                const float s = soft_mask(fv[e], d.tau);
                const float tv = mv[e] ? 1.0f : 0.0f;
                ss += s;
                tt += tv;
                st += s * tv;
            }
        }
    }
    __shared__ double w3[3][NTH / 32];
    double a0 = ss, a1 = tt, a2 = st;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        a0 += __shfl_down_sync(0xffffffffu, a0, o);
        a1 += __shfl_down_sync(0xffffffffu, a1, o);
        a2 += __shfl_down_sync(0xffffffffu, a2, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        w3[0][warp] = a0;
        w3[1][warp] = a1;
        w3[2][warp] = a2;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int q = 0; q < NTH / 32; ++q) t += w3[threadIdx.x][q];
        d.part[3 * (size_t)blockIdx.x + threadIdx.x] = t;
    }
}

// lambda_K = dloss/dphi_K on the bricks the reverse reads it at (those
// within one brick of some A_k; elsewhere lambda passes through untouched to
// lambda_0, which nothing reads), with the two contribution fields cleared
// on the same voxels (the reverse reads and scatters into them there only).
// Item i: group i mod G (four voxels of a brick row) of brick i div G.
// Every block adds the blocks' sums in the same order (the same totals in
// every block and every call); block 0 publishes them for the loss.
__device__ void adj_lambda_k(const DiceArgs& d) {
    __shared__ double tot[3];
    if (threadIdx.x < 32) {
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        for (uint32_t b = threadIdx.x; b < d.nparts; b += 32) {
            a0 += d.part[3 * (size_t)b];
            a1 += d.part[3 * (size_t)b + 1];
            a2 += d.part[3 * (size_t)b + 2];
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            a0 += __shfl_down_sync(0xffffffffu, a0, o);
            a1 += __shfl_down_sync(0xffffffffu, a1, o);
            a2 += __shfl_down_sync(0xffffffffu, a2, o);
        }
        if (threadIdx.x == 0) {
            tot[0] = a0;
            tot[1] = a1;
            tot[2] = a2;
            if (blockIdx.x == 0) {
                d.gsum[4] = a0;
                d.gsum[5] = a1;
                d.gsum[6] = a2;
            }
        }
    }
    __syncthreads();
    // dloss/ds = (2 st - 2 t den) / den^2 with den = sum s + sum t.
    const double den = tot[0] + tot[1], sst = tot[2];
    const float c_out = (float)(2.0 * sst / (den * den)), c_in = (float)(2.0 * sst / (den * den) - 2.0 / den);
    const uint32_t G = (uint32_t)(d.bx * d.by * d.bz) / 4, n = d.nb * G;
    const uint32_t nt = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += kDiceUnroll * nt) {
        float4 f[kDiceUnroll];
        uchar4 m[kDiceUnroll];
        uint64_t g[kDiceUnroll];
        uint32_t x0[kDiceUnroll];
#pragma unroll
        for (int u = 0; u < kDiceUnroll; ++u) {
            const uint32_t i = i0 + u * nt;
            x0[u] = 0xFFFFFFFFu;
            if (i < n && d.reached[i / G] == d.gen) {
                const uint32_t b = i / G, j = (i - b * G) * 4;
                const uint32_t kx = b % (uint32_t)d.nbx, r = b / (uint32_t)d.nbx;
                const uint32_t ky = r % (uint32_t)d.nby, kz = r / (uint32_t)d.nby;
                const uint32_t x = kx * d.bx + j % d.bx, y = ky * d.by + (j / d.bx) % d.by,
                               z = kz * d.bz + j / (d.bx * d.by);
                if (y < (uint32_t)d.ny && z < (uint32_t)d.nz) {
                    x0[u] = x;
                    g[u] = (((uint64_t)z * d.py + y) * d.px + x) / 4;
                    f[u] = reinterpret_cast<const float4*>(d.phi)[g[u]];
                    m[u] = reinterpret_cast<const uchar4*>(d.tgt)[g[u]];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kDiceUnroll; ++u) {
            if (x0[u] == 0xFFFFFFFFu) continue;
            const float fv[4] = {f[u].x, f[u].y, f[u].z, f[u].w};
            const unsigned char mv[4] = {m[u].x, m[u].y, m[u].z, m[u].w};
            float l[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const float s = soft_mask(fv[e], d.tau);
                l[e] = x0[u] + e < (uint32_t)d.nx ? (mv[e] ? c_in : c_out) * (-s * (1.0f - s) / d.tau) : 0.0f;
            }
            reinterpret_cast<float4*>(d.lam)[g[u]] = make_float4(l[0], l[1], l[2], l[3]);
            reinterpret_cast<float4*>(d.z0)[g[u]] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            reinterpret_cast<float4*>(d.z1)[g[u]] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
}

// Everything one call works on.  Per-iteration arrays are evenly spaced in
// the workspace: act[k] = act0 + k * astride words, list[k] = list0 +
// k * lstride, flag[k] = flag0 + k * lstride; the checkpoints are fstride
// floats apart, the brick logs lgstride.
struct AdjPlan {
    NsVol V;                    // the one volume (brick_base 0)
    float* ck0;                 // checkpoint s < nck - 1 = ck0 + s * fstride (phi_{s * every}, sparse)
    float* qb[2];               // second field of a recomputed segment's pair (by parity)
    float* fw[2];               // the forward's ping-pong pair
    float* log0;                // brick logs: set (s & 1), slot t - s * every, lgstride floats each
    float* lam;                 // lambda = lam + Z[(k + 1) & 1] entering reverse iteration k
    float* Z[2];                // lambda contributions of the last reverse iteration, by parity
    float* dbias;               // nullable
    const uint8_t* tgt;
    unsigned long long* act0;   // [K+1][NB * WORDS]: the recorded brick masks of A_k
    uint32_t* list0;            // [K+1][NB]
    uint32_t* flag0;            // [K+1][NB]
    uint32_t* counts;           // [K+1]
    uint32_t* flagT[2];         // [NB]: bricks reverse iteration k scatters into, in flagT[(k - 1) & 1]
    uint32_t* need;             // [NB]: s + 1 once segment s's checkpoint holds the brick
    uint32_t* reached;          // [NB]: gen once within one brick of some A_k (lambda is read there only)
    uint32_t* nlist0;           // [nck - 1][NB]: the bricks of checkpoint s
    uint32_t* ncount;           // [nck]
    double* gsum;               // [8]: the soft-Dice totals in 4..6 (nact follows)
    double* gpart;              // [grid][3]: each block's dT, deps, dalpha
    unsigned long long* nact;   // active-voxel updates of the forward
    uint64_t fstride, astride, lstride, lgstride, P;
    const float* phi0;                     // the engine's phi at the start
    const unsigned long long* act_src;     // and its masks of A_0
    uint64_t mwords;                       // mask words a set
    uint64_t dbias_n;                      // floats of d_bias cleared (a multiple of 4)
    DiceArgs dice;                         // the loss phases' view (phi_K, target, lambda, sums)
    uint32_t gen;                          // this call's stamp in `reached` (>= 1)
    int32_t partial;                       // 1: the pair holds phi_0 but in the bricks stamped gen - 1
    uint32_t nb;
    int32_t K, every, nck;
    float tau;
};

__device__ __forceinline__ unsigned long long* plan_act(const AdjPlan& a, int k) { return a.act0 + (uint64_t)k * a.astride; }
__device__ __forceinline__ uint32_t* plan_list(const AdjPlan& a, int k) { return a.list0 + (uint64_t)k * a.lstride; }
__device__ __forceinline__ uint32_t* plan_flag(const AdjPlan& a, int k) { return a.flag0 + (uint64_t)k * a.lstride; }
__device__ __forceinline__ uint32_t* plan_need(const AdjPlan& a, int s) { return a.nlist0 + (uint64_t)s * a.lstride; }
// The log of iteration t of segment s: the bricks of list_t before the
// update, brick b at b * VOX.
__device__ __forceinline__ float* plan_log(const AdjPlan& a, int s, int t) {
    return a.log0 + ((uint64_t)(s & 1) * a.every + (uint64_t)(t - s * a.every)) * a.lgstride;
}

// The pair of fields segment s runs on in the reverse: state t in
// f[(t - base) & 1].  The last segment: the forward's pair.  The others:
// their checkpoint and a second field.
struct SegPair {
    float* f[2];
    int base;
};
__device__ __forceinline__ SegPair seg_pair(const AdjPlan& a, int s) {
    SegPair p;
    if (s == a.nck - 1) {
        p.f[0] = a.fw[0];
        p.f[1] = a.fw[1];
        p.base = 0;
    } else {
        p.f[0] = a.ck0 + (uint64_t)s * a.fstride;
        p.f[1] = a.qb[s & 1];
        p.base = s * a.every;
    }
    return p;
}

// Per-iteration brick lists: list[k][0 .. count[k]) = the bricks of A_k in
// no particular order (each brick once), flag[k][b] = b is in it.  Brick
// logs are indexed by brick: brick b of a log at b * VOX.

// flag_0 of every brick from the masks of A_0 (the first iteration's scan
// lists its bricks).
template <class S>
__device__ __forceinline__ void adj_flag0(const unsigned long long* act, uint32_t* flag, uint32_t nb) {
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        unsigned long long any = 0ull;
#pragma unroll
        for (int w = 0; w < S::WORDS; ++w) any |= act[(size_t)b * S::WORDS + w];
        flag[b] = any ? 1u : 0u;
    }
}

// The changed-voxel bits of one brick (chg, CHG 32-bit words) dilated
// (V.nbh = 6 or 26) into its 27 neighbours' masks of A_{k+1} (nxt); each
// neighbour reached is marked in flag_next with a plain store (the next
// iteration finds its bricks by a scan of the flags).  Threads t0, t0 +
// stride, ... take the (neighbour, mask word) pairs.
template <class S>
__device__ __forceinline__ void adj_dilate_brick(const NsVol& V, uint32_t b, const uint32_t* chg, int t0, int stride,
                                                 unsigned long long* nxt, uint32_t* flag_next) {
    const int3 o = brick_origin<S>(V, b + V.brick_base);
    for (int r = t0; r < 27 * S::WORDS; r += stride) {
        const int slot = r / S::WORDS, w = r % S::WORDS;
        const int ox = slot % 3 - 1, oy = (slot / 3) % 3 - 1, oz = slot / 9 - 1;
        const int bx = o.x / S::X + ox, by = o.y / S::Y + oy, bz = o.z / S::Z + oz;
        const int lx = V.nx - bx * S::X, ly = V.ny - by * S::Y, lz = V.nz - bz * S::Z;
        if (bx < 0 || by < 0 || bz < 0 || lx <= 0 || ly <= 0 || lz <= 0) continue;
        uint64_t x = dilate_word<S>(chg, ox, oy, oz, w, V.nbh);
        if (lx < S::X || ly < S::Y || lz < S::Z)
            x &= inside_mask<S>(w, min(lx, S::X), min(ly, S::Y), min(lz, S::Z));
        if (!x) continue;
        const uint32_t nbi = b + (int32_t)((oz * V.nby + oy) * V.nbx + ox);
        atomicOr(&nxt[(size_t)nbi * S::WORDS + w], (unsigned long long)x);
        flag_next[nbi] = 1u;
    }
}

// Forward iteration k.  Its bricks are found by a scan of the flags: block
// g looks at bricks c + t * grid + g (thread t, chunks c of grid * threads
// bricks, so consecutive bricks go to different blocks); flag_k set: a brick
// of A_k, written whole into out (active voxels updated from in, the others
// copied) and recorded in list_k; else flag_{k-1} set: a brick of A_{k-1}
// that left the set, copied from in to out.  So out equals in outside the
// bricks of A_k (both fields of the pair stay current).  Each updated
// brick's changed voxels are dilated into A_{k+1} by the same block, which
// marks the bricks reached in flag_{k+1}.  With log (the last segment):
// brick b of A_k is logged as it was before the update (in) at log + b *
// VOX.  Every brick within one brick of A_k is marked in `reached`.  With
// cap = s + 1 (segment s has a checkpoint): the 27 bricks around
// each brick of A_k (the update's reads and writes, a superset) join the
// segment's checkpoint the first time the segment reaches them, copied from
// in: a brick no earlier iteration of the segment reached still holds phi at
// the segment's start.  The checkpoint is that sparse field ck, and the
// bricks it holds are listed for the reverse.  Returns the active voxels
// this thread updated.
template <class S>
__device__ uint32_t adj_forward_step(const AdjPlan& a, int k, const float* in, float* out, float* log, uint32_t cap,
                                     float* ck) {
    const NsVol& V = a.V;
    __shared__ uint32_t chg[S::CHG];
    __shared__ uint32_t any, ncap, nfound;
    __shared__ uint32_t capl[27];
    __shared__ uint32_t found[kAdjThreads];
    constexpr int G = S::VOX / 4;
    constexpr uint32_t kUpd = 0x80000000u;
    const unsigned long long* act = plan_act(a, k);
    const uint32_t* flag_k = plan_flag(a, k);
    const uint32_t* flag_p = k ? plan_flag(a, k - 1) : nullptr;
    uint32_t mine = 0;
    const uint64_t chunk = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t c0 = 0; c0 < a.nb; c0 += chunk) {
        __syncthreads();  // found and nfound free
        if (threadIdx.x == 0) nfound = 0u;
        __syncthreads();
        const uint64_t mb = c0 + (uint64_t)threadIdx.x * gridDim.x + blockIdx.x;
        bool upd_mine = false;
        uint32_t pos = 0u;
        if (mb < a.nb) {
            const uint32_t b = (uint32_t)mb;
            upd_mine = flag_k[b] != 0u;
            if (upd_mine || (flag_p && flag_p[b] != 0u)) found[atomicAdd(&nfound, 1u)] = b | (upd_mine ? kUpd : 0u);
            // The list position is stored at the end of the chunk: the
            // atomic's latency hides behind the bricks' work.
            if (upd_mine) pos = atomicAdd(&a.counts[k], 1u);
        }
        __syncthreads();  // found complete
        const uint32_t nf = nfound;
        for (uint32_t f = 0; f < nf; ++f) {
            const bool upd = (found[f] & kUpd) != 0u;
            const uint32_t b = found[f] & ~kUpd;
            const int3 o = brick_origin<S>(V, b + V.brick_base);
            if (upd) {
                __syncthreads();  // chg, any, ncap and capl free: the previous brick is done
                if (threadIdx.x == 0) {
                    any = 0u;
                    ncap = 0u;
                }
                __syncthreads();
            }
            // Thread r < 27 marks neighbour r as reached (the reverse reads
            // lambda there only) and claims it for the checkpoint before the
            // update, so the atomic's latency hides behind the update.
            uint32_t nbr = 0u;
            bool won = false;
            if (upd && threadIdx.x < 27) {
                const int ox = (int)threadIdx.x % 3 - 1, oy = ((int)threadIdx.x / 3) % 3 - 1,
                          oz = (int)threadIdx.x / 9 - 1;
                const int bx = o.x / S::X + ox, by = o.y / S::Y + oy, bz = o.z / S::Z + oz;
                if (bx >= 0 && by >= 0 && bz >= 0 && bx < V.nbx && by < V.nby && bz < V.nbz) {
                    nbr = b + (uint32_t)((oz * V.nby + oy) * V.nbx + ox);
                    a.reached[nbr] = a.gen;
                    if (cap) won = atomicExch(&a.need[nbr], cap) != cap;
                }
            }
            for (int j = threadIdx.x; j < S::VOX; j += blockDim.x) {
                const int3 p = make_int3(o.x + j % S::X, o.y + (j / S::X) % S::Y, o.z + j / (S::X * S::Y));
                bool changed = false;
                if (p.x < V.nx && p.y < V.ny && p.z < V.nz) {
                    const size_t idx = ((size_t)p.z * V.py + p.y) * V.px + p.x;
                    const float c = in[idx];
                    if (upd && log) log[(size_t)b * S::VOX + j] = c;
                    if (upd && ((act[(size_t)b * S::WORDS + (j >> 6)] >> (j & 63)) & 1ull)) {
                        auto P = [&](int dx, int dy, int dz) {
                            return in[((size_t)clampi(p.z + dz, V.nz) * V.py + clampi(p.y + dy, V.ny)) * V.px +
                                      clampi(p.x + dx, V.nx)];
                        };
                        const float nv = ns_update_f32(P, V.img[idx], V.bias ? V.bias[idx] : 0.0f, V);
                        changed = fabsf(nv - c) > V.thr_t;
                        out[idx] = nv;
                        ++mine;
                    } else {
                        out[idx] = c;
                    }
                }
                // VOX is a multiple of 32: a warp's slots are all in or all out.
                if (upd) {
                    const uint32_t bal = __ballot_sync(0xffffffffu, changed);
                    if ((threadIdx.x & 31) == 0) {
                        chg[j >> 5] = bal;
                        if (bal) any = 1u;
                    }
                }
            }
            if (!upd) continue;
            __syncthreads();  // chg and any complete
            if (any) adj_dilate_brick<S>(V, b, chg, threadIdx.x, blockDim.x, plan_act(a, k + 1), plan_flag(a, k + 1));
            if (cap) {
                if (won) {
                    capl[atomicAdd(&ncap, 1u)] = nbr;
                    plan_need(a, (int)cap - 1)[atomicAdd(&a.ncount[cap - 1], 1u)] = nbr;
                }
                __syncthreads();  // capl complete
                const uint32_t nc = ncap;
                const float4* in4 = reinterpret_cast<const float4*>(in);
                float4* ck4 = reinterpret_cast<float4*>(ck);
                for (uint32_t q = threadIdx.x; q < nc * G; q += blockDim.x) {
                    const uint32_t cb = capl[q / G];
                    const int jj = (int)(q % G) * 4;
                    const int3 c = brick_origin<S>(V, cb + V.brick_base);
                    const size_t idx = ((size_t)(c.z + jj / (S::X * S::Y)) * V.py + c.y + (jj / S::X) % S::Y) * V.px +
                                       c.x + jj % S::X;
                    ck4[idx / 4] = in4[idx / 4];
                }
            }
        }
        if (upd_mine) plan_list(a, k)[pos] = (uint32_t)mb;
    }
    __syncthreads();  // the shared words are reused by the next call
    return mine;
}

// Brick parts, the work split of the reverse: a brick's voxels in N runs
// of TPG consecutive voxels (whole z-planes), one voxel a thread.  A block
// holds GROUPS groups of TPG threads; item i of a phase (brick i / N, part
// i mod N) goes to the group whose slot is i mod (GROUPS * grid), slot =
// group * grid + (block + offset) mod grid.  So the parts of one brick run
// on different SMs: an iteration holds a few dozen bricks of ~150 active
// voxels each, and one SM a brick would leave most SMs idle.
template <class S>
struct Parts {
    static constexpr int TPG = S::VOX < 128 ? S::VOX : 128;
    static constexpr int N = S::VOX / TPG;
    static constexpr int GROUPS = kAdjThreads / TPG;
    static_assert(kAdjThreads % TPG == 0, "groups tile the block");
    // Items of the reverse iteration proper: with 128-thread groups, 64
    // voxels an item and two threads a voxel (t and t + 64, in different
    // warps, each half of the transposed Jacobian); else TPG voxels, one
    // thread each.
    static constexpr bool SPLIT = TPG == 128;
    static constexpr int AV = SPLIT ? 64 : TPG;
    static constexpr int NA = S::VOX / AV;
    uint32_t slot, nslots;
    int t;
    __device__ __forceinline__ explicit Parts(uint32_t offset) {
        const uint32_t g = threadIdx.x / TPG;
        t = (int)(threadIdx.x % TPG);
        slot = g * gridDim.x + (blockIdx.x + offset) % gridDim.x;
        nslots = GROUPS * gridDim.x;
    }
    // Brick voxel of item i for this thread.
    __device__ __forceinline__ int voxel(uint32_t i) const { return (int)(i % N) * TPG + t; }
    // Brick voxel of reverse-iteration item i, and this thread's half of the
    // Jacobian (-1: all of it).
    __device__ __forceinline__ int avoxel(uint32_t i) const { return (int)(i % NA) * AV + (SPLIT ? (t & 63) : t); }
    __device__ __forceinline__ int half() const { return SPLIT ? (t >> 6) : -1; }
};

// One item of the restore of phi_kr into dst (holding phi_{kr+2}) from the
// logs of segment s: the bricks of list_kr from log_kr, those of
// list_{kr+1} outside list_kr from log_{kr+1}; n0 = count_kr.  Item i:
// brick i / N of list_kr followed by list_{kr+1}.
template <class S>
__device__ __forceinline__ void restore_item(const AdjPlan& a, int s, int kr, float* dst, uint32_t n0, uint32_t i,
                                             const Parts<S>& pt) {
    const NsVol& V = a.V;
    const uint32_t bi = i / Parts<S>::N;
    const bool first = bi < n0;
    const uint32_t pos = first ? bi : bi - n0;
    const uint32_t b = plan_list(a, first ? kr : kr + 1)[pos];
    if (!first && plan_flag(a, kr)[b]) return;
    const int j = pt.voxel(i);
    const int3 p = voxel_of<S>(V, b, j);
    if (p.x < V.nx && p.y < V.ny && p.z < V.nz)
        dst[((size_t)p.z * V.py + p.y) * V.px + p.x] = plan_log(a, s, first ? kr : kr + 1)[(size_t)b * S::VOX + j];
}

// One item of recomputed iteration t of segment s (list_t then, for t past
// the segment's first iteration, list_{t-1}; n = count_t): the bricks of
// list_t written whole into out (active voxels updated from in, the others
// copied) and logged as they were (brick b at log_t + b * VOX); the bricks
// of list_{t-1} outside list_t copied from in to out.
template <class S>
__device__ __forceinline__ void rec_item(const AdjPlan& a, int s, int t, const float* in, float* out, uint32_t n,
                                         uint32_t i, const Parts<S>& pt) {
    const NsVol& V = a.V;
    const uint32_t bi = i / Parts<S>::N;
    const bool upd = bi < n;
    const uint32_t b = upd ? plan_list(a, t)[bi] : plan_list(a, t - 1)[bi - n];
    if (!upd && plan_flag(a, t)[b]) return;
    const int j = pt.voxel(i);
    const int3 p = voxel_of<S>(V, b, j);
    if (p.x >= V.nx || p.y >= V.ny || p.z >= V.nz) return;
    const size_t idx = ((size_t)p.z * V.py + p.y) * V.px + p.x;
    const float c = in[idx];
    if (!upd) {
        out[idx] = c;
        return;
    }
    plan_log(a, s, t)[(size_t)b * S::VOX + j] = c;
    if (!((plan_act(a, t)[(size_t)b * S::WORDS + (j >> 6)] >> (j & 63)) & 1ull)) {
        out[idx] = c;
        return;
    }
    auto P = [&](int dx, int dy, int dz) {
        return in[((size_t)clampi(p.z + dz, V.nz) * V.py + clampi(p.y + dy, V.ny)) * V.px + clampi(p.x + dx, V.nx)];
    };
    out[idx] = ns_update_f32(P, V.img[idx], V.bias ? V.bias[idx] : 0.0f, V);
}

// One item of the seeding of a recomputed segment's pair: brick i / N of
// segment s's checkpoint list copied from the checkpoint ck to its second
// field q (the recomputation reads and writes no other brick).
template <class S>
__device__ __forceinline__ void seed_item(const AdjPlan& a, int s, const float* ck, float* q, uint32_t i,
                                          const Parts<S>& pt) {
    const NsVol& V = a.V;
    const int3 p = voxel_of<S>(V, plan_need(a, s)[i / Parts<S>::N], pt.voxel(i));
    if (p.x < V.nx && p.y < V.ny && p.z < V.nz) {
        const size_t idx = ((size_t)p.z * V.py + p.y) * V.px + p.x;
        q[idx] = ck[idx];
    }
}

// Vector-Jacobian product of ns_update_f32 at one voxel with upstream lam:
// scatters dloss/dphi onto the stencil (add(dx, dy, dz, g)) and returns the
// parameter terms in g4 = (T, eps, alpha, bias).  Same derivation as the FP64
// oracle (oracle/ns_adjoint.hpp), in fp32.  part 0: the centre, face and
// upwind terms; part 1: the cross-derivative and parameter terms; part 2:
// all (two threads with parts 0 and 1 together do what one with part 2 does).
template <class PF, class AF>
__device__ __forceinline__ void ns_update_vjp_f32(PF P, AF add, float I, float bias, const NsVol& V, float lam,
                                                  float* g4, int part = 2) {
    const float c = P(0, 0, 0);
    const float xm = P(-1, 0, 0), xp = P(1, 0, 0);
    const float ym = P(0, -1, 0), yp = P(0, 1, 0);
    const float zm = P(0, 0, -1), zp = P(0, 0, 1);
    const float cx = (xp - xm) * 0.5f, cy = (yp - ym) * 0.5f, cz = (zp - zm) * 0.5f;
    const float fxx = xp - 2.0f * c + xm, fyy = yp - 2.0f * c + ym, fzz = zp - 2.0f * c + zm;
    const float fxy = (P(1, 1, 0) - P(1, -1, 0) - P(-1, 1, 0) + P(-1, -1, 0)) * 0.25f;
    const float fxz = (P(1, 0, 1) - P(1, 0, -1) - P(-1, 0, 1) + P(-1, 0, -1)) * 0.25f;
    const float fyz = (P(0, 1, 1) - P(0, 1, -1) - P(0, -1, 1) + P(0, -1, -1)) * 0.25f;
    const float g2 = cx * cx + cy * cy + cz * cz;
    const bool has_curv = g2 > 1e-12f;
    float curv = 0.0f;
    if (has_curv) {
        const float num = fxx * (cy * cy + cz * cz) + fyy * (cx * cx + cz * cz) + fzz * (cx * cx + cy * cy) -
                          2.0f * (cx * cy * fxy + cx * cz * fxz + cy * cz * fyz);
        curv = num / g2;
    }
    const float Draw = V.data_literal ? V.eps - fabsf(I - V.T) : (V.eps - fabsf(I - V.T)) / V.eps;
    const bool dclamp = Draw < V.dlo || Draw > V.dhi;
    const float Dt = fminf(fmaxf(Draw, V.dlo), V.dhi) + bias;
    const float F = V.wd * Dt;
    const float dxm = c - xm, dxp = xp - c, dym = c - ym, dyp = yp - c, dzm = c - zm, dzp = zp - c;
    float a, b, e, f, h, k;
    if (F > 0.0f) {
        a = fmaxf(dxm, 0.0f); b = fminf(dxp, 0.0f); e = fmaxf(dym, 0.0f);
        f = fminf(dyp, 0.0f); h = fmaxf(dzm, 0.0f); k = fminf(dzp, 0.0f);
    } else {
        a = fminf(dxm, 0.0f); b = fmaxf(dxp, 0.0f); e = fminf(dym, 0.0f);
        f = fmaxf(dyp, 0.0f); h = fminf(dzm, 0.0f); k = fmaxf(dzp, 0.0f);
    }
    const float gn = sqrtf(a * a + b * b + e * e + f * f + h * h + k * k);
    const float u = c + V.dt * (V.wc * curv - F * gn);
    if (u < V.lo || u > V.hi) return;  // clamped: no gradient
    const bool p0 = part != 1, p1 = part != 0;
    if (p0) add(0, 0, 0, lam);
    const float gcurv = lam * V.dt * V.wc, gF = -lam * V.dt * gn, ggn = -lam * V.dt * F;
    if (has_curv) {
        const float gnum = gcurv / g2, gg2 = -gcurv * curv / g2;
        if (p0) {
            const float gcx = gnum * (2.0f * cx * (fyy + fzz) - 2.0f * (cy * fxy + cz * fxz)) + gg2 * 2.0f * cx;
            const float gcy = gnum * (2.0f * cy * (fxx + fzz) - 2.0f * (cx * fxy + cz * fyz)) + gg2 * 2.0f * cy;
            const float gcz = gnum * (2.0f * cz * (fxx + fyy) - 2.0f * (cx * fxz + cy * fyz)) + gg2 * 2.0f * cz;
            const float gfxx = gnum * (cy * cy + cz * cz), gfyy = gnum * (cx * cx + cz * cz),
                        gfzz = gnum * (cx * cx + cy * cy);
            add(1, 0, 0, 0.5f * gcx + gfxx);
            add(-1, 0, 0, -0.5f * gcx + gfxx);
            add(0, 1, 0, 0.5f * gcy + gfyy);
            add(0, -1, 0, -0.5f * gcy + gfyy);
            add(0, 0, 1, 0.5f * gcz + gfzz);
            add(0, 0, -1, -0.5f * gcz + gfzz);
            add(0, 0, 0, -2.0f * (gfxx + gfyy + gfzz));
        }
    }
    if (has_curv && p1) {
        const float gnum = gcurv / g2;
        const float gfxy = -2.0f * gnum * cx * cy, gfxz = -2.0f * gnum * cx * cz, gfyz = -2.0f * gnum * cy * cz;
        add(1, 1, 0, 0.25f * gfxy);
        add(1, -1, 0, -0.25f * gfxy);
        add(-1, 1, 0, -0.25f * gfxy);
        add(-1, -1, 0, 0.25f * gfxy);
        add(1, 0, 1, 0.25f * gfxz);
        add(1, 0, -1, -0.25f * gfxz);
        add(-1, 0, 1, -0.25f * gfxz);
        add(-1, 0, -1, 0.25f * gfxz);
        add(0, 1, 1, 0.25f * gfyz);
        add(0, 1, -1, -0.25f * gfyz);
        add(0, -1, 1, -0.25f * gfyz);
        add(0, -1, -1, 0.25f * gfyz);
    }
    if (p0 && gn > 0.0f) {
        const float s = ggn / gn;
        add(0, 0, 0, s * (a - b + e - f + h - k));
        add(-1, 0, 0, -s * a);
        add(1, 0, 0, s * b);
        add(0, -1, 0, -s * e);
        add(0, 1, 0, s * f);
        add(0, 0, -1, -s * h);
        add(0, 0, 1, s * k);
    }
    if (!p1) return;
    const float gDt = gF * V.wd;
    g4[3] += gDt;
    if (!dclamp) {
        const float sg = I > V.T ? 1.0f : (I < V.T ? -1.0f : 0.0f);
        if (V.data_literal) {  // D = eps - |I - T|
            g4[0] += gDt * sg;
            g4[1] += gDt;
        } else {  // D = (eps - |I - T|) / eps
            g4[0] += gDt * sg / V.eps;
            g4[1] += gDt * fabsf(I - V.T) / (V.eps * V.eps);
        }
    }
    const float du_dalpha = V.dt * (-curv - Dt * gn);
    g4[2] += lam * (V.alpha_data ? du_dalpha : -du_dalpha);
}

// Block sum of three doubles added into the block's own three words (slot;
// no other block writes them, so no atomics, and the host adds the blocks'
// slots in a fixed order).
__device__ __forceinline__ void block_sum3(double a0, double a1, double a2, double* slot) {
    __shared__ double s[3][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        a0 += __shfl_down_sync(0xffffffffu, a0, o);
        a1 += __shfl_down_sync(0xffffffffu, a1, o);
        a2 += __shfl_down_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) { s[0][warp] = a0; s[1][warp] = a1; s[2][warp] = a2; }
    __syncthreads();
    if (warp == 0) {
        a0 = lane < nw ? s[0][lane] : 0.0;
        a1 = lane < nw ? s[1][lane] : 0.0;
        a2 = lane < nw ? s[2][lane] : 0.0;
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            a0 += __shfl_down_sync(0xffffffffu, a0, o);
            a1 += __shfl_down_sync(0xffffffffu, a1, o);
            a2 += __shfl_down_sync(0xffffffffu, a2, o);
        }
        if (lane == 0) {
            slot[0] += a0;
            slot[1] += a1;
            slot[2] += a2;
        }
    }
    __syncthreads();
}

// The bricks one brick's reverse iteration scatters into: the 26-dilation of
// its voxels of A_k (act, a superset of the update's stencil), clipped to
// the volume; each gets mark[brick] = 1.  Threads t0, t0 + stride, ... take
// the (neighbour, mask word) pairs.
template <class S>
__device__ __forceinline__ void adj_mark_brick(const NsVol& V, uint32_t b, const unsigned long long* act, int t0,
                                               int stride, uint32_t* mark) {
    const uint32_t* bits = reinterpret_cast<const uint32_t*>(act + (size_t)b * S::WORDS);
    const int3 o = brick_origin<S>(V, b + V.brick_base);
    for (int r = t0; r < 27 * S::WORDS; r += stride) {
        const int slot = r / S::WORDS, w = r % S::WORDS;
        const int ox = slot % 3 - 1, oy = (slot / 3) % 3 - 1, oz = slot / 9 - 1;
        const int bx = o.x / S::X + ox, by = o.y / S::Y + oy, bz = o.z / S::Z + oz;
        const int lx = V.nx - bx * S::X, ly = V.ny - by * S::Y, lz = V.nz - bz * S::Z;
        if (bx < 0 || by < 0 || bz < 0 || lx <= 0 || ly <= 0 || lz <= 0) continue;
        uint64_t x = dilate_word<S>(bits, ox, oy, oz, w, 26);
        if (lx < S::X || ly < S::Y || lz < S::Z)
            x &= inside_mask<S>(w, min(lx, S::X), min(ly, S::Y), min(lz, S::Z));
        if (x) mark[b + (int32_t)((oz * V.nby + oy) * V.nbx + ox)] = 1u;
    }
}

// Reverse iteration k.  With p = (k + 1) & 1, lambda_{k+1} = lam + Z[p] on
// entry, where Z[p] (the previous reverse iteration's scatter) is zero
// outside the bricks marked in flagT[k & 1], and Z[1-p] is zero everywhere.
// At each voxel v visited:
//   lambda_{k+1}[v] = lam[v] + Z[p][v];  Z[p][v] = 0;
//   v not in A_k: lam[v] = lambda_{k+1}[v] (the pass-through);
//   v in A_k:     lam[v] = 0, and lambda_{k+1}[v] is scattered through the
//                 transposed stencil Jacobian of the update into Z[1-p]
//                 (fp32 atomics), the parameter terms (T, eps, alpha) added
//                 to s3 (FP64, per thread) and the bias gradient to dbias;
// so lambda_k = lam + Z[1-p] on exit, with the bricks Z[1-p] reaches marked
// in flagT[(k - 1) & 1] (by each brick's part 0).  Part one (brick parts of
// A_k) visits the bricks of A_k whole; part two (adj_rev_touched) the
// marked bricks outside A_k.  Every field of a voxel is written by one
// thread only (with two threads a voxel: lambda and Z by half 0, d_bias by
// half 1).
//
// half (Parts::half): -1, the thread does the voxel alone; 0 or 1, the
// voxel's two threads of a 128-thread group (in different warps, so the
// halves run side by side) both load, a barrier of the group orders every
// load before the folds, then half 0 folds lambda and scatters part 0 of
// the transposed Jacobian, half 1 scatters part 1 and adds the parameter
// and bias gradients.  Every thread of a split group reaches the barrier.
template <class S>
__device__ __forceinline__ void rev_voxel(const AdjPlan& a, const float* phi, float* zin, float* zout, uint32_t b,
                                          int j, bool in_a, double* s3, int half) {
    const NsVol& V = a.V;
    const int3 pv = voxel_of<S>(V, b, j);
    const bool inside = pv.x < V.nx && pv.y < V.ny && pv.z < V.nz;
    const size_t idx = inside ? ((size_t)pv.z * V.py + pv.y) * V.px + pv.x : 0;
    auto at = [&](int dx, int dy, int dz) {
        return ((size_t)clampi(pv.z + dz, V.nz) * V.py + clampi(pv.y + dy, V.ny)) * V.px + clampi(pv.x + dx, V.nx);
    };
    // Every load of the voxel is issued before any store or branch, by the
    // lanes outside A_k too (a warp runs both kinds of lane one after the
    // other, so this keeps it to one round trip): the stencil of phi_k (the
    // update's 19 points), I, the bias, lambda's two parts.
    float st[3][3][3];
    float I = 0.0f, bias = 0.0f, x = 0.0f, z = 0.0f;
    if (inside) {
#pragma unroll
        for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                for (int dx = -1; dx <= 1; ++dx)
                    st[dz + 1][dy + 1][dx + 1] = (dx != 0 && dy != 0 && dz != 0) ? 0.0f : phi[at(dx, dy, dz)];
        I = V.img[idx];
        bias = V.bias ? V.bias[idx] : 0.0f;
        x = a.lam[idx];
        z = zin[idx];
    }
    // The group's 128 threads, barrier 1 + group (the non-aligned form: the
    // lanes may reach it from the divergent loads above).
    if (half >= 0) asm volatile("barrier.sync %0, 128;" ::"r"(1 + (int)(threadIdx.x >> 7)) : "memory");
    if (!inside) return;
    const float u = x + z;
    if (half != 1) {
        if (z != 0.0f) zin[idx] = 0.0f;
        if (!in_a) {
            if (z != 0.0f) a.lam[idx] = u;
            return;
        }
        if (x != 0.0f) a.lam[idx] = 0.0f;
    }
    if (!in_a || u == 0.0f) return;
    auto P = [&](int dx, int dy, int dz) { return st[dz + 1][dy + 1][dx + 1]; };
    auto add = [&](int dx, int dy, int dz, float g) {
        if (g != 0.0f) atomicAdd(&zout[at(dx, dy, dz)], g);
    };
    float g4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    ns_update_vjp_f32(P, add, I, bias, V, u, g4, half < 0 ? 2 : half);
    if (half == 0) return;
    s3[0] += g4[0];
    s3[1] += g4[1];
    s3[2] += g4[2];
    if (a.dbias) a.dbias[idx] += g4[3];
}

// One phase of the reverse: reverse iteration k of segment s (k < 0:
// none), with the restore of phi_kr beside it (kr < 0: none) and step r of
// the recomputation of segment rs (r < 0: none; r = 0 seeds the pair's
// second field with the checkpoint, r >= 1 runs iteration t = rs * every +
// r - 1).  Its work items (brick parts: reverse iteration, then the
// recomputed iteration, then the restore) share one item space, so the
// kinds run side by side on different SMs.  Everything here is read from
// the recorded lists before the barrier that precedes the phase.
struct RevPhase {
    int k, s, kr, rs, r, t;
    const float* phi;   // phi_k
    float* rdst;        // the field restored to phi_kr
    const float* rin;   // the recomputation's fields
    float* rout;
    uint32_t nA, nC, nR;  // items of each kind
    uint32_t cnt_t, cnt_kr;
    uint32_t b0;          // brick of this thread's first item (reverse iteration)
    unsigned long long w0;  // and its mask word of the thread's voxel
};

template <class S>
__device__ __forceinline__ int rev_phases(const AdjPlan& a, int s) {
    const int len = min(a.K, (s + 1) * a.every) - s * a.every;
    return max(len, (s > 0 && a.every > 1) ? a.every : 0);
}

template <class S>
__device__ RevPhase rev_phase(const AdjPlan& a, int s, int j) {
    constexpr uint32_t N = Parts<S>::N;
    RevPhase ph;
    ph.k = ph.kr = ph.rs = ph.r = ph.t = -1;
    ph.s = s;
    ph.phi = nullptr;
    ph.rdst = ph.rout = nullptr;
    ph.rin = nullptr;
    ph.nA = ph.nC = ph.nR = ph.cnt_t = ph.cnt_kr = ph.b0 = 0u;
    ph.w0 = 0ull;
    const int s0 = s * a.every, s1 = min(a.K, s0 + a.every);
    const SegPair pr = seg_pair(a, s);
    // The highest state the pair holds (with the one below it): phi_K for
    // the last segment, phi_{s1 - 1} after a recomputation.
    const int top = s == a.nck - 1 ? a.K : s1 - 1;
    if (j < s1 - s0) {
        const int k = s1 - 1 - j;
        ph.k = k;
        ph.phi = pr.f[(k - pr.base) & 1];
        ph.nA = a.counts[k] * (uint32_t)Parts<S>::NA;
        const Parts<S> pt(0);
        if (pt.slot < ph.nA) {
            ph.b0 = plan_list(a, k)[pt.slot / Parts<S>::NA];
            ph.w0 = plan_act(a, k)[(size_t)ph.b0 * S::WORDS + (pt.avoxel(pt.slot) >> 6)];
        }
        // The pair's other field steps down to phi_{k-1} unless it holds it.
        if (k - 1 >= s0 && k - 1 < top - 1) {
            ph.kr = k - 1;
            ph.rdst = pr.f[(k - 1 - pr.base) & 1];
            ph.cnt_kr = a.counts[k - 1];
            ph.nR = (ph.cnt_kr + a.counts[k]) * N;
        }
    }
    // Segment s - 1 (full length) is recomputed beside this one, one step a
    // phase: its checkpoint's bricks copied into the pair's second field,
    // then its iterations s0' .. s0' + every - 2, logged.
    if (s > 0 && a.every > 1 && j < a.every) {
        const SegPair rp = seg_pair(a, s - 1);
        ph.rs = s - 1;
        ph.r = j;
        if (j == 0) {
            ph.rin = rp.f[0];
            ph.rout = rp.f[1];
            ph.nC = a.ncount[s - 1] * N;
        } else {
            ph.t = rp.base + j - 1;
            ph.rin = rp.f[(j - 1) & 1];
            ph.rout = rp.f[j & 1];
            ph.cnt_t = a.counts[ph.t];
            ph.nC = (ph.cnt_t + (j >= 2 ? a.counts[ph.t - 1] : 0u)) * N;
        }
    }
    return ph;
}

// Part two of reverse iteration k: the bricks marked in flagT[k & 1] that
// are not in A_k hold no active voxel, so lambda_{k+1} passes through:
// lam += Z[p], Z[p] = 0, four voxels a lane-step (brick rows of 4 or 8
// voxels are 16-byte aligned: px is a multiple of 8; padding voxels hold
// Z = 0 and stay as they are).  Warp w scans bricks w + l * NW (lane l; NW
// warps), so a cluster of consecutive marked bricks spreads over the warps;
// every mark is cleared for reverse iteration k - 2.  Warp w of the nw
// warps doing this part.
template <class S>
__device__ void adj_rev_touched(const AdjPlan& a, int k, uint32_t w, uint32_t nw) {
    const NsVol& V = a.V;
    const int p = (k + 1) & 1;
    float4* const lam4 = reinterpret_cast<float4*>(a.lam);
    float4* const z4 = reinterpret_cast<float4*>(a.Z[p]);
    uint32_t* flag = a.flagT[k & 1];
    const uint32_t* in_a = plan_flag(a, k);
    const int lane = threadIdx.x & 31;
    constexpr int G = S::VOX / 4, PER = (G + 31) / 32;
    for (uint64_t base = 0; base < a.nb; base += 32ull * nw) {
        const uint64_t bl = base + (uint64_t)lane * nw + w;
        bool fold = false;
        if (bl < a.nb && flag[bl]) {
            flag[bl] = 0u;
            fold = !in_a[bl];
        }
        uint32_t bal = __ballot_sync(0xffffffffu, fold);
        while (bal) {
            const int l = __ffs(bal) - 1;
            bal &= bal - 1u;
            const uint32_t b = (uint32_t)(base + (uint64_t)l * nw + w);
            const int3 o = brick_origin<S>(V, b + V.brick_base);
            size_t g4[PER];
            float4 zz[PER], xx[PER];
#pragma unroll
            for (int u = 0; u < PER; ++u) {
                const int q = lane + 32 * u, j = 4 * q;
                g4[u] = q < G ? (((size_t)(o.z + j / (S::X * S::Y)) * V.py + o.y + (j / S::X) % S::Y) * V.px + o.x +
                                 j % S::X) / 4
                              : 0;
                if (q < G) {
                    zz[u] = z4[g4[u]];
                    xx[u] = lam4[g4[u]];
                }
            }
#pragma unroll
            for (int u = 0; u < PER; ++u) {
                if (lane + 32 * u >= G) continue;
                if (zz[u].x != 0.0f || zz[u].y != 0.0f || zz[u].z != 0.0f || zz[u].w != 0.0f) {
                    lam4[g4[u]] = make_float4(xx[u].x + zz[u].x, xx[u].y + zz[u].y, xx[u].z + zz[u].z,
                                              xx[u].w + zz[u].w);
                    z4[g4[u]] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                }
            }
        }
    }
}

template <class S>
__device__ void adj_rev_phase(const AdjPlan& a, const RevPhase& ph, double* s3) {
    const Parts<S> pt(0);
    // Part two of the reverse iteration goes to the warps of the groups
    // without a brick part of A_k (all warps when every group has one), so
    // the parts of A_k, the longest work of the phase, start at once.
    if (ph.k >= 0) {
        constexpr uint32_t WPG = Parts<S>::TPG / 32;
        const uint32_t wig = (uint32_t)pt.t / 32;
        if (ph.nA < pt.nslots) {
            if (pt.slot >= ph.nA) adj_rev_touched<S>(a, ph.k, (pt.slot - ph.nA) * WPG + wig, (pt.nslots - ph.nA) * WPG);
        } else {
            adj_rev_touched<S>(a, ph.k, pt.slot * WPG + wig, pt.nslots * WPG);
        }
    }
    const uint32_t nAC = ph.nA + ph.nC, total = nAC + ph.nR;
    for (uint32_t it = pt.slot; it < total; it += pt.nslots) {
        if (it < ph.nA) {
            const int k = ph.k, p = (k + 1) & 1;
            const bool first = it == pt.slot;
            const unsigned long long* act = plan_act(a, k);
            const uint32_t b = first ? ph.b0 : plan_list(a, k)[it / Parts<S>::NA];
            const int jv = pt.avoxel(it);
            const unsigned long long wj = first ? ph.w0 : act[(size_t)b * S::WORDS + (jv >> 6)];
            rev_voxel<S>(a, ph.phi, a.Z[p], a.Z[p ^ 1], b, jv, (wj >> (jv & 63)) & 1ull, s3, pt.half());
            if (it % Parts<S>::NA == 0 && k > 0)
                adj_mark_brick<S>(a.V, b, act, pt.t, Parts<S>::TPG, a.flagT[(k - 1) & 1]);
        } else if (it < nAC) {
            if (ph.r == 0) {
                seed_item<S>(a, ph.rs, ph.rin, ph.rout, it - ph.nA, pt);
            } else {
                rec_item<S>(a, ph.rs, ph.t, ph.rin, ph.rout, ph.cnt_t, it - ph.nA, pt);
            }
        } else {
            restore_item<S>(a, ph.s, ph.kr, ph.rdst, ph.cnt_kr, it - nAC, pt);
        }
    }
}

// The call's set-up, grid-stride over the whole grid (one pass instead of a
// dozen memsets and copies): both fields of the forward's pair <- phi_0, the
// recorded masks of A_0 <- the engine's, those of A_1..A_K, the membership
// flags of A_1..A_K, counts, marks and sums <- 0, and d_bias <- 0.  A call
// writes the pair in the bricks of its A_k only, all stamped in `reached`;
// when the engine's phi and the workspace are those of the previous call
// (partial), the pair still holds phi_0 elsewhere and only the bricks that
// call stamped (gen - 1) are copied again, and the stamps stay (this call's
// are gen); otherwise the whole field is copied and the stamps cleared.
template <class S>
__device__ void adj_setup(const AdjPlan& a) {
    const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, nt = (uint64_t)gridDim.x * blockDim.x;
    const float4* src4 = reinterpret_cast<const float4*>(a.phi0);
    float4* f0 = reinterpret_cast<float4*>(a.fw[0]);
    float4* f1 = reinterpret_cast<float4*>(a.fw[1]);
    if (a.partial) {
        // Item i: float4 q of brick b (rows of X / 4 float4, x fastest).
        constexpr uint32_t Q = S::X / 4, PER = S::VOX / 4;
        const uint32_t prev = a.gen - 1u;
        for (uint64_t i = t0; i < (uint64_t)a.nb * PER; i += nt) {
            const uint32_t b = (uint32_t)(i / PER), q = (uint32_t)(i % PER);
            if (a.reached[b] != prev) continue;
            const int3 o = brick_origin<S>(a.V, b + a.V.brick_base);
            const uint32_t row = q / Q, ly = row % S::Y, lz = row / S::Y;
            const uint64_t g = (((uint64_t)(o.z + lz) * a.V.py + (o.y + ly)) * a.V.px + o.x) / 4 + q % Q;
            const float4 v = src4[g];
            f0[g] = v;
            f1[g] = v;
        }
    } else {
        for (uint64_t i = t0; i < a.P / 4; i += nt) {
            const float4 v = src4[i];
            f0[i] = v;
            f1[i] = v;
        }
    }
    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
    // act_0 (mwords u64, copied) then act_1 .. act_K (astride u64 each, cleared).
    for (uint64_t i = t0; i < a.mwords; i += nt) a.act0[i] = a.act_src[i];
    uint4* act4 = reinterpret_cast<uint4*>(a.act0 + a.astride);
    for (uint64_t i = t0; i < (uint64_t)a.K * a.astride / 2; i += nt) act4[i] = z;
    // flag_1 .. flag_K (flag_0 is written whole by adj_flag0 in this phase).
    uint4* flag4 = reinterpret_cast<uint4*>(a.flag0 + a.lstride);
    for (uint64_t i = t0; i < (uint64_t)a.K * a.lstride / 4; i += nt) flag4[i] = z;
    if (a.dbias) {
        float4* d4 = reinterpret_cast<float4*>(a.dbias);
        for (uint64_t i = t0; i < a.dbias_n / 4; i += nt) d4[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    for (uint64_t i = t0; i < a.nb; i += nt) {
        a.flagT[0][i] = 0u;
        a.flagT[1][i] = 0u;
        a.need[i] = 0u;
        if (!a.partial) a.reached[i] = 0u;
    }
    for (uint64_t i = t0; i <= (uint64_t)a.K; i += nt) a.counts[i] = 0u;
    for (uint64_t i = t0; i < (uint64_t)a.nck; i += nt) a.ncount[i] = 0u;
    for (uint64_t i = t0; i < 9; i += nt) a.gsum[i] = 0.0;  // the sums and the update count
    for (uint64_t i = t0; i < 3ull * gridDim.x; i += nt) a.gpart[i] = 0.0;  // the reverse's grid is this one
}

// The forward: list_0, then K iterations; every segment but the last
// builds its sparse checkpoint as it goes, the last one logs its bricks.
template <class S>
__global__ void __launch_bounds__(kAdjThreads) k_adj_forward(const AdjPlan a) {
    cg::grid_group grid = cg::this_grid();
    adj_setup<S>(a);
    adj_flag0<S>(a.act_src, plan_flag(a, 0), a.nb);  // from the engine's masks: no wait for the copy
    grid.sync();
    uint32_t mine = 0;
    const int last = a.nck - 1;
    for (int k = 0; k < a.K; ++k) {
        const float* src = a.fw[k & 1];
        float* dst = a.fw[(k + 1) & 1];
        const int s = k / a.every;
        mine += adj_forward_step<S>(a, k, src, dst, s == last ? plan_log(a, last, k) : nullptr,
                                    s < last ? (uint32_t)s + 1u : 0u,
                                    s < last ? a.ck0 + (uint64_t)s * a.fstride : nullptr);
        grid.sync();
    }
    __shared__ uint32_t s_cnt;
    if (threadIdx.x == 0) s_cnt = 0u;
    __syncthreads();
    mine = __reduce_add_sync(0xffffffffu, mine);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(&s_cnt, mine);
    __syncthreads();
    if (threadIdx.x == 0 && s_cnt) atomicAdd(a.nact, (unsigned long long)s_cnt);
    // The loss: phi_K is whole (the last iteration's barrier), the sums,
    // one barrier, lambda_K.
    adj_dice_sums<kAdjThreads>(a.dice);
    grid.sync();
    adj_lambda_k(a.dice);
}

// The reverse: the segments from the last (lambda_K is in lam).
template <class S>
__global__ void __launch_bounds__(kAdjThreads) k_adj_reverse(const AdjPlan a) {
    cg::grid_group grid = cg::this_grid();
    // Segments from the last; each phase's descriptor is read before the
    // barrier that precedes it.
    int s = a.nck - 1, j = 0;
    RevPhase ph = rev_phase<S>(a, s, j);
    double s3[3] = {0.0, 0.0, 0.0};
    for (;;) {
        adj_rev_phase<S>(a, ph, s3);
        if (++j == rev_phases<S>(a, s)) {
            --s;
            j = 0;
        }
        if (s < 0) break;  // the sums below are the block's own
        ph = rev_phase<S>(a, s, j);
        grid.sync();
    }
    block_sum3(s3[0], s3[1], s3[2], a.gpart + 3 * (size_t)blockIdx.x);
}

template <class S>
void run_adjoint(NsCore& core, int K, int every, const uint8_t* target, float tau, const float* bias,
                 float* dbias, lss_grads* out) {
    EngineBase* owner = core.owner();
    cudaStream_t st = owner->stream;
    NsVol V = core.descriptor(0);
    V.brick_base = 0;
    const uint32_t nb = (uint32_t)core.bricks();
    const uint64_t P = (uint64_t)V.px * V.py * V.pz;
    const size_t mwords = (size_t)nb * S::WORDS;
    const int nck = (K + every - 1) / every;
    const int grid = owner->num_sms * 8;  // the upload and download kernels
    const void* kf = (const void*)&k_adj_forward<S>;
    const void* kr = (const void*)&k_adj_reverse<S>;
    // Cooperative grids: every block resident.
    auto coop = [&](const void* k) {
        int per_sm = 0;
        LSS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kAdjThreads, 0));
        LSS_REQUIRE(per_sm > 0, LSS_ERR_CUDA, "adjoint kernel does not fit on an SM");
        return owner->num_sms * std::min(per_sm, kAdjBlocksPerSm);
    };
    const int gf = coop(kf), gr = coop(kr);
    // One device workspace (kept by the engine between calls), carved into
    // 256-byte aligned parts.
    auto al = [](uint64_t b) { return (b + 255) / 256 * 256; };
    // Fields: the checkpoints of every segment but the last, the second
    // fields of two recomputed segments' pairs, the forward's pair, lambda
    // and its two contribution fields, d_bias, bias; then two sets of
    // `every` brick logs (one set with a single segment), a brick list's
    // worth of voxels each.
    const int nqb = (nck > 1 && every > 1) ? 2 : 0, nsets = std::min(nck, 2);
    const uint64_t nfields = (uint64_t)(nck - 1) + nqb + 5 + (dbias ? 1 : 0) + (bias ? 1 : 0);
    const uint64_t logb = al((uint64_t)nb * S::VOX * 4);
    const uint64_t total = nfields * al(P * 4) + (uint64_t)nsets * every * logb + (uint64_t)(K + 1) * al(mwords * 8) +
                           2 * (uint64_t)(K + 1) * al((uint64_t)nb * 4) + al((uint64_t)(K + 1) * 4) + al(P) +
                           2 * al((uint64_t)nb * 4) + (uint64_t)(nck + 2) * al((uint64_t)nb * 4) + al((uint64_t)nck * 4) +
                           al(8 * sizeof(double) + 8) + al((uint64_t)gr * 3 * sizeof(double)) +
                           al((uint64_t)gf * 3 * sizeof(double));
    char* base = (char*)core.workspace(total);
    char* const end = base + total;
    auto carve = [&](uint64_t bytes) {
        char* p = base;
        base += al(bytes);
        LSS_REQUIRE(base <= end, LSS_ERR_CAPACITY, "adjoint workspace layout");
        return p;
    };
    auto F = [&]() { return (float*)carve(P * 4); };
    AdjPlan a;
    std::memset(&a, 0, sizeof(a));
    a.fstride = al(P * 4) / 4;
    a.ck0 = nck > 1 ? F() : nullptr;
    for (int s = 1; s < nck - 1; ++s) F();
    for (int q = 0; q < nqb; ++q) a.qb[q] = F();
    a.fw[0] = F();
    a.fw[1] = F();
    a.lam = F();
    a.Z[0] = F();
    a.Z[1] = F();
    a.lgstride = logb / 4;
    a.log0 = (float*)carve(logb);
    for (int i = 1; i < nsets * every; ++i) carve(logb);
    a.astride = al(mwords * 8) / 8;
    a.act0 = (unsigned long long*)carve(mwords * 8);
    for (int k = 1; k <= K; ++k) carve(mwords * 8);
    a.lstride = al((uint64_t)nb * 4) / 4;
    a.list0 = (uint32_t*)carve((uint64_t)nb * 4);
    for (int k = 1; k <= K; ++k) carve((uint64_t)nb * 4);
    a.flag0 = (uint32_t*)carve((uint64_t)nb * 4);
    for (int k = 1; k <= K; ++k) carve((uint64_t)nb * 4);
    a.counts = (uint32_t*)carve((uint64_t)(K + 1) * 4);
    for (int q = 0; q < 2; ++q) a.flagT[q] = (uint32_t*)carve((uint64_t)nb * 4);
    a.need = (uint32_t*)carve((uint64_t)nb * 4);
    a.reached = (uint32_t*)carve((uint64_t)nb * 4);
    a.nlist0 = (uint32_t*)carve((uint64_t)nb * 4);  // lstride apart, like the brick lists
    for (int q = 1; q < nck - 1; ++q) carve((uint64_t)nb * 4);
    a.ncount = (uint32_t*)carve((uint64_t)nck * 4);
    uint8_t* const tgt_field = (uint8_t*)carve(P);
    a.gsum = (double*)carve(8 * sizeof(double) + 8);
    a.nact = (unsigned long long*)(a.gsum + 8);
    a.gpart = (double*)carve((uint64_t)gr * 3 * sizeof(double));
    double* dpart = (double*)carve((uint64_t)gf * 3 * sizeof(double));  // the loss's block sums
    a.dbias = dbias ? F() : nullptr;
    a.P = P;
    a.nb = nb;
    a.K = K;
    a.every = every;
    a.nck = nck;
    a.tau = tau;
    // Target, bias and the bias gradient.  Device memory of a volume whose
    // rows need no padding (px = nx, py = ny: the caller's layout is the
    // padded one up to z = nz, the only part any kernel touches) is used in
    // place.  Otherwise the padded copies in the workspace: pinned host or
    // device memory is read (written) in place by the scatter (gather)
    // kernel, pageable memory goes through the copy engine into fw[0] (free
    // until the forward starts and after the reverse ends).  The padding of
    // these fields is never read.
    const uint64_t n = (uint64_t)V.nx * V.ny * V.nz;
    const bool flat = V.px == V.nx && V.py == V.ny;
    auto in_place = [&](const void* p) { return flat && device_memory(p) && (uintptr_t)p % 16 == 0; };
    bool staged = false;  // fw[0] used as a staging buffer before the forward
    auto upload = [&](auto* dst, const auto* host) {
        using T = std::remove_cv_t<std::remove_pointer_t<decltype(host)>>;
        const T* src = (const T*)device_view(host);
        if (!src) {
            T* stage = (T*)(void*)a.fw[0];
            LSS_CUDA(cudaMemcpyAsync(stage, host, n * sizeof(T), cudaMemcpyDefault, st));
            src = stage;
            staged = true;
        }
        k_ns_scatter<<<grid, 256, 0, st>>>(dst, src, V.nx, V.ny, V.nz, V.px, V.py);
        count_launch(owner);
    };
    if (in_place(target)) {
        a.tgt = target;
    } else {
        upload(tgt_field, target);
        a.tgt = tgt_field;
    }
    if (bias) {
        float* bd = F();
        if (in_place(bias)) {
            V.bias = bias;
        } else {
            upload(bd, bias);
            V.bias = bd;
        }
    }
    a.V = V;
    const bool dbias_in_place = dbias && in_place(dbias);
    if (dbias_in_place) a.dbias = dbias;
    // Everything else of the set-up (clears, the pair's copies of phi_0, the
    // masks of A_0) is the forward kernel's first phase.
    a.dbias_n = a.dbias ? (dbias_in_place ? n : P) : 0;
    a.phi0 = V.phi[core.parity()];
    a.act_src = core.masks(core.parity());
    a.mwords = mwords;
    // The pair is copied whole unless the previous call left it holding
    // phi_0 outside its stamped bricks: the engine unchanged since (epoch),
    // the same fields, stamps and phi_0 (key), and fw[0] not used for
    // staging since.  The record is void until this call has completed.
    NsCore::AdjointRecord& rec = core.adjoint_record();
    const void* key[4] = {a.fw[0], a.fw[1], a.reached, a.phi0};
    const bool same = rec.valid && rec.epoch == core.epoch() && !staged &&
                      std::equal(key, key + 4, rec.key) && rec.gen < 0xFFFFFF00u;
    a.partial = same ? 1 : 0;
    a.gen = same ? rec.gen + 1u : 1u;
    rec.valid = false;
    LSS_REQUIRE(gf == gr, LSS_ERR_CUDA, "adjoint grids differ");
    void* params[] = {(void*)&a};
    a.dice = DiceArgs{a.fw[K & 1], a.tgt, a.lam, dpart, a.gsum, V.nx, V.ny, V.nz, V.px, V.py, (uint32_t)gf, tau,
                      a.reached, a.Z[0], a.Z[1], nb, S::X, S::Y, S::Z, V.nbx, V.nby, a.gen};
    LSS_CUDA(cudaLaunchCooperativeKernel(kf, dim3(gf), dim3(kAdjThreads), params, 0, st));
    count_launch(owner);
    LSS_CUDA(cudaLaunchCooperativeKernel(kr, dim3(gr), dim3(kAdjThreads), params, 0, st));
    count_launch(owner);
    // d_bias back to the caller's unpadded layout (written in place when the
    // device can address it).
    bool staged_out = false;  // fw[0] used as a staging buffer after the reverse
    if (dbias && !dbias_in_place) {
        float* dev = (float*)device_view(dbias);
        k_ns_gather<<<grid, 256, 0, st>>>(dev ? dev : a.fw[0], a.dbias, V.nx, V.ny, V.nz, V.px, V.py);
        count_launch(owner);
        if (!dev) LSS_CUDA(cudaMemcpyAsync(dbias, a.fw[0], n * 4, cudaMemcpyDefault, st));
        staged_out = !dev;
    }
    double h[8];
    unsigned long long na = 0;
    std::vector<double> parts((size_t)gr * 3);
    LSS_CUDA(cudaMemcpyAsync(h, a.gsum, sizeof(h), cudaMemcpyDeviceToHost, st));
    LSS_CUDA(cudaMemcpyAsync(&na, a.nact, 8, cudaMemcpyDeviceToHost, st));
    LSS_CUDA(cudaMemcpyAsync(parts.data(), a.gpart, parts.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    owner->sync();
    rec.epoch = core.epoch();
    std::copy(key, key + 4, rec.key);
    rec.gen = a.gen;
    rec.valid = !staged_out;
    // The blocks' parameter sums, added in block order (the same every call).
    double g3[3] = {0.0, 0.0, 0.0};
    for (int b = 0; b < gr; ++b)
        for (int q = 0; q < 3; ++q) g3[q] += parts[(size_t)3 * b + q];
    const double den = h[4] + h[5];
    out->loss = 1.0 - 2.0 * h[6] / den;
    out->d_target = g3[0];
    out->d_window = g3[1];
    out->d_curvature = g3[2];
    out->active_voxel_iterations = na;
}

}  // namespace

void ns_adjoint(NsCore& core, int K, int every, const uint8_t* target, float tau, const float* bias,
                float* dbias, lss_grads* out) {
    LSS_REQUIRE(core.nvol() == 1, LSS_ERR_UNSUPPORTED, "the adjoint runs on a single volume");
    LSS_REQUIRE(core.initialized(), LSS_ERR_STATE, "no seed or phi set");
    LSS_REQUIRE(K > 0 && every > 0 && target && out && tau > 0.0f, LSS_ERR_INVALID_ARGUMENT,
                "bad adjoint arguments");
    every = std::min(every, K);  // one segment holds all K iterations at most
    const BrickConfig& c = core.config();
    if (c.bx == 8 && c.by == 8 && c.bz == 8) return run_adjoint<Brick<8, 8, 8>>(core, K, every, target, tau, bias, dbias, out);
    if (c.bx == 8 && c.by == 8 && c.bz == 4) return run_adjoint<Brick<8, 8, 4>>(core, K, every, target, tau, bias, dbias, out);
    if (c.bx == 4 && c.by == 4 && c.bz == 4) return run_adjoint<Brick<4, 4, 4>>(core, K, every, target, tau, bias, dbias, out);
    throw Error(LSS_ERR_UNSUPPORTED, "unsupported brick shape");
}

}  // namespace lss
