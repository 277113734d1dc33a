// The differentiation form of LSS_MODE_NS (lss_adjoint_run): K unrolled
// iterations of the spec update from the engine's current state, with
// the active set of every iteration recorded in the forward pass and held
// fixed, the soft-Dice loss of sigmoid(-phi/tau) against a target mask, and
// its gradients with respect to T, eps, alpha and a per-voxel speed bias.
//
// Work-efficient like the forward engine: every iteration touches the bricks
// of its active set only.  The forward keeps the brick list of each A_k
// (built while dilating: the first thread to put a word into a brick appends
// it; the block that updates a brick dilates it) beside the recorded brick
// masks.  It runs over a ping-pong pair in
// which both buffers stay current: iteration k writes the bricks of A_k
// whole (active voxels updated, the rest copied) and copies across the
// bricks of A_{k-1} that left the set; the changed voxels' ballot words are
// dilated into A_{k+1} exactly as in the persistent kernel, so the recorded
// sets are the sparse engine's sets.  phi is checkpointed every `every`
// iterations (a device copy); the reverse pass recomputes each segment from
// its checkpoint (a copy of the previous state plus the sparse update:
// bit-identical, the arithmetic is deterministic) and runs the segment's
// iterations backwards on one lambda field, in place:
//   take:  U = lambda_{k+1} at the voxels of A_k, lambda = 0 there (lambda
//          keeps lambda_{k+1} everywhere else: the pass-through);
//   vjp:   every active voxel v scatters U[v] through the transposed stencil
//          Jacobian of the update onto its 19 stencil voxels (fp32 atomics);
// parameter gradients are reduced per block in FP64 (the gradient-check
// reduction) and the bias gradient accumulates per voxel.
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

// Per-iteration brick lists: list[k][0 .. count[k]) = the bricks of A_k in
// no particular order (each brick once), flag[k][b] = b is in it.

// list_0 and flag_0 from the recorded masks of A_0.
template <class S>
__global__ void __launch_bounds__(256) k_adj_list0(const unsigned long long* __restrict__ act, uint32_t* flag,
                                                   uint32_t* list, uint32_t* count, uint32_t nb) {
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        unsigned long long any = 0ull;
#pragma unroll
        for (int w = 0; w < S::WORDS; ++w) any |= act[(size_t)b * S::WORDS + w];
        if (any) {
            flag[b] = 1u;
            list[atomicAdd(count, 1u)] = b;
        }
    }
}

// The changed-voxel ballot words of one brick (chg, CHG words) dilated into
// its 27 neighbours' masks of A_{k+1}; the first thread to put a word into a
// brick appends the brick to list_{k+1}.  Threads t0, t0 + stride, ... take
// the (neighbour, mask word) pairs.
template <class S>
__device__ __forceinline__ void adj_dilate_brick(const NsVol& V, uint32_t b, const uint32_t* chg, int t0, int stride,
                                                 unsigned long long* nxt, uint32_t* flag_next, uint32_t* list_next,
                                                 uint32_t* count_next) {
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
        if (*(volatile uint32_t*)&flag_next[nbi] == 0u && atomicExch(&flag_next[nbi], 1u) == 0u)
            list_next[atomicAdd(count_next, 1u)] = nbi;
    }
}

// Iteration k: block per brick.  The bricks of list_k are written whole into
// out (active voxels updated from in, the others copied); with `prev` (the
// recorded forward's ping-pong pair), the bricks of list_{k-1} not in
// list_k (flag_k clear) are copied from in to out, so that out equals in
// outside the bricks of A_k.  With nxt (the recorded forward, not a
// recomputation): each updated brick's changed voxels are dilated into A_{k+1}
// by the same block (adj_dilate_brick) and the updated voxels are counted
// into *nact.
template <class S>
__global__ void __launch_bounds__(256) k_adj_update(NsVol V, const float* __restrict__ in, float* __restrict__ out,
                                                    const unsigned long long* __restrict__ act,
                                                    const uint32_t* __restrict__ list, const uint32_t* count,
                                                    const uint32_t* __restrict__ prev, const uint32_t* prev_count,
                                                    const uint32_t* __restrict__ flag_k, unsigned long long* nxt,
                                                    uint32_t* flag_next, uint32_t* list_next, uint32_t* count_next,
                                                    unsigned long long* nact) {
    __shared__ uint32_t chg[S::CHG];
    __shared__ uint32_t any;
    const uint32_t n = *count, np = prev ? *prev_count : 0u;
    uint32_t mine = 0;
    for (uint32_t i = blockIdx.x; i < n + np; i += gridDim.x) {
        const bool upd = i < n;
        const uint32_t b = upd ? list[i] : prev[i - n];
        if (!upd && flag_k[b]) continue;  // also in list_k: written above (uniform over the block)
        const bool dil = nxt && upd;      // uniform over the block
        if (dil) {
            __syncthreads();  // chg and any free: the previous brick's dilation is done
            if (threadIdx.x == 0) any = 0u;
            __syncthreads();
        }
        for (int j = threadIdx.x; j < S::VOX; j += blockDim.x) {
            const int3 p = voxel_of<S>(V, b, j);
            bool changed = false;
            if (p.x < V.nx && p.y < V.ny && p.z < V.nz) {
                const size_t idx = ((size_t)p.z * V.py + p.y) * V.px + p.x;
                const float c = in[idx];
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
            if (dil) {
                const uint32_t bal = __ballot_sync(0xffffffffu, changed);
                if ((threadIdx.x & 31) == 0) {
                    chg[j >> 5] = bal;
                    if (bal) any = 1u;
                }
            }
        }
        if (dil) {
            __syncthreads();  // chg and any complete
            if (any) adj_dilate_brick<S>(V, b, chg, threadIdx.x, blockDim.x, nxt, flag_next, list_next, count_next);
        }
    }
    if (nact) {  // uniform: one atomic per block on the shared counter, not one per warp
        __shared__ uint32_t s_cnt;
        if (threadIdx.x == 0) s_cnt = 0u;
        __syncthreads();
        mine = __reduce_add_sync(0xffffffffu, mine);
        if ((threadIdx.x & 31) == 0 && mine) atomicAdd(&s_cnt, mine);
        __syncthreads();
        if (threadIdx.x == 0 && s_cnt) atomicAdd(nact, (unsigned long long)s_cnt);
    }
}

// The bricks of lists k_lo .. k_hi (list k at lists + k * stride, count k at
// counts[k]; bricks may repeat) copied from src to dst, a brick a block.
template <class S>
__global__ void __launch_bounds__(256) k_adj_copy_bricks(NsVol V, const float* __restrict__ src,
                                                         float* __restrict__ dst, const uint32_t* __restrict__ lists,
                                                         uint64_t stride, const uint32_t* __restrict__ counts,
                                                         int k_lo, int k_hi) {
    for (int k = k_lo; k <= k_hi; ++k) {
        const uint32_t n = counts[k];
        const uint32_t* list = lists + (uint64_t)k * stride;
        for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
            const uint32_t b = list[i];
            for (int j = threadIdx.x; j < S::VOX; j += blockDim.x) {
                const int3 p = voxel_of<S>(V, b, j);
                if (p.x < V.nx && p.y < V.ny && p.z < V.nz) {
                    const size_t idx = ((size_t)p.z * V.py + p.y) * V.px + p.x;
                    dst[idx] = src[idx];
                }
            }
        }
    }
}

// Reverse iteration k, first half (block per brick of list_k): U =
// lambda_{k+1} at the voxels of A_k and lambda = 0 there; lambda keeps
// lambda_{k+1} at every other voxel.
template <class S>
__global__ void __launch_bounds__(256) k_adj_take(NsVol V, const unsigned long long* __restrict__ act,
                                                  const uint32_t* __restrict__ list, const uint32_t* count,
                                                  float* __restrict__ lam, float* __restrict__ U) {
    const uint32_t n = *count;
    for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
        const uint32_t b = list[i];
        for (int j = threadIdx.x; j < S::VOX; j += blockDim.x) {
            if (!((act[(size_t)b * S::WORDS + (j >> 6)] >> (j & 63)) & 1ull)) continue;
            const int3 p = voxel_of<S>(V, b, j);
            if (p.x >= V.nx || p.y >= V.ny || p.z >= V.nz) continue;
            const size_t idx = ((size_t)p.z * V.py + p.y) * V.px + p.x;
            U[idx] = lam[idx];
            lam[idx] = 0.0f;
        }
    }
}

// Vector-Jacobian product of ns_update_f32 at one voxel with upstream lam:
// scatters dloss/dphi onto the stencil (add(dx, dy, dz, g)) and returns the
// parameter terms in g4 = (T, eps, alpha, bias).  Same derivation as the FP64
// oracle (oracle/ns_adjoint.hpp), in fp32.
template <class PF, class AF>
__device__ __forceinline__ void ns_update_vjp_f32(PF P, AF add, float I, float bias, const NsVol& V, float lam,
                                                  float* g4) {
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
    add(0, 0, 0, lam);
    const float gcurv = lam * V.dt * V.wc, gF = -lam * V.dt * gn, ggn = -lam * V.dt * F;
    if (has_curv) {
        const float gnum = gcurv / g2, gg2 = -gcurv * curv / g2;
        const float gcx = gnum * (2.0f * cx * (fyy + fzz) - 2.0f * (cy * fxy + cz * fxz)) + gg2 * 2.0f * cx;
        const float gcy = gnum * (2.0f * cy * (fxx + fzz) - 2.0f * (cx * fxy + cz * fyz)) + gg2 * 2.0f * cy;
        const float gcz = gnum * (2.0f * cz * (fxx + fyy) - 2.0f * (cx * fxz + cy * fyz)) + gg2 * 2.0f * cz;
        const float gfxx = gnum * (cy * cy + cz * cz), gfyy = gnum * (cx * cx + cz * cz),
                    gfzz = gnum * (cx * cx + cy * cy);
        const float gfxy = -2.0f * gnum * cx * cy, gfxz = -2.0f * gnum * cx * cz, gfyz = -2.0f * gnum * cy * cz;
        add(1, 0, 0, 0.5f * gcx + gfxx);
        add(-1, 0, 0, -0.5f * gcx + gfxx);
        add(0, 1, 0, 0.5f * gcy + gfyy);
        add(0, -1, 0, -0.5f * gcy + gfyy);
        add(0, 0, 1, 0.5f * gcz + gfzz);
        add(0, 0, -1, -0.5f * gcz + gfzz);
        add(0, 0, 0, -2.0f * (gfxx + gfyy + gfzz));
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
    if (gn > 0.0f) {
        const float s = ggn / gn;
        add(0, 0, 0, s * (a - b + e - f + h - k));
        add(-1, 0, 0, -s * a);
        add(1, 0, 0, s * b);
        add(0, -1, 0, -s * e);
        add(0, 1, 0, s * f);
        add(0, 0, -1, -s * h);
        add(0, 0, 1, s * k);
    }
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

// Block sum of three doubles into gsum[0..2]: one atomic each per block (none
// for a zero sum, which changes nothing), or, with Slot, added into the
// block's own three words (gsum = its slot; no other block writes them, so
// no atomics, and launches of the same grid accumulate in a fixed order).
template <bool Slot = false>
__device__ __forceinline__ void block_sum3(double a0, double a1, double a2, double* gsum) {
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
        if (lane == 0 && Slot) {
            gsum[0] += a0;
            gsum[1] += a1;
            gsum[2] += a2;
        } else if (lane == 0) {
            if (a0 != 0.0) atomicAdd(&gsum[0], a0);
            if (a1 != 0.0) atomicAdd(&gsum[1], a1);
            if (a2 != 0.0) atomicAdd(&gsum[2], a2);
        }
    }
    __syncthreads();
}

// Reverse iteration k, second half (block per brick of list_k): scatters U
// (lambda_{k+1}) of the voxels of A_k through the update's transposed
// Jacobian into lam, adds the bias gradient and the parameter gradients
// (T, eps, alpha; FP64) into the block's slot gpart[3 * blockIdx.x ..].
template <class S>
__global__ void __launch_bounds__(256) k_adj_vjp(NsVol V, const float* __restrict__ phi,
                                                 const unsigned long long* __restrict__ act,
                                                 const uint32_t* __restrict__ list, const uint32_t* count,
                                                 const float* __restrict__ U, float* lam, float* dbias,
                                                 double* gpart) {
    const uint32_t n = *count;
    double sT = 0.0, sE = 0.0, sA = 0.0;
    for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
        const uint32_t b = list[i];
        for (int j = threadIdx.x; j < S::VOX; j += blockDim.x) {
            if (!((act[(size_t)b * S::WORDS + (j >> 6)] >> (j & 63)) & 1ull)) continue;
            const int3 p = voxel_of<S>(V, b, j);
            if (p.x >= V.nx || p.y >= V.ny || p.z >= V.nz) continue;
            const size_t idx = ((size_t)p.z * V.py + p.y) * V.px + p.x;
            const float u = U[idx];
            if (u == 0.0f) continue;
            auto at = [&](int dx, int dy, int dz) {
                return ((size_t)clampi(p.z + dz, V.nz) * V.py + clampi(p.y + dy, V.ny)) * V.px +
                       clampi(p.x + dx, V.nx);
            };
            auto P = [&](int dx, int dy, int dz) { return phi[at(dx, dy, dz)]; };
            auto add = [&](int dx, int dy, int dz, float g) {
                if (g != 0.0f) atomicAdd(&lam[at(dx, dy, dz)], g);
            };
            float g4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            ns_update_vjp_f32(P, add, V.img[idx], V.bias ? V.bias[idx] : 0.0f, V, u, g4);
            sT += g4[0];
            sE += g4[1];
            sA += g4[2];
            if (dbias) dbias[idx] += g4[3];
        }
    }
    block_sum3<true>(sT, sE, sA, gpart + 3 * (size_t)blockIdx.x);  // every thread of the block reaches it
}

// Soft-Dice sums over the volume: gsum[0..2] = (sum s, sum t, sum s t).
// Per voxel in fp32 (a thread sums a few tens of voxels); the block and grid
// reduction in FP64.
__global__ void __launch_bounds__(256) k_adj_dice_sums(NsVol V, const float* __restrict__ phi,
                                                       const uint8_t* __restrict__ target, float tau,
                                                       double* gsum) {
    const uint32_t rows = (uint32_t)V.ny * (uint32_t)V.nz;
    float ss = 0.0f, tt = 0.0f, st = 0.0f;
    // Block per row (y, z), threads over x (every thread reaches block_sum3).
    for (uint32_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const uint32_t z = r / (uint32_t)V.ny, y = r - z * (uint32_t)V.ny;
        const size_t row = ((size_t)z * V.py + y) * V.px;
        for (int x = threadIdx.x; x < V.nx; x += blockDim.x) {
            const float s = 1.0f / (1.0f + expf(phi[row + x] / tau));
            const float tv = target[row + x] ? 1.0f : 0.0f;
            ss += s;
            tt += tv;
            st += s * tv;
        }
    }
    block_sum3(ss, tt, st, gsum);
}

// lambda_K = dloss/dphi_K of the soft-Dice loss, per voxel in fp32 from the
// FP64 sums: dloss/ds = (2 st - 2 t den) / den^2.
__global__ void __launch_bounds__(256) k_adj_dice_grad(NsVol V, const float* __restrict__ phi,
                                                       const uint8_t* __restrict__ target, float tau,
                                                       const double* __restrict__ sums, float* lam) {
    const double den = sums[0] + sums[1], st = sums[2];
    const float c_out = (float)(2.0 * st / (den * den)), c_in = (float)(2.0 * st / (den * den) - 2.0 / den);
    const uint32_t rows = (uint32_t)V.ny * (uint32_t)V.nz;
    for (uint32_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const uint32_t z = r / (uint32_t)V.ny, y = r - z * (uint32_t)V.ny;
        const size_t row = ((size_t)z * V.py + y) * V.px;
        for (int x = threadIdx.x; x < V.nx; x += blockDim.x) {
            const float s = 1.0f / (1.0f + expf(phi[row + x] / tau));
            const float dl_ds = target[row + x] ? c_in : c_out;
            lam[row + x] = dl_ds * (-s * (1.0f - s) / tau);
        }
    }
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
    const int grid = owner->num_sms * 8;        // element-wise kernels
    const int bgrid = owner->num_sms * 4;       // block-per-brick kernels
    // One device workspace (kept by the engine between calls), carved into
    // 256-byte aligned parts.
    auto al = [](uint64_t b) { return (b + 255) / 256 * 256; };
    const uint64_t nfields = (uint64_t)nck + (every - 1) + 4 + (dbias ? 1 : 0) + (bias ? 1 : 0);
    const uint64_t total = nfields * al(P * 4) + (uint64_t)(K + 1) * al(mwords * 8) +
                           2 * (uint64_t)(K + 1) * al((uint64_t)nb * 4) + al((uint64_t)(K + 1) * 4) + al(P) + 256 +
                           al((uint64_t)bgrid * 3 * sizeof(double));
    char* base = (char*)core.workspace(total);
    auto carve = [&](uint64_t bytes) {
        char* p = base;
        base += al(bytes);
        return p;
    };
    auto F = [&]() { return (float*)carve(P * 4); };
    std::vector<float*> ck(nck), seg(every);
    for (auto& p : ck) p = F();
    for (int i = 1; i < every; ++i) seg[i] = F();
    float* fw[2] = {F(), F()};  // the forward's ping-pong pair
    float* lam = F();
    float* U = F();
    std::vector<unsigned long long*> act(K + 1);
    for (auto& a : act) a = (unsigned long long*)carve(mwords * 8);
    std::vector<uint32_t*> list(K + 1), flag(K + 1);
    for (auto& l : list) l = (uint32_t*)carve((uint64_t)nb * 4);
    for (auto& f : flag) f = (uint32_t*)carve((uint64_t)nb * 4);
    uint32_t* counts = (uint32_t*)carve((uint64_t)(K + 1) * 4);
    uint8_t* tgt = (uint8_t*)carve(P);
    double* gsum = (double*)carve(8 * sizeof(double) + 8);
    unsigned long long* nact = (unsigned long long*)(gsum + 8);
    double* gpart = (double*)carve((uint64_t)bgrid * 3 * sizeof(double));  // per-block dT, deps, dalpha
    float* dbias_d = dbias ? F() : nullptr;
    auto count_k = [&](int k) { return counts + k; };
    // Target and bias into the padded layout on the device (pinned host
    // buffers are read in place, pageable ones through the copy engine into
    // fw[0], which is free until the forward starts).
    const uint64_t n = (uint64_t)V.nx * V.ny * V.nz;
    auto upload = [&](auto* dst, const auto* host) {
        using T = std::remove_cv_t<std::remove_pointer_t<decltype(host)>>;
        const T* src = (const T*)pinned_device_ptr(host);
        if (!src) {
            T* stage = (T*)(void*)fw[0];
            LSS_CUDA(cudaMemcpyAsync(stage, host, n * sizeof(T), cudaMemcpyHostToDevice, st));
            src = stage;
        }
        k_ns_scatter<<<grid, 256, 0, st>>>(dst, src, V.nx, V.ny, V.nz, V.px, V.py);
        count_launch(owner);
    };
    LSS_CUDA(cudaMemsetAsync(tgt, 0, P, st));
    upload(tgt, target);
    if (bias) {
        float* bd = F();
        LSS_CUDA(cudaMemsetAsync(bd, 0, P * 4, st));
        upload(bd, bias);
        V.bias = bd;
    }
    if (dbias_d) LSS_CUDA(cudaMemsetAsync(dbias_d, 0, P * 4, st));
    LSS_CUDA(cudaMemsetAsync(gsum, 0, 8 * sizeof(double) + 8, st));
    LSS_CUDA(cudaMemsetAsync(gpart, 0, (uint64_t)bgrid * 3 * sizeof(double), st));
    LSS_CUDA(cudaMemsetAsync(act[1], 0, (uint64_t)K * al(mwords * 8), st));  // act[1..K] are contiguous
    LSS_CUDA(cudaMemsetAsync(flag[0], 0, (uint64_t)(K + 1) * al((uint64_t)nb * 4), st));
    LSS_CUDA(cudaMemsetAsync(counts, 0, (uint64_t)(K + 1) * 4, st));
    auto count = [&]() { count_launch(owner); };
    // Forward from the engine's current phi and active set: both buffers of
    // the pair and the first checkpoint hold phi_0.
    const float* phi0 = V.phi[core.parity()];
    for (float* d : {ck[0], fw[0], fw[1]})
        LSS_CUDA(cudaMemcpyAsync(d, phi0, P * 4, cudaMemcpyDeviceToDevice, st));
    LSS_CUDA(cudaMemcpyAsync(act[0], core.masks(core.parity()), mwords * 8, cudaMemcpyDeviceToDevice, st));
    k_adj_list0<S><<<(nb + 255) / 256, 256, 0, st>>>(act[0], flag[0], list[0], count_k(0), nb);
    count();
    for (int k = 0; k < K; ++k) {
        const float* src = fw[k & 1];
        float* dst = fw[(k + 1) & 1];
        k_adj_update<S><<<bgrid, 256, 0, st>>>(V, src, dst, act[k], list[k], count_k(k),
                                               k ? list[k - 1] : nullptr, k ? count_k(k - 1) : nullptr, flag[k],
                                               act[k + 1], flag[k + 1], list[k + 1], count_k(k + 1), nact);
        count();
        if ((k + 1) % every == 0 && k + 1 < K)
            LSS_CUDA(cudaMemcpyAsync(ck[(k + 1) / every], dst, P * 4, cudaMemcpyDeviceToDevice, st));
    }
    const float* phiK = fw[K & 1];
    // Loss and lambda_K.
    k_adj_dice_sums<<<grid, 256, 0, st>>>(V, phiK, tgt, tau, gsum + 4);
    count();
    k_adj_dice_grad<<<grid, 256, 0, st>>>(V, phiK, tgt, tau, gsum + 4, lam);
    count();
    // Reverse, segment by segment from the last checkpoint.  seg[i] holds
    // phi_{held[i]} (-1: nothing of this call): to turn it into phi_{k+1}
    // only the bricks of lists k+1 .. held[i]-1 can differ from phi_k (the
    // bricks of list_k are rewritten whole by the update), so only those are
    // copied from seg[i-1] = phi_k; the first use copies the whole field.
    const uint64_t lstride = al((uint64_t)nb * 4) / 4;
    std::vector<int> held(every, -1);
    for (int sgi = nck - 1; sgi >= 0; --sgi) {
        const int s0 = sgi * every, s1 = std::min(K, s0 + every);
        seg[0] = ck[sgi];
        for (int k = s0; k + 1 < s1; ++k) {
            const int i = k - s0 + 1;
            float* d = seg[i];
            if (held[i] < 0) {
                LSS_CUDA(cudaMemcpyAsync(d, seg[i - 1], P * 4, cudaMemcpyDeviceToDevice, st));
            } else if (held[i] - 1 >= k + 1) {
                k_adj_copy_bricks<S><<<bgrid, 256, 0, st>>>(V, seg[i - 1], d, list[0], lstride, counts, k + 1,
                                                            held[i] - 1);
                count();
            }
            k_adj_update<S><<<bgrid, 256, 0, st>>>(V, seg[i - 1], d, act[k], list[k], count_k(k), nullptr,
                                                   nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
            count();
            held[i] = k + 1;
        }
        for (int k = s1 - 1; k >= s0; --k) {
            k_adj_take<S><<<bgrid, 256, 0, st>>>(V, act[k], list[k], count_k(k), lam, U);
            count();
            k_adj_vjp<S><<<bgrid, 256, 0, st>>>(V, seg[k - s0], act[k], list[k], count_k(k), U, lam, dbias_d, gpart);
            count();
        }
    }
    // d_bias back to the caller's unpadded layout (in place when pinned).
    if (dbias) {
        float* dev = (float*)pinned_device_ptr(dbias);
        k_ns_gather<<<grid, 256, 0, st>>>(dev ? dev : fw[0], dbias_d, V.nx, V.ny, V.nz, V.px, V.py);
        count();
        if (!dev) LSS_CUDA(cudaMemcpyAsync(dbias, fw[0], n * 4, cudaMemcpyDeviceToHost, st));
    }
    double h[8];
    unsigned long long na = 0;
    std::vector<double> parts((size_t)bgrid * 3);
    LSS_CUDA(cudaMemcpyAsync(h, gsum, sizeof(h), cudaMemcpyDeviceToHost, st));
    LSS_CUDA(cudaMemcpyAsync(&na, nact, 8, cudaMemcpyDeviceToHost, st));
    LSS_CUDA(cudaMemcpyAsync(parts.data(), gpart, parts.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    owner->sync();
    // The blocks' parameter sums, added in block order (the same every call).
    double g3[3] = {0.0, 0.0, 0.0};
    for (int b = 0; b < bgrid; ++b)
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
