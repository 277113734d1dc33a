// The differentiation form of LSS_MODE_NS (lss_adjoint_run): K unrolled
// iterations of the spec update from the engine's current state, with
// the active set of every iteration recorded in the forward pass and held
// fixed, the soft-Dice loss of sigmoid(-phi/tau) against a target mask, and
// its gradients with respect to T, eps, alpha and a per-voxel speed bias.
//
// Forward: iteration k updates the voxels of A_k (brick masks, the layout of
// the sparse engine) and writes every other voxel through; the changed
// voxels' ballot words are dilated into A_{k+1} exactly as in the persistent
// kernel, so the recorded sets are the sparse engine's sets.  phi is
// checkpointed every `every` iterations; the reverse pass recomputes each
// segment from its checkpoint (bit-identical: the update arithmetic is
// deterministic) and runs the segment's iterations backwards:
//   lambda_k = lambda_{k+1} on inactive voxels (pass-through), and for every
//   active voxel v the transposed stencil Jacobian of the update scatters
//   lambda_{k+1}[v] onto its 19 stencil voxels (fp32 atomics);
// parameter gradients are reduced per block in FP64 (the gradient-check
// reduction) and the bias gradient accumulates per voxel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "ns_core.hpp"
#include "ns_kernels.cuh"

namespace lss {
namespace {

__device__ __forceinline__ int clampi(int v, int n) { return v < 0 ? 0 : (v >= n ? n - 1 : v); }

// Voxel j of local brick b of a one-volume descriptor.
template <class S>
__device__ __forceinline__ int3 voxel_of(const NsVol& V, uint32_t b, int j) {
    const int3 o = brick_origin<S>(V, b + V.brick_base);
    return make_int3(o.x + j % S::X, o.y + (j / S::X) % S::Y, o.z + j / (S::X * S::Y));
}

// Forward iteration: phi_out = update of phi_in on A_k (act), pass-through
// elsewhere; changed voxels -> ballot words chg[brick * CHG + j / 32] (when
// chg is not null).  One thread per voxel slot in brick-major order.
template <class S>
__global__ void __launch_bounds__(256) k_adj_update(NsVol V, const float* __restrict__ in, float* __restrict__ out,
                                                    const unsigned long long* __restrict__ act,
                                                    uint32_t* __restrict__ chg, uint32_t nb) {
    const uint64_t total = (uint64_t)nb * S::VOX;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = (uint32_t)(t / S::VOX);
        const int j = (int)(t % S::VOX);
        const int3 p = voxel_of<S>(V, b, j);
        bool changed = false;
        if (p.x < V.nx && p.y < V.ny && p.z < V.nz) {
            const size_t idx = ((size_t)p.z * V.py + p.y) * V.px + p.x;
            const float c = in[idx];
            if ((act[(size_t)b * S::WORDS + (j >> 6)] >> (j & 63)) & 1ull) {
                auto P = [&](int dx, int dy, int dz) {
                    return in[((size_t)clampi(p.z + dz, V.nz) * V.py + clampi(p.y + dy, V.ny)) * V.px +
                              clampi(p.x + dx, V.nx)];
                };
                const float nv = ns_update_f32(P, V.img[idx], V.bias ? V.bias[idx] : 0.0f, V);
                changed = fabsf(nv - c) > V.thr_t;
                out[idx] = nv;
            } else {
                out[idx] = c;
            }
        }
        if (chg) {
            const uint32_t bal = __ballot_sync(0xffffffffu, changed);
            if ((threadIdx.x & 31) == 0) chg[t >> 5] = bal;
        }
    }
}

// A_{k+1}: the changed words of every brick dilated into its 27 neighbours
// (one thread per neighbour mask word).
template <class S>
__global__ void __launch_bounds__(256) k_adj_dilate(NsVol V, const uint32_t* __restrict__ chg,
                                                    unsigned long long* __restrict__ nxt, uint32_t nb) {
    constexpr int PER = 27 * S::WORDS;
    const uint64_t total = (uint64_t)nb * PER;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = (uint32_t)(t / PER);
        const int r = (int)(t % PER), slot = r / S::WORDS, w = r % S::WORDS;
        const uint32_t* cb = chg + (size_t)b * S::CHG;
        uint32_t any = 0;
#pragma unroll
        for (int q = 0; q < S::CHG; ++q) any |= cb[q];
        if (!any) continue;
        const int3 o = brick_origin<S>(V, b + V.brick_base);
        const int ox = slot % 3 - 1, oy = (slot / 3) % 3 - 1, oz = slot / 9 - 1;
        const int bx = o.x / S::X + ox, by = o.y / S::Y + oy, bz = o.z / S::Z + oz;
        const int lx = V.nx - bx * S::X, ly = V.ny - by * S::Y, lz = V.nz - bz * S::Z;
        if (bx < 0 || by < 0 || bz < 0 || lx <= 0 || ly <= 0 || lz <= 0) continue;
        uint64_t x = dilate_word<S>(cb, ox, oy, oz, w, V.nbh);
        if (lx < S::X || ly < S::Y || lz < S::Z)
            x &= inside_mask<S>(w, min(lx, S::X), min(ly, S::Y), min(lz, S::Z));
        const uint32_t nbi = b + (int32_t)((oz * V.nby + oy) * V.nbx + ox);
        if (x) atomicOr(&nxt[(size_t)nbi * S::WORDS + w], (unsigned long long)x);
    }
}

// lambda_k = lambda_{k+1} on the voxels outside A_k, 0 on A_k (their
// contributions are scattered by k_adj_vjp).
template <class S>
__global__ void __launch_bounds__(256) k_adj_lambda_init(NsVol V, const unsigned long long* __restrict__ act,
                                                         const float* __restrict__ nxt, float* __restrict__ lam,
                                                         uint32_t nb) {
    const uint64_t total = (uint64_t)nb * S::VOX;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = (uint32_t)(t / S::VOX);
        const int j = (int)(t % S::VOX);
        const int3 p = voxel_of<S>(V, b, j);
        if (p.x >= V.nx || p.y >= V.ny || p.z >= V.nz) continue;
        const size_t idx = ((size_t)p.z * V.py + p.y) * V.px + p.x;
        const bool a = (act[(size_t)b * S::WORDS + (j >> 6)] >> (j & 63)) & 1ull;
        lam[idx] = a ? 0.0f : nxt[idx];
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
    const float Draw = (V.eps - fabsf(I - V.T)) / V.eps;
    const bool dclamp = Draw < -1.0f || Draw > 1.0f;
    const float Dt = fminf(fmaxf(Draw, -1.0f), 1.0f) + bias;
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
        g4[0] += gDt * sg / V.eps;
        g4[1] += gDt * fabsf(I - V.T) / (V.eps * V.eps);
    }
    const float du_dalpha = V.dt * (-curv - Dt * gn);
    g4[2] += lam * (V.alpha_data ? du_dalpha : -du_dalpha);
}

// Block sum of three doubles into gsum[0..2] (one atomic each per block).
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
        if (lane == 0) {
            atomicAdd(&gsum[0], a0);
            atomicAdd(&gsum[1], a1);
            atomicAdd(&gsum[2], a2);
        }
    }
    __syncthreads();
}

// Reverse iteration k: scatters lambda_{k+1} of the voxels of A_k through the
// update's transposed Jacobian into lam, adds the bias gradient and the
// parameter gradients (gsum[0..2] = T, eps, alpha; FP64).
template <class S>
__global__ void __launch_bounds__(256) k_adj_vjp(NsVol V, const float* __restrict__ phi,
                                                 const unsigned long long* __restrict__ act,
                                                 const float* __restrict__ nxt, float* lam, float* dbias,
                                                 double* gsum, uint32_t nb) {
    const uint64_t total = (uint64_t)nb * S::VOX;
    double sT = 0.0, sE = 0.0, sA = 0.0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    // Every thread runs the same number of loop trips (block_sum3 below).
    for (uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x; t0 < total; t0 += stride) {
        const uint64_t t = t0 + threadIdx.x;
        if (t >= total) continue;
        const uint32_t b = (uint32_t)(t / S::VOX);
        const int j = (int)(t % S::VOX);
        if (!((act[(size_t)b * S::WORDS + (j >> 6)] >> (j & 63)) & 1ull)) continue;
        const int3 p = voxel_of<S>(V, b, j);
        if (p.x >= V.nx || p.y >= V.ny || p.z >= V.nz) continue;
        const size_t idx = ((size_t)p.z * V.py + p.y) * V.px + p.x;
        const float u = nxt[idx];
        if (u == 0.0f) continue;
        auto at = [&](int dx, int dy, int dz) {
            return ((size_t)clampi(p.z + dz, V.nz) * V.py + clampi(p.y + dy, V.ny)) * V.px + clampi(p.x + dx, V.nx);
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
    block_sum3(sT, sE, sA, gsum);
}

// Soft-Dice sums over the volume: gsum[0..2] = (sum s, sum t, sum s t), FP64.
__global__ void __launch_bounds__(256) k_adj_dice_sums(NsVol V, const float* __restrict__ phi,
                                                       const uint8_t* __restrict__ target, float tau,
                                                       double* gsum) {
    const uint64_t total = (uint64_t)V.nx * V.ny * V.nz;
    double ss = 0.0, tt = 0.0, st = 0.0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x; t0 < total; t0 += stride) {
        const uint64_t t = t0 + threadIdx.x;
        if (t >= total) continue;
        const int x = (int)(t % V.nx), y = (int)((t / V.nx) % V.ny), z = (int)(t / ((uint64_t)V.nx * V.ny));
        const size_t idx = ((size_t)z * V.py + y) * V.px + x;
        const double s = 1.0 / (1.0 + (double)expf(phi[idx] / tau));
        const double tv = target[idx] ? 1.0 : 0.0;
        ss += s;
        tt += tv;
        st += s * tv;
    }
    block_sum3(ss, tt, st, gsum);
}

// lambda_K = dloss/dphi_K of the soft-Dice loss.
__global__ void __launch_bounds__(256) k_adj_dice_grad(NsVol V, const float* __restrict__ phi,
                                                       const uint8_t* __restrict__ target, float tau,
                                                       const double* __restrict__ sums, float* lam) {
    const uint64_t total = (uint64_t)V.nx * V.ny * V.nz;
    const double den = sums[0] + sums[1], st = sums[2];
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const int x = (int)(t % V.nx), y = (int)((t / V.nx) % V.ny), z = (int)(t / ((uint64_t)V.nx * V.ny));
        const size_t idx = ((size_t)z * V.py + y) * V.px + x;
        const float s = 1.0f / (1.0f + expf(phi[idx] / tau));
        const double dl_ds = -2.0 * ((target[idx] ? 1.0 : 0.0) * den - st) / (den * den);
        lam[idx] = (float)(dl_ds * (double)(-s * (1.0f - s) / tau));
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
    DeviceArena mem(core.budget_left());
    auto F = [&]() { return (float*)mem.alloc(P * 4); };
    std::vector<float*> ck(nck), seg(every);
    for (auto& p : ck) p = F();
    for (int i = 1; i < every; ++i) seg[i] = F();
    float* fw[2] = {F(), F()};
    float* lam[2] = {F(), F()};
    std::vector<unsigned long long*> act(K + 1);
    for (auto& a : act) a = (unsigned long long*)mem.alloc(mwords * 8);
    uint32_t* chg = (uint32_t*)mem.alloc((size_t)nb * S::CHG * 4);
    uint8_t* tgt = (uint8_t*)mem.alloc(P);
    double* gsum = (double*)mem.alloc(8 * sizeof(double));
    float* dbias_d = dbias ? F() : nullptr;
    // Target and bias, padded on the host.
    {
        std::vector<uint8_t> t(P, 0);
        std::vector<float> bb(bias ? P : 0, 0.0f);
        for (int z = 0; z < V.nz; ++z)
            for (int y = 0; y < V.ny; ++y)
                for (int x = 0; x < V.nx; ++x) {
                    const size_t i = ((size_t)z * V.ny + y) * V.nx + x, o = ((size_t)z * V.py + y) * V.px + x;
                    t[o] = target[i] ? 1 : 0;
                    if (bias) bb[o] = bias[i];
                }
        LSS_CUDA(cudaMemcpyAsync(tgt, t.data(), P, cudaMemcpyHostToDevice, st));
        if (bias) {
            float* bd = F();
            LSS_CUDA(cudaMemcpyAsync(bd, bb.data(), P * 4, cudaMemcpyHostToDevice, st));
            V.bias = bd;
        }
        owner->sync();  // host staging buffers go out of scope
    }
    for (float* p : {fw[0], fw[1], lam[0], lam[1]}) LSS_CUDA(cudaMemsetAsync(p, 0, P * 4, st));
    if (dbias_d) LSS_CUDA(cudaMemsetAsync(dbias_d, 0, P * 4, st));
    LSS_CUDA(cudaMemsetAsync(gsum, 0, 8 * sizeof(double), st));
    const int grid = owner->num_sms * 8;
    auto count = [&]() { ++owner->launches; LSS_CUDA(cudaGetLastError()); };
    // Forward from the engine's current phi and active set.
    LSS_CUDA(cudaMemcpyAsync(ck[0], V.phi[core.parity()], P * 4, cudaMemcpyDeviceToDevice, st));
    LSS_CUDA(cudaMemcpyAsync(act[0], core.masks(core.parity()), mwords * 8, cudaMemcpyDeviceToDevice, st));
    const float* cur = ck[0];
    for (int k = 0; k < K; ++k) {
        float* dst = ((k + 1) % every == 0 && k + 1 < K) ? ck[(k + 1) / every] : fw[k & 1];
        LSS_CUDA(cudaMemsetAsync(act[k + 1], 0, mwords * 8, st));
        k_adj_update<S><<<grid, 256, 0, st>>>(V, cur, dst, act[k], chg, nb);
        count();
        k_adj_dilate<S><<<grid, 256, 0, st>>>(V, chg, act[k + 1], nb);
        count();
        cur = dst;
    }
    // Loss and lambda_K.
    k_adj_dice_sums<<<grid, 256, 0, st>>>(V, cur, tgt, tau, gsum + 4);
    count();
    k_adj_dice_grad<<<grid, 256, 0, st>>>(V, cur, tgt, tau, gsum + 4, lam[K & 1]);
    count();
    // Reverse, segment by segment from the last checkpoint.
    for (int sgi = nck - 1; sgi >= 0; --sgi) {
        const int s0 = sgi * every, s1 = std::min(K, s0 + every);
        seg[0] = ck[sgi];
        for (int k = s0; k + 1 < s1; ++k) {
            k_adj_update<S><<<grid, 256, 0, st>>>(V, seg[k - s0], seg[k - s0 + 1], act[k], nullptr, nb);
            count();
        }
        for (int k = s1 - 1; k >= s0; --k) {
            float* nxt = lam[(k + 1) & 1];
            float* l = lam[k & 1];
            k_adj_lambda_init<S><<<grid, 256, 0, st>>>(V, act[k], nxt, l, nb);
            count();
            k_adj_vjp<S><<<grid, 256, 0, st>>>(V, seg[k - s0], act[k], nxt, l, dbias_d, gsum, nb);
            count();
        }
    }
    double h[8];
    LSS_CUDA(cudaMemcpyAsync(h, gsum, sizeof(h), cudaMemcpyDeviceToHost, st));
    std::vector<float> db;
    if (dbias) {
        db.resize(P);
        LSS_CUDA(cudaMemcpyAsync(db.data(), dbias_d, P * 4, cudaMemcpyDeviceToHost, st));
    }
    owner->sync();
    const double den = h[4] + h[5];
    out->loss = 1.0 - 2.0 * h[6] / den;
    out->d_target = h[0];
    out->d_window = h[1];
    out->d_curvature = h[2];
    if (dbias)
        for (int z = 0; z < V.nz; ++z)
            for (int y = 0; y < V.ny; ++y)
                for (int x = 0; x < V.nx; ++x)
                    dbias[((size_t)z * V.ny + y) * V.nx + x] = db[((size_t)z * V.py + y) * V.px + x];
}

}  // namespace

void ns_adjoint(NsCore& core, int K, int every, const uint8_t* target, float tau, const float* bias,
                float* dbias, lss_grads* out) {
    LSS_REQUIRE(core.nvol() == 1, LSS_ERR_UNSUPPORTED, "the adjoint runs on a single volume");
    LSS_REQUIRE(core.initialized(), LSS_ERR_STATE, "no seed or phi set");
    LSS_REQUIRE(K > 0 && every > 0 && target && out && tau > 0.0f, LSS_ERR_INVALID_ARGUMENT,
                "bad adjoint arguments");
    const BrickConfig& c = core.config();
    if (c.bx == 8 && c.by == 8 && c.bz == 8) return run_adjoint<Brick<8, 8, 8>>(core, K, every, target, tau, bias, dbias, out);
    if (c.bx == 8 && c.by == 8 && c.bz == 4) return run_adjoint<Brick<8, 8, 4>>(core, K, every, target, tau, bias, dbias, out);
    if (c.bx == 4 && c.by == 4 && c.bz == 4) return run_adjoint<Brick<4, 4, 4>>(core, K, every, target, tau, bias, dbias, out);
    throw Error(LSS_ERR_UNSUPPORTED, "unsupported brick shape");
}

}  // namespace lss
