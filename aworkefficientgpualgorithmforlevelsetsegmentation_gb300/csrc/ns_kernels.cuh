// LSS_MODE_NS device code: the persistent bricked iteration kernel and its
// helpers.  One launch runs many iterations (and, in the batched form, many
// volumes) with two bounded grid barriers per iteration:
//
//   phase 1  every active brick of A_k: TMA-load the brick's phi with a
//            one-voxel halo (and its intensities) into shared memory, update
//            the active voxels (upwind |grad phi|, mean curvature, speed
//            D = eps - |I - T|), TMA-store the brick into the other phi
//            buffer, flag changed voxels with warp ballots, dilate the changed
//            bitmask by the 26- (or 6-) neighbourhood and OR it into the next
//            masks of the brick and its 26 neighbours; every brick of F_k
//            (active at k-1, not at k) copies phi across so that both buffers
//            stay current.
//   barrier
//   phase 2  single-pass decoupled-lookback compaction of the brick bitmaps
//            into the sorted lists A_{k+1} (non-empty next mask) and F_{k+1}
//            (in A_k, not in A_{k+1}); active voxels of A_{k+1} are counted per
//            volume (popc of the masks).
//   barrier  then every block evaluates the stopping rule on the same counts.
//
// The reference keeps one dense list of voxel coordinates and rebuilds it
// with seven offset buffers, a tag-volume filter and CUDPP compaction per
// iteration (UpdateActiveElementsVolume.cu:110-363, FilterDuplicates.cu,
// Cuda.cpp:699-758), with a host round trip for the count; here the active
// set is a per-brick voxel bitmask plus a sorted brick list, so duplicates
// cannot arise and the count never leaves the device.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"
#include "tma.cuh"

namespace lss {

struct NsVol {
    int32_t nx, ny, nz;     // logical dims
    int32_t px, py, pz;     // padded dims (multiples of the brick dims)
    int32_t nbx, nby, nbz;  // bricks per axis
    uint32_t brick_base;    // global index of the volume's first brick
    float* phi[2];          // ping-pong fields, padded, x fastest
    const float* img;       // intensities, padded
    const float* bias;      // per-voxel speed bias (padded) or null
    float T, eps, alpha, dt, lo, hi, thr_t, thr_s;
    int32_t alpha_data;     // 1: alpha weights the data term, 0: the curvature term
    int32_t nbh;            // 26 or 6
    uint32_t tmap_base;     // 5 maps: phi0 halo-load, phi1 halo-load, phi0 store, phi1 store, img
    int32_t pad;
};

struct NsVolState {
    unsigned long long n0;          // active voxels after seeding
    unsigned long long n_cur;       // active voxels of the current list
    unsigned long long updates;     // voxel updates so far
    unsigned long long bricks;      // brick updates so far
    unsigned long long iterations;  // iterations so far
    int32_t streak, done, parity, pad;
};

struct NsCtl {
    uint32_t nA, nF;          // lengths of A_k and F_k
    uint32_t err;
    uint32_t bar_count, bar_gen;
    uint32_t scan_tile;       // dynamic tile counter of the phase-2 compaction
    uint32_t iters_run;       // iterations run by the last launch
    uint32_t all_done;
};

struct NsArgs {
    const NsVol* vols;
    NsVolState* vstate;
    int32_t nvol;
    const CUtensorMap* tmaps;
    unsigned long long* masks[2];  // [NB][WORDS]
    uint32_t* bits[2];             // [NW]
    const uint16_t* brick_vol;     // [NB]
    uint32_t* A_list;
    uint32_t* F_list;
    unsigned long long* cnt[2];    // [nvol]
    uint64_t* status;              // decoupled-lookback status words
    NsCtl* ctl;
    uint32_t NB, NW;
    uint32_t parity0;              // phi parity of the launch's first iteration
    int32_t max_iters;
    int32_t conv_mode;             // 0: exactly max_iters, 1: stopping rule
    double rel;
    int32_t patience;
    unsigned long long abs_thr;
};

template <int BX, int BY, int BZ>
struct Brick {
    static constexpr int X = BX, Y = BY, Z = BZ;
    static constexpr int VOX = BX * BY * BZ;
    static constexpr int WORDS = (VOX + 63) / 64;
    static constexpr int CHG = VOX / 32;
    static constexpr int TX = BX + 8, TY = BY + 2, TZ = BZ + 2;  // halo tile
    static constexpr int TILE = TX * TY * TZ;
    static constexpr int EXT = (BX + 2) * (BY + 2) * (BZ + 2);
    static_assert(VOX % 64 == 0, "brick must hold a multiple of 64 voxels");
    static_assert(BX == 4 || BX == 8, "brick x must be 4 or 8");
};

// Bounded sense-reversing grid barrier (all blocks co-resident: cooperative
// launch).  Returns false if this block gave up waiting.
__device__ __forceinline__ bool grid_barrier(NsCtl* ctl, uint32_t& gen, uint32_t nblocks) {
    __shared__ uint32_t s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        s_ok = 1;
        const uint32_t target = gen + 1;
        __threadfence();
        const uint32_t arrived = atomicAdd(&ctl->bar_count, 1u) + 1u;
        if (arrived == nblocks) {
            ctl->bar_count = 0;
            __threadfence();
            asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(&ctl->bar_gen), "r"(target) : "memory");
        } else {
            uint64_t t0 = globaltimer_ns();
            while (ld_acquire_u32(&ctl->bar_gen) != target) {
                if (globaltimer_ns() - t0 > kWaitLimitNs) {
                    set_error(&ctl->err, ERR_BARRIER_TIMEOUT);
                    s_ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        gen = target;
        __threadfence();
    }
    __syncthreads();
    return s_ok != 0;
}

// The spec update of one voxel from the shared-memory halo tile.
// P(dx,dy,dz) reads the tile around the voxel.  Mirrors ns_update() of the
// FP64 oracle in fp32.
template <class PF>
__device__ __forceinline__ float ns_update_f32(PF P, float I, float bias, const NsVol& V) {
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
    float curv = 0.0f;
    if (g2 > 1e-12f) {
        const float num = fxx * (cy * cy + cz * cz) + fyy * (cx * cx + cz * cz) +
                          fzz * (cx * cx + cy * cy) -
                          2.0f * (cx * cy * fxy + cx * cz * fxz + cy * cz * fyz);
        curv = num / g2;
    }
    float D = (V.eps - fabsf(I - V.T)) / V.eps;
    D = fminf(fmaxf(D, -1.0f), 1.0f) + bias;
    const float wc = V.alpha_data ? 1.0f - V.alpha : V.alpha;
    const float wd = 1.0f - wc;
    const float F = wd * D;
    const float dxm = c - xm, dxp = xp - c, dym = c - ym, dyp = yp - c, dzm = c - zm, dzp = zp - c;
    float g;
    if (F > 0.0f) {
        const float a = fmaxf(dxm, 0.0f), b = fminf(dxp, 0.0f), e = fmaxf(dym, 0.0f),
                    f = fminf(dyp, 0.0f), h = fmaxf(dzm, 0.0f), k = fminf(dzp, 0.0f);
        g = sqrtf(a * a + b * b + e * e + f * f + h * h + k * k);
    } else {
        const float a = fminf(dxm, 0.0f), b = fmaxf(dxp, 0.0f), e = fminf(dym, 0.0f),
                    f = fmaxf(dyp, 0.0f), h = fminf(dzm, 0.0f), k = fmaxf(dzp, 0.0f);
        g = sqrtf(a * a + b * b + e * e + f * f + h * h + k * k);
    }
    float nv = c + V.dt * (wc * curv - F * g);
    return fminf(fmaxf(nv, V.lo), V.hi);
}

template <class S, int NT>
struct NsSmem {
    alignas(128) float phi[2][S::TILE];  // halo tiles, double buffered
    alignas(128) float img[2][S::VOX];
    alignas(128) float out[2][S::VOX];
    unsigned long long act[S::WORDS];
    unsigned long long next[27 * S::WORDS];
    uint32_t chg[S::CHG];
    alignas(8) uint64_t bar[2];
};

// Bits of one brick row (BX voxels) of the changed mask.
template <class S>
__device__ __forceinline__ uint32_t chg_row(const uint32_t* chg, int ly, int lz) {
    const int off = (lz * S::Y + ly) * S::X;
    return (chg[off >> 5] >> (off & 31)) & ((1u << S::X) - 1u);
}

template <class S>
__device__ __forceinline__ bool chg_bit(const uint32_t* chg, int lx, int ly, int lz) {
    const int j = (lz * S::Y + ly) * S::X + lx;
    return (chg[j >> 5] >> (j & 31)) & 1u;
}

// Brick origin of global brick b.
template <class S>
__device__ __forceinline__ int3 brick_origin(const NsVol& V, uint32_t b) {
    const uint32_t lb = b - V.brick_base;
    const int kx = lb % V.nbx, ky = (lb / V.nbx) % V.nby, kz = lb / (V.nbx * V.nby);
    return make_int3(kx * S::X, ky * S::Y, kz * S::Z);
}

// Issues the TMA loads of brick b (halo tile of phi[p] and the intensities)
// into buffer `buf` (thread 0 only).
template <class S, int NT>
__device__ __forceinline__ void ns_issue_loads(const NsArgs& a, NsSmem<S, NT>& sm, uint32_t b,
                                               uint32_t p, int buf) {
    const NsVol& V = a.vols[a.brick_vol[b]];
    const int3 o = brick_origin<S>(V, b);
    mbar_expect_tx(&sm.bar[buf], (uint32_t)(S::TILE + S::VOX) * 4u);
    tma_load_3d(sm.phi[buf], &a.tmaps[V.tmap_base + p], o.x - 4, o.y - 1, o.z - 1, &sm.bar[buf]);
    tma_load_3d(sm.img[buf], &a.tmaps[V.tmap_base + 4], o.x, o.y, o.z, &sm.bar[buf]);
}

// Per-block running totals of updated voxels and bricks of one volume,
// flushed with one atomic each when the volume changes or the phase ends.
struct BlockTally {
    uint32_t v = 0xFFFFFFFFu;
    unsigned long long upd = 0, brk = 0;
    __device__ void add(NsVolState* vs, uint32_t vol, unsigned long long n) {
        if (vol != v) {
            flush(vs);
            v = vol;
        }
        upd += n;
        brk += 1;
    }
    __device__ void flush(NsVolState* vs) {
        if (v != 0xFFFFFFFFu && brk) {
            atomicAdd(&vs[v].updates, upd);
            atomicAdd(&vs[v].bricks, brk);
        }
        upd = brk = 0;
    }
};

// Phase-1 work on one active brick whose loads were issued into `buf`.
template <class S, int NT>
__device__ __forceinline__ void ns_process_brick(const NsArgs& a, NsSmem<S, NT>& sm, uint32_t b,
                                                 uint32_t p, int buf, uint32_t* mphase,
                                                 BlockTally& tally) {
    const int tid = threadIdx.x;
    const uint32_t v = a.brick_vol[b];
    const NsVol& V = a.vols[v];
    const int3 o = brick_origin<S>(V, b);
    const int x0 = o.x, y0 = o.y, z0 = o.z;
    unsigned long long* cur = a.masks[p] + (size_t)b * S::WORDS;
    if (tid < S::WORDS) {
        sm.act[tid] = cur[tid];
        cur[tid] = 0ull;
    }
    for (int t = tid; t < 27 * S::WORDS; t += NT) sm.next[t] = 0ull;
    if (!mbar_wait(&sm.bar[buf], mphase[buf])) set_error(&a.ctl->err, ERR_TMA_TIMEOUT);
    mphase[buf] ^= 1u;
    __syncthreads();
    float* phi = sm.phi[buf];
    // Clamp-to-edge halo where the tile leaves the volume (TMA filled zeros).
    const bool edge = x0 < 4 || y0 < 1 || z0 < 1 || x0 + S::X + 4 > V.nx || y0 + S::Y + 1 > V.ny ||
                      z0 + S::Z + 1 > V.nz;
    if (edge) {
        for (int t = tid; t < S::TILE; t += NT) {
            const int tx = t % S::TX, ty = (t / S::TX) % S::TY, tz = t / (S::TX * S::TY);
            const int gx = x0 - 4 + tx, gy = y0 - 1 + ty, gz = z0 - 1 + tz;
            const int cx = min(max(gx, 0), V.nx - 1), cy = min(max(gy, 0), V.ny - 1),
                      cz = min(max(gz, 0), V.nz - 1);
            if (cx != gx || cy != gy || cz != gz)
                phi[t] = phi[((cz - z0 + 1) * S::TY + (cy - y0 + 1)) * S::TX + (cx - x0 + 4)];
        }
        __syncthreads();
    }
    // The store issued from out[buf] two bricks ago must have read its source.
    if (tid == 0) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
    __syncthreads();
    float* out = sm.out[buf];
    constexpr int VPT = (S::VOX + NT - 1) / NT;
    const float* bias = V.bias;
#pragma unroll
    for (int k = 0; k < VPT; ++k) {
        const int j = tid + k * NT;
        bool chg = false;
        if (j < S::VOX) {
            const int lx = j % S::X, ly = (j / S::X) % S::Y, lz = j / (S::X * S::Y);
            const int ti = ((lz + 1) * S::TY + (ly + 1)) * S::TX + (lx + 4);
            const float c = phi[ti];
            float nv = c;
            if ((sm.act[j >> 6] >> (j & 63)) & 1ull) {
                auto P = [&](int dx, int dy, int dz) { return phi[ti + (dz * S::TY + dy) * S::TX + dx]; };
                float bb = 0.0f;
                if (bias) bb = bias[((size_t)(z0 + lz) * V.py + (y0 + ly)) * V.px + (x0 + lx)];
                nv = ns_update_f32(P, sm.img[buf][j], bb, V);
                chg = fabsf(nv - c) > V.thr_t;
            }
            out[j] = nv;
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, chg);
        const int word = (tid >> 5) + k * (NT / 32);
        if ((tid & 31) == 0 && word < S::CHG) sm.chg[word] = bal;
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
        tma_store_3d(&a.tmaps[V.tmap_base + 2 + (p ^ 1u)], x0, y0, z0, out);
        tma_store_commit();
    }
    // Dilation of the changed mask into the 27 bricks around (and including) b.
    bool any = false;
#pragma unroll 1
    for (int w = 0; w < S::CHG; ++w) any |= sm.chg[w] != 0u;
    if (any) {
        const int EX = S::X + 2, EY = S::Y + 2;
        for (int e = tid; e < S::EXT; e += NT) {
            const int ex = e % EX - 1, ey = (e / EX) % EY - 1, ez = e / (EX * EY) - 1;
            const int gx = x0 + ex, gy = y0 + ey, gz = z0 + ez;
            if (gx < 0 || gy < 0 || gz < 0 || gx >= V.nx || gy >= V.ny || gz >= V.nz) continue;
            bool hit = false;
            if (V.nbh == 26) {
                const int lo = max(ex - 1, 0), hi = min(ex + 1, S::X - 1);
                if (lo <= hi) {
                    const uint32_t m = ((1u << (hi - lo + 1)) - 1u) << lo;
                    for (int dz = -1; dz <= 1 && !hit; ++dz) {
                        const int z = ez + dz;
                        if (z < 0 || z >= S::Z) continue;
                        for (int dy = -1; dy <= 1; ++dy) {
                            const int y = ey + dy;
                            if (y < 0 || y >= S::Y) continue;
                            if (chg_row<S>(sm.chg, y, z) & m) { hit = true; break; }
                        }
                    }
                }
            } else {
                const bool in = ex >= 0 && ex < S::X && ey >= 0 && ey < S::Y && ez >= 0 && ez < S::Z;
                if (in && chg_bit<S>(sm.chg, ex, ey, ez)) hit = true;
                const int nb[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
                for (int q = 0; q < 6 && !hit; ++q) {
                    const int x = ex + nb[q][0], y = ey + nb[q][1], z = ez + nb[q][2];
                    if (x >= 0 && x < S::X && y >= 0 && y < S::Y && z >= 0 && z < S::Z &&
                        chg_bit<S>(sm.chg, x, y, z))
                        hit = true;
                }
            }
            if (!hit) continue;
            const int ox = ex < 0 ? -1 : (ex >= S::X ? 1 : 0);
            const int oy = ey < 0 ? -1 : (ey >= S::Y ? 1 : 0);
            const int oz = ez < 0 ? -1 : (ez >= S::Z ? 1 : 0);
            const int lx = ex - ox * S::X, ly = ey - oy * S::Y, lz = ez - oz * S::Z;
            const int jj = (lz * S::Y + ly) * S::X + lx;
            const int slot = (oz + 1) * 9 + (oy + 1) * 3 + (ox + 1);
            atomicOr(&sm.next[slot * S::WORDS + (jj >> 6)], 1ull << (jj & 63));
        }
        __syncthreads();
        for (int t = tid; t < 27 * S::WORDS; t += NT) {
            const unsigned long long w = sm.next[t];
            if (!w) continue;
            const int slot = t / S::WORDS, word = t % S::WORDS;
            const int ox = slot % 3 - 1, oy = (slot / 3) % 3 - 1, oz = slot / 9 - 1;
            const uint32_t nb = b + (int32_t)((oz * V.nby + oy) * V.nbx + ox);
            atomicOr(&a.masks[p ^ 1u][(size_t)nb * S::WORDS + word], w);
            uint32_t* bw = &a.bits[p ^ 1u][nb >> 5];
            const uint32_t bit = 1u << (nb & 31);
            if (!(*(volatile uint32_t*)bw & bit)) atomicOr(bw, bit);
        }
    }
    if (tid == 0) {
        unsigned long long n = 0;
        for (int w = 0; w < S::WORDS; ++w) n += __popcll(sm.act[w]);
        tally.add(a.vstate, v, n);
    }
    __syncthreads();
}

// Phase-1 work on one brick of F_k: phi[p] -> phi[p^1].
template <class S, int NT>
__device__ __forceinline__ void ns_flush_brick(const NsArgs& a, uint32_t b, uint32_t p) {
    const NsVol& V = a.vols[a.brick_vol[b]];
    const uint32_t lb = b - V.brick_base;
    const int kx = lb % V.nbx, ky = (lb / V.nbx) % V.nby, kz = lb / (V.nbx * V.nby);
    const float* src = V.phi[p];
    float* dst = V.phi[p ^ 1u];
    constexpr int Q = S::X / 4;  // float4 per row
    for (int t = threadIdx.x; t < S::Y * S::Z * Q; t += NT) {
        const int q = t % Q, ly = (t / Q) % S::Y, lz = t / (Q * S::Y);
        const size_t off = ((size_t)(kz * S::Z + lz) * V.py + (ky * S::Y + ly)) * V.px + kx * S::X + 4 * q;
        *reinterpret_cast<float4*>(dst + off) = *reinterpret_cast<const float4*>(src + off);
    }
}

// Phase 2 (and list construction at initialisation): compaction of the brick
// bitmaps.  next: bricks with a non-empty next mask (-> A); cur (nullable):
// bricks of A_k (cur & ~next -> F, and cur is cleared).  done (nullable)
// drops bricks of finished volumes.  Counts the voxels of A per volume into
// cnt.  The last tile publishes the list lengths.
template <int WORDS, int NT>
__device__ __forceinline__ void ns_scan(const NsArgs& a, uint32_t* next, uint32_t* cur,
                                        const unsigned long long* nmask, unsigned long long* cnt,
                                        const int32_t* done) {
    __shared__ uint32_t s_tile;
    const uint32_t ntiles = (a.NW + NT - 1) / NT;
    constexpr uint64_t M31 = (1ull << 31) - 1;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&a.ctl->scan_tile, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        __syncthreads();
        if (tile >= ntiles) break;
        const uint32_t w = tile * NT + threadIdx.x;
        uint32_t an = 0, c = 0;
        if (w < a.NW) {
            an = next[w];
            if (cur) c = cur[w];
            if (done && (an | c)) {
                uint32_t all = an | c;
                while (all) {
                    const int bit = __ffs(all) - 1;
                    all &= all - 1;
                    if (done[a.brick_vol[w * 32 + bit]]) {
                        an &= ~(1u << bit);
                        c &= ~(1u << bit);
                    }
                }
            }
        }
        const uint32_t fb = c & ~an;
        const uint64_t val = ((uint64_t)__popc(an) << 31) | (uint64_t)__popc(fb);
        uint64_t total;
        const uint64_t excl = block_exclusive_sum64(val, &total);
        const uint64_t prefix = tile_exclusive_prefix(a.status, tile, total, &a.ctl->err);
        const uint32_t a0 = (uint32_t)(prefix >> 31);  // this tile's first A position
        uint32_t pa = a0 + (uint32_t)(excl >> 31);
        uint32_t pf = (uint32_t)((prefix & M31) + (excl & M31));
        uint32_t m = an;
        while (m) {
            const int bit = __ffs(m) - 1;
            m &= m - 1;
            a.A_list[pa++] = w * 32 + bit;
        }
        m = fb;
        while (m) {
            const int bit = __ffs(m) - 1;
            m &= m - 1;
            a.F_list[pf++] = w * 32 + bit;
        }
        if (cur && w < a.NW) cur[w] = 0u;
        if (tile == ntiles - 1 && threadIdx.x == 0) {
            const uint64_t t = prefix + total;
            a.ctl->nA = (uint32_t)(t >> 31);
            a.ctl->nF = (uint32_t)(t & M31);
        }
        // Voxel count of this tile's A bricks, spread over the block; one
        // atomic per warp and volume run.
        __syncthreads();
        const uint32_t a1 = a0 + (uint32_t)(total >> 31);
        uint32_t vol = 0xFFFFFFFFu;
        unsigned long long sum = 0;
        for (uint32_t i = a0 + threadIdx.x; i < a1; i += NT) {
            const uint32_t bk = a.A_list[i];
            const uint32_t bv = a.brick_vol[bk];
            if (bv != vol) {
                if (sum) atomicAdd(&cnt[vol], sum);
                vol = bv;
                sum = 0;
            }
            for (int q = 0; q < WORDS; ++q) sum += __popcll(nmask[(size_t)bk * WORDS + q]);
        }
        const uint32_t v0 = __reduce_min_sync(0xffffffffu, sum ? vol : 0xFFFFFFFFu);
        const bool uniform = __all_sync(0xffffffffu, vol == v0 || sum == 0);
        if (uniform) {
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
            if ((threadIdx.x & 31) == 0 && sum) atomicAdd(&cnt[v0], sum);
        } else if (sum) {
            atomicAdd(&cnt[vol], sum);
        }
        __syncthreads();
    }
}

// Per-volume stopping state kept identically by every block (dynamic shared
// memory): done, streak, stop iteration, current count.
struct StopState {
    int32_t* done;
    int32_t* streak;
    int32_t* stop;
    unsigned long long* n;
};

__host__ __device__ constexpr size_t stop_state_bytes(int nvol) {
    return (size_t)16 * ((3 * nvol + 3) / 4) + 8 * (size_t)nvol;
}

__device__ __forceinline__ StopState stop_state(int32_t* base, int nvol) {
    StopState s;
    s.done = base;
    s.streak = base + nvol;
    s.stop = base + 2 * nvol;
    s.n = reinterpret_cast<unsigned long long*>(base + 4 * ((3 * nvol + 3) / 4));
    return s;
}

template <int NT>
__device__ __forceinline__ void ns_begin(const NsArgs& a, StopState& ss, uint32_t* s_gen) {
    const int tid = threadIdx.x;
    if (tid == 0) {
        *s_gen = ld_acquire_u32(&a.ctl->bar_gen);
        for (int v = 0; v < a.nvol; ++v)
            for (int m = 0; m < 5; ++m) tmap_acquire(&a.tmaps[a.vols[v].tmap_base + m]);
    }
    for (int v = tid; v < a.nvol; v += NT) {
        ss.done[v] = 0;
        ss.streak[v] = 0;
        ss.stop[v] = -1;
        ss.n[v] = a.vstate[v].n_cur;
    }
}

// Start of an iteration (block 0): clear this iteration's count slot, the
// compaction status words and the tile counter.
template <int NT>
__device__ __forceinline__ void ns_iteration_prologue(const NsArgs& a, uint32_t p) {
    if (blockIdx.x != 0) return;
    const int tid = threadIdx.x;
    for (int v = tid; v < a.nvol; v += NT) a.cnt[p ^ 1u][v] = 0ull;
    const uint32_t ntiles = (a.NW + NT - 1) / NT;
    for (uint32_t t = tid; t < ntiles; t += NT) a.status[t] = 0ull;
    if (tid == 0) a.ctl->scan_tile = 0u;
}

// After phase 1: barrier, phase-2 compaction, barrier, stopping rule.
// Returns false when the loop must end (*it_out then holds the iterations run).
template <int WORDS, int NT>
__device__ __forceinline__ bool ns_iteration_epilogue(const NsArgs& a, StopState& ss, uint32_t& gen,
                                                      uint32_t p, int it, int* it_out) {
    const int tid = threadIdx.x;
    const uint32_t G = gridDim.x;
    *it_out = it;
    __syncthreads();
    if (!grid_barrier(a.ctl, gen, G)) return false;
    ns_scan<WORDS, NT>(a, a.bits[p ^ 1u], a.bits[p], a.masks[p ^ 1u], a.cnt[p ^ 1u],
                       a.nvol > 1 ? ss.done : nullptr);
    if (!grid_barrier(a.ctl, gen, G)) return false;
    if (tid == 0) asm volatile("fence.proxy.async.global;" ::: "memory");
    if (*(volatile uint32_t*)&a.ctl->err) return false;
    __shared__ int32_t s_live;
    if (tid == 0) s_live = 0;
    __syncthreads();
    for (int v = tid; v < a.nvol; v += NT) {
        if (ss.done[v]) continue;
        const unsigned long long n = *(volatile unsigned long long*)&a.cnt[p ^ 1u][v];
        ss.n[v] = n;
        bool stop;
        if (a.conv_mode) {
            const unsigned long long n0 = a.vstate[v].n0;
            ss.streak[v] = ((double)n < a.rel * (double)n0) ? ss.streak[v] + 1 : 0;
            stop = ss.streak[v] >= a.patience || n <= a.abs_thr || it + 1 >= a.max_iters;
        } else {
            stop = it + 1 >= a.max_iters;
        }
        if (stop) {
            ss.done[v] = 1;
            ss.stop[v] = it;
        } else {
            atomicAdd(&s_live, 1);
        }
    }
    __syncthreads();
    *it_out = it + 1;
    return s_live != 0;
}

template <int NT>
__device__ __forceinline__ void ns_finish(const NsArgs& a, const StopState& ss, int it) {
    if (blockIdx.x != 0) return;
    const int tid = threadIdx.x;
    for (int v = tid; v < a.nvol; v += NT) {
        NsVolState& st = a.vstate[v];
        const int ran = ss.stop[v] >= 0 ? ss.stop[v] + 1 : it;
        st.iterations += (unsigned long long)ran;
        st.parity = (int32_t)((a.parity0 + (uint32_t)ran) & 1u);
        st.n_cur = ss.n[v];
        st.streak = ss.streak[v];
        st.done = a.conv_mode ? ss.done[v] : 0;
    }
    if (tid == 0) a.ctl->iters_run = (uint32_t)it;
}

// One block per brick (NT threads per brick), loads double buffered.
template <int BX, int BY, int BZ, int NT>
__global__ void __launch_bounds__(NT) k_ns_persistent(NsArgs a) {
    using S = Brick<BX, BY, BZ>;
    __shared__ NsSmem<S, NT> sm;
    extern __shared__ int32_t s_dyn[];
    StopState ss = stop_state(s_dyn, a.nvol);
    const int tid = threadIdx.x;
    const uint32_t G = gridDim.x;
    __shared__ uint32_t s_gen;
    if (tid == 0) {
        mbar_init(&sm.bar[0], 1);
        mbar_init(&sm.bar[1], 1);
    }
    ns_begin<NT>(a, ss, &s_gen);
    __syncthreads();
    uint32_t gen = s_gen;
    uint32_t mphase[2] = {0u, 0u};
    int it = 0, ran = 0;
    for (; it < a.max_iters; ++it) {
        const uint32_t p = (a.parity0 + (uint32_t)it) & 1u;
        const uint32_t nA = *(volatile uint32_t*)&a.ctl->nA;
        const uint32_t nF = *(volatile uint32_t*)&a.ctl->nF;
        ns_iteration_prologue<NT>(a, p);
        BlockTally tally;
        int buf = 0;
        if (tid == 0 && blockIdx.x < nA) ns_issue_loads<S, NT>(a, sm, a.A_list[blockIdx.x], p, 0);
        for (uint32_t w = blockIdx.x; w < nA; w += G) {
            const uint32_t b = a.A_list[w];
            if (tid == 0 && w + G < nA) ns_issue_loads<S, NT>(a, sm, a.A_list[w + G], p, buf ^ 1);
            if (!ss.done[a.brick_vol[b]]) {
                ns_process_brick<S, NT>(a, sm, b, p, buf, mphase, tally);
            } else {
                if (!mbar_wait(&sm.bar[buf], mphase[buf])) set_error(&a.ctl->err, ERR_TMA_TIMEOUT);
                mphase[buf] ^= 1u;
                __syncthreads();
            }
            buf ^= 1;
        }
        if (tid == 0) tally.flush(a.vstate);
        for (uint32_t w = blockIdx.x; w < nF; w += G) {
            const uint32_t b = a.F_list[w];
            if (!ss.done[a.brick_vol[b]]) ns_flush_brick<S, NT>(a, b, p);
        }
        if (tid == 0) {
            tma_store_wait_all();
            asm volatile("fence.proxy.async.global;" ::: "memory");
        }
        if (!ns_iteration_epilogue<S::WORDS, NT>(a, ss, gen, p, it, &ran)) break;
    }
    if (it == a.max_iters) ran = it;
    ns_finish<NT>(a, ss, ran);
}

// ---------------------------------------------------------------------------
// One warp per brick: each warp owns a shared-memory slice and an mbarrier and
// synchronises with __syncwarp only, so an SM keeps as many bricks in flight
// as it holds warps.
template <class S>
struct WarpSmem {
    alignas(128) float phi[S::TILE];
    alignas(128) float img[S::VOX];
    alignas(128) float out[S::VOX];
    unsigned long long act[S::WORDS];
    unsigned long long next[27 * S::WORDS];
    uint32_t chg[S::CHG];
    alignas(8) uint64_t bar;
};

template <class S>
__device__ __forceinline__ void ns_process_brick_warp(const NsArgs& a, WarpSmem<S>& sm, uint32_t b,
                                                      uint32_t p, uint32_t& mphase,
                                                      BlockTally& tally) {
    const int lane = threadIdx.x & 31;
    const uint32_t v = a.brick_vol[b];
    const NsVol& V = a.vols[v];
    const int3 o = brick_origin<S>(V, b);
    const int x0 = o.x, y0 = o.y, z0 = o.z;
    unsigned long long* cur = a.masks[p] + (size_t)b * S::WORDS;
    if (lane == 0) {
        // The previous brick's store must have read its source before the
        // update overwrites it.
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        mbar_expect_tx(&sm.bar, (uint32_t)(S::TILE + S::VOX) * 4u);
        tma_load_3d(sm.phi, &a.tmaps[V.tmap_base + p], x0 - 4, y0 - 1, z0 - 1, &sm.bar);
        tma_load_3d(sm.img, &a.tmaps[V.tmap_base + 4], x0, y0, z0, &sm.bar);
    }
    for (int t = lane; t < S::WORDS; t += 32) {
        sm.act[t] = cur[t];
        cur[t] = 0ull;
    }
    for (int t = lane; t < 27 * S::WORDS; t += 32) sm.next[t] = 0ull;
    if (!mbar_wait(&sm.bar, mphase)) set_error(&a.ctl->err, ERR_TMA_TIMEOUT);
    mphase ^= 1u;
    __syncwarp();
    float* phi = sm.phi;
    const bool edge = x0 < 4 || y0 < 1 || z0 < 1 || x0 + S::X + 4 > V.nx || y0 + S::Y + 1 > V.ny ||
                      z0 + S::Z + 1 > V.nz;
    if (edge) {
        for (int t = lane; t < S::TILE; t += 32) {
            const int tx = t % S::TX, ty = (t / S::TX) % S::TY, tz = t / (S::TX * S::TY);
            const int gx = x0 - 4 + tx, gy = y0 - 1 + ty, gz = z0 - 1 + tz;
            const int cx = min(max(gx, 0), V.nx - 1), cy = min(max(gy, 0), V.ny - 1),
                      cz = min(max(gz, 0), V.nz - 1);
            if (cx != gx || cy != gy || cz != gz)
                phi[t] = phi[((cz - z0 + 1) * S::TY + (cy - y0 + 1)) * S::TX + (cx - x0 + 4)];
        }
        __syncwarp();
    }
    const float* bias = V.bias;
    bool any = false;
#pragma unroll 2
    for (int k = 0; k < S::CHG; ++k) {
        const int j = lane + 32 * k;
        const int lx = j % S::X, ly = (j / S::X) % S::Y, lz = j / (S::X * S::Y);
        const int ti = ((lz + 1) * S::TY + (ly + 1)) * S::TX + (lx + 4);
        const float c = phi[ti];
        float nv = c;
        bool chg = false;
        if ((sm.act[j >> 6] >> (j & 63)) & 1ull) {
            auto P = [&](int dx, int dy, int dz) { return phi[ti + (dz * S::TY + dy) * S::TX + dx]; };
            float bb = 0.0f;
            if (bias) bb = bias[((size_t)(z0 + lz) * V.py + (y0 + ly)) * V.px + (x0 + lx)];
            nv = ns_update_f32(P, sm.img[j], bb, V);
            chg = fabsf(nv - c) > V.thr_t;
        }
        sm.out[j] = nv;
        const uint32_t bal = __ballot_sync(0xffffffffu, chg);
        any |= bal != 0u;
        if (lane == 0) sm.chg[k] = bal;
    }
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) {
        tma_store_3d(&a.tmaps[V.tmap_base + 2 + (p ^ 1u)], x0, y0, z0, sm.out);
        tma_store_commit();
    }
    if (any) {
        const int EX = S::X + 2, EY = S::Y + 2;
        for (int e = lane; e < S::EXT; e += 32) {
            const int ex = e % EX - 1, ey = (e / EX) % EY - 1, ez = e / (EX * EY) - 1;
            const int gx = x0 + ex, gy = y0 + ey, gz = z0 + ez;
            if (gx < 0 || gy < 0 || gz < 0 || gx >= V.nx || gy >= V.ny || gz >= V.nz) continue;
            bool hit = false;
            if (V.nbh == 26) {
                const int lo = max(ex - 1, 0), hi = min(ex + 1, S::X - 1);
                if (lo <= hi) {
                    const uint32_t m = ((1u << (hi - lo + 1)) - 1u) << lo;
                    for (int dz = -1; dz <= 1 && !hit; ++dz) {
                        const int z = ez + dz;
                        if (z < 0 || z >= S::Z) continue;
                        for (int dy = -1; dy <= 1; ++dy) {
                            const int y = ey + dy;
                            if (y < 0 || y >= S::Y) continue;
                            if (chg_row<S>(sm.chg, y, z) & m) { hit = true; break; }
                        }
                    }
                }
            } else {
                const bool in = ex >= 0 && ex < S::X && ey >= 0 && ey < S::Y && ez >= 0 && ez < S::Z;
                if (in && chg_bit<S>(sm.chg, ex, ey, ez)) hit = true;
                const int nb[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
                for (int q = 0; q < 6 && !hit; ++q) {
                    const int x = ex + nb[q][0], y = ey + nb[q][1], z = ez + nb[q][2];
                    if (x >= 0 && x < S::X && y >= 0 && y < S::Y && z >= 0 && z < S::Z &&
                        chg_bit<S>(sm.chg, x, y, z))
                        hit = true;
                }
            }
            if (!hit) continue;
            const int ox = ex < 0 ? -1 : (ex >= S::X ? 1 : 0);
            const int oy = ey < 0 ? -1 : (ey >= S::Y ? 1 : 0);
            const int oz = ez < 0 ? -1 : (ez >= S::Z ? 1 : 0);
            const int lx = ex - ox * S::X, ly = ey - oy * S::Y, lz = ez - oz * S::Z;
            const int jj = (lz * S::Y + ly) * S::X + lx;
            const int slot = (oz + 1) * 9 + (oy + 1) * 3 + (ox + 1);
            atomicOr(&sm.next[slot * S::WORDS + (jj >> 6)], 1ull << (jj & 63));
        }
        __syncwarp();
        for (int t = lane; t < 27 * S::WORDS; t += 32) {
            const unsigned long long w = sm.next[t];
            if (!w) continue;
            const int slot = t / S::WORDS, word = t % S::WORDS;
            const int ox = slot % 3 - 1, oy = (slot / 3) % 3 - 1, oz = slot / 9 - 1;
            const uint32_t nb = b + (int32_t)((oz * V.nby + oy) * V.nbx + ox);
            atomicOr(&a.masks[p ^ 1u][(size_t)nb * S::WORDS + word], w);
            atomicOr(&a.bits[p ^ 1u][nb >> 5], 1u << (nb & 31));
        }
    }
    if (lane == 0) {
        unsigned long long n = 0;
        for (int w = 0; w < S::WORDS; ++w) n += __popcll(sm.act[w]);
        tally.add(a.vstate, v, n);
    }
    __syncwarp();
}

template <class S>
__device__ __forceinline__ void ns_flush_brick_warp(const NsArgs& a, uint32_t b, uint32_t p) {
    const NsVol& V = a.vols[a.brick_vol[b]];
    const int3 o = brick_origin<S>(V, b);
    const float* src = V.phi[p];
    float* dst = V.phi[p ^ 1u];
    constexpr int Q = S::X / 4;
    for (int t = threadIdx.x & 31; t < S::Y * S::Z * Q; t += 32) {
        const int q = t % Q, ly = (t / Q) % S::Y, lz = t / (Q * S::Y);
        const size_t off = ((size_t)(o.z + lz) * V.py + (o.y + ly)) * V.px + o.x + 4 * q;
        *reinterpret_cast<float4*>(dst + off) = *reinterpret_cast<const float4*>(src + off);
    }
}

template <class S>
__host__ __device__ constexpr size_t warp_smem_offset(int nvol) {
    return (stop_state_bytes(nvol) + 127) / 128 * 128 + 128;  // + slack for base alignment
}

// NT/32 warps per block, one brick per warp at a time.
template <int BX, int BY, int BZ, int NT>
__global__ void __launch_bounds__(NT) k_ns_persistent_warp(NsArgs a) {
    using S = Brick<BX, BY, BZ>;
    constexpr int W = NT / 32;
    extern __shared__ __align__(128) unsigned char s_raw[];
    StopState ss = stop_state(reinterpret_cast<int32_t*>(s_raw), a.nvol);
    uintptr_t wb = reinterpret_cast<uintptr_t>(s_raw) + (stop_state_bytes(a.nvol) + 127) / 128 * 128;
    wb = (wb + 127) & ~(uintptr_t)127;
    WarpSmem<S>* wsm = reinterpret_cast<WarpSmem<S>*>(wb);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    WarpSmem<S>& sm = wsm[warp];
    const uint32_t GW = gridDim.x * W;
    const uint32_t gw = blockIdx.x * W + warp;
    __shared__ uint32_t s_gen;
    if (lane == 0) mbar_init(&sm.bar, 1);
    ns_begin<NT>(a, ss, &s_gen);
    __syncthreads();
    uint32_t gen = s_gen;
    uint32_t mphase = 0;
    int it = 0, ran = 0;
    for (; it < a.max_iters; ++it) {
        const uint32_t p = (a.parity0 + (uint32_t)it) & 1u;
        const uint32_t nA = *(volatile uint32_t*)&a.ctl->nA;
        const uint32_t nF = *(volatile uint32_t*)&a.ctl->nF;
        ns_iteration_prologue<NT>(a, p);
        BlockTally tally;
        for (uint32_t w = gw; w < nA; w += GW) {
            const uint32_t b = a.A_list[w];
            if (!ss.done[a.brick_vol[b]]) ns_process_brick_warp<S>(a, sm, b, p, mphase, tally);
        }
        if (lane == 0) tally.flush(a.vstate);
        for (uint32_t w = gw; w < nF; w += GW) {
            const uint32_t b = a.F_list[w];
            if (!ss.done[a.brick_vol[b]]) ns_flush_brick_warp<S>(a, b, p);
        }
        if (lane == 0) {
            tma_store_wait_all();
            asm volatile("fence.proxy.async.global;" ::: "memory");
        }
        if (!ns_iteration_epilogue<S::WORDS, NT>(a, ss, gen, p, it, &ran)) break;
    }
    if (it == a.max_iters) ran = it;
    ns_finish<NT>(a, ss, ran);
}

// Initial active set of every brick: voxels whose 6-neighbours differ by more
// than thr_s (clamped coordinates), one block per brick.
template <int BX, int BY, int BZ, int NT>
__global__ void __launch_bounds__(NT) k_ns_init_active(NsArgs a, uint32_t p) {
    using S = Brick<BX, BY, BZ>;
    __shared__ uint32_t s_w[S::CHG];
    for (uint32_t b = blockIdx.x; b < a.NB; b += gridDim.x) {
        const NsVol& V = a.vols[a.brick_vol[b]];
        const uint32_t lb = b - V.brick_base;
        const int kx = lb % V.nbx, ky = (lb / V.nbx) % V.nby, kz = lb / (V.nbx * V.nby);
        const float* ph = V.phi[p];
        constexpr int VPT = (S::VOX + NT - 1) / NT;
        for (int k = 0; k < VPT; ++k) {
            const int j = threadIdx.x + k * NT;
            bool act = false;
            if (j < S::VOX) {
                const int x = kx * S::X + j % S::X, y = ky * S::Y + (j / S::X) % S::Y,
                          z = kz * S::Z + j / (S::X * S::Y);
                if (x < V.nx && y < V.ny && z < V.nz) {
                    auto at = [&](int xx, int yy, int zz) {
                        xx = min(max(xx, 0), V.nx - 1);
                        yy = min(max(yy, 0), V.ny - 1);
                        zz = min(max(zz, 0), V.nz - 1);
                        return ph[((size_t)zz * V.py + yy) * V.px + xx];
                    };
                    const float c = at(x, y, z);
                    float m = fabsf(at(x - 1, y, z) - c);
                    m = fmaxf(m, fabsf(at(x + 1, y, z) - c));
                    m = fmaxf(m, fabsf(at(x, y - 1, z) - c));
                    m = fmaxf(m, fabsf(at(x, y + 1, z) - c));
                    m = fmaxf(m, fabsf(at(x, y, z - 1) - c));
                    m = fmaxf(m, fabsf(at(x, y, z + 1) - c));
                    act = m > V.thr_s;
                }
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, act);
            const int word = (threadIdx.x >> 5) + k * (NT / 32);
            if ((threadIdx.x & 31) == 0 && word < S::CHG) s_w[word] = bal;
        }
        __syncthreads();
        if (threadIdx.x < S::WORDS) {
            const unsigned long long w =
                (unsigned long long)s_w[2 * threadIdx.x] | ((unsigned long long)s_w[2 * threadIdx.x + 1] << 32);
            a.masks[p][(size_t)b * S::WORDS + threadIdx.x] = w;
            if (w) atomicOr(&a.bits[p][b >> 5], 1u << (b & 31));
        }
        __syncthreads();
    }
}

// List construction from bits[p] (no F list, bits kept).
template <int WORDS, int NT>
__global__ void __launch_bounds__(NT) k_ns_build_list(NsArgs a, uint32_t p) {
    ns_scan<WORDS, NT>(a, a.bits[p], nullptr, a.masks[p], a.cnt[p], nullptr);
}

}  // namespace lss
