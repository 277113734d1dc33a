// LSS_MODE_NS device code: the persistent bricked iteration kernel and its
// helpers.  One launch runs many iterations (and, in the batched form, many
// volumes) with ONE bounded grid barrier per iteration k:
//
//   every block ranks the bricks of A_k (and of A_{k-1} \ A_k) with a block
//     prefix sum over the membership words and takes the ranks i, i+G, ...
//     (block i of G): every block gets ceil(n/G) or floor(n/G) bricks, with
//     no global list and no atomics;
//   every owned brick of A_k: TMA-load the brick's phi with a one-voxel halo
//     (and its speed, computed once per volume and parameter set from D =
//     eps - |I - T|) into shared memory, with the next brick's loads and mask
//     words in flight (double buffered); update the active voxels (upwind
//     |grad phi| times the speed, mean curvature), TMA-store
//     the brick into the other phi buffer, flag changed voxels with warp
//     ballots, dilate the changed bitmask by the 26- (or 6-) neighbourhood and
//     OR it into the next masks and membership bits of the brick and its 26
//     neighbours (fire-and-forget reductions);
//   every owned brick of A_{k-1} that is not in A_k copies phi across, so
//     both phi buffers stay current;
//   barrier, then every block evaluates the stopping rule on the same counts.
//
// Membership bits, masks and phi are order independent, so results are
// deterministic.  The ordered (brick-major) voxel list is produced on demand
// by a single-pass decoupled-lookback compaction over the membership bits
// (k_ns_emit).
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
    const float* speed;     // ns_speed_f32 of every voxel (padded): what the iterations read
    float T, eps, alpha, dt, lo, hi, thr_t, thr_s;
    int32_t alpha_data;     // 1: alpha weights the data term, 0: the curvature term
    int32_t nbh;            // 26 or 6
    uint32_t tmap_base;     // 5 maps: phi0 halo-load, phi1 halo-load, phi0 store, phi1 store, speed
    float inv_eps;          // 1 / eps (LSS_DATA_NORMALISED), 1 (LSS_DATA_LITERAL)
    float dlo, dhi;         // clamp of the data term: -1, 1 or -inf, +inf (literal)
    int32_t data_literal;   // 1: D = eps - |I - T| as written
    float wc, wd;           // curvature and data weights (from alpha and alpha_data)
    uint32_t mnbx, mnbxy;   // 0xFFFFFFFF / nbx + 1 and / (nbx * nby) + 1 (div_magic)
};

struct NsVolState {
    unsigned long long n0;          // active voxels after seeding
    unsigned long long n_cur;       // active voxels of the current list
    unsigned long long updates;     // voxel updates so far
    unsigned long long bricks;      // brick updates so far
    unsigned long long iterations;  // iterations so far
    int32_t streak, done, parity, pad;
};

// Grid-barrier words.  Arrival: blocks arrived (low 16 bits) + voxel updates
// of the iteration summed over the blocks (high 48 bits), so the last block
// to arrive knows the iteration's count without another memory round trip.
// Release (own 128-byte line, polled): generation (low 32 bits) | streak of
// the stopping rule (bits 32..47) | stop flag (bit 48).
constexpr int kArriveShift = 16;
constexpr uint64_t kArriveMask = (1ull << kArriveShift) - 1ull;
constexpr int kRelStreakShift = 32;
constexpr uint64_t kRelStop = 1ull << 48;

struct NsCtl {
    unsigned long long bar_arrive;
    unsigned long long n_last;  // updates of the last iteration (one-volume path)
    uint32_t err;
    uint32_t iters_run;         // iterations run by the last launch
    uint32_t emit_tile;         // tile counter of the voxel-list emission
    uint32_t pad;
    unsigned long long t_phase1_ns, t_barrier_ns;  // block 0's time split
    alignas(128) unsigned long long bar_release;
    unsigned long long pad2[15];
    // Counter barrier (grids of at most kCounterBarrierMax blocks): arrivals
    // counted since the control block was cleared, and the one-volume update
    // counts summed by iteration parity; all only grow.
    alignas(128) unsigned long long arrivals;
    unsigned long long pad3[15];
    alignas(128) unsigned long long upd_sum[2];
    unsigned long long pad4[14];
};

// Up to this many blocks the grid barrier is a counter that every block
// polls (one hop after the last arrival).  Measured alone, with every block
// arriving at once, the counter is faster at 152 blocks (1.23 against
// 1.80 us) and slower at 608 (2.18 against 1.93 us); in the solver, where
// arrivals spread over the iteration, it is 1 % faster at 608 as well.
// Above, polling that one line costs more than the last arriver's release
// word.
constexpr uint32_t kCounterBarrierMax = 640;

struct NsArgs {
    const NsVol* vols;
    NsVolState* vstate;
    int32_t nvol;
    const CUtensorMap* tmaps;
    unsigned long long* masks[2];  // [NB][WORDS], by phi parity
    uint32_t* bits[4];             // [NW] brick membership, by iteration mod 4
    const uint16_t* brick_vol;     // [NB]
    unsigned long long* cnt[3];    // [nvol] active voxels updated, by iteration mod 3
    uint64_t* status;              // decoupled-lookback status words
    NsCtl* ctl;
    uint32_t NB, NW;
    uint32_t k0;                   // global iteration index of the launch's first iteration
    int32_t max_iters;
    int32_t conv_mode;             // 0: exactly max_iters, 1: stopping rule
    double rel;
    int32_t patience;
    unsigned long long abs_thr;
    unsigned long long arrivals0;   // NsCtl::arrivals and upd_sum at the launch
    unsigned long long upd_sum0[2];
};

template <int BX, int BY, int BZ>
struct Brick {
    static constexpr int X = BX, Y = BY, Z = BZ;
    static constexpr int VOX = BX * BY * BZ;
    static constexpr int WORDS = (VOX + 63) / 64;
    static constexpr int CHG = VOX / 32;
    static constexpr int TX = BX + 8, TY = BY + 2, TZ = BZ + 2;  // halo tile
    static constexpr int TILE = TX * TY * TZ;
    static constexpr int TILE_PAD = (TILE + 31) / 32 * 32;  // 128-byte stride between tiles
    static constexpr int XY = BX * BY;
    static_assert(VOX % 64 == 0, "brick must hold a multiple of 64 voxels");
    static_assert(BX == 4 || BX == 8, "brick x must be 4 or 8");
    // Mask words: one z-plane a word (XY == 64) or the whole brick in one word.
    static_assert(XY == 64 || VOX == 64, "mask word layout");
};

// The speed of one voxel, F = w_d (clamp(D(I)) + bias), the part of the
// LSS_MODE_NS update that no iteration changes: the engine computes it once
// per volume and parameter set (k_ns_speed, no bias) and the iterations read
// it; the adjoint, whose bias changes every call, computes it in place.
// Every operation is an explicit round-to-nearest intrinsic, so both give
// the same bits.  Literal data term: inv_eps = 1 (an exact product) and an
// infinite clamp, so both readings share one instruction sequence.
__device__ __forceinline__ float ns_speed_f32(float I, float bias, const NsVol& V) {
    float D = __fmul_rn(__fsub_rn(V.eps, fabsf(__fsub_rn(I, V.T))), V.inv_eps);
    D = __fadd_rn(fminf(fmaxf(D, V.dlo), V.dhi), bias);
    return __fmul_rn(V.wd, D);
}

// The LSS_MODE_NS update of one voxel of speed F from the shared-memory halo
// tile.  P(dx,dy,dz) reads the tile around the voxel.  Mirrors ns_update()
// of the FP64 oracle in fp32, with the central differences kept unscaled:
//   X = 2 phi_x, Fxx = phi_xx, Fxy = 4 phi_xy, so
//   kappa |grad phi| = [Fxx (Y^2+Z^2) + Fyy (X^2+Z^2) + Fzz (X^2+Y^2)
//                       - (XY Fxy + XZ Fxz + YZ Fyz) / 2] / (X^2+Y^2+Z^2).
// Every operation is an explicit round-to-nearest intrinsic (no contraction
// or reassociation left to the compiler), so the result is the same bit for
// bit in every kernel that inlines it.  The paired FP32 intrinsics
// (__ffma2_rn and kin) are not used: chained, they gave results an ulp off
// the IEEE operation sequence in about 1.4 % of updates, where the scalar
// form matched a CPU restatement of the sequence bit for bit.  The
// evaluation order keeps few values live; it changes no result.
template <class PF>
__device__ __forceinline__ float ns_update_speed_f32(PF P, float F, const NsVol& V) {
    const float c = P(0, 0, 0);
    const float xm = P(-1, 0, 0), xp = P(1, 0, 0);
    const float ym = P(0, -1, 0), yp = P(0, 1, 0);
    const float zm = P(0, 0, -1), zp = P(0, 0, 1);
    const float X = __fsub_rn(xp, xm), Y = __fsub_rn(yp, ym), Z = __fsub_rn(zp, zm);
    const float Fxx = __fmaf_rn(-2.0f, c, __fadd_rn(xp, xm));
    const float Fyy = __fmaf_rn(-2.0f, c, __fadd_rn(yp, ym));
    const float Fzz = __fmaf_rn(-2.0f, c, __fadd_rn(zp, zm));
    const float dxm = __fsub_rn(c, xm), dxp = __fsub_rn(xp, c), dym = __fsub_rn(c, ym),
                dyp = __fsub_rn(yp, c), dzm = __fsub_rn(c, zm), dzp = __fsub_rn(zp, c);
    // Osher-Sethian upwind |grad phi| for the speed F: one-sided differences
    // selected by the sign of F.
    float a, b, e, f, h, k;
    if (F > 0.0f) {
        a = fmaxf(dxm, 0.0f); b = fminf(dxp, 0.0f); e = fmaxf(dym, 0.0f);
        f = fminf(dyp, 0.0f); h = fmaxf(dzm, 0.0f); k = fminf(dzp, 0.0f);
    } else {
        a = fminf(dxm, 0.0f); b = fmaxf(dxp, 0.0f); e = fminf(dym, 0.0f);
        f = fmaxf(dyp, 0.0f); h = fminf(dzm, 0.0f); k = fmaxf(dzp, 0.0f);
    }
    const float s2 = __fmaf_rn(k, k, __fmaf_rn(h, h, __fmaf_rn(f, f, __fmaf_rn(e, e,
                               __fmaf_rn(b, b, __fmul_rn(a, a))))));
    const float Fg = __fmul_rn(F, __fsqrt_rn(s2));
    auto cross = [&](float pp, float pm, float mp, float mm) {
        return __fsub_rn(__fadd_rn(pp, mm), __fadd_rn(pm, mp));
    };
    const float Fxy = cross(P(1, 1, 0), P(1, -1, 0), P(-1, 1, 0), P(-1, -1, 0));
    const float Fxz = cross(P(1, 0, 1), P(1, 0, -1), P(-1, 0, 1), P(-1, 0, -1));
    const float Fyz = cross(P(0, 1, 1), P(0, 1, -1), P(0, -1, 1), P(0, -1, -1));
    const float xx = __fmul_rn(X, X), yy = __fmul_rn(Y, Y), zz = __fmul_rn(Z, Z);
    const float g2 = __fadd_rn(__fadd_rn(xx, yy), zz);  // 4 |grad phi|^2
    float curv = 0.0f;
    if (g2 > 4e-12f) {
        const float t = __fmaf_rn(Fzz, __fadd_rn(xx, yy),
                                  __fmaf_rn(Fyy, __fadd_rn(xx, zz), __fmul_rn(Fxx, __fadd_rn(yy, zz))));
        const float x = __fmaf_rn(__fmul_rn(Y, Z), Fyz, __fmaf_rn(__fmul_rn(X, Z), Fxz, __fmul_rn(__fmul_rn(X, Y), Fxy)));
        curv = __fdividef(__fmaf_rn(-0.5f, x, t), g2);  // g2 in (4e-12, 192]: within 2 ulp
    }
    const float nv = __fmaf_rn(V.dt, __fsub_rn(__fmul_rn(V.wc, curv), Fg), c);
    return fminf(fmaxf(nv, V.lo), V.hi);
}

// The update from the intensity and the bias (the speed computed in place).
template <class PF>
__device__ __forceinline__ float ns_update_f32(PF P, float I, float bias, const NsVol& V) {
    return ns_update_speed_f32(P, ns_speed_f32(I, bias, V), V);
}

// Every TMA destination / source below starts on a 128-byte boundary: the
// arrays are 128-byte aligned and every per-buffer stride is a multiple of
// 128 bytes (TILE_PAD floats; VOX floats = 256 B or more).
template <class S, int NT>
struct NsSmem {
    static_assert((S::TILE_PAD * 4) % 128 == 0 && (S::VOX * 4) % 128 == 0, "TMA smem alignment");
    // The thread that issues, commits and awaits the brick stores and keeps
    // the tally: lane 0 of the last warp, which has no xy-plane dilation work
    // (9 x WORDS <= NT - 32), so the store issue delays no barrier.
    static constexpr int STORE_TID = NT - 32;
    alignas(128) float phi[2][S::TILE_PAD];  // halo tiles, double buffered
    alignas(128) float spd[2][S::VOX];         // the brick's speed
    alignas(128) float out[2][S::VOX];
    unsigned long long act[2][S::WORDS];     // the brick's active mask, double buffered
    uint32_t chg[2][S::CHG];                 // changed voxels of the brick (ballot words)
    unsigned long long xy[9 * S::WORDS];     // xy-dilated planes per (ox, oy) pair
    int4 org[2];                             // origin (x, y, z) and volume of the brick in each buffer
    alignas(8) uint64_t bar[2];
};

// Bit-parallel dilation of a brick's changed mask.  Voxel (lx, ly, lz) is
// bit j = (lz*Y + ly)*X + lx of the mask (word j/64, bit j%64).  The box
// (26-neighbour) dilation is separable: x, then y, then z; the part of the
// result that lands in the neighbour brick at offset (ox, oy, oz) is
// Z_oz(Y_oy(X_ox(c))), where X_0 dilates within the brick and X_{-1} / X_{+1}
// move the edge column x = 0 / x = X-1 to the far column of the neighbour
// (likewise for y and z).  The 6-neighbour dilation is c | X_0 | Y_0 | Z_0 in
// the brick itself and X_{+-1}, Y_{+-1}, Z_{+-1} in the six face neighbours.
template <class S>
struct BitGeo {
    // Bits of a mask word whose voxel satisfies a predicate of (lx, ly, plane).
    template <class F>
    static constexpr uint64_t where(F f) {
        uint64_t m = 0;
        for (int b = 0; b < 64; ++b)
            if (f(b % S::X, (b / S::X) % S::Y, b / S::XY)) m |= 1ull << b;
        return m;
    }
    static constexpr uint64_t CX0 = where([](int x, int, int) { return x == 0; });
    static constexpr uint64_t CXL = where([](int x, int, int) { return x == S::X - 1; });
    static constexpr uint64_t RY0 = where([](int, int y, int) { return y == 0; });
    static constexpr uint64_t RYL = where([](int, int y, int) { return y == S::Y - 1; });
    static constexpr uint64_t PZ0 = where([](int, int, int z) { return z == 0; });
    static constexpr uint64_t PZL = where([](int, int, int z) { return z == S::Z - 1; });
};

template <class S>
__host__ __device__ __forceinline__ uint64_t dil_x(uint64_t v, int o) {
    using G = BitGeo<S>;
    const uint64_t d0 = v | ((v & ~G::CXL) << 1) | ((v & ~G::CX0) >> 1);
    const uint64_t dm = (v & G::CX0) << (S::X - 1), dp = (v & G::CXL) >> (S::X - 1);
    return o == 0 ? d0 : (o < 0 ? dm : dp);
}

template <class S>
__host__ __device__ __forceinline__ uint64_t dil_y(uint64_t v, int o) {
    using G = BitGeo<S>;
    const uint64_t d0 = v | ((v & ~G::RYL) << S::X) | ((v & ~G::RY0) >> S::X);
    const uint64_t dm = (v & G::RY0) << (S::X * (S::Y - 1)), dp = (v & G::RYL) >> (S::X * (S::Y - 1));
    return o == 0 ? d0 : (o < 0 ? dm : dp);
}

// z step over the whole mask (in place).
template <class S>
__host__ __device__ __forceinline__ void dil_z(uint64_t (&v)[S::WORDS], int o) {
    using G = BitGeo<S>;
    if constexpr (S::WORDS == 1) {
        constexpr int sh = S::XY * (S::Z - 1);
        if (o == 0) v[0] = v[0] | ((v[0] & ~G::PZL) << S::XY) | ((v[0] & ~G::PZ0) >> S::XY);
        else v[0] = o < 0 ? (v[0] & G::PZ0) << sh : (v[0] & G::PZL) >> sh;
    } else {
        uint64_t r[S::WORDS];
#pragma unroll
        for (int w = 0; w < S::WORDS; ++w) {
            if (o == 0) r[w] = v[w] | (w > 0 ? v[w - 1] : 0ull) | (w + 1 < S::WORDS ? v[w + 1] : 0ull);
            else if (o < 0) r[w] = w == S::WORDS - 1 ? v[0] : 0ull;
            else r[w] = w == 0 ? v[S::WORDS - 1] : 0ull;
        }
#pragma unroll
        for (int w = 0; w < S::WORDS; ++w) v[w] = r[w];
    }
}

// The part of the dilated mask m (in place) that lands in the neighbour
// brick at offset (ox, oy, oz); nbh = 26 or 6.
template <class S>
__host__ __device__ __forceinline__ void dilate_slot(uint64_t (&m)[S::WORDS], int ox, int oy, int oz, int nbh) {
    const int moved = (ox != 0) + (oy != 0) + (oz != 0);
    if (nbh == 6 && moved > 1) {
        for (int w = 0; w < S::WORDS; ++w) m[w] = 0ull;
    } else if (nbh == 6 && moved == 1) {  // face neighbour: one axis moves
        for (int w = 0; w < S::WORDS; ++w) m[w] = ox ? dil_x<S>(m[w], ox) : (oy ? dil_y<S>(m[w], oy) : m[w]);
        if (oz) dil_z<S>(m, oz);
    } else if (nbh == 6) {  // the brick itself: c | X_0 | Y_0 | Z_0
        uint64_t zz[S::WORDS];
        for (int w = 0; w < S::WORDS; ++w) zz[w] = m[w];
        dil_z<S>(zz, 0);
        for (int w = 0; w < S::WORDS; ++w) m[w] = dil_x<S>(m[w], 0) | dil_y<S>(m[w], 0) | zz[w];
    } else {
        for (int w = 0; w < S::WORDS; ++w) m[w] = dil_y<S>(dil_x<S>(m[w], ox), oy);
        dil_z<S>(m, oz);
    }
}

// Word w of dilate_slot's result, from the changed mask given as 32-bit
// words (chg[2q] | chg[2q+1] << 32 is mask word q).  With one z-plane a word,
// word w of the neighbour depends on planes w-1, w, w+1 only, so the 27 x
// WORDS words are computed by independent threads.
template <class S>
__host__ __device__ __forceinline__ uint64_t dilate_word(const uint32_t* chg, int ox, int oy, int oz, int w,
                                                         int nbh) {
    auto W = [&](int q) -> uint64_t { return (uint64_t)chg[2 * q] | ((uint64_t)chg[2 * q + 1] << 32); };
    if constexpr (S::WORDS == 1) {
        uint64_t m[1] = {W(0)};
        dilate_slot<S>(m, ox, oy, oz, nbh);
        return m[0];
    } else {
        if (nbh == 6) {
            if ((ox != 0) + (oy != 0) + (oz != 0) > 1) return 0ull;
            if (oz) return oz < 0 ? (w == S::WORDS - 1 ? W(0) : 0ull) : (w == 0 ? W(S::WORDS - 1) : 0ull);
            const uint64_t c = W(w);
            if (ox) return dil_x<S>(c, ox);
            if (oy) return dil_y<S>(c, oy);
            uint64_t r = dil_x<S>(c, 0) | dil_y<S>(c, 0);
            if (w > 0) r |= W(w - 1);
            if (w + 1 < S::WORDS) r |= W(w + 1);
            return r;
        }
        auto xy = [&](uint64_t c) { return dil_y<S>(dil_x<S>(c, ox), oy); };
        if (oz < 0) return w == S::WORDS - 1 ? xy(W(0)) : 0ull;
        if (oz > 0) return w == 0 ? xy(W(S::WORDS - 1)) : 0ull;
        uint64_t r = xy(W(w));
        if (w > 0) r |= xy(W(w - 1));
        if (w + 1 < S::WORDS) r |= xy(W(w + 1));
        return r;
    }
}

// Voxels of a brick inside the volume when only the first lim_x, lim_y,
// lim_z voxels of each axis are (the far edge of the volume), for word w.
template <class S>
__host__ __device__ __forceinline__ uint64_t inside_mask(int w, int lx, int ly, int lz) {
    using G = BitGeo<S>;
    const uint64_t mx = (uint64_t)((1u << lx) - 1u) * G::CX0;
    uint64_t my;
    if constexpr (S::XY == 64) my = ly >= S::Y ? ~0ull : (1ull << (S::X * ly)) - 1ull;
    else my = (uint64_t)((1u << (S::X * ly)) - 1u) * G::where([](int x, int y, int) { return x == 0 && y == 0; });
    uint64_t mz;
    if constexpr (S::WORDS == 1) mz = lz >= S::Z ? ~0ull : (1ull << (S::XY * lz)) - 1ull;
    else mz = w < lz ? ~0ull : 0ull;
    return mx & my & mz;
}

// x / g for x < 2^31, given gm = 0xFFFFFFFF / g + 1: the high half of x * gm
// overshoots x / g by less than one and is corrected once (g = 1: gm wraps).
__host__ __device__ __forceinline__ uint32_t div_magic(uint32_t x, uint32_t g, uint32_t gm) {
    if (g == 1u) return x;
#ifdef __CUDA_ARCH__
    const uint32_t d = __umulhi(x, gm);
#else
    const uint32_t d = (uint32_t)(((uint64_t)x * gm) >> 32);
#endif
    return d * g > x ? d - 1u : d;
}

// Brick origin of global brick b.
template <class S>
__device__ __forceinline__ int3 brick_origin(const NsVol& V, uint32_t b) {
    const uint32_t lb = b - V.brick_base;
    const uint32_t nbx = (uint32_t)V.nbx, nbxy = nbx * (uint32_t)V.nby;
    const uint32_t kz = div_magic(lb, nbxy, V.mnbxy), r = lb - kz * nbxy;
    const uint32_t ky = div_magic(r, nbx, V.mnbx), kx = r - ky * nbx;
    return make_int3((int)kx * S::X, (int)ky * S::Y, (int)kz * S::Z);
}

// A brick tile (origin x0, y0, z0 at tile column 4, row 1, plane 1) whose
// read region [-1, X] x [-1, Y] x [-1, Z] leaves the volume.
template <class S>
__device__ __forceinline__ bool tile_at_edge(const NsVol& V, int x0, int y0, int z0) {
    return x0 < 1 || y0 < 1 || z0 < 1 || x0 + S::X + 1 > V.nx || y0 + S::Y + 1 > V.ny || z0 + S::Z + 1 > V.nz;
}

// Clamp-to-edge halo: every element of the read region outside the volume
// (zero-filled by the TMA load) takes the value of the nearest voxel inside,
// which no thread writes, so one pass needs no ordering.  Threads t0,
// t0 + stride, ... each fix whole rows (y, z) of the region.
template <class S>
__device__ __forceinline__ void clamp_tile_halo(float* phi, const NsVol& V, int x0, int y0, int z0, int t0,
                                                int stride) {
    for (int r = t0; r < (S::Y + 2) * (S::Z + 2); r += stride) {
        const int ly = r % (S::Y + 2) - 1, lz = r / (S::Y + 2) - 1;
        const int gy = y0 + ly, gz = z0 + lz;
        const int cy = min(max(gy, 0), V.ny - 1), cz = min(max(gz, 0), V.nz - 1);
        float* d = phi + ((lz + 1) * S::TY + (ly + 1)) * S::TX + 4;
        const float* src = phi + ((cz - z0 + 1) * S::TY + (cy - y0 + 1)) * S::TX + 4;
        const bool row_out = cy != gy || cz != gz;
#pragma unroll
        for (int lx = -1; lx <= S::X; ++lx) {
            const int gx = x0 + lx, cx = min(max(gx, 0), V.nx - 1);
            if (row_out || cx != gx) d[lx] = src[cx - x0];
        }
    }
}

// Issues the TMA loads of brick b (halo tile of phi[p] and the speed)
// into buffer `buf` and records the brick's origin and volume beside them
// (thread 0 only: the brick's index arithmetic is done once, not by every
// thread).
template <class S, int NT>
__device__ __forceinline__ void ns_issue_loads(const NsArgs& a, NsSmem<S, NT>& sm, uint32_t b,
                                               uint32_t p, int buf, const NsVol* vone) {
    const uint32_t vol = vone ? 0u : a.brick_vol[b];
    const NsVol& V = vone ? *vone : a.vols[vol];
    const int3 o = brick_origin<S>(V, b);
    sm.org[buf] = make_int4(o.x, o.y, o.z, (int)vol);
    mbar_expect_tx(&sm.bar[buf], (uint32_t)(S::TILE + S::VOX) * 4u);
    tma_load_3d(sm.phi[buf], &a.tmaps[V.tmap_base + p], o.x - 4, o.y - 1, o.z - 1, &sm.bar[buf]);
    tma_load_3d(sm.spd[buf], &a.tmaps[V.tmap_base + 4], o.x, o.y, o.z, &sm.bar[buf]);
}

// Per-block running totals of updated voxels and bricks of one volume,
// flushed with one atomic each when the volume changes or the phase ends.
// `iter` sums the block's updates over all volumes of the iteration.  cnt
// may be null (one volume: the count travels with the barrier arrival).
// Plain data (it may live in shared memory): reset() before first use.
struct BlockTally {
    uint32_t v;
    unsigned long long upd, brk, iter;
    __device__ void reset() {
        v = 0xFFFFFFFFu;
        upd = brk = iter = 0;
    }
    __device__ void add(NsVolState* vs, unsigned long long* cnt, uint32_t vol, unsigned long long n) {
        if (vol != v) {
            flush(vs, cnt);
            v = vol;
        }
        upd += n;
        brk += 1;
        iter += n;
    }
    __device__ void flush(NsVolState* vs, unsigned long long* cnt) {
        if (v != 0xFFFFFFFFu && brk) {
            atomicAdd(&vs[v].updates, upd);
            atomicAdd(&vs[v].bricks, brk);
            if (cnt) atomicAdd(&cnt[v], upd);
        }
        upd = brk = 0;
    }
};

// The threads that work on one brick together, and how they synchronise:
// the whole block (BlockTeam: __syncthreads), or one of several groups of NT
// threads in a block (GroupTeam: named barrier 1 + g, NT threads), so that
// one block per SM can run several bricks at once with one rank selection
// and one grid-barrier participant.  Named barriers order shared and global
// memory among their threads as __syncthreads does.
struct BlockTeam {
    __device__ int tid() const { return threadIdx.x; }
    __device__ void sync() const { __syncthreads(); }
    __device__ int sync_or(int pred) const { return __syncthreads_or(pred); }
};

template <int NT>
struct GroupTeam {
    int g;  // group index; barrier id 1 + g
    __device__ int tid() const { return (int)threadIdx.x - g * NT; }
    __device__ void sync() const { asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(NT) : "memory"); }
    __device__ int sync_or(int pred) const {
        int r;
        asm volatile(
            "{\n\t.reg .pred p, q;\n\t"
            "setp.ne.s32 q, %1, 0;\n\t"
            "bar.red.or.pred p, %2, %3, q;\n\t"
            "selp.s32 %0, 1, 0, p;\n\t}"
            : "=r"(r)
            : "r"(pred), "r"(1 + g), "r"(NT)
            : "memory");
        return r;
    }
};

// Work on one brick of A_k whose loads were issued into `buf`.
// The brick's mask words -> act[buf] (threads < WORDS), cleared in global
// memory: the mask array of parity p becomes the accumulator of iteration k+1.
template <class S, int NT>
__device__ __forceinline__ void ns_fetch_mask(const NsArgs& a, NsSmem<S, NT>& sm, uint32_t b, uint32_t p,
                                              int buf, int tid) {
    if (tid < S::WORDS) {
        unsigned long long* cur = a.masks[p] + (size_t)b * S::WORDS;
        sm.act[buf][tid] = cur[tid];
        cur[tid] = 0ull;
    }
}

// The xy-dilated plane of mask word c for the pair of xy offsets `pair`
// ((ox + 1) + 3 (oy + 1)): its part that lands in that neighbour column.
template <class S>
__host__ __device__ __forceinline__ uint64_t xy_plane(uint64_t c, int pair, int nbh) {
    const int ox = pair % 3 - 1, oy = pair / 3 - 1;
    if (nbh == 26) return dil_y<S>(dil_x<S>(c, ox), oy);
    if (ox == 0 && oy == 0) return dil_x<S>(c, 0) | dil_y<S>(c, 0);
    if (ox == 0 || oy == 0) return ox ? dil_x<S>(c, ox) : dil_y<S>(c, oy);
    return 0ull;
}

// Word w of the neighbour at (ox, oy, oz), with one z-plane per mask word,
// from the 9 x WORDS xy-dilated planes xyp (xy_plane, WORDS per pair) and
// the changed mask word W(q): an OR of up to three planes.  Equals
// dilate_word.
template <class S, class WF>
__host__ __device__ __forceinline__ uint64_t plane_word(const unsigned long long* xyp, WF W, int ox, int oy, int oz,
                                                        int w, int nbh) {
    const unsigned long long* xy = xyp + ((oy + 1) * 3 + (ox + 1)) * S::WORDS;
    const bool center = ox == 0 && oy == 0;
    if (nbh == 26)
        return oz == 0 ? (xy[w] | (w > 0 ? xy[w - 1] : 0ull) | (w < S::WORDS - 1 ? xy[w + 1] : 0ull))
                       : (oz < 0 ? (w == S::WORDS - 1 ? xy[0] : 0ull) : (w == 0 ? xy[S::WORDS - 1] : 0ull));
    if (oz == 0) return xy[w] | (center ? ((w > 0 ? W(w - 1) : 0ull) | (w < S::WORDS - 1 ? W(w + 1) : 0ull)) : 0ull);
    return center ? (oz < 0 ? (w == S::WORDS - 1 ? W(0) : 0ull) : (w == 0 ? W(S::WORDS - 1) : 0ull)) : 0ull;
}

// The work items of a brick's neighbour words.  With one z-plane per mask
// word a neighbour above or below the brick receives one word only (the
// plane next to the brick), so the 9 neighbours of the brick's own layer
// take WORDS items each and the 18 others one item each; otherwise item t is
// word t % WORDS of neighbour t / WORDS.  Item t (< dilate_items<S>()) ->
// neighbour slot (ox + 1) + 3 (oy + 1) + 9 (oz + 1) and word w; returns
// whether it is the only word of its neighbour.
template <class S>
__host__ __device__ constexpr int dilate_layer_items() {
    return S::XY == 64 ? 9 * S::WORDS : 27 * S::WORDS;
}
template <class S>
__host__ __device__ constexpr int dilate_items() {
    return S::XY == 64 ? dilate_layer_items<S>() + 18 : dilate_layer_items<S>();
}
template <class S>
__host__ __device__ __forceinline__ bool dilate_item(int t, int& slot, int& w) {
    constexpr int LAYER = dilate_layer_items<S>();
    if (t < LAYER) {
        slot = (S::XY == 64 ? 9 : 0) + t / S::WORDS;  // with planes: the layer oz = 0
        w = t % S::WORDS;
        return false;
    }
    const int q = t - LAYER;  // q < 9: the layer below, else above
    slot = q < 9 ? q : q + 9;
    w = q < 9 ? S::WORDS - 1 : 0;
    return true;
}

// Phase 1 of a brick's dilation with one z-plane per mask word (XY == 64):
// the 9 x WORDS xy-dilated planes of the changed mask cw (ballot words),
// once each, into xy.  Threads t0, t0 + stride, ...
template <class S>
__device__ __forceinline__ void dilate_planes(const NsVol& V, const uint32_t* cw, unsigned long long* xy,
                                              int t0, int stride) {
    for (int t = t0; t < 9 * S::WORDS; t += stride) {
        const int w = t % S::WORDS;
        xy[t] = xy_plane<S>((uint64_t)cw[2 * w] | ((uint64_t)cw[2 * w + 1] << 32), t / S::WORDS, V.nbh);
    }
}

// Phase 2: each thread computes one word of one neighbour of brick b (origin
// x0, y0, z0; the items of dilate_item) and ORs it into the next masks
// (parity p ^ 1); one thread per neighbour sets its membership bit in
// bits[sn] (reductions, no round trip).  Threads t0, t0 + STRIDE, ...;
// STRIDE is a multiple of 32 and every lane of a calling warp takes part
// (ballots).
template <class S, int STRIDE>
__device__ __forceinline__ void dilate_scatter(const NsArgs& a, const NsVol& V, const uint32_t* cw,
                                               const unsigned long long* xyp, uint32_t b, int x0, int y0,
                                               int z0, uint32_t p, uint32_t sn, int t0) {
    static_assert(STRIDE % 32 == 0, "whole warps");
    auto W = [&](int q) -> uint64_t { return (uint64_t)cw[2 * q] | ((uint64_t)cw[2 * q + 1] << 32); };
    constexpr int ITEMS = dilate_items<S>();
    constexpr int ROUNDS = (ITEMS + STRIDE - 1) / STRIDE;
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
        const int t = t0 + r * STRIDE;
        int slot, w;
        const bool single = dilate_item<S>(t, slot, w);
        uint64_t x = 0ull;
        uint32_t nb = 0;
        if (t < ITEMS) {
            const int ox = slot % 3 - 1, oy = (slot / 3) % 3 - 1, oz = slot / 9 - 1;
            const int bx = x0 / S::X + ox, by = y0 / S::Y + oy, bz = z0 / S::Z + oz;
            // Voxels of the neighbour inside the volume along each axis
            // (bricks in the padding beyond the volume hold none).
            const int lx = V.nx - bx * S::X, ly = V.ny - by * S::Y, lz = V.nz - bz * S::Z;
            if (bx >= 0 && by >= 0 && bz >= 0 && lx > 0 && ly > 0 && lz > 0) {
                if constexpr (S::XY == 64) x = plane_word<S>(xyp, W, ox, oy, oz, w, V.nbh);
                else x = dilate_word<S>(cw, ox, oy, oz, w, V.nbh);
                if (lx < S::X || ly < S::Y || lz < S::Z)
                    x &= inside_mask<S>(w, min(lx, S::X), min(ly, S::Y), min(lz, S::Z));
                nb = b + (int32_t)((oz * V.nby + oy) * V.nbx + ox);
                if (x) atomicOr(&a.masks[p ^ 1u][(size_t)nb * S::WORDS + w], (unsigned long long)x);
            }
        }
        // The WORDS threads of a grouped neighbour are adjacent lanes of one
        // warp (the layer's item count is a multiple of WORDS).
        const uint32_t bal = __ballot_sync(0xffffffffu, x != 0ull);
        const int lane = t & 31, g0 = lane & ~(S::WORDS - 1);
        const uint32_t gmask = (S::WORDS >= 32 ? 0xffffffffu : ((1u << S::WORDS) - 1u)) << g0;
        if (single ? x != 0ull : (lane == g0 && (bal & gmask)))
            atomicOr(&a.bits[sn][nb >> 5], 1u << (nb & 31));
    }
}

// One brick of A_k by the whole block: wait for its loads, update its active
// voxels in place of a copy of the tile centre (each thread its own voxels:
// compacting the active voxels first measured slower, it costs two more block
// barriers per brick), changed flags -> ballot words, TMA store, dilation.
// vone: the volume descriptor in shared memory when the launch has one
// volume (else null: descriptors are read per brick).
template <class S, int NT, class Team = BlockTeam>
__device__ __forceinline__ void ns_process_brick(const NsArgs& a, NsSmem<S, NT>& sm, uint32_t b,
                                                 uint32_t p, uint32_t sn, int buf, uint32_t& mphase,
                                                 BlockTally& tally, unsigned long long* cnt,
                                                 const NsVol* vone, const Team team = Team{}) {
    const int tid = team.tid();
    // Written by thread 0 with the loads, before a block barrier.
    const int4 og = sm.org[buf];
    const uint32_t v = (uint32_t)og.w;
    const NsVol& V = vone ? *vone : a.vols[v];
    const int x0 = og.x, y0 = og.y, z0 = og.z;
    const unsigned long long* act = sm.act[buf];
    // Every thread waits for the loads itself.  out[buf] is free: the store
    // issued from it two bricks ago was waited for (read) by the store thread
    // before the previous brick's block barrier.
    if (!mbar_wait(&sm.bar[buf], (mphase >> buf) & 1u)) set_error(&a.ctl->err, ERR_TMA_TIMEOUT);
    mphase ^= 1u << buf;  // bit b: phase of load barrier b
    float* phi = sm.phi[buf];
    if (tile_at_edge<S>(V, x0, y0, z0)) {
        clamp_tile_halo<S>(phi, V, x0, y0, z0, tid, NT);
        team.sync();
    }
    float* out = sm.out[buf];
    auto tile_index = [](int j) {
        const int lx = j % S::X, ly = (j / S::X) % S::Y, lz = j / (S::X * S::Y);
        return ((lz + 1) * S::TY + (ly + 1)) * S::TX + (lx + 4);
    };
    // The store thread's warp: the brick's active voxels (one mask word a
    // lane), read before the block barrier and tallied after it.
    constexpr int STORE_TID = NsSmem<S, NT>::STORE_TID;
    static_assert(NT >= 64 && S::WORDS <= 32 && (S::XY != 64 || 9 * S::WORDS <= STORE_TID), "store warp");
    uint32_t nact = 0;
    if ((tid >> 5) == (STORE_TID >> 5))
        nact = __reduce_add_sync(0xffffffffu, (tid & 31) < S::WORDS ? __popcll(act[tid & 31]) : 0u);
    constexpr int VPT = (S::VOX + NT - 1) / NT;
    bool anyl = false;
    if constexpr (VPT == 2 && S::VOX == 2 * NT && S::Z % 2 == 0) {
        // Two voxels a thread, z-adjacent at the same (x, y): updated in one
        // straight-line block (their chains interleave) when either is
        // active, the ten tile reads they share loaded once.
        const int lo = tid % S::XY;
        const int j0 = lo + 2 * S::XY * (tid / S::XY), j1 = j0 + S::XY;
        const int t0 = tile_index(j0), t1 = t0 + S::TY * S::TX;
        const float c0 = phi[t0], c1 = phi[t1];
        const bool a0 = (act[j0 >> 6] >> (j0 & 63)) & 1ull, a1 = (act[j1 >> 6] >> (j1 & 63)) & 1ull;
        float nv0 = c0, nv1 = c1;
        bool ch0 = false, ch1 = false;
        if (a0 || a1) {
            auto P0 = [&](int dx, int dy, int dz) { return phi[t0 + (dz * S::TY + dy) * S::TX + dx]; };
            auto P1 = [&](int dx, int dy, int dz) { return phi[t1 + (dz * S::TY + dy) * S::TX + dx]; };
            const float u0 = ns_update_speed_f32(P0, sm.spd[buf][j0], V);
            const float u1 = ns_update_speed_f32(P1, sm.spd[buf][j1], V);
            if (a0) {
                nv0 = u0;
                ch0 = fabsf(nv0 - c0) > V.thr_t;
            }
            if (a1) {
                nv1 = u1;
                ch1 = fabsf(nv1 - c1) > V.thr_t;
            }
        }
        out[j0] = nv0;
        out[j1] = nv1;
        const uint32_t bal0 = __ballot_sync(0xffffffffu, ch0), bal1 = __ballot_sync(0xffffffffu, ch1);
        anyl = (bal0 | bal1) != 0u;
        if ((tid & 31) == 0) {
            sm.chg[buf][j0 >> 5] = bal0;
            sm.chg[buf][j1 >> 5] = bal1;
        }
    } else {
#pragma unroll
    for (int k = 0; k < VPT; ++k) {
        const int j = tid + k * NT;
        bool chg = false;
        if (j < S::VOX) {
            const int ti = tile_index(j);
            const float c = phi[ti];
            float nv = c;
            if ((act[j >> 6] >> (j & 63)) & 1ull) {
                auto P = [&](int dx, int dy, int dz) { return phi[ti + (dz * S::TY + dy) * S::TX + dx]; };
                nv = ns_update_speed_f32(P, sm.spd[buf][j], V);
                chg = fabsf(nv - c) > V.thr_t;
            }
            out[j] = nv;
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, chg);
        anyl |= bal != 0u;
        const int word = (tid >> 5) + k * (NT / 32);
        if ((tid & 31) == 0 && word < S::CHG) sm.chg[buf][word] = bal;
    }
    }
    fence_proxy_async_smem();
    // The previous brick's store (from out[buf ^ 1], overwritten by the next
    // brick after this barrier) has read its source.
    if (tid == STORE_TID) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    // The one block barrier of a brick: out[] and chg[buf] complete; after it
    // nothing reads phi[buf], spd[buf] or act[buf] of this brick, so the next
    // loads into this buffer may be issued while the dilation below runs.
    const int any = team.sync_or(anyl ? 1 : 0);
    if (tid == STORE_TID) {
        tma_store_3d(&a.tmaps[V.tmap_base + 2 + (p ^ 1u)], x0, y0, z0, out);
        tma_store_commit();
        tally.add(a.vstate, cnt, v, nact);
    }
    // Dilation of the changed mask into the 27 bricks around (and including)
    // b (dilate_planes, dilate_scatter).
    if (any) {
        if constexpr (S::XY == 64) {
            dilate_planes<S>(V, sm.chg[buf], sm.xy, tid, NT);
            team.sync();  // uniform: `any` is
        }
        dilate_scatter<S, NT>(a, V, sm.chg[buf], sm.xy, b, x0, y0, z0, p, sn, tid);
    }
    // No barrier here: the next brick uses the other buffers, and this
    // brick's buffers are reused two bricks later, behind the next brick's
    // barrier.
}

// A brick of A_{k-1} not in A_k: phi[p] -> phi[p^1].
// Threads t0, t0 + stride, ... copy.
template <class S>
__device__ __forceinline__ void ns_flush_brick(const NsArgs& a, uint32_t b, uint32_t p, const NsVol* vone,
                                               int t0, int stride) {
    const NsVol& V = vone ? *vone : a.vols[a.brick_vol[b]];
    const int3 o = brick_origin<S>(V, b);
    const float* src = V.phi[p];
    float* dst = V.phi[p ^ 1u];
    constexpr int Q = S::X / 4;  // float4 per row
    for (int t = t0; t < S::Y * S::Z * Q; t += stride) {
        const int q = t % Q, ly = (t / Q) % S::Y, lz = t / (Q * S::Y);
        const size_t off = ((size_t)(o.z + lz) * V.py + (o.y + ly)) * V.px + o.x + 4 * q;
        *reinterpret_cast<float4*>(dst + off) = *reinterpret_cast<const float4*>(src + off);
    }
}

// Per-volume stopping state kept identically by every block (dynamic shared
// memory): done, streak, stop iteration, last count.
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

// Unpadded fields (x fastest, rows of nx) <-> padded device fields (pitch px,
// py).  Block i takes the rows (y, z) i, i + gridDim.x, ... and its threads
// cover x, so there is one division a row, none an element.  The unpadded
// side may be pinned host memory read or written in place.
template <class T>
__global__ void k_ns_scatter(T* dst, const T* src, int nx, int ny, int nz, int px, int py) {
    const uint32_t rows = (uint32_t)ny * (uint32_t)nz;
    for (uint32_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const uint32_t z = r / (uint32_t)ny, y = r - z * (uint32_t)ny;
        const T* s = src + (size_t)r * nx;
        T* d = dst + ((size_t)z * py + y) * px;
        for (int x = threadIdx.x; x < nx; x += blockDim.x) d[x] = s[x];
    }
}

template <class T>
__global__ void k_ns_gather(T* dst, const T* src, int nx, int ny, int nz, int px, int py) {
    const uint32_t rows = (uint32_t)ny * (uint32_t)nz;
    for (uint32_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const uint32_t z = r / (uint32_t)ny, y = r - z * (uint32_t)ny;
        const T* s = src + ((size_t)z * py + y) * px;
        T* d = dst + (size_t)r * nx;
        for (int x = threadIdx.x; x < nx; x += blockDim.x) d[x] = s[x];
    }
}

constexpr uint32_t kNoBrick = 0xFFFFFFFFu;  // a brick of a finished volume

// Position of the s-th set bit (from 0, counted from bit 0) of m; s < popc(m).
__host__ __device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t s) {
    uint32_t pos = 0;
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) {
        const uint32_t low = m & ((1u << h) - 1u);
#ifdef __CUDA_ARCH__
        const uint32_t c = __popc(low);
#else
        const uint32_t c = (uint32_t)__builtin_popcount(low);
#endif
        if (s >= c) {
            s -= c;
            pos += (uint32_t)h;
            m >>= h;
        }
    }
    return pos;
}
constexpr int kScanCache = 4;               // membership words per thread kept in shared memory
constexpr int kSearchBatch = 8;             // words past the cache loaded at once by a rank search

// Shared state of the iteration driver (static shared memory).
template <int NT>
struct IterShared {
    NsVol vol;                     // the descriptor of a one-volume launch
    uint32_t gen, abort;
    unsigned long long rel, n0, upd, t0, t1;  // t0, t1: block 0's phase clock
    unsigned long long upd_seen[2];           // counter barrier: upd_sum read so far, by parity
    int32_t live;
    uint32_t work[NT], flush[NT];  // this block's bricks of the chunk
    uint2 scan[kScanCache][NT];    // (A_k word, A_{k-1} \ A_k word) per thread
};

// The iteration driver shared by the persistent kernels.  Per iteration k:
//   every block ranks the bricks of A_k (and of A_{k-1} \ A_k) with a block
//     prefix sum over the membership words and takes the ranks i, i+G, ...
//     (block i of G): every block gets ceil(n/G) or floor(n/G) bricks, with
//     no global list and no atomics;
//   Proc::chunk updates the block's bricks of A_k and copies its bricks of
//     A_{k-1} \ A_k across (phi[p] -> phi[p^1]), so both buffers stay current;
//   Proc::finish closes the iteration (tallies, TMA stores complete);
//   one bounded grid barrier; its arrival word carries the block's voxel
//     updates, so the last block to arrive evaluates the one-volume stopping
//     rule and releases the others with the decision in the release word
//     (several volumes: every block evaluates the rule on the same counts).
// Slots at iteration k: membership bits B[k%4] = A_k, B[(k+1)%4] = A_{k+1}
// (being built), B[(k+3)%4] = A_{k-1}, B[(k+2)%4] cleared for reuse; voxel
// counts cnt[k%3].  Stopping rule after iteration k, per volume: n_k = active
// voxels updated at k; streak = consecutive iterations with n_k < rel * n0;
// stop when streak >= patience, n_k <= abs_thr, or the budget is used.
template <int NT, class Proc>
__device__ __forceinline__ void ns_drive(const NsArgs& a, IterShared<NT>& sh, StopState ss, Proc& proc) {
    const int tid = threadIdx.x;
    const uint32_t G = gridDim.x;
    if (tid == 0) {
        sh.gen = (uint32_t)ld_acquire_u64((const uint64_t*)&a.ctl->bar_release);
        sh.abort = 0;
        sh.upd = 0;
        sh.n0 = a.vstate[0].n0;
        sh.upd_seen[0] = a.upd_sum0[0];
        sh.upd_seen[1] = a.upd_sum0[1];
        if (a.nvol == 1) sh.vol = a.vols[0];
        for (int v = 0; v < a.nvol; ++v)
            for (int m = 0; m < 5; ++m) tmap_acquire(&a.tmaps[a.vols[v].tmap_base + m]);
    }
    for (int v = tid; v < a.nvol; v += NT) {
        ss.done[v] = 0;
        ss.streak[v] = 0;
        ss.stop[v] = -1;
        ss.n[v] = 0;
    }
    proc.init();
    __syncthreads();
    uint32_t gen = sh.gen;
    const bool one = a.nvol == 1;  // one volume: the stopping rule rides on the barrier
    const NsVol* vone = one ? &sh.vol : nullptr;
    uint32_t streak = 0;
    const uint32_t patience = (uint32_t)min(max(a.patience, 0), 0xFFFF);
    int ran = 0;
    for (int it = 0; it < a.max_iters; ++it) {
        const uint32_t k = a.k0 + (uint32_t)it;
        const uint32_t p = k & 1u, c3 = k % 3u, c3n = (k + 1u) % 3u;
        const uint32_t* cur = a.bits[k % 4u];
        const uint32_t* prev = a.bits[(k + 3u) % 4u];
        const uint32_t sn = (k + 1u) % 4u, sz = (k + 2u) % 4u;
        unsigned long long* cnt = one ? nullptr : a.cnt[c3];
        if (blockIdx.x == 0 && tid == 0) sh.t0 = globaltimer_ns();
        if (blockIdx.x == 0)
            for (int v = tid; v < a.nvol; v += NT) a.cnt[c3n][v] = 0ull;
        // Ranks: thread t counts the words t, t+NT, ...; ranks follow (thread,
        // word).  The first kScanCache words of each thread stay in shared
        // memory for the second pass.
        uint32_t ca = 0, cf = 0;
#pragma unroll
        for (int m = 0; m < kScanCache; ++m) {
            const uint32_t w = tid + (uint32_t)m * NT;
            const uint32_t c = w < a.NW ? cur[w] : 0u;
            const uint32_t f = w < a.NW ? prev[w] & ~c : 0u;
            sh.scan[m][tid] = make_uint2(c, f);
            ca += __popc(c);
            cf += __popc(f);
        }
        for (uint32_t w = tid + kScanCache * NT; w < a.NW; w += NT) {
            const uint32_t c = cur[w];
            ca += __popc(c);
            cf += __popc(prev[w] & ~c);
        }
        uint64_t tot;
        // (No closing barrier: the next call is many block barriers away.)
        const uint64_t ex = block_exclusive_sum64<false>(((uint64_t)cf << 32) | ca, &tot);
        const uint32_t na = (uint32_t)tot, nfl = (uint32_t)(tot >> 32);
        // Block i takes the ranks i, i+G, i+2G, ... of both kinds.
        const uint32_t bi = blockIdx.x;
        const uint32_t gm = 0xFFFFFFFFu / G + 1u;
        auto divg = [&](uint32_t x) { return div_magic(x, G, gm); };
        const uint32_t mya = na > bi ? divg(na - bi + G - 1) : 0u;
        const uint32_t myf = nfl > bi ? divg(nfl - bi + G - 1) : 0u;
        for (uint32_t c0 = 0; c0 < mya || c0 < myf; c0 += NT) {
            // Chunk c0: this block's j-th brick for j in [c0, c0 + NT).
            const uint32_t nw = min(mya - min(mya, c0), (uint32_t)NT);
            const uint32_t nf = min(myf - min(myf, c0), (uint32_t)NT);
            {
                const uint32_t lo = bi + c0 * G;
                const uint32_t hia = bi + (c0 + nw) * G, hif = bi + (c0 + nf) * G;
                // This thread's ranks are [ra, ra + ca) and [rf, rf + cf),
                // its words in order; the block's ranks q = bi (mod G) among
                // them (at most one while a thread holds fewer than G bricks)
                // are located word by word.
                const uint32_t ra = (uint32_t)ex, rf = (uint32_t)(ex >> 32);
                auto take = [&](uint32_t r0, uint32_t n, uint32_t hi, bool fl, uint32_t* out) {
                    uint32_t q = max(r0, lo);
                    q = bi + divg(q - bi + G - 1) * G;
                    for (; q < r0 + n && q < hi; q += G) {
                        uint32_t s = q - r0, b = 0xFFFFFFFFu;
                        for (int m = 0; m < kScanCache; ++m) {
                            const uint2 cf2 = sh.scan[m][tid];
                            const uint32_t bits = fl ? cf2.y : cf2.x;
                            const uint32_t c = __popc(bits);
                            if (s < c) {
                                b = (tid + (uint32_t)m * NT) * 32u + nth_set_bit(bits, s);
                                break;
                            }
                            s -= c;
                        }
                        // Words past the cache, kSearchBatch at a time:
                        // their loads are independent, so a search costs
                        // one memory round trip per batch, not per word.
                        for (uint32_t w0 = tid + kScanCache * NT; b == 0xFFFFFFFFu && w0 < a.NW;
                             w0 += kSearchBatch * NT) {
                            uint32_t bw[kSearchBatch];
#pragma unroll
                            for (int u = 0; u < kSearchBatch; ++u) {
                                const uint32_t w = w0 + (uint32_t)u * NT;
                                const uint32_t cw = w < a.NW ? cur[w] : 0u;
                                bw[u] = fl ? (w < a.NW ? prev[w] : 0u) & ~cw : cw;
                            }
#pragma unroll
                            for (int u = 0; u < kSearchBatch; ++u) {
                                const uint32_t c = __popc(bw[u]);
                                if (b == 0xFFFFFFFFu) {
                                    if (s < c) b = (w0 + (uint32_t)u * NT) * 32u + nth_set_bit(bw[u], s);
                                    else s -= c;
                                }
                            }
                        }
                        const uint32_t slot = divg(q - bi) - c0;
                        if (slot >= (uint32_t)NT || b >= a.NB) {  // a rank outside this chunk: report, skip
                            set_error(&a.ctl->err, ERR_BOUNDS);
                            continue;
                        }
                        out[slot] = (!one && ss.done[a.brick_vol[b]]) ? kNoBrick : b;
                    }
                };
                take(ra, ca, hia, false, sh.work);
                take(rf, cf, hif, true, sh.flush);
            }
            __syncthreads();
            proc.chunk(a, sh, nw, nf, p, sn, cnt, vone);  // ends with a block barrier
        }
        proc.finish(a, sh, cnt);
        for (uint32_t w = blockIdx.x * NT + tid; w < a.NW; w += G * NT) a.bits[sz][w] = 0u;
        if (blockIdx.x == 0 && tid == 0) sh.t1 = globaltimer_ns();
        __syncthreads();
        if (tid == 0 && G <= kCounterBarrierMax) {
            // Counter barrier: the block's count, then a release add of one
            // arrival; every block polls the counter until the iteration's
            // arrivals are all in and evaluates the one-volume stopping rule
            // on the same sum (the counts of one parity slot cannot gain the
            // next iteration's before every block has read them).
            const unsigned long long mine = sh.upd;
            sh.upd = 0;
            const uint32_t target = gen + 1;
            const uint32_t par = k & 1u;
            if (one && mine)
                asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(&a.ctl->upd_sum[par]), "l"(mine)
                             : "memory");
            asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(&a.ctl->arrivals), "l"(1ull) : "memory");
            const unsigned long long want = a.arrivals0 + (unsigned long long)G * (unsigned long long)(it + 1);
            const uint64_t w0 = globaltimer_ns();
            uint32_t ns = 16;
            unsigned long long rel = target;
            for (;;) {
                if (ld_acquire_u64((const uint64_t*)&a.ctl->arrivals) >= want) break;
                if (globaltimer_ns() - w0 > kWaitLimitNs) {
                    set_error(&a.ctl->err, ERR_BARRIER_TIMEOUT);
                    sh.abort = 1;
                    break;
                }
                __nanosleep(ns);
                if (ns < 64) ns <<= 1;
            }
            if (one) {
                const unsigned long long tot = *(volatile unsigned long long*)&a.ctl->upd_sum[par];
                const unsigned long long n = tot - sh.upd_seen[par];
                sh.upd_seen[par] = tot;
                if (blockIdx.x == 0) a.ctl->n_last = n;
                uint32_t st = streak;
                bool stop = it + 1 >= a.max_iters;
                if (a.conv_mode) {
                    st = ((double)n < a.rel * (double)sh.n0) ? min(st + 1u, 0xFFFFu) : 0u;
                    stop = stop || st >= patience || n <= a.abs_thr;
                }
                rel = (unsigned long long)target | ((unsigned long long)st << kRelStreakShift) |
                      (stop ? kRelStop : 0ull);
            }
            sh.rel = rel;
            gen = target;
            asm volatile("fence.proxy.async.global;" ::: "memory");
            if (blockIdx.x == 0) {
                const uint64_t t2 = globaltimer_ns();
                a.ctl->t_phase1_ns += sh.t1 - sh.t0;
                a.ctl->t_barrier_ns += t2 - sh.t1;
            }
        } else if (tid == 0) {
            const unsigned long long mine = sh.upd;
            sh.upd = 0;
            const uint32_t target = gen + 1;
            // Arrival: one acquire-release add (the block's writes, ordered
            // before it by the block barrier, are released; the last block
            // to arrive acquires everyone's).
            unsigned long long old;
            asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], %2;"
                         : "=l"(old)
                         : "l"(&a.ctl->bar_arrive), "l"((mine << kArriveShift) | 1ull)
                         : "memory");
            unsigned long long rel;
            if ((old & kArriveMask) == G - 1) {
                // Last to arrive: evaluate the one-volume stopping rule, release.
                a.ctl->bar_arrive = 0ull;
                uint32_t st = streak;
                bool stop = it + 1 >= a.max_iters;
                if (one) {
                    const unsigned long long n = (old >> kArriveShift) + mine;
                    a.ctl->n_last = n;
                    if (a.conv_mode) {
                        st = ((double)n < a.rel * (double)sh.n0) ? min(st + 1u, 0xFFFFu) : 0u;
                        stop = stop || st >= patience || n <= a.abs_thr;
                    }
                }
                rel = (unsigned long long)target | ((unsigned long long)st << kRelStreakShift) |
                      (stop ? kRelStop : 0ull);
                st_release_u64((uint64_t*)&a.ctl->bar_release, rel);  // orders the stores above
            } else {
                const uint64_t w0 = globaltimer_ns();
                uint32_t ns = 16;
                for (;;) {
                    rel = ld_acquire_u64((const uint64_t*)&a.ctl->bar_release);
                    if ((uint32_t)rel == target) break;
                    if (globaltimer_ns() - w0 > kWaitLimitNs) {
                        set_error(&a.ctl->err, ERR_BARRIER_TIMEOUT);
                        sh.abort = 1;
                        break;
                    }
                    __nanosleep(ns);
                    if (ns < 64) ns <<= 1;
                }
            }
            sh.rel = rel;
            gen = target;
            asm volatile("fence.proxy.async.global;" ::: "memory");
            if (blockIdx.x == 0) {
                const uint64_t t2 = globaltimer_ns();
                a.ctl->t_phase1_ns += sh.t1 - sh.t0;
                a.ctl->t_barrier_ns += t2 - sh.t1;
            }
        }
        __syncthreads();
        // A block that gave up leaves; the others then give up at the next
        // barrier (bounded), so every block ends.
        if (sh.abort) { ran = it; break; }
        if (one) {
            const unsigned long long rel = sh.rel;
            streak = (uint32_t)(rel >> kRelStreakShift) & 0xFFFFu;
            ran = it + 1;
            if (rel & kRelStop) {
                if (tid == 0) {
                    ss.done[0] = 1;
                    ss.stop[0] = it;
                }
                break;
            }
            continue;
        }
        // Stopping rule, evaluated identically by every block.
        if (tid == 0) sh.live = 0;
        __syncthreads();
        for (int v = tid; v < a.nvol; v += NT) {
            if (ss.done[v]) continue;
            const unsigned long long n = *(volatile unsigned long long*)&a.cnt[c3][v];
            ss.n[v] = n;
            bool stop;
            if (a.conv_mode) {
                const unsigned long long nv0 = a.vstate[v].n0;
                ss.streak[v] = ((double)n < a.rel * (double)nv0) ? ss.streak[v] + 1 : 0;
                stop = ss.streak[v] >= a.patience || n <= a.abs_thr || it + 1 >= a.max_iters;
            } else {
                stop = it + 1 >= a.max_iters;
            }
            if (stop) {
                ss.done[v] = 1;
                ss.stop[v] = it;
            } else {
                atomicAdd(&sh.live, 1);
            }
        }
        __syncthreads();
        ran = it + 1;
        if (sh.live == 0) break;
    }
    __syncthreads();
    if (one && tid == 0) {
        ss.n[0] = *(volatile unsigned long long*)&a.ctl->n_last;
        ss.streak[0] = (int32_t)streak;
    }
    __syncthreads();
    if (blockIdx.x == 0) {
        for (int v = tid; v < a.nvol; v += NT) {
            NsVolState& st = a.vstate[v];
            const int r = ss.stop[v] >= 0 ? ss.stop[v] + 1 : ran;
            st.iterations += (unsigned long long)r;
            st.parity = (int32_t)((a.k0 + (uint32_t)r) & 1u);
            st.n_cur = ss.n[v];
            st.streak = ss.streak[v];
            st.done = a.conv_mode ? ss.done[v] : 0;
        }
        if (tid == 0) a.ctl->iters_run = (uint32_t)ran;
    }
}

// Block-per-brick processing: all NT threads of the block work on one brick
// at a time (the next brick's loads in flight).
template <class S, int NT>
struct BlockProc {
    NsSmem<S, NT>& sm;
    BlockTally& tally;  // the store thread's; in shared memory, off the threads' registers
    uint32_t mphase;    // bit b: phase of load barrier b
    int buf;
    __device__ BlockProc(NsSmem<S, NT>& s, BlockTally& t) : sm(s), tally(t), mphase(0u), buf(0) {}
    __device__ void init() {
        if (threadIdx.x == 0) {
            mbar_init(&sm.bar[0], 1);
            mbar_init(&sm.bar[1], 1);
            tally.reset();
        }
    }
    __device__ void chunk(const NsArgs& a, IterShared<NT>& sh, uint32_t nw, uint32_t nf, uint32_t p,
                          uint32_t sn, unsigned long long* cnt, const NsVol* vone) {
        const int tid = threadIdx.x;
        uint32_t q = 0;
        while (q < nw && sh.work[q] == kNoBrick) ++q;
        if (q < nw) {
            if (tid == 0) ns_issue_loads<S, NT>(a, sm, sh.work[q], p, buf, vone);
            ns_fetch_mask<S, NT>(a, sm, sh.work[q], p, buf, tid);
            __syncthreads();  // act[buf] of the first brick (later ones are fetched a brick ahead)
        }
        while (q < nw) {
            uint32_t q2 = q + 1;
            while (q2 < nw && sh.work[q2] == kNoBrick) ++q2;
            if (q2 < nw) {
                if (tid == 0) ns_issue_loads<S, NT>(a, sm, sh.work[q2], p, buf ^ 1, vone);
                ns_fetch_mask<S, NT>(a, sm, sh.work[q2], p, buf ^ 1, tid);
            }
            ns_process_brick<S, NT>(a, sm, sh.work[q], p, sn, buf, mphase, tally, cnt, vone);
            buf ^= 1;
            q = q2;
        }
        for (uint32_t r = 0; r < nf; ++r)
            if (sh.flush[r] != kNoBrick) ns_flush_brick<S>(a, sh.flush[r], p, vone, tid, NT);
        __syncthreads();
    }
    __device__ void finish(const NsArgs& a, IterShared<NT>& sh, unsigned long long* cnt) {
        if (threadIdx.x == NsSmem<S, NT>::STORE_TID) {
            sh.upd = tally.iter;
            tally.flush(a.vstate, cnt);
            tally.reset();
            tma_store_wait_all();
            asm volatile("fence.proxy.async.global;" ::: "memory");
        }
    }
};

// The persistent kernel, block per brick.  MINB resident blocks per SM (the
// register cap follows: 1024 threads -> 64 registers a thread; 1280 -> 48
// trades per-thread registers for more bricks in flight at full load).
template <int BX, int BY, int BZ, int NT, int MINB = 1024 / NT>
__global__ void __launch_bounds__(NT, MINB) k_ns_persistent(NsArgs a) {
    using S = Brick<BX, BY, BZ>;
    __shared__ NsSmem<S, NT> sm;
    __shared__ IterShared<NT> sh;
    __shared__ BlockTally tally;
    extern __shared__ int32_t s_dyn[];
    BlockProc<S, NT> proc(sm, tally);
    ns_drive<NT>(a, sh, stop_state(s_dyn, a.nvol), proc);
}

// ---------------------------------------------------------------------------
// Brick workers: one block per SM of GROUPS groups of NT threads; group g
// takes the block's bricks g, g + GROUPS, ... of each chunk and works on each
// exactly as a block-per-brick block does (its own double-buffered TMA loads,
// store thread and tally), synchronising on its named barrier only.  The
// iteration's rank selection and the grid-barrier arrival are done once per
// SM, and the SM's bricks are spread over its groups.
template <class S, int NT, int GROUPS>
struct GroupProc {
    NsSmem<S, NT>* sm;   // GROUPS of them (dynamic shared memory)
    BlockTally* tally;   // GROUPS of them (shared memory), one per store thread
    GroupTeam<NT> team;
    uint32_t mphase;     // bit b: phase of this group's load barrier b
    int buf;
    __device__ GroupProc(NsSmem<S, NT>* s, BlockTally* t) : sm(s), tally(t), mphase(0u), buf(0) {
        team.g = (int)threadIdx.x / NT;
    }
    __device__ void init() {
        if (team.tid() == 0) {
            mbar_init(&sm[team.g].bar[0], 1);
            mbar_init(&sm[team.g].bar[1], 1);
            tally[team.g].reset();
        }
    }
    template <int BT>
    __device__ void chunk(const NsArgs& a, IterShared<BT>& sh, uint32_t nw, uint32_t nf, uint32_t p, uint32_t sn,
                          unsigned long long* cnt, const NsVol* vone) {
        const int g = team.g, tid = team.tid();
        NsSmem<S, NT>& s = sm[g];
        uint32_t q = (uint32_t)g;
        while (q < nw && sh.work[q] == kNoBrick) q += GROUPS;
        if (q < nw) {
            if (tid == 0) ns_issue_loads<S, NT>(a, s, sh.work[q], p, buf, vone);
            ns_fetch_mask<S, NT>(a, s, sh.work[q], p, buf, tid);
            team.sync();  // act[buf] of the group's first brick
        }
        while (q < nw) {
            uint32_t q2 = q + GROUPS;
            while (q2 < nw && sh.work[q2] == kNoBrick) q2 += GROUPS;
            if (q2 < nw) {
                if (tid == 0) ns_issue_loads<S, NT>(a, s, sh.work[q2], p, buf ^ 1, vone);
                ns_fetch_mask<S, NT>(a, s, sh.work[q2], p, buf ^ 1, tid);
            }
            ns_process_brick<S, NT, GroupTeam<NT>>(a, s, sh.work[q], p, sn, buf, mphase, tally[g], cnt, vone, team);
            buf ^= 1;
            q = q2;
        }
        for (uint32_t r = (uint32_t)g; r < nf; r += GROUPS)
            if (sh.flush[r] != kNoBrick) ns_flush_brick<S>(a, sh.flush[r], p, vone, tid, NT);
        __syncthreads();
    }
    template <int BT>
    __device__ void finish(const NsArgs& a, IterShared<BT>& sh, unsigned long long* cnt) {
        if (team.tid() == NsSmem<S, NT>::STORE_TID) {
            BlockTally& t = tally[team.g];
            if (t.iter) atomicAdd(&sh.upd, t.iter);
            t.flush(a.vstate, cnt);
            t.reset();
            tma_store_wait_all();
            asm volatile("fence.proxy.async.global;" ::: "memory");
        }
    }
};

// Dynamic shared memory of the brick-worker kernel: 128 bytes of alignment
// slack, the GROUPS work areas, then the stopping state.
template <class S, int NT, int GROUPS>
__host__ __device__ constexpr size_t group_smem_fixed() {
    return 128 + (size_t)GROUPS * sizeof(NsSmem<S, NT>);
}

template <int BX, int BY, int BZ, int NT, int GROUPS>
__global__ void __launch_bounds__(NT * GROUPS, 1) k_ns_group(NsArgs a) {
    using S = Brick<BX, BY, BZ>;
    __shared__ IterShared<NT * GROUPS> sh;
    __shared__ BlockTally tally[GROUPS];
    extern __shared__ unsigned char s_dyn_raw[];
    unsigned char* dyn = s_dyn_raw + ((128u - (smem_addr(s_dyn_raw) & 127u)) & 127u);
    NsSmem<S, NT>* sm = reinterpret_cast<NsSmem<S, NT>*>(dyn);
    int32_t* state = reinterpret_cast<int32_t*>(s_dyn_raw + group_smem_fixed<S, NT, GROUPS>());
    GroupProc<S, NT, GROUPS> proc(sm, tally);
    ns_drive<NT * GROUPS>(a, sh, stop_state(state, a.nvol), proc);
}

// ---------------------------------------------------------------------------
// Warp per brick: one block per SM, W warps, every warp updates its own
// bricks with warp-level synchronisation only (no block barrier inside the
// brick work), so up to W bricks per SM are in flight at once and the grid
// barrier has one participant per SM.

template <class S>
struct WarpSlot {
    static_assert((S::TILE_PAD * 4) % 128 == 0 && (S::VOX * 4) % 128 == 0, "TMA smem alignment");
    alignas(128) float phi[S::TILE_PAD];  // halo tile of phi
    alignas(128) float spd[S::VOX];  // the brick's speed
    alignas(128) float out[S::VOX];
    unsigned long long act[S::WORDS];
    uint32_t chg[S::CHG];
    uint16_t list[S::VOX];
    uint8_t chgb[S::VOX];
    unsigned long long xy[9 * S::WORDS];  // xy-dilated planes per (ox, oy) pair
    alignas(8) uint64_t bar;
};

// One brick of A_k by one warp: TMA load (lane 0) + mask fetch, pass 1 (copy,
// ballot-prefix compaction of the active voxels), pass 2 (update), pass 3
// (changed bytes -> ballot words), TMA store (lane 0), dilation into the 27
// neighbours (one mask word per lane and round; one lane per neighbour sets
// its membership bit).
template <class S>
__device__ __forceinline__ void ns_warp_brick(const NsArgs& a, WarpSlot<S>& sl, uint32_t b, uint32_t p,
                                              uint32_t sn, uint32_t& phase, BlockTally& tally,
                                              unsigned long long* cnt, const NsVol* vone) {
    const int lane = threadIdx.x & 31;
    const uint32_t v = vone ? 0u : a.brick_vol[b];
    const NsVol& V = vone ? *vone : a.vols[v];
    const int3 o = brick_origin<S>(V, b);
    if (lane < S::WORDS) {
        unsigned long long* mp = a.masks[p] + (size_t)b * S::WORDS + lane;
        sl.act[lane] = *mp;
        *mp = 0ull;  // the mask array of parity p becomes the accumulator of iteration k+1
    }
    if (lane == 0) {
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // this warp's last store read out[]
        fence_proxy_async_smem();  // the warp's generic reads of the slot before the async writes
        mbar_expect_tx(&sl.bar, (uint32_t)(S::TILE + S::VOX) * 4u);
        tma_load_3d(sl.phi, &a.tmaps[V.tmap_base + p], o.x - 4, o.y - 1, o.z - 1, &sl.bar);
        tma_load_3d(sl.spd, &a.tmaps[V.tmap_base + 4], o.x, o.y, o.z, &sl.bar);
    }
    __syncwarp();
    if (!mbar_wait(&sl.bar, phase)) set_error(&a.ctl->err, ERR_TMA_TIMEOUT);
    phase ^= 1u;
    float* phi = sl.phi;
    if (tile_at_edge<S>(V, o.x, o.y, o.z)) {
        clamp_tile_halo<S>(phi, V, o.x, o.y, o.z, lane, 32);
        __syncwarp();
    }
    auto tile_index = [](int j) {
        const int lx = j % S::X, ly = (j / S::X) % S::Y, lz = j / (S::X * S::Y);
        return ((lz + 1) * S::TY + (ly + 1)) * S::TX + (lx + 4);
    };
    const uint32_t lt = (1u << lane) - 1u;
    // pass 1
    uint32_t nact = 0;
#pragma unroll 4
    for (int g = 0; g < S::VOX / 32; ++g) {
        const int j = lane + 32 * g;
        sl.out[j] = phi[tile_index(j)];
        sl.chgb[j] = 0;
        const bool act = (sl.act[j >> 6] >> (j & 63)) & 1ull;
        const uint32_t bal = __ballot_sync(0xffffffffu, act);
        if (act) sl.list[nact + __popc(bal & lt)] = (uint16_t)j;
        nact += __popc(bal);
    }
    __syncwarp();
    // pass 2
    for (uint32_t i = lane; i < nact; i += 32) {
        const int j = sl.list[i];
        const int ti = tile_index(j);
        auto P = [&](int dx, int dy, int dz) { return phi[ti + (dz * S::TY + dy) * S::TX + dx]; };
        const float c = phi[ti];
        const float nv = ns_update_speed_f32(P, sl.spd[j], V);
        sl.out[j] = nv;
        sl.chgb[j] = fabsf(nv - c) > V.thr_t;
    }
    fence_proxy_async_smem();
    __syncwarp();
    // pass 3
    bool any = false;
#pragma unroll 4
    for (int g = 0; g < S::VOX / 32; ++g) {
        const uint32_t bal = __ballot_sync(0xffffffffu, sl.chgb[lane + 32 * g] != 0);
        if (lane == 0) sl.chg[g] = bal;
        any |= bal != 0u;
    }
    __syncwarp();
    if (lane == 0) {
        tma_store_3d(&a.tmaps[V.tmap_base + 2 + (p ^ 1u)], o.x, o.y, o.z, sl.out);
        tma_store_commit();
        tally.add(a.vstate, cnt, v, nact);
    }
    if (any) {
        if constexpr (S::XY == 64) {
            dilate_planes<S>(V, sl.chg, sl.xy, lane, 32);
            __syncwarp();
        }
        dilate_scatter<S, 32>(a, V, sl.chg, sl.xy, b, o.x, o.y, o.z, p, sn, lane);
    }
    __syncwarp();
}

template <class S, int W>
struct WarpProc {
    static constexpr int NT = W * 32;
    WarpSlot<S>* slots;
    uint32_t phase;    // this warp's load barrier phase
    BlockTally tally;  // lane 0 of every warp
    __device__ explicit WarpProc(WarpSlot<S>* s) : slots(s), phase(0u) {}
    __device__ void init() {
        tally.reset();
        if ((threadIdx.x & 31) == 0) mbar_init(&slots[threadIdx.x >> 5].bar, 1);
    }
    __device__ void chunk(const NsArgs& a, IterShared<NT>& sh, uint32_t nw, uint32_t nf, uint32_t p,
                          uint32_t sn, unsigned long long* cnt, const NsVol* vone) {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        WarpSlot<S>& sl = slots[warp];
        for (uint32_t q = warp; q < nw; q += W)
            if (sh.work[q] != kNoBrick) ns_warp_brick<S>(a, sl, sh.work[q], p, sn, phase, tally, cnt, vone);
        for (uint32_t q = warp; q < nf; q += W)
            if (sh.flush[q] != kNoBrick) ns_flush_brick<S>(a, sh.flush[q], p, vone, lane, 32);
        __syncthreads();
    }
    __device__ void finish(const NsArgs& a, IterShared<NT>& sh, unsigned long long* cnt) {
        if ((threadIdx.x & 31) == 0) {
            if (tally.iter) atomicAdd(&sh.upd, tally.iter);
            tally.flush(a.vstate, cnt);
            tally.reset();
            tma_store_wait_all();
            asm volatile("fence.proxy.async.global;" ::: "memory");
        }
    }
};

// Dynamic shared memory of the warp kernel: 128 bytes of alignment slack, the
// W warp slots, then the stopping state.
template <class S, int W>
__host__ __device__ constexpr size_t warp_smem_fixed() {
    return 128 + (size_t)W * sizeof(WarpSlot<S>);
}

template <int BX, int BY, int BZ, int W>
__global__ void __launch_bounds__(W * 32, 1) k_ns_warp(NsArgs a) {
    using S = Brick<BX, BY, BZ>;
    __shared__ IterShared<W * 32> sh;
    extern __shared__ unsigned char s_dyn_raw[];
    unsigned char* dyn = s_dyn_raw + ((128u - (smem_addr(s_dyn_raw) & 127u)) & 127u);
    WarpSlot<S>* slots = reinterpret_cast<WarpSlot<S>*>(dyn);
    int32_t* state = reinterpret_cast<int32_t*>(s_dyn_raw + warp_smem_fixed<S, W>());
    WarpProc<S, W> proc(slots);
    ns_drive<W * 32>(a, sh, stop_state(state, a.nvol), proc);
}

// Initial active set of every brick: voxels whose 6-neighbours differ by more
// than thr_s (clamped coordinates).  One thread per voxel slot in brick-major
// order (grid-stride), so a warp covers 32 consecutive voxels of one brick
// and its ballot is one 32-bit half of a mask word, stored directly; bricks
// with a non-empty mask get their membership bit in bits[s].  Counts land in
// cnt[0] (one atomic per warp and volume run).
//
// box_n.x > 0 restricts the pass to the bricks [box_lo, box_lo + box_n) of a
// one-volume launch (brick coordinates); the other bricks are known empty.
template <int BX, int BY, int BZ, int NT>
__global__ void __launch_bounds__(NT) k_ns_init_active(NsArgs a, uint32_t p, uint32_t s, int3 box_lo,
                                                       int3 box_n) {
    using S = Brick<BX, BY, BZ>;
    const bool boxed = box_n.x > 0;
    const uint64_t nbricks = boxed ? (uint64_t)box_n.x * box_n.y * box_n.z : (uint64_t)a.NB;
    const uint64_t total = nbricks * S::VOX;
    uint32_t cur_v = 0xFFFFFFFFu;
    unsigned long long n = 0;
    auto flush = [&]() {
        for (int o = 16; o; o >>= 1) n += __shfl_down_sync(0xffffffffu, n, o);
        if ((threadIdx.x & 31) == 0 && n && cur_v != 0xFFFFFFFFu) atomicAdd(&a.cnt[0][cur_v], n);
        n = 0;
    };
    for (uint64_t t = blockIdx.x * (uint64_t)NT + threadIdx.x; t < total; t += (uint64_t)gridDim.x * NT) {
        uint32_t b = (uint32_t)(t / S::VOX);
        const int j = (int)(t % S::VOX);
        if (boxed) {
            const NsVol& V0 = a.vols[0];
            const int kx = box_lo.x + (int)(b % box_n.x), ky = box_lo.y + (int)((b / box_n.x) % box_n.y),
                      kz = box_lo.z + (int)(b / ((uint32_t)box_n.x * box_n.y));
            b = V0.brick_base + (uint32_t)((kz * V0.nby + ky) * V0.nbx + kx);
        }
        const uint32_t v = a.brick_vol[b];  // one brick per warp: uniform
        if (v != cur_v) {
            flush();
            cur_v = v;
        }
        const NsVol& V = a.vols[v];
        const int3 o = brick_origin<S>(V, b);
        const int x = o.x + j % S::X, y = o.y + (j / S::X) % S::Y, z = o.z + j / (S::X * S::Y);
        bool act = false;
        if (x < V.nx && y < V.ny && z < V.nz) {
            const float* ph = V.phi[p];
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
        const uint32_t bal = __ballot_sync(0xffffffffu, act);
        if ((threadIdx.x & 31) == 0) {
            // Half (j / 32) % 2 of mask word j / 64 (little-endian halves).
            reinterpret_cast<uint32_t*>(a.masks[p])[(size_t)b * S::WORDS * 2 + (j >> 5)] = bal;
            if (bal) atomicOr(&a.bits[s][b >> 5], 1u << (b & 31));
        }
        n += act ? 1u : 0u;
    }
    flush();
}

// The active voxels of A_k (membership slot s, masks of parity p) as one
// brick-major list: tiles of NT/32 membership words (a warp each) are placed
// by a single-pass decoupled lookback over their voxel counts; inside a word
// the warp emits brick after brick, its lanes splitting each brick's voxels
// (VOX/32 a lane) and placing them by a warp prefix sum.  Writes
// volume-local linear indices (x + nx*(y + ny*z)) when `out` is set and,
// from the last tile, the total count.
template <int BX, int BY, int BZ, int NT>
__global__ void __launch_bounds__(NT) k_ns_emit(NsArgs a, uint32_t p, uint32_t s, uint64_t* out,
                                               unsigned long long* total_out) {
    using S = Brick<BX, BY, BZ>;
    constexpr int NWARP = NT / 32;
    constexpr int VPL = S::VOX / 32;  // voxels of a brick a lane
    static_assert(VPL >= 1 && VPL <= 32 && 64 % VPL == 0, "voxels a lane");
    __shared__ uint32_t s_tile;
    __shared__ unsigned long long s_warp[NWARP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t ntiles = (a.NW + NWARP - 1) / NWARP;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&a.ctl->emit_tile, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        __syncthreads();
        if (tile >= ntiles) break;
        const uint32_t w = tile * NWARP + warp;
        const uint32_t bw = w < a.NW ? a.bits[s][w] : 0u;
        // Lane l: the voxel count of brick 32 w + l (if in A_k).
        uint32_t bc = 0;
        if ((bw >> lane) & 1u) {
            const uint32_t b = w * 32u + (uint32_t)lane;
#pragma unroll
            for (int q = 0; q < S::WORDS; ++q) bc += (uint32_t)__popcll(a.masks[p][(size_t)b * S::WORDS + q]);
        }
        uint32_t inc = bc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) s_warp[warp] = inc;
        __syncthreads();
        unsigned long long woff = 0, ttot = 0;
#pragma unroll
        for (int i = 0; i < NWARP; ++i) {
            const unsigned long long x = s_warp[i];
            if (i < warp) woff += x;
            ttot += x;
        }
        const uint64_t prefix = tile_exclusive_prefix(a.status, tile, ttot, &a.ctl->err);
        if (out) {
            const uint64_t base = prefix + woff;
            for (uint32_t m = bw; m; m &= m - 1u) {
                const int bl = __ffs(m) - 1;
                const uint32_t b = w * 32u + (uint32_t)bl;
                const uint64_t bstart = base + __shfl_sync(0xffffffffu, inc - bc, bl);
                const int j0 = lane * VPL;
                const unsigned long long word = a.masks[p][(size_t)b * S::WORDS + j0 / 64];
                const uint32_t chunk =
                    (uint32_t)((word >> (j0 % 64)) & (VPL == 32 ? 0xFFFFFFFFull : ((1ull << VPL) - 1ull)));
                const uint32_t cc = (uint32_t)__popc(chunk);
                uint32_t ci = cc;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, ci, o);
                    if (lane >= o) ci += y;
                }
                const NsVol& V = a.vols[a.brick_vol[b]];
                const int3 og = brick_origin<S>(V, b);
                uint64_t o = bstart + (ci - cc);
                for (uint32_t cm = chunk; cm; cm &= cm - 1u) {
                    const int j = j0 + __ffs(cm) - 1;
                    const uint64_t x = og.x + j % S::X, y = og.y + (j / S::X) % S::Y, z = og.z + j / (S::X * S::Y);
                    out[o++] = (z * V.ny + y) * V.nx + x;
                }
            }
        }
        if (tile == ntiles - 1 && threadIdx.x == 0) *total_out = prefix + ttot;
    }
}

}  // namespace lss
