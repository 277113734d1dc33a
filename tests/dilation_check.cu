// Host-side check of the bit-parallel brick dilation (dilate_slot,
// dilate_word, inside_mask in csrc/ns_kernels.cuh) against a brute-force
// dilation, for every brick shape, both neighbourhoods and every neighbour
// slot; of the kernels' work split of it (xy_plane, plane_word,
// dilate_item); and the rank-selection helpers nth_set_bit and div_magic
// against plain loops and division.  Built and run by tests/test_dilation_host.py
// (no GPU needed).
#include "ns_kernels.cuh"
#include <cstdio>
#include <random>
using namespace lss;
template <class S> int check(std::mt19937_64& rng, int nbh) {
    int bad = 0;
    auto bit = [&](const uint64_t* v, int x, int y, int z) {
        int j = (z * S::Y + y) * S::X + x; return (int)((v[j >> 6] >> (j & 63)) & 1); };
    for (int trial = 0; trial < 3000; ++trial) {
        uint64_t c[S::WORDS];
        const int dens = trial % 4;
        for (int w = 0; w < S::WORDS; ++w) {
            c[w] = rng();
            for (int q = 0; q < dens; ++q) c[w] &= rng();
        }
        for (int oz = -1; oz <= 1; ++oz) for (int oy = -1; oy <= 1; ++oy) for (int ox = -1; ox <= 1; ++ox) {
            uint64_t m[S::WORDS];
            for (int w = 0; w < S::WORDS; ++w) m[w] = c[w];
            dilate_slot<S>(m, ox, oy, oz, nbh);
            uint32_t c32[2 * S::WORDS];
            for (int w = 0; w < S::WORDS; ++w) { c32[2 * w] = (uint32_t)c[w]; c32[2 * w + 1] = (uint32_t)(c[w] >> 32); }
            for (int w = 0; w < S::WORDS; ++w) if (dilate_word<S>(c32, ox, oy, oz, w, nbh) != m[w]) ++bad;
            for (int z = 0; z < S::Z; ++z) for (int y = 0; y < S::Y; ++y) for (int x = 0; x < S::X; ++x) {
                // voxel of neighbour brick in center coordinates
                int gx = x + ox * S::X, gy = y + oy * S::Y, gz = z + oz * S::Z;
                int want = 0;
                for (int dz = -1; dz <= 1; ++dz) for (int dy = -1; dy <= 1; ++dy) for (int dx = -1; dx <= 1; ++dx) {
                    if (nbh == 6 && (dx != 0) + (dy != 0) + (dz != 0) > 1) continue;
                    int sx = gx + dx, sy = gy + dy, sz = gz + dz;
                    if (sx < 0 || sy < 0 || sz < 0 || sx >= S::X || sy >= S::Y || sz >= S::Z) continue;
                    want |= bit(c, sx, sy, sz);
                }
                if (want != bit(m, x, y, z)) ++bad;
            }
        }
    }
    // inside_mask
    for (int lx = 1; lx <= S::X; ++lx) for (int ly = 1; ly <= S::Y; ++ly) for (int lz = 1; lz <= S::Z; ++lz) {
        uint64_t m[S::WORDS];
        for (int w = 0; w < S::WORDS; ++w) m[w] = inside_mask<S>(w, lx, ly, lz);
        for (int z = 0; z < S::Z; ++z) for (int y = 0; y < S::Y; ++y) for (int x = 0; x < S::X; ++x)
            if (bit(m, x, y, z) != (x < lx && y < ly && z < lz)) ++bad;
    }
    return bad;
}
// The per-brick work split of the kernels' dilation: xy_plane + plane_word
// (one z-plane a mask word) equal dilate_word, and the items of dilate_item
// cover each (neighbour, word) at most once and every word that can be
// non-zero (the words they skip are zero for every mask).
template <class S> int check_items(std::mt19937_64& rng, int nbh) {
    int bad = 0;
    int seen[27][S::WORDS] = {};
    for (int t = 0; t < dilate_items<S>(); ++t) {
        int slot = -1, w = -1;
        const bool single = dilate_item<S>(t, slot, w);
        if (slot < 0 || slot >= 27 || w < 0 || w >= S::WORDS) { ++bad; continue; }
        ++seen[slot][w];
        if (single != (t >= dilate_layer_items<S>())) ++bad;
    }
    for (int slot = 0; slot < 27; ++slot)
        for (int w = 0; w < S::WORDS; ++w)
            if (seen[slot][w] > 1) ++bad;
    for (int trial = 0; trial < 2000; ++trial) {
        uint64_t c[S::WORDS];
        for (int w = 0; w < S::WORDS; ++w) {
            c[w] = rng();
            for (int q = 0; q < trial % 4; ++q) c[w] &= rng();
        }
        uint32_t c32[2 * S::WORDS];
        for (int w = 0; w < S::WORDS; ++w) { c32[2 * w] = (uint32_t)c[w]; c32[2 * w + 1] = (uint32_t)(c[w] >> 32); }
        unsigned long long xy[9 * S::WORDS];
        for (int t = 0; t < 9 * S::WORDS; ++t) xy[t] = xy_plane<S>(c[t % S::WORDS], t / S::WORDS, nbh);
        auto W = [&](int q) -> uint64_t { return c[q]; };
        for (int slot = 0; slot < 27; ++slot) {
            const int ox = slot % 3 - 1, oy = (slot / 3) % 3 - 1, oz = slot / 9 - 1;
            for (int w = 0; w < S::WORDS; ++w) {
                const uint64_t want = dilate_word<S>(c32, ox, oy, oz, w, nbh);
                if (!seen[slot][w] && want) ++bad;
                if constexpr (S::XY == 64)
                    if (plane_word<S>(xy, W, ox, oy, oz, w, nbh) != want) ++bad;
            }
        }
    }
    return bad;
}
int check_select(std::mt19937_64& rng) {
    int bad = 0;
    for (int trial = 0; trial < 20000; ++trial) {
        uint32_t m = (uint32_t)rng();
        if (trial % 3 == 1) m &= (uint32_t)rng();
        if (trial % 3 == 2) m |= (uint32_t)rng();
        uint32_t mm = m;
        for (uint32_t s = 0; mm; ++s, mm &= mm - 1u)
            if (nth_set_bit(m, s) != (uint32_t)__builtin_ctz(mm)) ++bad;
    }
    for (uint32_t g = 1; g <= 5000; ++g) {
        const uint32_t gm = 0xFFFFFFFFu / g + 1u;
        for (int t = 0; t < 200; ++t) {
            uint32_t x = (uint32_t)(rng() & 0x7FFFFFFFu);
            if (t % 4 == 1) x = (x / g) * g;
            if (t % 4 == 2) x = (x / g) * g + g - 1u;
            if (t % 4 == 3) x = (x / g) * g - 1u;
            x &= 0x7FFFFFFFu;
            if (div_magic(x, g, gm) != x / g) ++bad;
        }
        if (div_magic(0x7FFFFFFFu, g, gm) != 0x7FFFFFFFu / g) ++bad;
    }
    return bad;
}
int main() {
    std::mt19937_64 rng(7);
    int bad = check_select(rng);
    printf("selection helpers: %d\n", bad);
    for (int nbh : {26, 6}) {
        int a = check<Brick<8, 8, 8>>(rng, nbh), b = check<Brick<8, 8, 4>>(rng, nbh), c = check<Brick<4, 4, 4>>(rng, nbh);
        printf("nbh %d: 888 %d, 884 %d, 444 %d\n", nbh, a, b, c);
        bad += a + b + c;
        a = check_items<Brick<8, 8, 8>>(rng, nbh), b = check_items<Brick<8, 8, 4>>(rng, nbh),
        c = check_items<Brick<4, 4, 4>>(rng, nbh);
        printf("items, nbh %d: 888 %d, 884 %d, 444 %d\n", nbh, a, b, c);
        bad += a + b + c;
    }
    printf(bad ? "FAIL\n" : "OK\n");
    return bad != 0;
}
