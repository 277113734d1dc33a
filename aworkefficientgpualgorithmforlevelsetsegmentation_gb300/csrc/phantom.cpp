// Deterministic synthetic phantoms (host code).  See include/lss_phantom.h.
//
// The reference's accuracy and performance runs used BrainWeb volumes
// (code/gpuseg/code/src/Segmenter.cpp:1755-1864), which are absent; these
// seeded generators provide inputs of the same sizes and value ranges.
// Compiled with -ffp-contract=off so that aarch64 and x86-64 agree bit for bit.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "lss_phantom.h"

namespace {

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

inline double u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

// Sequential generator: SplitMix64 stream.
struct Stream {
    uint64_t s;
    explicit Stream(uint64_t seed) : s(splitmix64(seed ^ 0x5EEDull)) {}
    double next() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return u01(z);
    }
    // Irwin-Hall(4): sum of 4 uniforms has mean 2 and variance 1/3.
    double normal() {
        double a = next() + next() + next() + next();
        return (a - 2.0) * 1.7320508075688772;  // sqrt(3)
    }
};

bool dims_ok(int32_t nx, int32_t ny, int32_t nz) {
    return nx > 0 && ny > 0 && nz > 0 && (uint64_t)nx * ny * nz < (1ull << 40);
}

void add_noise(float* out, size_t n, float sigma, uint64_t seed) {
    if (sigma == 0.0f) return;
    Stream st(seed);
    for (size_t i = 0; i < n; ++i) out[i] = (float)((double)out[i] + (double)sigma * st.normal());
}

// Separable Gaussian blur, sigma = 1, radius 3, clamp-to-edge.  The weights
// are exp(-k^2/2) for k = 0..3, written as literals so no libm call is made.
void blur_sigma1(float* v, int32_t nx, int32_t ny, int32_t nz) {
    const double w[4] = {1.0, 0.60653065971263342, 0.13533528323661270, 0.011108996538242306};
    double sum = w[0] + 2.0 * (w[1] + w[2] + w[3]);
    double k[4];
    for (int i = 0; i < 4; ++i) k[i] = w[i] / sum;
    const size_t sx = 1, sy = (size_t)nx, sz = (size_t)nx * ny;
    std::vector<float> line;
    auto pass = [&](int32_t len, size_t stride, int32_t na, size_t sa, int32_t nb, size_t sb) {
        line.resize(len);
        for (int32_t b = 0; b < nb; ++b)
            for (int32_t a = 0; a < na; ++a) {
                float* base = v + (size_t)a * sa + (size_t)b * sb;
                for (int32_t i = 0; i < len; ++i) line[i] = base[(size_t)i * stride];
                for (int32_t i = 0; i < len; ++i) {
                    double acc = k[0] * line[i];
                    for (int t = 1; t <= 3; ++t) {
                        int32_t lo = i - t < 0 ? 0 : i - t;
                        int32_t hi = i + t >= len ? len - 1 : i + t;
                        acc += k[t] * ((double)line[lo] + (double)line[hi]);
                    }
                    base[(size_t)i * stride] = (float)acc;
                }
            }
    };
    pass(nx, sx, ny, sy, nz, sz);
    pass(ny, sy, nx, sx, nz, sz);
    pass(nz, sz, nx, sx, ny, sy);
}

// Trilinear value noise in [0,1) on a lattice of spacing L.
struct ValueNoise {
    int32_t L, gx, gy, gz;
    std::vector<double> g;
    ValueNoise(int32_t nx, int32_t ny, int32_t nz, int32_t L_, uint64_t seed) : L(L_) {
        gx = nx / L + 2; gy = ny / L + 2; gz = nz / L + 2;
        g.resize((size_t)gx * gy * gz);
        for (size_t i = 0; i < g.size(); ++i) g[i] = u01(splitmix64(seed * 0x100000001B3ull + i));
    }
    double at(int32_t x, int32_t y, int32_t z) const {
        int32_t ix = x / L, iy = y / L, iz = z / L;
        double fx = (double)(x - ix * L) / L, fy = (double)(y - iy * L) / L,
               fz = (double)(z - iz * L) / L;
        auto G = [&](int32_t a, int32_t b, int32_t c) {
            return g[((size_t)c * gy + b) * gx + a];
        };
        double c00 = G(ix, iy, iz) * (1 - fx) + G(ix + 1, iy, iz) * fx;
        double c10 = G(ix, iy + 1, iz) * (1 - fx) + G(ix + 1, iy + 1, iz) * fx;
        double c01 = G(ix, iy, iz + 1) * (1 - fx) + G(ix + 1, iy, iz + 1) * fx;
        double c11 = G(ix, iy + 1, iz + 1) * (1 - fx) + G(ix + 1, iy + 1, iz + 1) * fx;
        double c0 = c00 * (1 - fy) + c10 * fy;
        double c1 = c01 * (1 - fy) + c11 * fy;
        return c0 * (1 - fz) + c1 * fz;
    }
};

}  // namespace

extern "C" {

double lss_phantom_uniform(uint64_t seed, uint64_t index) {
    return u01(splitmix64(splitmix64(seed) ^ (index * 0xD1B54A32D192ED03ull)));
}

lss_status lss_phantom_ellipsoid(int32_t nx, int32_t ny, int32_t nz, const float* c,
                                 const float* a, float fg, float bg, float noise_sigma,
                                 uint64_t seed, float* out) {
    if (!dims_ok(nx, ny, nz) || !c || !a || !out) return LSS_ERR_INVALID_ARGUMENT;
    if (!(a[0] > 0 && a[1] > 0 && a[2] > 0)) return LSS_ERR_INVALID_ARGUMENT;
    for (int32_t z = 0; z < nz; ++z)
        for (int32_t y = 0; y < ny; ++y)
            for (int32_t x = 0; x < nx; ++x) {
                double dx = (x - (double)c[0]) / a[0], dy = (y - (double)c[1]) / a[1],
                       dz = (z - (double)c[2]) / a[2];
                double q = dx * dx + dy * dy + dz * dz;
                out[((size_t)z * ny + y) * nx + x] = q <= 1.0 ? fg : bg;
            }
    add_noise(out, (size_t)nx * ny * nz, noise_sigma, seed);
    return LSS_OK;
}

lss_status lss_phantom_shells(int32_t nx, int32_t ny, int32_t nz, int32_t nshells,
                              const float* axes, const float* values, float bg,
                              float disp_amp, int32_t lattice, uint64_t disp_seed,
                              float blur_sigma, float noise_sigma, uint64_t noise_seed,
                              float* out) {
    if (!dims_ok(nx, ny, nz) || nshells <= 0 || !axes || !values || !out || lattice <= 0)
        return LSS_ERR_INVALID_ARGUMENT;
    if (!(blur_sigma == 0.0f || blur_sigma == 1.0f)) return LSS_ERR_UNSUPPORTED;
    ValueNoise vn(nx, ny, nz, lattice, disp_seed);
    const double cx = (nx - 1) * 0.5, cy = (ny - 1) * 0.5, cz = (nz - 1) * 0.5;
    std::vector<double> amean(nshells);
    for (int32_t s = 0; s < nshells; ++s)
        amean[s] = ((double)axes[3 * s] + axes[3 * s + 1] + axes[3 * s + 2]) / 3.0;
    for (int32_t z = 0; z < nz; ++z)
        for (int32_t y = 0; y < ny; ++y)
            for (int32_t x = 0; x < nx; ++x) {
                double d = disp_amp == 0.0f ? 0.0 : disp_amp * (2.0 * vn.at(x, y, z) - 1.0);
                float val = bg;
                for (int32_t s = 0; s < nshells; ++s) {
                    double dx = (x - cx) / axes[3 * s], dy = (y - cy) / axes[3 * s + 1],
                           dz = (z - cz) / axes[3 * s + 2];
                    double q = dx * dx + dy * dy + dz * dz;
                    double r = 1.0 + d / amean[s];
                    if (r > 0 && q <= r * r) val = values[s];  // inner shells overwrite
                }
                out[((size_t)z * ny + y) * nx + x] = val;
            }
    if (blur_sigma == 1.0f) blur_sigma1(out, nx, ny, nz);
    add_noise(out, (size_t)nx * ny * nz, noise_sigma, noise_seed);
    return LSS_OK;
}

lss_status lss_phantom_sdf_spheres(int32_t nx, int32_t ny, int32_t nz, const float* s,
                                   int32_t count, float lo, float hi, float* out) {
    if (!dims_ok(nx, ny, nz) || !s || count <= 0 || !out || !(lo < hi))
        return LSS_ERR_INVALID_ARGUMENT;
    for (int32_t z = 0; z < nz; ++z)
        for (int32_t y = 0; y < ny; ++y)
            for (int32_t x = 0; x < nx; ++x) {
                double best = 1e300;
                for (int32_t k = 0; k < count; ++k) {
                    double dx = x - (double)s[4 * k], dy = y - (double)s[4 * k + 1],
                           dz = z - (double)s[4 * k + 2];
                    double d = std::sqrt(dx * dx + dy * dy + dz * dz) - s[4 * k + 3];
                    if (d < best) best = d;
                }
                if (best < lo) best = lo;
                if (best > hi) best = hi;
                out[((size_t)z * ny + y) * nx + x] = (float)best;
            }
    return LSS_OK;
}

}  // extern "C"
