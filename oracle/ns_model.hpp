// ORACLE — test infrastructure only (the checker for LSS_MODE_NS, and the
// timed CPU baseline of bench.py).  Nothing in the product links it.
//
// FP64 restatement of the sparse level-set iteration in its spec form:
//   phi <- clamp(phi + dt * (wc * kappa*|grad phi|  -  F * |grad phi|_upwind),
//                phi_min, phi_max)
//   kappa*|grad phi| = div(grad phi/|grad phi|) * |grad phi|  (central differences)
//   F  = wd * (clamp((eps - |I - T|) / eps, -1, 1) + bias)   (outward speed)
//   alpha_data = 1: wd = alpha, wc = 1 - alpha  (F = alpha*D + (1-alpha)*C, the
//                   Lefohn et al. 2004 weighting the workloads' alpha values need)
//   alpha_data = 0: wc = alpha, wd = 1 - alpha  (the reference's speed function,
//                   UpdateLevelSetVolume.cu:303, and the paper, main.tex:178)
// D is the paper's eps - |I - T| (main.tex:176) divided by eps as the
// reference's ComputeDensityTerm does (UpdateLevelSetVolume.cu:335-342), and
// clamped to [-1, 1] so that dt*|F| stays inside the upwind scheme's CFL bound.
// with the Osher-Sethian upwind gradient for F, inside = phi <= 0, and every
// stencil coordinate clamped independently to the volume (edge replication).
//
// Active-set tracking follows the paper's two culling conditions
// (main.tex:217-231): the initial set holds the voxels with a 6-neighbour
// whose phi differs by more than the spatial threshold; after each update the
// voxels whose |dphi| exceeds the temporal threshold activate themselves and
// their 26 (or 6) neighbours for the next iteration.  The list is kept in
// brick-major order (bricks x-fastest over the padded brick grid, voxels
// x-fastest inside a brick) — the order the GPU engine's decoupled-lookback
// compaction produces.
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace lssns {

struct Params {
    double T = 0.5, eps = 0.1, alpha = 0.5, dt = 0.5;
    double lo = -4.0, hi = 4.0;
    double thr_t = 0.01, thr_s = 0.0;
    int nbh = 26;
    int alpha_data = 1;       // 1: alpha weights the data term, 0: the curvature term
};

// The update of one voxel; shared by the oracle and the adjoint oracle.
// P(x,y,z) must clamp its coordinates.  bias is added to the data speed.
template <class Real, class PF>
inline Real ns_update(PF P, int x, int y, int z, Real I, Real bias, const Params& p) {
    Real c = P(x, y, z);
    Real xm = P(x - 1, y, z), xp = P(x + 1, y, z);
    Real ym = P(x, y - 1, z), yp = P(x, y + 1, z);
    Real zm = P(x, y, z - 1), zp = P(x, y, z + 1);
    Real cx = (xp - xm) * Real(0.5), cy = (yp - ym) * Real(0.5), cz = (zp - zm) * Real(0.5);
    Real fxx = xp - Real(2) * c + xm, fyy = yp - Real(2) * c + ym, fzz = zp - Real(2) * c + zm;
    Real fxy = (P(x + 1, y + 1, z) - P(x + 1, y - 1, z) - P(x - 1, y + 1, z) + P(x - 1, y - 1, z)) * Real(0.25);
    Real fxz = (P(x + 1, y, z + 1) - P(x + 1, y, z - 1) - P(x - 1, y, z + 1) + P(x - 1, y, z - 1)) * Real(0.25);
    Real fyz = (P(x, y + 1, z + 1) - P(x, y + 1, z - 1) - P(x, y - 1, z + 1) + P(x, y - 1, z - 1)) * Real(0.25);
    Real g2 = cx * cx + cy * cy + cz * cz;
    Real curv = 0;
    if (g2 > Real(1e-12)) {
        Real num = fxx * (cy * cy + cz * cz) + fyy * (cx * cx + cz * cz) + fzz * (cx * cx + cy * cy) -
                   Real(2) * (cx * cy * fxy + cx * cz * fxz + cy * cz * fyz);
        curv = num / g2;
    }
    Real D = (Real(p.eps) - std::fabs(I - Real(p.T))) / Real(p.eps);
    D = std::min(std::max(D, Real(-1)), Real(1)) + bias;
    Real wc = p.alpha_data ? Real(1) - Real(p.alpha) : Real(p.alpha);
    Real wd = Real(1) - wc;
    Real F = wd * D;
    Real dxm = c - xm, dxp = xp - c, dym = c - ym, dyp = yp - c, dzm = c - zm, dzp = zp - c;
    Real zero = 0, g;
    if (F > 0) {
        Real a = std::max(dxm, zero), b = std::min(dxp, zero);
        Real e = std::max(dym, zero), f = std::min(dyp, zero);
        Real h = std::max(dzm, zero), k = std::min(dzp, zero);
        g = std::sqrt(a * a + b * b + e * e + f * f + h * h + k * k);
    } else {
        Real a = std::min(dxm, zero), b = std::max(dxp, zero);
        Real e = std::min(dym, zero), f = std::max(dyp, zero);
        Real h = std::min(dzm, zero), k = std::max(dzp, zero);
        g = std::sqrt(a * a + b * b + e * e + f * f + h * h + k * k);
    }
    Real nv = c + Real(p.dt) * (wc * curv - F * g);
    if (nv < Real(p.lo)) nv = Real(p.lo);
    if (nv > Real(p.hi)) nv = Real(p.hi);
    return nv;
}

class NsOracle {
   public:
    int nx = 0, ny = 0, nz = 0;
    int bx = 8, by = 8, bz = 8;
    int NBx = 0, NBy = 0, NBz = 0;
    Params p;
    std::vector<double> phi;
    std::vector<float> I;
    std::vector<float> bias;      // empty = none
    std::vector<double> bias64;   // overrides bias when non-empty (finite differences)
    std::vector<uint64_t> active;  // linear indices, brick-major order
    std::vector<uint8_t> mark;     // scratch membership volume
    std::vector<uint8_t> bmark;    // scratch brick flags
    uint64_t n0 = 0, iterations = 0, updates = 0;
    int threads = 1;
    std::vector<double> last_old, last_new;  // values of the last step, list order

    size_t idx(int x, int y, int z) const { return ((size_t)z * ny + y) * nx + x; }

    double bias_at(uint64_t li) const {
        if (!bias64.empty()) return bias64[li];
        return bias.empty() ? 0.0 : (double)bias[li];
    }

    void init(int nx_, int ny_, int nz_, const float* img, int bx_, int by_, int bz_) {
        nx = nx_; ny = ny_; nz = nz_;
        bx = bx_; by = by_; bz = bz_;
        NBx = (nx + bx - 1) / bx; NBy = (ny + by - 1) / by; NBz = (nz + bz - 1) / bz;
        size_t N = (size_t)nx * ny * nz;
        I.assign(img, img + N);
        phi.assign(N, p.hi);
        mark.assign(N, 0);
        bmark.assign((size_t)NBx * NBy * NBz, 0);
        active.clear();
        bias.clear();
    }

    double at(int x, int y, int z) const {
        x = x < 0 ? 0 : (x >= nx ? nx - 1 : x);
        y = y < 0 ? 0 : (y >= ny ? ny - 1 : y);
        z = z < 0 ? 0 : (z >= nz ? nz - 1 : z);
        return phi[idx(x, y, z)];
    }

    void mark_voxel(int x, int y, int z) {
        mark[idx(x, y, z)] = 1;
        bmark[((size_t)(z / bz) * NBy + (y / by)) * NBx + (x / bx)] = 1;
    }

    // Collects the marked voxels in brick-major order and clears the marks.
    void collect() {
        active.clear();
        for (int kz = 0; kz < NBz; ++kz)
            for (int ky = 0; ky < NBy; ++ky)
                for (int kx = 0; kx < NBx; ++kx) {
                    size_t b = ((size_t)kz * NBy + ky) * NBx + kx;
                    if (!bmark[b]) continue;
                    bmark[b] = 0;
                    for (int lz = 0; lz < bz; ++lz)
                        for (int ly = 0; ly < by; ++ly)
                            for (int lx = 0; lx < bx; ++lx) {
                                int x = kx * bx + lx, y = ky * by + ly, z = kz * bz + lz;
                                if (x >= nx || y >= ny || z >= nz) continue;
                                size_t i = idx(x, y, z);
                                if (mark[i]) { mark[i] = 0; active.push_back(i); }
                            }
                }
    }

    // Initial active set: a 6-neighbour differs by more than thr_s.
    void init_active() {
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x) {
                    double c = phi[idx(x, y, z)];
                    double m = 0;
                    m = std::max(m, std::fabs(at(x - 1, y, z) - c));
                    m = std::max(m, std::fabs(at(x + 1, y, z) - c));
                    m = std::max(m, std::fabs(at(x, y - 1, z) - c));
                    m = std::max(m, std::fabs(at(x, y + 1, z) - c));
                    m = std::max(m, std::fabs(at(x, y, z - 1) - c));
                    m = std::max(m, std::fabs(at(x, y, z + 1) - c));
                    if (m > p.thr_s) mark_voxel(x, y, z);
                }
        collect();
        n0 = active.size();
        iterations = 0;
        updates = 0;
    }

    void set_phi(const float* ph) {
        for (size_t i = 0; i < phi.size(); ++i) phi[i] = ph[i];
        init_active();
    }

    template <class F>
    void parallel_for(size_t n, F f) {
        int T = std::max(1, threads);
        if (T == 1 || n < 4096) { f(0, n); return; }
        std::vector<std::thread> pool;
        size_t chunk = (n + T - 1) / T;
        for (int t = 0; t < T; ++t) {
            size_t a = t * chunk, b = std::min(n, a + chunk);
            if (a >= b) break;
            pool.emplace_back([=] { f(a, b); });
        }
        for (auto& th : pool) th.join();
    }

    // Expansion of the changed set into the next active list.
    void expand(const std::vector<uint8_t>& changed) {
        const std::vector<uint64_t>& cur = active;
        for (size_t i = 0; i < cur.size(); ++i) {
            if (!changed[i]) continue;
            uint64_t li = cur[i];
            int x = (int)(li % nx), y = (int)((li / nx) % ny), z = (int)(li / ((size_t)nx * ny));
            for (int dz = -1; dz <= 1; ++dz)
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        if (p.nbh == 6 && (dx != 0) + (dy != 0) + (dz != 0) > 1) continue;
                        int X = x + dx, Y = y + dy, Z = z + dz;
                        if (X < 0 || Y < 0 || Z < 0 || X >= nx || Y >= ny || Z >= nz) continue;
                        mark_voxel(X, Y, Z);
                    }
        }
        collect();
    }

    // One iteration; returns the new active count.
    size_t step() {
        size_t n = active.size();
        last_old.resize(n);
        last_new.resize(n);
        std::vector<uint8_t> changed(n);
        parallel_for(n, [&](size_t a, size_t b) {
            auto P = [&](int x, int y, int z) { return at(x, y, z); };
            for (size_t i = a; i < b; ++i) {
                uint64_t li = active[i];
                int x = (int)(li % nx), y = (int)((li / nx) % ny), z = (int)(li / ((size_t)nx * ny));
                double bb = bias_at(li);
                double nv = ns_update<double>(P, x, y, z, (double)I[li], bb, p);
                last_old[i] = phi[li];
                last_new[i] = nv;
                changed[i] = std::fabs(nv - phi[li]) > p.thr_t;
            }
        });
        for (size_t i = 0; i < n; ++i) phi[active[i]] = last_new[i];
        updates += n;
        ++iterations;
        expand(changed);
        return active.size();
    }
};

}  // namespace lssns
