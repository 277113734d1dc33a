// ORACLE — test infrastructure only (the parity reference for LSS_MODE_NS,
// and the timed CPU baseline of bench.py).  Nothing in the product links it.
//
// FP64 restatement of the sparse level-set iteration in its LSS_MODE_NS form:
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
// clamped to [-1, 1] so that dt*|F| stays inside the upwind scheme's CFL bound;
// with data_literal it is eps - |I - T| as written.
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
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace lssns {

// A fixed set of worker threads reused by every parallel loop of an oracle
// (starting threads per iteration cost more than the work of a thin band).
// run(n, f) calls f(a, b) on the parts of [0, n) split into one contiguous
// part per thread; the calling thread takes part 0.
class Pool {
   public:
    explicit Pool(int threads) : T_(std::max(1, threads)) {
        for (int t = 1; t < T_; ++t) workers_.emplace_back([this, t] { loop(t); });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> g(mu_);
            quit_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto& w : workers_) w.join();
    }
    int size() const { return T_; }
    void run(size_t n, const std::function<void(size_t, size_t)>& f) {
        {
            std::lock_guard<std::mutex> g(mu_);
            f_ = &f;
            n_ = n;
            pending_ = T_ - 1;
            ++gen_;
        }
        cv_.notify_all();
        part(0);
        std::unique_lock<std::mutex> g(mu_);
        done_.wait(g, [this] { return pending_ == 0; });
        f_ = nullptr;
    }

   private:
    void part(int t) {
        const size_t chunk = (n_ + T_ - 1) / T_;
        const size_t a = std::min(n_, (size_t)t * chunk), b = std::min(n_, a + chunk);
        if (a < b) (*f_)(a, b);
    }
    void loop(int t) {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> g(mu_);
                cv_.wait(g, [&] { return gen_ != seen; });
                seen = gen_;
                if (quit_) return;
            }
            part(t);
            {
                std::lock_guard<std::mutex> g(mu_);
                if (--pending_ == 0) done_.notify_one();
            }
        }
    }
    int T_;
    std::vector<std::thread> workers_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    const std::function<void(size_t, size_t)>* f_ = nullptr;
    size_t n_ = 0;
    int pending_ = 0;
    uint64_t gen_ = 0;
    bool quit_ = false;
};

struct Params {
    double T = 0.5, eps = 0.1, alpha = 0.5, dt = 0.5;
    double lo = -4.0, hi = 4.0;
    double thr_t = 0.01, thr_s = 0.0;
    int nbh = 26;
    int alpha_data = 1;       // 1: alpha weights the data term, 0: the curvature term
    int data_literal = 0;     // 1: D = eps - |I - T| as written (no scaling, no clamp)
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
    Real D;
    if (p.data_literal) {
        D = Real(p.eps) - std::fabs(I - Real(p.T)) + bias;
    } else {
        D = (Real(p.eps) - std::fabs(I - Real(p.T))) / Real(p.eps);
        D = std::min(std::max(D, Real(-1)), Real(1)) + bias;
    }
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
    std::unique_ptr<Pool> pool;              // `threads` workers, made on first use
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

    // Marks are set from several threads at once: every store writes 1, so
    // relaxed atomic byte stores give the same marks in any order.
    void mark_voxel(int x, int y, int z) {
        __atomic_store_n(&mark[idx(x, y, z)], (uint8_t)1, __ATOMIC_RELAXED);
        __atomic_store_n(&bmark[((size_t)(z / bz) * NBy + (y / by)) * NBx + (x / bx)], (uint8_t)1,
                         __ATOMIC_RELAXED);
    }

    // Collects the marked voxels in brick-major order (bricks x fastest over
    // the brick grid, voxels x fastest inside a brick) and clears the marks.
    // The marked bricks are listed in order, split into contiguous parts
    // collected in parallel, and the parts concatenated in order.
    void collect() {
        std::vector<uint32_t> bricks;
        for (size_t b = 0; b < bmark.size(); ++b)
            if (bmark[b]) {
                bmark[b] = 0;
                bricks.push_back((uint32_t)b);
            }
        const int T = std::max(1, std::min(threads, (int)(bricks.size() / 8 + 1)));
        std::vector<std::vector<uint64_t>> parts(T);
        parallel_for(bricks.size(), [&](size_t a, size_t e) {
            const size_t chunk = (bricks.size() + T - 1) / T;
            std::vector<uint64_t>& out = parts[std::min((size_t)T - 1, a / std::max<size_t>(1, chunk))];
            for (size_t q = a; q < e; ++q) {
                const uint32_t b = bricks[q];
                const int kx = (int)(b % NBx), ky = (int)((b / NBx) % NBy), kz = (int)(b / ((size_t)NBx * NBy));
                for (int lz = 0; lz < bz; ++lz)
                    for (int ly = 0; ly < by; ++ly)
                        for (int lx = 0; lx < bx; ++lx) {
                            const int x = kx * bx + lx, y = ky * by + ly, z = kz * bz + lz;
                            if (x >= nx || y >= ny || z >= nz) continue;
                            const size_t i = idx(x, y, z);
                            if (mark[i]) { mark[i] = 0; out.push_back(i); }
                        }
            }
        }, T);
        active.clear();
        size_t tot = 0;
        for (auto& v : parts) tot += v.size();
        active.reserve(tot);
        for (auto& v : parts) active.insert(active.end(), v.begin(), v.end());
    }

    // Initial active set: a 6-neighbour differs by more than thr_s.
    void init_active() {
        parallel_for((size_t)nz, [&](size_t z0, size_t z1) {
            for (int z = (int)z0; z < (int)z1; ++z)
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
        }, threads, 1);
        collect();
        n0 = active.size();
        iterations = 0;
        updates = 0;
    }

    void set_phi(const float* ph) {
        for (size_t i = 0; i < phi.size(); ++i) phi[i] = ph[i];
        init_active();
    }

    // f(a, b) over [0, n) split into `parts` contiguous parts (default: one
    // per thread) run on the pool; serial below `min_n` items.
    template <class F>
    void parallel_for(size_t n, F f, int parts = 0, size_t min_n = 4096) {
        const int T = std::max(1, parts > 0 ? std::min(parts, threads) : threads);
        if (T == 1 || n < min_n) { f(0, n); return; }
        if (!pool || pool->size() != threads) pool.reset(new Pool(threads));
        if (T == pool->size()) {
            pool->run(n, f);
            return;
        }
        // Fewer parts than threads: part t of T on pool thread t, the rest idle.
        const size_t chunk = (n + T - 1) / T;
        pool->run((size_t)pool->size(), [&](size_t a, size_t b) {
            for (size_t t = a; t < b; ++t) {
                if ((int)t >= T) continue;
                const size_t s = t * chunk, e = std::min(n, s + chunk);
                if (s < e) f(s, e);
            }
        });
    }

    // Expansion of the changed set into the next active list.
    void expand(const std::vector<uint8_t>& changed) {
        const std::vector<uint64_t>& cur = active;
        parallel_for(cur.size(), [&](size_t a, size_t e) {
            for (size_t i = a; i < e; ++i) {
                if (!changed[i]) continue;
                uint64_t li = cur[i];
                int x = (int)(li % nx), y = (int)((li / nx) % ny), z = (int)(li / ((size_t)nx * ny));
                // Per axis: the neighbour coordinate and its brick coordinate
                // (three values each, so no division per neighbour).
                int bxs[3], bys[3], bzs[3];
                for (int d = 0; d < 3; ++d) {
                    bxs[d] = (x + d - 1) >= 0 ? (x + d - 1) / bx : -1;
                    bys[d] = (y + d - 1) >= 0 ? (y + d - 1) / by : -1;
                    bzs[d] = (z + d - 1) >= 0 ? (z + d - 1) / bz : -1;
                }
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            if (p.nbh == 6 && (dx != 0) + (dy != 0) + (dz != 0) > 1) continue;
                            int X = x + dx, Y = y + dy, Z = z + dz;
                            if (X < 0 || Y < 0 || Z < 0 || X >= nx || Y >= ny || Z >= nz) continue;
                            // Test before setting: most neighbours are marked
                            // already, and a store would dirty the line.
                            uint8_t* m = &mark[idx(X, Y, Z)];
                            if (__atomic_load_n(m, __ATOMIC_RELAXED)) continue;
                            __atomic_store_n(m, (uint8_t)1, __ATOMIC_RELAXED);
                            uint8_t* bm = &bmark[((size_t)bzs[dz + 1] * NBy + bys[dy + 1]) * NBx + bxs[dx + 1]];
                            if (!__atomic_load_n(bm, __ATOMIC_RELAXED)) __atomic_store_n(bm, (uint8_t)1, __ATOMIC_RELAXED);
                        }
            }
        });
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
