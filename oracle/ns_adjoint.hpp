// ORACLE — test infrastructure only (the FP64 parity reference of the GPU
// adjoint in LSS_MODE_NS).  Nothing in the product links it.
//
// Differentiation of K unrolled iterations of the LSS_MODE_NS update
// (ns_update in ns_model.hpp) with the active set of every iteration recorded
// in the forward pass and then held fixed:
//   phi_{k+1}[v] = ns_update(phi_k)[v]  for v in A_k,   phi_k[v] otherwise;
//   loss = 1 - 2 sum(s t) / (sum s + sum t),  s = sigmoid(-phi_K / tau),
//   t = target mask.
// The reverse pass propagates lambda_k = dloss/dphi_k through the transposed
// stencil Jacobian of every active voxel and accumulates dloss/dT, dloss/deps,
// dloss/dalpha and dloss/dbias[v].  The reference has no differentiation
// form; this restatement is pinned by central finite differences of the same
// FP64 forward (tests/test_adjoint_oracle.py).
#pragma once

#include <cmath>
#include <vector>

#include "ns_model.hpp"

namespace lssns {

// Vector-Jacobian product of ns_update at (x, y, z) with upstream gradient
// lam = dloss/dnv.  addphi(x', y', z', g) receives dloss/dphi at every stencil
// point (coordinates not yet clamped); the parameter gradients are added to
// g[0..3] = (T, eps, alpha, bias).
template <class PF, class AF>
inline void ns_update_vjp(PF P, AF addphi, int x, int y, int z, double I, double bias, const Params& p,
                          double lam, double* g) {
    const double c = P(x, y, z);
    const double xm = P(x - 1, y, z), xp = P(x + 1, y, z);
    const double ym = P(x, y - 1, z), yp = P(x, y + 1, z);
    const double zm = P(x, y, z - 1), zp = P(x, y, z + 1);
    const double cx = (xp - xm) * 0.5, cy = (yp - ym) * 0.5, cz = (zp - zm) * 0.5;
    const double fxx = xp - 2 * c + xm, fyy = yp - 2 * c + ym, fzz = zp - 2 * c + zm;
    const double fxy = (P(x + 1, y + 1, z) - P(x + 1, y - 1, z) - P(x - 1, y + 1, z) + P(x - 1, y - 1, z)) * 0.25;
    const double fxz = (P(x + 1, y, z + 1) - P(x + 1, y, z - 1) - P(x - 1, y, z + 1) + P(x - 1, y, z - 1)) * 0.25;
    const double fyz = (P(x, y + 1, z + 1) - P(x, y + 1, z - 1) - P(x, y - 1, z + 1) + P(x, y - 1, z - 1)) * 0.25;
    const double g2 = cx * cx + cy * cy + cz * cz;
    double curv = 0, num = 0;
    const bool has_curv = g2 > 1e-12;
    if (has_curv) {
        num = fxx * (cy * cy + cz * cz) + fyy * (cx * cx + cz * cz) + fzz * (cx * cx + cy * cy) -
              2 * (cx * cy * fxy + cx * cz * fxz + cy * cz * fyz);
        curv = num / g2;
    }
    const double Draw = p.data_literal ? p.eps - std::fabs(I - p.T) : (p.eps - std::fabs(I - p.T)) / p.eps;
    const bool dclamp = !p.data_literal && (Draw < -1 || Draw > 1);
    const double Dt = (p.data_literal ? Draw : std::min(std::max(Draw, -1.0), 1.0)) + bias;
    const double wc = p.alpha_data ? 1 - p.alpha : p.alpha;
    const double wd = 1 - wc;
    const double F = wd * Dt;
    const double dxm = c - xm, dxp = xp - c, dym = c - ym, dyp = yp - c, dzm = c - zm, dzp = zp - c;
    double a, b, e, f, h, k;
    if (F > 0) {
        a = std::max(dxm, 0.0); b = std::min(dxp, 0.0); e = std::max(dym, 0.0);
        f = std::min(dyp, 0.0); h = std::max(dzm, 0.0); k = std::min(dzp, 0.0);
    } else {
        a = std::min(dxm, 0.0); b = std::max(dxp, 0.0); e = std::min(dym, 0.0);
        f = std::max(dyp, 0.0); h = std::min(dzm, 0.0); k = std::max(dzp, 0.0);
    }
    const double gn = std::sqrt(a * a + b * b + e * e + f * f + h * h + k * k);
    const double u = c + p.dt * (wc * curv - F * gn);
    if (u < p.lo || u > p.hi) return;  // clamped: no gradient
    // u = c + dt (wc curv - F gn)
    addphi(x, y, z, lam);
    const double gcurv = lam * p.dt * wc, gF = -lam * p.dt * gn, ggn = -lam * p.dt * F;
    if (has_curv) {
        const double gnum = gcurv / g2, gg2 = -gcurv * curv / g2;
        const double gcx = gnum * (2 * cx * (fyy + fzz) - 2 * (cy * fxy + cz * fxz)) + gg2 * 2 * cx;
        const double gcy = gnum * (2 * cy * (fxx + fzz) - 2 * (cx * fxy + cz * fyz)) + gg2 * 2 * cy;
        const double gcz = gnum * (2 * cz * (fxx + fyy) - 2 * (cx * fxz + cy * fyz)) + gg2 * 2 * cz;
        const double gfxx = gnum * (cy * cy + cz * cz), gfyy = gnum * (cx * cx + cz * cz),
                     gfzz = gnum * (cx * cx + cy * cy);
        const double gfxy = -2 * gnum * cx * cy, gfxz = -2 * gnum * cx * cz, gfyz = -2 * gnum * cy * cz;
        addphi(x + 1, y, z, 0.5 * gcx + gfxx);
        addphi(x - 1, y, z, -0.5 * gcx + gfxx);
        addphi(x, y + 1, z, 0.5 * gcy + gfyy);
        addphi(x, y - 1, z, -0.5 * gcy + gfyy);
        addphi(x, y, z + 1, 0.5 * gcz + gfzz);
        addphi(x, y, z - 1, -0.5 * gcz + gfzz);
        addphi(x, y, z, -2 * (gfxx + gfyy + gfzz));
        addphi(x + 1, y + 1, z, 0.25 * gfxy);
        addphi(x + 1, y - 1, z, -0.25 * gfxy);
        addphi(x - 1, y + 1, z, -0.25 * gfxy);
        addphi(x - 1, y - 1, z, 0.25 * gfxy);
        addphi(x + 1, y, z + 1, 0.25 * gfxz);
        addphi(x + 1, y, z - 1, -0.25 * gfxz);
        addphi(x - 1, y, z + 1, -0.25 * gfxz);
        addphi(x - 1, y, z - 1, 0.25 * gfxz);
        addphi(x, y + 1, z + 1, 0.25 * gfyz);
        addphi(x, y + 1, z - 1, -0.25 * gfyz);
        addphi(x, y - 1, z + 1, -0.25 * gfyz);
        addphi(x, y - 1, z - 1, 0.25 * gfyz);
    }
    if (gn > 0) {
        // d gn / d(one-sided difference d) = d / gn where the difference is selected.
        const double s = ggn / gn;
        addphi(x, y, z, s * (a - b + e - f + h - k));
        addphi(x - 1, y, z, -s * a);
        addphi(x + 1, y, z, s * b);
        addphi(x, y - 1, z, -s * e);
        addphi(x, y + 1, z, s * f);
        addphi(x, y, z - 1, -s * h);
        addphi(x, y, z + 1, s * k);
    }
    // F = wd (Dc + bias); Dc = (eps - |I - T|) / eps unless clamped, or
    // eps - |I - T| (literal).
    const double gDt = gF * wd;
    g[3] += gDt;
    if (!dclamp) {
        const double sg = I > p.T ? 1.0 : (I < p.T ? -1.0 : 0.0);
        if (p.data_literal) {  // D = eps - |I - T|
            g[0] += gDt * sg;
            g[1] += gDt;
        } else {  // D = (eps - |I - T|) / eps
            g[0] += gDt * sg / p.eps;
            g[1] += gDt * std::fabs(I - p.T) / (p.eps * p.eps);
        }
    }
    // alpha: u = c + dt (wc curv - wd Dt gn), (wc, wd) = (1 - alpha, alpha) or (alpha, 1 - alpha).
    const double du_dalpha = p.dt * (-curv - Dt * gn);
    g[2] += lam * (p.alpha_data ? du_dalpha : -du_dalpha);
}

struct AdjointResult {
    double loss = 0, dT = 0, deps = 0, dalpha = 0;
    std::vector<double> dbias;  // per voxel (nx*ny*nz)
};

// Compensated (Neumaier) running sum: the rounding error of a sum over
// millions of voxels stays at one ulp of the result, so that two losses whose
// fields differ in a few voxels (central finite differences of a single bias
// voxel) differ by what those voxels contribute, not by rounding noise.
struct CompensatedSum {
    double sum = 0, c = 0;
    void add(double x) {
        const double t = sum + x;
        c += std::fabs(sum) >= std::fabs(x) ? (sum - t) + x : (x - t) + sum;
        sum = t;
    }
    double value() const { return sum + c; }
};

// Soft-Dice loss of sigmoid(-phi/tau) against target, and dloss/dphi.
inline double soft_dice(const std::vector<double>& phi, const uint8_t* target, double tau,
                        std::vector<double>* grad, double* coefficient = nullptr) {
    CompensatedSum css, cst;
    double tt = 0;
    const size_t N = phi.size();
    std::vector<double> s(N);
    for (size_t i = 0; i < N; ++i) {
        s[i] = 1.0 / (1.0 + std::exp(phi[i] / tau));
        css.add(s[i]);
        tt += target[i] ? 1.0 : 0.0;
        if (target[i]) cst.add(s[i]);
    }
    const double ss = css.value(), st = cst.value();
    const double den = ss + tt;
    const double loss = 1.0 - 2.0 * st / den;
    if (coefficient) *coefficient = 2.0 * st / den;
    if (grad) {
        grad->assign(N, 0.0);
        for (size_t i = 0; i < N; ++i) {
            const double dL_ds = -2.0 * ((target[i] ? 1.0 : 0.0) * den - st) / (den * den);
            const double ds_dphi = -s[i] * (1.0 - s[i]) / tau;
            (*grad)[i] = dL_ds * ds_dphi;
        }
    }
    return loss;
}

// K iterations of o (from its current phi and active list), recording the
// active lists in `sets` (or replaying them when `replay`), then the loss.
// o's phi / active / counters are restored on return.
// With `coefficient`, returns the soft-Dice coefficient 2 sum(s t) / (sum s +
// sum t) instead of the loss 1 - coefficient: near a loss of 1 the
// coefficient keeps ~1000x finer resolution (the subtraction from 1 rounds to
// the ulp of 1), which central differences of one bias voxel need.
inline double adjoint_forward(NsOracle& o, int K, const uint8_t* target, double tau,
                              std::vector<std::vector<uint64_t>>& sets, bool replay,
                              std::vector<std::vector<double>>* history, bool coefficient = false) {
    const std::vector<double> phi0 = o.phi;
    const std::vector<uint64_t> act0 = o.active;
    const uint64_t it0 = o.iterations, up0 = o.updates;
    if (!replay) sets.assign(1, act0);
    if (history) history->assign(1, o.phi);
    for (int k = 0; k < K; ++k) {
        o.active = sets[k];
        o.step();
        if (!replay) sets.push_back(o.active);
        if (history) history->push_back(o.phi);
    }
    double coef = 0;
    const double loss = soft_dice(o.phi, target, tau, nullptr, &coef);
    o.phi = phi0;
    o.active = act0;
    o.iterations = it0;
    o.updates = up0;
    return coefficient ? coef : loss;
}

inline AdjointResult adjoint_run(NsOracle& o, int K, const uint8_t* target, double tau,
                                 std::vector<std::vector<uint64_t>>& sets) {
    std::vector<std::vector<double>> hist;
    AdjointResult r;
    adjoint_forward(o, K, target, tau, sets, false, &hist);
    std::vector<double> lam;
    r.loss = soft_dice(hist[K], target, tau, &lam);
    const size_t N = lam.size();
    r.dbias.assign(N, 0.0);
    std::vector<double> nxt(N);
    const int nx = o.nx, ny = o.ny, nz = o.nz;
    auto clampi = [](int v, int n) { return v < 0 ? 0 : (v >= n ? n - 1 : v); };
    for (int k = K - 1; k >= 0; --k) {
        const std::vector<double>& ph = hist[k];
        auto P = [&](int x, int y, int z) {
            return ph[((size_t)clampi(z, nz) * ny + clampi(y, ny)) * nx + clampi(x, nx)];
        };
        // Inactive voxels pass lambda through; active ones are replaced by
        // their update, whose transposed Jacobian scatters lambda.
        nxt = lam;
        for (uint64_t li : sets[k]) nxt[li] = 0.0;
        auto add = [&](int x, int y, int z, double g) {
            nxt[((size_t)clampi(z, nz) * ny + clampi(y, ny)) * nx + clampi(x, nx)] += g;
        };
        for (uint64_t li : sets[k]) {
            const int x = (int)(li % nx), y = (int)((li / nx) % ny), z = (int)(li / ((size_t)nx * ny));
            const double bb = o.bias_at(li);
            double g[4] = {0, 0, 0, 0};
            ns_update_vjp(P, add, x, y, z, (double)o.I[li], bb, o.p, lam[li], g);
            r.dT += g[0];
            r.deps += g[1];
            r.dalpha += g[2];
            r.dbias[li] += g[3];
        }
        lam.swap(nxt);
    }
    return r;
}

}  // namespace lssns
