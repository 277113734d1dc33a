// ORACLE — test infrastructure only.  C entry points over the CPU
// restatements in ref_model.hpp (LSS_MODE_REF) and ns_model.hpp
// (LSS_MODE_NS), loaded by tests/, __graft_entry__.smoke() and bench.py's CPU
// legs through oracle/oracle.py.  Built by oracle/build.py with
// -ffp-contract=off so that every float operation is a single IEEE-754
// operation on x86-64 and aarch64 alike.
#include <cstdint>
#include <cstring>
#include <exception>
#include <string>

#ifdef LSS_ORACLE_REFERENCE_KERNELS
#include "ref_shim/ref_backend.hpp"
#endif
#include "ns_adjoint.hpp"
#include "ns_model.hpp"
#include "ref_model.hpp"

using lssref::RefSegmenter;
using lssref::RestatedBackend;

#ifdef LSS_ORACLE_REFERENCE_KERNELS
using Backend = lssrefshim::ReferenceBackend;
#define OREF(name) oref_refk_##name
#else
using Backend = RestatedBackend;
#define OREF(name) oref_##name
#endif
using Seg = RefSegmenter<Backend>;

static thread_local std::string g_err;

#define GUARD(body)                                   \
    try {                                             \
        body;                                         \
        return 0;                                     \
    } catch (const std::exception& ex) {              \
        g_err = ex.what();                            \
        return 1;                                     \
    }

extern "C" {

const char* OREF(last_error)() { return g_err.c_str(); }

void* OREF(create)(const void* data, uint32_t nx, uint32_t ny, uint32_t nz, int dtype,
                   float aniso, int quirk) {
    try {
        Seg* s = new Seg();
#ifndef LSS_ORACLE_REFERENCE_KERNELS
        s->be.quirk_i3 = quirk != 0;
#else
        (void)quirk;
#endif
        s->load(data, nx, ny, nz, dtype, aniso);
        return s;
    } catch (const std::exception& ex) {
        g_err = ex.what();
        return nullptr;
    }
}

void OREF(destroy)(void* h) { delete (Seg*)h; }

int OREF(set_params)(void* h, float t, float w, float a, float dt, float conv) {
    GUARD(((Seg*)h)->set_params(t, w, a, dt, conv))
}

int OREF(initialize_seed)(void* h, float cx, float cy, float cz, float r) {
    GUARD(((Seg*)h)->initialize_seed(cx, cy, cz, r))
}

int OREF(set_phi)(void* h, const float* phi) { GUARD(((Seg*)h)->set_phi(phi)) }

int OREF(step)(void* h, int k) {
    try {
        return ((Seg*)h)->request_update(k);
    } catch (const std::exception& ex) {
        g_err = ex.what();
        return -1;
    }
}

uint64_t OREF(active_count)(void* h) { return ((Seg*)h)->n; }
int OREF(iterations)(void* h) { return ((Seg*)h)->iterations; }
int OREF(finished)(void* h) { return ((Seg*)h)->finished() ? 1 : 0; }

void OREF(padded_dims)(void* h, uint32_t* out3) {
    Seg* s = (Seg*)h;
    out3[0] = s->d.x; out3[1] = s->d.y; out3[2] = s->d.z;
}

// which: 0 phi read (int8 tiled), 1 phi write, 2 export (u8 linear), 3 tag,
// 4 coord (u32), 5 valid (u32), 6 active (u32, first n), 7 frozen.
int OREF(get_buffer)(void* h, int which, void* out) {
    Seg* s = (Seg*)h;
    size_t N = s->N;
    switch (which) {
        case 0: std::memcpy(out, s->rd, N); return 0;
        case 1: std::memcpy(out, s->wr, N); return 0;
        case 2: std::memcpy(out, s->exportv.data(), N); return 0;
        case 3: std::memcpy(out, s->tag.data(), N); return 0;
        case 4: std::memcpy(out, s->coord.data(), N * 4); return 0;
        case 5: std::memcpy(out, s->valid.data(), N * 4); return 0;
        case 6: std::memcpy(out, s->active.data(), s->n * 4); return 0;
        case 7: std::memcpy(out, s->frozen.data(), N); return 0;
    }
    return 1;
}

int OREF(read_mask)(void* h, uint8_t* out) { GUARD(((Seg*)h)->read_mask(out)) }
int OREF(read_phi)(void* h, float* out) { GUARD(((Seg*)h)->read_phi(out)) }
int OREF(read_export)(void* h, int8_t* out) { GUARD(((Seg*)h)->read_export(out)) }
int OREF(read_active_volume)(void* h, uint8_t* out) { GUARD(((Seg*)h)->read_active_volume(out)) }
int OREF(freeze)(void* h) { GUARD(((Seg*)h)->freeze()) }
int OREF(clear_current)(void* h) { GUARD(((Seg*)h)->clear_current()) }
int OREF(clear_all)(void* h) { GUARD(((Seg*)h)->clear_all()) }
int OREF(estimate_params)(void* h, float* t, float* w) { GUARD(((Seg*)h)->estimate_params(t, w)) }

#ifndef LSS_ORACLE_REFERENCE_KERNELS
// ---------------------------------------------------------------------------
// LSS_MODE_NS oracle.
using lssns::NsOracle;

void* ons_create(int nx, int ny, int nz, const float* img, int bx, int by, int bz) {
    try {
        NsOracle* o = new NsOracle();
        o->init(nx, ny, nz, img, bx, by, bz);
        return o;
    } catch (const std::exception& ex) {
        g_err = ex.what();
        return nullptr;
    }
}

void ons_destroy(void* h) { delete (NsOracle*)h; }

void ons_set_params(void* h, double T, double eps, double alpha, double dt, double lo, double hi,
                    double thr_t, double thr_s, int nbh) {
    NsOracle* o = (NsOracle*)h;
    o->p.T = T; o->p.eps = eps; o->p.alpha = alpha; o->p.dt = dt;
    o->p.lo = lo; o->p.hi = hi; o->p.thr_t = thr_t; o->p.thr_s = thr_s; o->p.nbh = nbh;
}

void ons_set_alpha_role(void* h, int alpha_data) { ((NsOracle*)h)->p.alpha_data = alpha_data; }

void ons_set_data_term(void* h, int literal) { ((NsOracle*)h)->p.data_literal = literal; }

void ons_set_threads(void* h, int t) { ((NsOracle*)h)->threads = t; }

void ons_set_bias(void* h, const float* b) {
    NsOracle* o = (NsOracle*)h;
    o->bias64.clear();
    if (!b) { o->bias.clear(); return; }
    o->bias.assign(b, b + o->phi.size());
}

void ons_set_phi(void* h, const float* phi) { ((NsOracle*)h)->set_phi(phi); }

// Sets phi and an explicit active list (linear indices, any order; stored
// sorted into brick-major order).
void ons_set_state(void* h, const float* phi, const uint64_t* act, uint64_t n) {
    NsOracle* o = (NsOracle*)h;
    for (size_t i = 0; i < o->phi.size(); ++i) o->phi[i] = phi[i];
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t li = act[i];
        int x = (int)(li % o->nx), y = (int)((li / o->nx) % o->ny), z = (int)(li / ((uint64_t)o->nx * o->ny));
        o->mark_voxel(x, y, z);
    }
    o->collect();
}

uint64_t ons_step(void* h, int k) {
    NsOracle* o = (NsOracle*)h;
    for (int i = 0; i < k; ++i) o->step();
    return o->active.size();
}

// Runs to the stopping rule, evaluated after each iteration on n_k, the
// number of active voxels that iteration updated: stop once n_k < rel*n0 for
// `patience` consecutive iterations, once n_k <= abs_thr, or after max_it
// iterations.  Returns the iterations run.
int ons_run(void* h, double rel, int patience, int max_it, uint64_t abs_thr) {
    NsOracle* o = (NsOracle*)h;
    int streak = 0, it = 0;
    while (it < max_it) {
        const size_t n = o->active.size();
        o->step();
        ++it;
        if ((double)n < rel * (double)o->n0) ++streak; else streak = 0;
        if (streak >= patience || n <= abs_thr) break;
    }
    return it;
}

uint64_t ons_active_count(void* h) { return ((NsOracle*)h)->active.size(); }
uint64_t ons_initial_count(void* h) { return ((NsOracle*)h)->n0; }
uint64_t ons_updates(void* h) { return ((NsOracle*)h)->updates; }

void ons_read_active(void* h, uint64_t* out) {
    NsOracle* o = (NsOracle*)h;
    std::memcpy(out, o->active.data(), o->active.size() * 8);
}

void ons_read_phi(void* h, float* out) {
    NsOracle* o = (NsOracle*)h;
    for (size_t i = 0; i < o->phi.size(); ++i) out[i] = (float)o->phi[i];
}

void ons_read_phi64(void* h, double* out) {
    NsOracle* o = (NsOracle*)h;
    std::memcpy(out, o->phi.data(), o->phi.size() * 8);
}

// The expansion rule alone, for "bit-exact given identical phi" checks:
// given the active list (linear indices), the values before and after one
// update (list order), returns the next list in brick-major order.
uint64_t ons_expand_given(void* h, const uint64_t* act, uint64_t n, const float* before,
                          const float* after, uint64_t* out) {
    NsOracle* o = (NsOracle*)h;
    o->active.assign(act, act + n);
    std::vector<uint8_t> changed(n);
    for (uint64_t i = 0; i < n; ++i)
        changed[i] = std::fabs(after[i] - before[i]) > (float)o->p.thr_t;  // the kernel's fp32 test
    o->expand(changed);
    std::memcpy(out, o->active.data(), o->active.size() * 8);
    return o->active.size();
}

// ---- FP64 adjoint (ns_adjoint.hpp) ----------------------------------------
// Active sets recorded by the last ons_adj_run of each handle.
static std::vector<std::vector<uint64_t>>& adj_sets(void* h) {
    static thread_local std::vector<std::pair<void*, std::vector<std::vector<uint64_t>>>> table;
    for (auto& e : table)
        if (e.first == h) return e.second;
    table.push_back({h, {}});
    return table.back().second;
}

// K iterations from the current state (recorded active sets), the soft-Dice
// loss and its gradients: out[0..3] = loss, dT, deps, dalpha; dbias (nullable,
// nx*ny*nz doubles).  The oracle's state is unchanged.
void ons_adj_run(void* h, int K, const uint8_t* target, double tau, double* out, double* dbias) {
    NsOracle* o = (NsOracle*)h;
    lssns::AdjointResult r = lssns::adjoint_run(*o, K, target, tau, adj_sets(h));
    out[0] = r.loss; out[1] = r.dT; out[2] = r.deps; out[3] = r.dalpha;
    if (dbias) std::memcpy(dbias, r.dbias.data(), r.dbias.size() * 8);
}

// The loss of K iterations replaying the active sets of the last
// ons_adj_run (finite differences under the fixed-set convention).
double ons_adj_loss(void* h, int K, const uint8_t* target, double tau) {
    NsOracle* o = (NsOracle*)h;
    return lssns::adjoint_forward(*o, K, target, tau, adj_sets(h), true, nullptr);
}

// The soft-Dice coefficient (1 - loss) of the same replay, at full
// resolution (finite differences of single bias voxels).
double ons_adj_dice(void* h, int K, const uint8_t* target, double tau) {
    NsOracle* o = (NsOracle*)h;
    return lssns::adjoint_forward(*o, K, target, tau, adj_sets(h), true, nullptr, true);
}

// Sets one parameter: 0 T, 1 eps, 2 alpha.
void ons_set_param(void* h, int which, double v) {
    NsOracle* o = (NsOracle*)h;
    if (which == 0) o->p.T = v;
    if (which == 1) o->p.eps = v;
    if (which == 2) o->p.alpha = v;
}

// Bias from doubles (finite differences need perturbations below fp32 ulp).
void ons_set_bias64(void* h, const double* b) {
    NsOracle* o = (NsOracle*)h;
    if (!b) { o->bias64.clear(); return; }
    o->bias64.assign(b, b + o->phi.size());
}
#endif

}  // extern "C"
