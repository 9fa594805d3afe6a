// C ABI of the H/S generation library (include/hsdla.h).
//
// Host side of the drop-in for create_HS2 (flapw_opt/src/h_and_s.cpp:591-893):
// validation of the AtomData-like inputs, upload of per-run tables, device
// workspace, and the per-call pipeline
//
//   (a) construct_AB            -> C = [A_a; B_a] per atom          (kernel a)
//   (b) X_a = T_a C_a           -> per-atom T application           (kernel b)
//   (c) S = C^H diag(w) C, H = C^H X, lower triangles               (kernel c)
//
// in either plain FP64 or the Ozaki FP8 form.  Errors are returned as status
// codes with a message in the context (the reference prints and exits,
// h_and_s.cpp:712-723).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "ozaki.cuh"

using namespace hsdla;

struct hsdla_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int64_t mem_cap = 0;       // 0 = no cap
    int64_t mem_used = 0;
    int nsm = 0;
    // persistent workspace reused across calls (grows on demand)
    void *ws = nullptr;
    int64_t ws_bytes = 0;
    // device H/S buffer of the host-buffer entry points, kept across calls (grows on demand)
    void *hout = nullptr;
    int64_t hout_bytes = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evs[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // host-buffer entry points: downloads overlapped with the last combine run on this stream
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copy = nullptr;
    // device blocks of at most kCacheBlockMax released by plans, kept for the next plan (a plan's
    // tables and job lists come and go with every hsdla_create_hs): size -> pointer, and the live
    // blocks' sizes
    std::multimap<int64_t, void *> cache;
    std::map<void *, int64_t> live;
    int64_t cached_bytes = 0;
    // page-locked staging of a plan's table upload (grows on demand; a plan's upload completes
    // before hsdla_plan_create returns, so the next plan reuses it)
    void *staging = nullptr;
    int64_t staging_bytes = 0;
    std::set<hsdla_plan *> plans;   // live plans, destroyed with the context
    // slice autotuner results: (L, atoms, types, n_G bucket, target) -> (slices, predicted error)
    std::map<std::tuple<int, int, int, int64_t, double>, std::pair<int, double>> tune_cache;
    // the BLAS-shaped plugin's Ozaki state (its device error word), set up on first use
    OzakiPlan plugin_oz{};
    // tile tuner results of the structure-factor form: (2L, row sets, k-points of the first group,
    // its largest n_G bucket, slices) -> (halves, merged)
    std::map<std::tuple<int, int, int, int64_t, int>, std::pair<int, int>> tile_cache;
};

struct PlanKpoint {
    DevKpoint dk;
    int64_t n_g;
};

struct hsdla_plan {
    hsdla_context *ctx = nullptr;
    hsdla_opts opts{};
    int L = 0, na = 0, nt = 0, max_lmax = 0;
    int64_t twoLa = 0;
    DevSystem dsys{};
    std::vector<PlanKpoint> kps;
    std::vector<int32_t> atom_type;
    double flop = 0.0;
    // device allocations owned by the plan
    void *tables = nullptr;          // system arrays, T blocks, weights, G lists
    int64_t tables_bytes = 0;
    double2 *Tfull = nullptr;        // [nt][2L][2L]
    double *w = nullptr;             // [2La] S row weights
    double *wsqrt = nullptr;         // [2La] sqrt of the S row weights (Ozaki left operand)
    Fp64Job *d_jobs = nullptr;       // job table (device)
    int64_t jobs_cap = 0;
    std::vector<Fp64Job> h_jobs;
    OzakiPlan oz{};
    // k-point groups, prepared against the context workspace (re-prepared when it moves)
    struct Group {
        std::vector<int> kidx;           // plan k-point indices
        KTable ktab;                     // construct / phase tables (C, M, Z, X per k-point)
        OzGroup *oz = nullptr;           // Ozaki engine state
        Fp64Job *d_jobs_t = nullptr;     // FP64: T application jobs (device, in the workspace)
        int n_jobs_t = 0;
        int64_t tiles_t = 0;
        Fp64Job *d_jobs_sh = nullptr;    // FP64: S/H jobs (device) and their pinned host copy
        Fp64Job *h_jobs_sh = nullptr;
        int64_t tiles_sh = 0;
        void *persist = nullptr;         // prepared tables (not shared with other groups)
        int64_t persist_bytes = 0;
        // event pairs around the S/H product launches (one pair, or one per type in the
        // structure-factor form; recorded under graph capture too)
        std::vector<cudaEvent_t> ev_dom;
        // event pairs around the T-application launches (un-graphed runs; the report's ms_tapply)
        std::vector<cudaEvent_t> ev_t;
        SfTab sft{};                     // structure-factor combine of this group (outputs per run)
    };
    std::vector<Group> groups;
    void *prepared_ws = nullptr;
    int64_t group_ws_bytes = 0;          // workspace of the largest group
    cudaGraphExec_t graph = nullptr;     // captured execution
    std::vector<void *> graph_outputs;   // output pointers the graph was captured with
    cudaStream_t graph_stream = nullptr;
    bool graph_failed = false;
    bool autotune = false;           // Ozaki slice count still to be chosen from the data
    bool hoist = false;              // T application per type (no atom carries its own rotation)
    bool external = false;           // C is supplied by the caller (contraction-only entry)
    int panels = 1;                  // atom panels of the Ozaki contraction (memory-bounded streaming)
    // structure-factor form (atoms share their type's rotation): per-type S weights [nt][2L] and
    // the structure factors SF_t over the box of G-vector differences
    bool sf = false;
    int classes = 0;                 // (type, rotation) classes the structure-factor form runs over (0: types)
    // T-block check read after the call's own synchronisation (hsdla_create_hs): the device's
    // statistics land in the context's page-locked staging, checked once the stream is idle
    bool tcheck_pending = false;
    const unsigned long long *tcheck_host = nullptr;
    std::vector<int32_t> tcheck_class_type;
    double *wt = nullptr;
    double2 *sf_tab = nullptr;
    SfTab sf_dims{};                 // box extents and offsets (entries filled per group)
    int tbatch = 1;                  // types whose products are combined into S and H in one pass
    // hsdla_create_hs: the host outputs the last combine of each group downloads column block by
    // column block on the context's copy stream (structure-factor form, no graph); `done` reports it
    struct Download {
        std::vector<hsdla_cx *> H, S;
        std::vector<int64_t> ld;
        bool direct = false;   // every output is page-locked host memory the GPU can write
        bool done = false;
        bool in_place = false;   // the combine wrote the host outputs
        int blocks = 0;          // ... in column blocks while the products of the next ran (0: after them)
    };
    Download *dl = nullptr;
    double est_err = 0.0;            // autotuner's predicted relative error
    int launches = 0;
    bool tiles_tuned = false;        // the S/H tile configuration came from the tile tuner
    bool tiles_done = false;         // nothing (more) to tune
    int tile_h = 0, tile_m = 0;      // the tuned configuration (re-applied when groups are re-prepared)
};

namespace {

int set_err(hsdla_context *ctx, int code, const char *fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return code;
}

#define CUDA_TRY(ctx, call)                                                                           \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return set_err((ctx), HSDLA_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));    \
    } while (0)

// Environment switch: unset or empty -> dflt, "0" -> false, anything else -> true.
bool env_flag(const char *name, bool dflt) {
    const char *v = getenv(name);
    if (!v || !*v) return dflt;
    return strcmp(v, "0") != 0;
}

constexpr int64_t kCacheBlockMax = (int64_t)256 << 20;    // larger blocks are freed, not kept
constexpr int64_t kCacheBytesMax = (int64_t)1 << 30;       // at most this much kept

// Returns every kept block to the driver.
void ctx_cache_release(hsdla_context *ctx) {
    if (ctx->cache.empty()) return;
    cudaDeviceSynchronize();
    for (auto &b : ctx->cache) cudaFree(b.second);
    ctx->mem_used -= ctx->cached_bytes;
    ctx->cache.clear();
    ctx->cached_bytes = 0;
}

// Device allocations of the context.  Blocks up to kCacheBlockMax are served from the blocks
// earlier plans released when one of at most twice the size is kept; the memory cap counts kept
// blocks as used (they are released first when a request would exceed it).
int ctx_malloc(hsdla_context *ctx, void **p, int64_t bytes) {
    *p = nullptr;
    if (bytes <= 0) return HSDLA_OK;
    // a cap below what the context holds: kept blocks go first, and every request is checked
    if (ctx->mem_cap > 0 && ctx->mem_used > ctx->mem_cap) ctx_cache_release(ctx);
    if (bytes <= kCacheBlockMax && (ctx->mem_cap == 0 || ctx->mem_used <= ctx->mem_cap)) {
        auto it = ctx->cache.lower_bound(bytes);
        if (it != ctx->cache.end() && it->first <= 2 * bytes) {
            *p = it->second;
            ctx->live[*p] = it->first;
            ctx->cached_bytes -= it->first;
            ctx->cache.erase(it);
            return HSDLA_OK;
        }
    }
    if (ctx->mem_cap > 0 && ctx->mem_used + bytes > ctx->mem_cap) ctx_cache_release(ctx);
    if (ctx->mem_cap > 0 && ctx->mem_used + bytes > ctx->mem_cap)
        return set_err(ctx, HSDLA_ERR_NOMEM, "device allocation of %lld bytes exceeds the cap (%lld used of %lld)",
                       (long long)bytes, (long long)ctx->mem_used, (long long)ctx->mem_cap);
    cudaError_t e = cudaMalloc(p, (size_t)bytes);
    if (e != cudaSuccess && !ctx->cache.empty()) {
        cudaGetLastError();
        ctx_cache_release(ctx);
        e = cudaMalloc(p, (size_t)bytes);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return set_err(ctx, HSDLA_ERR_NOMEM, "cudaMalloc(%lld) failed: %s", (long long)bytes, cudaGetErrorString(e));
    }
    ctx->mem_used += bytes;
    ctx->live[*p] = bytes;
    return HSDLA_OK;
}

// Releases a block of ctx_malloc.  Callers release only blocks no queued work still uses (they
// synchronise first where it could); a kept block is handed out again in stream order only after
// that.
void ctx_free(hsdla_context *ctx, void *p, int64_t bytes) {
    if (!p) return;
    auto it = ctx->live.find(p);
    const int64_t size = it != ctx->live.end() ? it->second : bytes;
    if (it != ctx->live.end()) ctx->live.erase(it);
    if (size <= kCacheBlockMax && ctx->cached_bytes + size <= kCacheBytesMax) {
        ctx->cache.emplace(size, p);
        ctx->cached_bytes += size;
        return;
    }
    cudaFree(p);
    ctx->mem_used -= size;
}

// Workspace of at least `bytes`, owned by the context (reused across calls).
int ctx_host_out(hsdla_context *ctx, int64_t bytes, void **out) {
    if (bytes <= ctx->hout_bytes && ctx->hout) { *out = ctx->hout; return HSDLA_OK; }
    if (ctx->hout) {
        cudaStreamSynchronize(ctx->stream);
        ctx_free(ctx, ctx->hout, ctx->hout_bytes);
        ctx->hout = nullptr;
        ctx->hout_bytes = 0;
    }
    int rc = ctx_malloc(ctx, &ctx->hout, bytes);
    if (rc) return rc;
    ctx->hout_bytes = bytes;
    *out = ctx->hout;
    return HSDLA_OK;
}

// Download of the lower triangle of a column-major n x n device matrix into a host matrix of
// leading dimension ld: column blocks of kDownBlock, each from its first row down (the strict
// upper triangle outside the diagonal blocks is not copied; ~half the bytes of the full matrix).
constexpr int64_t kDownBlock = 512;
cudaError_t download_lower(hsdla_cx *host, int64_t ld, const hsdla_cx *dev, int64_t n, cudaStream_t st) {
    for (int64_t c0 = 0; c0 < n; c0 += kDownBlock) {
        const int64_t w = std::min(kDownBlock, n - c0);
        const cudaError_t e = cudaMemcpy2DAsync(host + c0 + ld * c0, ld * sizeof(hsdla_cx), dev + c0 + n * c0,
                                                n * sizeof(hsdla_cx), (n - c0) * sizeof(hsdla_cx), w,
                                                cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

int ctx_workspace(hsdla_context *ctx, int64_t bytes, void **out) {
    if (bytes <= ctx->ws_bytes && ctx->ws) { *out = ctx->ws; return HSDLA_OK; }
    if (ctx->ws) {
        cudaStreamSynchronize(ctx->stream);
        ctx_free(ctx, ctx->ws, ctx->ws_bytes);
        ctx->ws = nullptr;
        ctx->ws_bytes = 0;
    }
    int rc = ctx_malloc(ctx, &ctx->ws, bytes);
    if (rc) return rc;
    ctx->ws_bytes = bytes;
    *out = ctx->ws;
    return HSDLA_OK;
}

bool finite_all(const double *p, int64_t n) {
    for (int64_t i = 0; i < n; ++i)
        if (!std::isfinite(p[i])) return false;
    return true;
}

// ylmnorm (external/compat/fleur/ylm4.f:111-137), pimach() = 3.1415926535897932
std::vector<double> ylm_norms(int lmax) {
    std::vector<double> yn((lmax + 1) * (lmax + 1));
    const double fpi = 4.0 * 3.1415926535897932;
    for (int l = 0; l <= lmax; ++l) {
        const int lm0 = l * (l + 1);
        double cd = 1.0;
        const double a = std::sqrt((2 * l + 1) / fpi);
        yn[lm0] = a;
        for (int m = 1; m <= l; ++m) {
            cd = cd / ((l + 1 - m) * (l + m));
            yn[lm0 + m] = a * std::sqrt(cd);
            yn[lm0 - m] = ((m & 1) ? -1.0 : 1.0) * yn[lm0 + m];
        }
    }
    return yn;
}

int validate(hsdla_context *ctx, const hsdla_system *s, const hsdla_kpoint *kpts, int nk) {
    if (!s) return set_err(ctx, HSDLA_ERR_ARG, "system is NULL");
    if (s->num_atoms < 1 || s->num_types < 1 || s->num_types > kMaxTypes)
        return set_err(ctx, HSDLA_ERR_ARG, "num_atoms=%d num_types=%d out of range", s->num_atoms, s->num_types);
    if (s->max_lmax < 1 || s->max_lmax > kMaxLmax)
        return set_err(ctx, HSDLA_ERR_UNSUPPORTED, "max_lmax=%d outside [1, %d]", s->max_lmax, kMaxLmax);
    if (!s->atom_type || !s->atom_pos || !s->type_rmt || !s->type_lmax || !s->type_u || !s->type_u_dr ||
        !s->type_dE_u || !s->type_dE_u_dr || !s->type_dE_u_norm || !s->type_t_aa || !s->type_t_ab || !s->type_t_bb)
        return set_err(ctx, HSDLA_ERR_ARG, "a required system array is NULL");
    if (!(s->vol_cell > 0.0) || !std::isfinite(s->vol_cell))
        return set_err(ctx, HSDLA_ERR_INPUT, "vol_cell must be positive and finite");
    if (!finite_all(s->bmat, 9)) return set_err(ctx, HSDLA_ERR_INPUT, "bmat is not finite");
    const int na = s->num_atoms, nt = s->num_types, nl = s->max_lmax + 1;
    for (int j = 0; j < na; ++j)
        if (s->atom_type[j] < 0 || s->atom_type[j] >= nt)
            return set_err(ctx, HSDLA_ERR_ARG, "atom_type[%d]=%d out of range", j, s->atom_type[j]);
    if (!finite_all(s->atom_pos, 3 * (int64_t)na)) return set_err(ctx, HSDLA_ERR_INPUT, "atom_pos not finite");
    if (s->atom_rotmat && !finite_all(s->atom_rotmat, 9 * (int64_t)na))
        return set_err(ctx, HSDLA_ERR_INPUT, "atom_rotmat not finite");
    for (int t = 0; t < nt; ++t) {
        if (s->type_lmax[t] < 1 || s->type_lmax[t] > s->max_lmax)
            return set_err(ctx, HSDLA_ERR_ARG, "type_lmax[%d]=%d outside [1, max_lmax]", t, s->type_lmax[t]);
        if (!(s->type_rmt[t] > 0.0) || !std::isfinite(s->type_rmt[t]))
            return set_err(ctx, HSDLA_ERR_INPUT, "type_rmt[%d] must be positive", t);
        for (int l = 0; l <= s->type_lmax[t]; ++l) {
            const int tl = t * nl + l;
            const double v[5] = {s->type_u[tl], s->type_u_dr[tl], s->type_dE_u[tl], s->type_dE_u_dr[tl],
                                 s->type_dE_u_norm[tl]};
            if (!finite_all(v, 5))
                return set_err(ctx, HSDLA_ERR_INPUT, "radial data of type %d, l=%d not finite", t, l);
            const double w = s->type_dE_u[tl] * s->type_u_dr[tl] - s->type_u[tl] * s->type_dE_u_dr[tl];
            if (w == 0.0 || !std::isfinite(1.0 / w))
                return set_err(ctx, HSDLA_ERR_INPUT, "zero Wronskian for type %d, l=%d", t, l);
            if (s->type_dE_u_norm[tl] < 0.0)
                return set_err(ctx, HSDLA_ERR_INPUT, "negative ||udot||^2 for type %d, l=%d", t, l);
        }
        // the T blocks are checked on the device as they are assembled (check_tmats)
    }
    if (nk < 0 || (nk > 0 && !kpts)) return set_err(ctx, HSDLA_ERR_ARG, "bad k-point list");
    for (int i = 0; i < nk; ++i) {
        if (kpts[i].n_g < 0) return set_err(ctx, HSDLA_ERR_ARG, "k-point %d: n_g < 0", i);
        if (kpts[i].n_g > 0 && !kpts[i].g) return set_err(ctx, HSDLA_ERR_ARG, "k-point %d: g is NULL", i);
        if (!finite_all(kpts[i].k, 3)) return set_err(ctx, HSDLA_ERR_INPUT, "k-point %d not finite", i);
        if (kpts[i].n_g > (int64_t)1 << 31) return set_err(ctx, HSDLA_ERR_UNSUPPORTED, "n_g too large");
    }
    return HSDLA_OK;
}

// (type, rotation) classes.  The reference gives every atom its own rotation mrot bmat
// (FleurData.cpp:52-62, 453-455) and builds its rows with it (tensor_AB_match.cpp:97) while its
// type supplies the radial data and T blocks.  Atoms of one type whose rotations are equal have
// the same rows up to their structure phase, so the structure-factor form runs per class instead
// of per type: a derived system whose types are the classes (each with its type's tables) and
// whose rows carry the class's rotation.
struct ClassSystem {
    hsdla_system sys{};
    int n = 0;                            // classes
    std::vector<int32_t> atom_class, class_type, class_rot, lmax;
    std::vector<double> rots, rmt, u, u_dr, dE_u, dE_u_dr, dE_u_norm;
    std::vector<hsdla_cx> taa, tab, tbb;
};

// Builds the class system when it shrinks the work: the classes' rows (2L per class) are few
// enough against the per-atom rows (2L per atom) to pay for the structure-factor combine, and
// their table fits the per-type rows kernel.  Returns false otherwise (per-atom form).
bool make_classes(const hsdla_system *s, ClassSystem &cs) {
    if (!s->atom_rotmat) return false;
    const int na = s->num_atoms, nt = s->num_types, nl = s->max_lmax + 1, L = nl * nl;
    std::map<std::vector<uint64_t>, int> rot_id;
    std::map<std::pair<int, int>, int> cls;
    cs.atom_class.resize(na);
    for (int j = 0; j < na; ++j) {
        std::vector<uint64_t> bits(9);
        memcpy(bits.data(), s->atom_rotmat + 9 * (size_t)j, 9 * sizeof(double));
        auto r = rot_id.find(bits);
        if (r == rot_id.end()) {
            r = rot_id.emplace(bits, (int)rot_id.size()).first;
            cs.rots.insert(cs.rots.end(), s->atom_rotmat + 9 * (size_t)j, s->atom_rotmat + 9 * (size_t)j + 9);
        }
        const auto key = std::make_pair((int)s->atom_type[j], r->second);
        auto c = cls.find(key);
        if (c == cls.end()) {
            c = cls.emplace(key, (int)cls.size()).first;
            cs.class_type.push_back(key.first);
            cs.class_rot.push_back(key.second);
        }
        cs.atom_class[j] = c->second;
    }
    cs.n = (int)cls.size();
    if (4 * cs.n > 3 * na || cs.n > kMaxTypes || rows_kernel_smem(L, s->max_lmax, cs.n) > kRowsKernelSmemMax)
        return false;
    const int n = cs.n;
    cs.rmt.resize(n); cs.lmax.resize(n);
    for (auto *v : {&cs.u, &cs.u_dr, &cs.dE_u, &cs.dE_u_dr, &cs.dE_u_norm}) v->resize((size_t)n * nl);
    for (auto *v : {&cs.taa, &cs.tab, &cs.tbb}) v->resize((size_t)n * L * L);
    for (int c = 0; c < n; ++c) {
        const int t = cs.class_type[c];
        cs.rmt[c] = s->type_rmt[t];
        cs.lmax[c] = s->type_lmax[t];
        const double *src[5] = {s->type_u, s->type_u_dr, s->type_dE_u, s->type_dE_u_dr, s->type_dE_u_norm};
        std::vector<double> *dst[5] = {&cs.u, &cs.u_dr, &cs.dE_u, &cs.dE_u_dr, &cs.dE_u_norm};
        for (int q = 0; q < 5; ++q) memcpy(dst[q]->data() + (size_t)c * nl, src[q] + (size_t)t * nl, nl * sizeof(double));
        const hsdla_cx *tsrc[3] = {s->type_t_aa, s->type_t_ab, s->type_t_bb};
        std::vector<hsdla_cx> *tdst[3] = {&cs.taa, &cs.tab, &cs.tbb};
        for (int q = 0; q < 3; ++q)
            memcpy(tdst[q]->data() + (size_t)c * L * L, tsrc[q] + (size_t)t * L * L, (size_t)L * L * sizeof(hsdla_cx));
    }
    hsdla_system &d = cs.sys;
    d = *s;
    d.num_types = n;
    d.atom_type = cs.atom_class.data();
    d.type_rmt = cs.rmt.data();
    d.type_lmax = cs.lmax.data();
    d.type_u = cs.u.data(); d.type_u_dr = cs.u_dr.data(); d.type_dE_u = cs.dE_u.data();
    d.type_dE_u_dr = cs.dE_u_dr.data(); d.type_dE_u_norm = cs.dE_u_norm.data();
    d.type_t_aa = cs.taa.data(); d.type_t_ab = cs.tab.data(); d.type_t_bb = cs.tbb.data();
    return true;
}

// The T blocks' checks, made on the device while they were assembled (launch_tfull): finite
// values, and T_AA and T_BB Hermitian (AtomData.cpp:138-139 asserts it), |T - T^H|^2 against
// |T|^2 over the lower triangle (its mirror element is the pair's other half).
int check_tmats(hsdla_context *ctx, const std::vector<unsigned long long> &st, int nt,
                const std::vector<int32_t> *class_type = nullptr) {
    auto as_double = [](unsigned long long b) { double d; memcpy(&d, &b, sizeof(d)); return d; };
    for (int t = 0; t < nt; ++t) {
        const int ty = class_type ? (*class_type)[t] : t;    // the caller's type of a class
        const unsigned long long fl = st[5 * (size_t)t];
        for (int q = 0; q < 3; ++q)
            if (fl & (1ull << q)) return set_err(ctx, HSDLA_ERR_INPUT, "T block %d of type %d not finite", q, ty);
        for (int q = 0; q < 2; ++q) {
            const double mx2 = as_double(st[5 * (size_t)t + 1 + 2 * q]), dev2 = as_double(st[5 * (size_t)t + 2 + 2 * q]);
            if (dev2 > 1e-24 * std::max(mx2, 1e-300))
                return set_err(ctx, HSDLA_ERR_INPUT, "T_%s of type %d is not Hermitian (|T-T^H| = %.3g)",
                               q == 0 ? "AA" : "BB", ty, std::sqrt(dev2));
        }
    }
    return HSDLA_OK;
}

template <typename T>
T *carve(char *&p, int64_t count) {
    T *r = reinterpret_cast<T *>(p);
    p += ((int64_t)sizeof(T) * count + 255) & ~int64_t(255);
    return r;
}

int upload_jobs(hsdla_plan *pl, cudaStream_t st) {
    hsdla_context *ctx = pl->ctx;
    const int64_t n = (int64_t)pl->h_jobs.size();
    if (n > pl->jobs_cap) {
        if (pl->d_jobs) { cudaStreamSynchronize(st); ctx_free(ctx, pl->d_jobs, pl->jobs_cap * sizeof(Fp64Job)); }
        pl->d_jobs = nullptr;
        int rc = ctx_malloc(ctx, (void **)&pl->d_jobs, n * sizeof(Fp64Job));
        if (rc) return rc;
        pl->jobs_cap = n;
    }
    CUDA_TRY(ctx, cudaMemcpyAsync(pl->d_jobs, pl->h_jobs.data(), n * sizeof(Fp64Job), cudaMemcpyHostToDevice, st));
    // the host vector must outlive the async copy: synchronise before it can change
    CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return HSDLA_OK;
}

int64_t assign_tiles(std::vector<Fp64Job> &jobs, size_t first) {
    int64_t t = 0;
    for (size_t i = first; i < jobs.size(); ++i) {
        jobs[i].tiles_n = (int32_t)((jobs[i].n + kFp64Tile - 1) / kFp64Tile);
        jobs[i].tile_begin = t;
        t += fp64_job_tiles(jobs[i]);
    }
    return t;
}

// Lower-triangle relative errors (Frobenius, max) of X against R, both n x n column-major.
void lower_errors(const std::vector<std::complex<double>> &X, const std::vector<std::complex<double>> &R, int64_t n,
                  double &fro, double &mx) {
    double d2 = 0, r2 = 0, dm = 0, rm = 0;
    for (int64_t c = 0; c < n; ++c)
        for (int64_t r = c; r < n; ++r) {
            const auto d = X[r + n * c] - R[r + n * c];
            d2 += std::norm(d); r2 += std::norm(R[r + n * c]);
            dm = std::max(dm, std::abs(d)); rm = std::max(rm, std::abs(R[r + n * c]));
        }
    fro = r2 > 0 ? std::sqrt(d2 / r2) : 0.0;
    mx = rm > 0 ? dm / rm : 0.0;
}

// Slice autotuner: an a-posteriori check of the Ozaki contraction on a column sample
// re-done in FP64.  The error of the S and H sample tiles at a probe slice count is
// extrapolated by 2^-5 per extra digit (each digit carries 5 bits) and, for the
// Frobenius ratio, by sqrt(n_G / n_sample) (digit errors are uniform over the matrix
// while its norm is carried by the diagonal); the smallest slice count whose
// prediction stays below a quarter of the target is kept for the plan.
int autotune_slices(hsdla_plan *pl, double2 *C, cudaStream_t st) {
    hsdla_context *ctx = pl->ctx;
    constexpr int kProbe = 8;
    int ik = 0;
    for (int i = 0; i < (int)pl->kps.size(); ++i)
        if (pl->kps[i].n_g > pl->kps[ik].n_g) ik = i;
    const int64_t G = pl->kps[ik].n_g;
    if (G == 0) { pl->autotune = false; return HSDLA_OK; }
    // systems of one shape share a dynamic range closely enough to share the choice
    const auto key = std::make_tuple(pl->L, pl->na, pl->nt, (G + 511) / 512, pl->opts.target_rel_err);
    const auto hit = ctx->tune_cache.find(key);
    if (hit != ctx->tune_cache.end()) {
        pl->oz.num_slices = hit->second.first;
        pl->est_err = hit->second.second;
        pl->autotune = false;
        return HSDLA_OK;
    }
    const int64_t ns = std::min<int64_t>(G, 384), step = G / ns;
    const int64_t K = pl->twoLa, twoL = 2 * (int64_t)pl->L;
    OzakiPlan probe{};
    int rc = ozaki_plan_init(probe, kProbe, pl->opts.target_rel_err);
    if (rc) return set_err(ctx, rc, "autotune: %s", ozaki_last_error());
    const int64_t bytes_sample = 2 * K * ns * (int64_t)sizeof(double2) + 4 * ns * ns * (int64_t)sizeof(double2);
    const int64_t bytes_oz = ozaki_pipeline_workspace(kProbe, twoL, pl->na, pl->nt, ns) + 1024;
    void *buf = nullptr;
    rc = ctx_malloc(ctx, &buf, bytes_sample + bytes_oz);
    if (rc) { ozaki_plan_release(probe); return rc; }
    double2 *Cs = reinterpret_cast<double2 *>(buf), *Xs = Cs + K * ns;
    double2 *Sr = Xs + K * ns, *Hr = Sr + ns * ns, *So = Hr + ns * ns, *Ho = So + ns * ns;
    char *wz = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(Ho + ns * ns) + 1023) & ~uintptr_t(1023));
    auto fail = [&](int code, const char *what) {
        cudaStreamSynchronize(st);
        ctx_free(ctx, buf, bytes_sample + bytes_oz);
        ozaki_plan_release(probe);
        return set_err(ctx, code, "autotune: %s", what);
    };
    if (launch_construct_ab(pl->dsys, pl->kps[ik].dk, C, K, st) != cudaSuccess) return fail(HSDLA_ERR_CUDA, "construct_ab");
    if (cudaMemcpy2DAsync(Cs, K * sizeof(double2), C, step * K * sizeof(double2), K * sizeof(double2), ns,
                          cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return fail(HSDLA_ERR_CUDA, "sample gather");
    // FP64 reference on the sample
    pl->h_jobs.clear();
    for (int j = 0; j < pl->na; ++j) {
        Fp64Job jb{};
        jb.P = pl->Tfull + (int64_t)pl->atom_type[j] * twoL * twoL; jb.ldp = twoL;
        jb.Q = Cs + twoL * j; jb.ldq = K; jb.out = Xs + twoL * j; jb.ldo = K;
        jb.m = twoL; jb.n = ns; jb.k = twoL;
        pl->h_jobs.push_back(jb);
    }
    const int64_t t1 = assign_tiles(pl->h_jobs, 0);
    const size_t nb = pl->h_jobs.size();
    Fp64Job js{};
    js.P = Cs; js.ldp = K; js.Q = Cs; js.ldq = K; js.w = pl->w; js.out = Sr; js.ldo = ns;
    js.m = ns; js.n = ns; js.k = K; js.lower = 1;
    Fp64Job jh = js;
    jh.Q = Xs; jh.w = nullptr; jh.out = Hr;
    pl->h_jobs.push_back(js);
    pl->h_jobs.push_back(jh);
    const int64_t t2 = assign_tiles(pl->h_jobs, nb);
    if (upload_jobs(pl, st)) return fail(HSDLA_ERR_CUDA, "job upload");
    if (launch_fp64_jobs(pl->d_jobs, (int)nb, t1, st) != cudaSuccess ||
        launch_fp64_jobs(pl->d_jobs + nb, 2, t2, st) != cudaSuccess)
        return fail(HSDLA_ERR_CUDA, "fp64 sample");
    // Ozaki at the probe slice count (overwrites Xs after the FP64 H job, in stream order)
    OzakiInputs in;
    in.C = Cs; in.Tfull = pl->Tfull; in.w = pl->w; in.atom_type = pl->atom_type.data(); in.X = Xs;
    in.twoL = twoL; in.na = pl->na; in.nt = pl->nt; in.G = ns;
    int nl = 0;
    rc = ozaki_pipeline(probe, in, So, Ho, ns, wz, st, &nl);
    if (rc) return fail(rc, ozaki_last_error());
    std::vector<std::complex<double>> h[4];
    double2 *src[4] = {Sr, Hr, So, Ho};
    for (int q = 0; q < 4; ++q) {
        h[q].resize(ns * ns);
        if (cudaMemcpyAsync(h[q].data(), src[q], ns * ns * sizeof(double2), cudaMemcpyDeviceToHost, st) != cudaSuccess)
            return fail(HSDLA_ERR_CUDA, "sample download");
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail(HSDLA_ERR_CUDA, "sync");
    if (ozaki_check_device_error(probe)) return fail(HSDLA_ERR_TIMEOUT, ozaki_last_error());
    double fS, mS, fH, mH;
    lower_errors(h[2], h[0], ns, fS, mS);
    lower_errors(h[3], h[1], ns, fH, mH);
    const double grow = std::sqrt((double)G / (double)ns);
    const double e = std::max(std::max(fS, fH) * grow, std::max(mS, mH));
    int s = kProbe;
    double pred = e;
    while (s < kOzMaxSlices && pred > 0.25 * pl->opts.target_rel_err) {
        ++s;
        pred *= 1.0 / 32.0;
    }
    pl->oz.num_slices = s;
    pl->est_err = pred;
    pl->autotune = false;
    ctx->tune_cache[key] = std::make_pair(s, pred);
    ctx_free(ctx, buf, bytes_sample + bytes_oz);
    ozaki_plan_release(probe);
    return HSDLA_OK;
}

}  // namespace

// =====================================================================================
extern "C" {

int hsdla_context_create(int device, hsdla_context **out) {
    if (!out) return HSDLA_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) { cudaGetLastError(); return HSDLA_ERR_DEVICE; }
    if (device < 0 || device >= ndev) return HSDLA_ERR_ARG;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return HSDLA_ERR_DEVICE;
    if (prop.major * 10 + prop.minor < 100) return HSDLA_ERR_DEVICE;
    auto *ctx = new hsdla_context();
    ctx->device = device;
    ctx->nsm = prop.multiProcessorCount;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return HSDLA_ERR_CUDA;
    }
    cudaEventCreate(&ctx->ev0);
    cudaEventCreate(&ctx->ev1);
    cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming);
    for (auto &e : ctx->evs) cudaEventCreate(&e);
    *out = ctx;
    return HSDLA_OK;
}

void hsdla_context_destroy(hsdla_context *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    while (!ctx->plans.empty()) hsdla_plan_destroy(*ctx->plans.begin());
    if (ctx->ws) ctx_free(ctx, ctx->ws, ctx->ws_bytes);
    if (ctx->hout) ctx_free(ctx, ctx->hout, ctx->hout_bytes);
    ozaki_plan_release(ctx->plugin_oz);
    ctx_cache_release(ctx);
    if (ctx->staging) cudaFreeHost(ctx->staging);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev_copy) cudaEventDestroy(ctx->ev_copy);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (auto &e : ctx->evs) if (e) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

// With a context: its last message.  Without one: the calling thread's last message of an entry
// point that takes no context (hsdla_zherkx_lower_noalloc).
const char *hsdla_last_error(const hsdla_context *ctx) { return ctx ? ctx->err.c_str() : ozaki_last_error(); }

int hsdla_set_mem_cap(hsdla_context *ctx, int64_t bytes) {
    if (!ctx || bytes < 0) return HSDLA_ERR_ARG;
    ctx->mem_cap = bytes;
    return HSDLA_OK;
}

int hsdla_prepare_tmat(int32_t lmax, int32_t lmax_nonsph, const hsdla_cx *taa, const hsdla_cx *tbb,
                       const hsdla_cx *tab, const hsdla_cx *tba, const double *E_l, const double *dE_u_norm,
                       hsdla_cx *aa_o, hsdla_cx *ab_o, hsdla_cx *bb_o) {
    if (lmax < 0 || lmax > kMaxLmax || lmax_nonsph < 0 || !taa || !tbb || !tab || !tba || !E_l || !dE_u_norm ||
        !aa_o || !ab_o || !bb_o)
        return HSDLA_ERR_ARG;
    using cx = std::complex<double>;
    const int n = (lmax + 1) * (lmax + 1);
    const cx *Taa = reinterpret_cast<const cx *>(taa), *Tbb = reinterpret_cast<const cx *>(tbb);
    const cx *Tab = reinterpret_cast<const cx *>(tab), *Tba = reinterpret_cast<const cx *>(tba);
    cx *aa = reinterpret_cast<cx *>(aa_o), *ab = reinterpret_cast<cx *>(ab_o), *bb = reinterpret_cast<cx *>(bb_o);
    // TMat::TMat: symmatl for aa/bb; ab = trimatl(tab) + trimatu(tba^H), diagonal from tab
    for (int r = 0; r < n; ++r)
        if (std::abs(Tab[r + (int64_t)n * r] - Tba[r + (int64_t)n * r]) >= 1e-15) return HSDLA_ERR_INPUT;
    for (int c = 0; c < n; ++c)
        for (int r = 0; r < n; ++r) {
            const int64_t i = r + (int64_t)n * c, iT = c + (int64_t)n * r;
            aa[i] = (r >= c) ? Taa[i] : std::conj(Taa[iT]);
            bb[i] = (r >= c) ? Tbb[i] : std::conj(Tbb[iT]);
            ab[i] = (r >= c) ? Tab[i] : std::conj(Tba[iT]);
        }
    // zero_nonsph (types_helper.cpp:72-88)
    const int s0 = (lmax_nonsph + 1) * (lmax_nonsph + 1);
    if (s0 < n)
        for (int c = 0; c < n; ++c)
            for (int r = 0; r < n; ++r)
                if (r >= s0 || c >= s0) {
                    const int64_t i = r + (int64_t)n * c;
                    aa[i] = 0.0; ab[i] = 0.0; bb[i] = 0.0;
                }
    // augment_tmats diagonal terms (AtomData.cpp:127-136)
    for (int l = 0; l <= lmax; ++l)
        for (int m = -l; m <= l; ++m) {
            const int64_t d = (int64_t)(l * (l + 1) + m) * (n + 1);
            aa[d] += E_l[l];
            bb[d] += E_l[l] * dE_u_norm[l];
            ab[d] += 0.5;
        }
    return HSDLA_OK;
}

}  // extern "C"

namespace {
int plan_create_impl(hsdla_context *ctx, const hsdla_system *s, const hsdla_kpoint *kpts, int32_t nk,
                     const hsdla_opts *opts, hsdla_plan **out, bool defer_tcheck);
}

extern "C" {

int hsdla_plan_create(hsdla_context *ctx, const hsdla_system *s, const hsdla_kpoint *kpts, int32_t nk,
                      const hsdla_opts *opts, hsdla_plan **out) {
    return plan_create_impl(ctx, s, kpts, nk, opts, out, false);
}

}  // extern "C"

namespace {
// defer_tcheck: leave the T-block check to the caller (after its own synchronisation), so that the
// device runs on while the host sets up the execution
int plan_create_impl(hsdla_context *ctx, const hsdla_system *s, const hsdla_kpoint *kpts, int32_t nk,
                     const hsdla_opts *opts, hsdla_plan **out, bool defer_tcheck) {
    if (!ctx || !out) return HSDLA_ERR_ARG;
    *out = nullptr;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    // HSDLA_TRACE=1: host time of the creation's phases on stderr
    using pclk = std::chrono::steady_clock;
    const bool ptrace = env_flag("HSDLA_TRACE", false);
    const pclk::time_point p0 = pclk::now();
    const auto pms = [&]() { return std::chrono::duration<double, std::milli>(pclk::now() - p0).count(); };
    int rc = validate(ctx, s, kpts, nk);
    if (rc) return rc;
    const double p_valid = pms();
    // atoms with rotations: (type, rotation) classes keep the structure-factor form where they
    // shrink the work (HSDLA_SF=0 or HSDLA_CLASSES=0 keeps the per-atom form)
    const char *sf_env0 = getenv("HSDLA_SF");
    ClassSystem cls;
    const bool use_classes = s->atom_rotmat && !(sf_env0 && strtol(sf_env0, nullptr, 10) == 0) &&
                             env_flag("HSDLA_CLASSES", true) && make_classes(s, cls);
    if (use_classes) s = &cls.sys;
    auto *pl = new hsdla_plan();
    pl->ctx = ctx;
    pl->classes = use_classes ? cls.n : 0;
    if (opts) pl->opts = *opts;
    if (pl->opts.precision != HSDLA_PREC_FP64 && pl->opts.precision != HSDLA_PREC_OZAKI_FP8) {
        delete pl;
        return set_err(ctx, HSDLA_ERR_ARG, "unknown precision %d", pl->opts.precision);
    }
    if (pl->opts.target_rel_err <= 0.0) pl->opts.target_rel_err = 1e-13;
    const int na = s->num_atoms, nt = s->num_types, nl = s->max_lmax + 1, L = nl * nl;
    pl->L = L; pl->na = na; pl->nt = nt; pl->max_lmax = s->max_lmax;
    pl->hoist = s->atom_rotmat == nullptr || use_classes;
    pl->twoLa = 2 * (int64_t)L * na;
    pl->atom_type.assign(s->atom_type, s->atom_type + na);

    // ---- host tables
    std::vector<double> inv_w((size_t)nt * nl, 0.0);
    for (int t = 0; t < nt; ++t)
        for (int l = 0; l <= s->type_lmax[t]; ++l) {
            const int tl = t * nl + l;
            inv_w[tl] = 1. / (s->type_dE_u[tl] * s->type_u_dr[tl] - s->type_u[tl] * s->type_dE_u_dr[tl]);
        }
    std::vector<double> yn = ylm_norms(s->max_lmax);
    std::vector<double> w(pl->twoLa), wsq(pl->twoLa);
    for (int j = 0; j < na; ++j) {
        const int t = s->atom_type[j];
        for (int l = 0; l < nl; ++l)
            for (int lm = l * l; lm < (l + 1) * (l + 1); ++lm) {
                const int64_t rA = 2 * (int64_t)L * j + lm, rB = rA + L;
                const double un = (l <= s->type_lmax[t]) ? s->type_dE_u_norm[t * nl + l] : 0.0;
                w[rA] = 1.0; wsq[rA] = 1.0;
                w[rB] = un; wsq[rB] = std::sqrt(un);
            }
    }
    const size_t tf_elems = (size_t)nt * 4 * L * L;
    const int64_t LLnt = (int64_t)nt * L * L;

    // ---- one device block for all tables: the uploaded part, then what the device fills
    int64_t bytes = 0;
    auto add = [&](int64_t b) { bytes += (b + 255) & ~int64_t(255); };
    add(sizeof(int32_t) * na); add(sizeof(double) * 3 * na); add(s->atom_rotmat ? sizeof(double) * 9 * na : 0);
    add(use_classes ? sizeof(double) * cls.rots.size() : 0); add(use_classes ? sizeof(int32_t) * nt : 0);
    add(sizeof(double) * nt); add(sizeof(int32_t) * nt);
    for (int q = 0; q < 5; ++q) add(sizeof(double) * nt * nl);
    add(sizeof(double) * L);
    for (int q = 0; q < 3; ++q) add(sizeof(double2) * LLnt);     // T_AA, T_AB, T_BB as given
    add(sizeof(double) * pl->twoLa); add(sizeof(double) * pl->twoLa);
    for (int i = 0; i < nk; ++i) add(sizeof(int32_t) * 3 * kpts[i].n_g);
    // structure-factor form: per-type weights, per-atom phase factors along each axis, the atoms
    // grouped by type and the table itself over the box of G-vector differences g_col - g_row
    const char *sf_env = getenv("HSDLA_SF");
    pl->sf = pl->hoist && !(sf_env && strtol(sf_env, nullptr, 10) == 0);
    int half[3] = {0, 0, 0}, ext[3] = {1, 1, 1};
    if (pl->sf) {
        for (int i = 0; i < nk; ++i)
            for (int64_t q = 0; q < kpts[i].n_g; ++q)
                for (int c = 0; c < 3; ++c) half[c] = std::max(half[c], 2 * std::abs(kpts[i].g[3 * q + c]));
        for (int c = 0; c < 3; ++c) ext[c] = 2 * half[c] + 1;
        add(sizeof(double) * 2 * L * nt);
        add(sizeof(int32_t) * (na + nt + 1));
    }
    const int64_t upload_bytes = bytes;
    // filled on the device: the assembled T blocks and their checks; the structure-factor form's
    // per-atom phase factors and its table
    add(sizeof(double2) * tf_elems);
    add(sizeof(unsigned long long) * 5 * nt);
    if (pl->sf) {
        add(sizeof(double2) * (int64_t)na * (ext[0] + ext[1] + ext[2]));
        add(sizeof(double2) * (int64_t)nt * ext[0] * ext[1] * ext[2]);
    }
    const double p_tables = pms();
    rc = ctx_malloc(ctx, &pl->tables, bytes);
    if (rc) { delete pl; return rc; }
    pl->tables_bytes = bytes;
    // staging of the uploaded part, page-locked and kept by the context (pageable if pinning
    // fails); left uninitialised: every byte that matters is written
    // (the T-block statistics come back behind the uploaded part)
    const int64_t stats_off = (upload_bytes + 255) & ~int64_t(255);
    const int64_t stage_need = stats_off + (int64_t)sizeof(unsigned long long) * 5 * nt;
    if (ctx->staging_bytes < stage_need) {
        if (ctx->staging) cudaFreeHost(ctx->staging);
        ctx->staging = nullptr;
        ctx->staging_bytes = 0;
        const int64_t want = std::max<int64_t>(stage_need, (int64_t)1 << 20);
        if (cudaHostAlloc(&ctx->staging, (size_t)want, cudaHostAllocDefault) == cudaSuccess) ctx->staging_bytes = want;
        else { cudaGetLastError(); ctx->staging = nullptr; }
    }
    std::unique_ptr<char[]> pageable;
    char *stage = reinterpret_cast<char *>(ctx->staging);
    if (!stage) { pageable.reset(new char[std::max<int64_t>(upload_bytes, 1)]); stage = pageable.get(); }
    char *hp = stage;
    char *dp = reinterpret_cast<char *>(pl->tables);
    // copies of 256 KB and more (the T blocks) are made together below, on several threads
    struct Pending { char *dst; const char *src; int64_t n; };
    std::vector<Pending> pend;
    auto put = [&](const void *src, int64_t b) -> void * {
        void *d = dp;
        if (b >= (int64_t)1 << 18 && src) pend.push_back({hp, reinterpret_cast<const char *>(src), b});
        else if (b > 0 && src) memcpy(hp, src, b);
        const int64_t adv = (b + 255) & ~int64_t(255);
        hp += adv; dp += adv;
        return d;
    };
    DevSystem &D = pl->dsys;
    D.num_atoms = na; D.num_types = nt; D.max_lmax = s->max_lmax; D.L = L;
    D.vol_prefac = 4 * kPi / std::sqrt(s->vol_cell);
    memcpy(D.bmat, s->bmat, sizeof(D.bmat));
    D.atom_type = (const int32_t *)put(s->atom_type, sizeof(int32_t) * na);
    D.atom_pos = (const double *)put(s->atom_pos, sizeof(double) * 3 * na);
    D.atom_rotmat = s->atom_rotmat ? (const double *)put(s->atom_rotmat, sizeof(double) * 9 * na) : nullptr;
    if (use_classes) {
        D.num_rots = (int)(cls.rots.size() / 9);
        D.rots = (const double *)put(cls.rots.data(), sizeof(double) * cls.rots.size());
        D.type_rot = (const int32_t *)put(cls.class_rot.data(), sizeof(int32_t) * nt);
    }
    D.type_rmt = (const double *)put(s->type_rmt, sizeof(double) * nt);
    D.type_lmax = (const int32_t *)put(s->type_lmax, sizeof(int32_t) * nt);
    D.u = (const double *)put(s->type_u, sizeof(double) * nt * nl);
    D.u_dr = (const double *)put(s->type_u_dr, sizeof(double) * nt * nl);
    D.dE_u = (const double *)put(s->type_dE_u, sizeof(double) * nt * nl);
    D.dE_u_dr = (const double *)put(s->type_dE_u_dr, sizeof(double) * nt * nl);
    D.inv_w = (const double *)put(inv_w.data(), sizeof(double) * nt * nl);
    D.ynorm = (const double *)put(yn.data(), sizeof(double) * L);
    const double2 *d_taa = (const double2 *)put(s->type_t_aa, sizeof(double2) * LLnt);
    const double2 *d_tab = (const double2 *)put(s->type_t_ab, sizeof(double2) * LLnt);
    const double2 *d_tbb = (const double2 *)put(s->type_t_bb, sizeof(double2) * LLnt);
    pl->w = (double *)put(w.data(), sizeof(double) * pl->twoLa);
    pl->wsqrt = (double *)put(wsq.data(), sizeof(double) * pl->twoLa);
    for (int i = 0; i < nk; ++i) {
        PlanKpoint pk;
        pk.n_g = kpts[i].n_g;
        memcpy(pk.dk.k, kpts[i].k, sizeof(pk.dk.k));
        pk.dk.n_g = kpts[i].n_g;
        pk.dk.g = (const int32_t *)put(kpts[i].g, sizeof(int32_t) * 3 * kpts[i].n_g);
        pl->kps.push_back(pk);
        const double G = (double)kpts[i].n_g;
        pl->flop += 20.0 * G * G * L * na + 24.0 * (double)L * L * na * G;
    }
    double2 *d_ex = nullptr;
    const int32_t *d_order = nullptr;
    if (pl->sf) {
        std::vector<double> wt((size_t)2 * L * nt);
        for (int t = 0; t < nt; ++t)
            for (int l = 0; l < nl; ++l)
                for (int lm = l * l; lm < (l + 1) * (l + 1); ++lm) {
                    wt[(size_t)2 * L * t + lm] = 1.0;
                    wt[(size_t)2 * L * t + L + lm] = (l <= s->type_lmax[t]) ? s->type_dE_u_norm[t * nl + l] : 0.0;
                }
        pl->wt = (double *)put(wt.data(), sizeof(double) * wt.size());
        std::vector<int32_t> ord;
        std::vector<int32_t> tb(nt + 1, 0);
        for (int t = 0; t < nt; ++t) {
            tb[t] = (int32_t)ord.size();
            for (int j = 0; j < na; ++j)
                if (s->atom_type[j] == t) ord.push_back(j);
        }
        tb[nt] = (int32_t)ord.size();
        ord.insert(ord.end(), tb.begin(), tb.end());
        d_order = (const int32_t *)put(ord.data(), sizeof(int32_t) * ord.size());
        SfTab &dm = pl->sf_dims;
        dm.dx = half[0]; dm.dy = half[1]; dm.dz = half[2];
        dm.ny = ext[1]; dm.nz = ext[2];
        dm.box = (int64_t)ext[0] * ext[1] * ext[2];
    }
    // past the uploaded part: what the device fills
    auto dev_only = [&](int64_t b) -> void * {
        void *d = dp;
        dp += (b + 255) & ~int64_t(255);
        return d;
    };
    pl->Tfull = (double2 *)dev_only(sizeof(double2) * tf_elems);
    unsigned long long *d_stats = (unsigned long long *)dev_only(sizeof(unsigned long long) * 5 * nt);
    if (pl->sf) {
        d_ex = (double2 *)dev_only(sizeof(double2) * (int64_t)na * (ext[0] + ext[1] + ext[2]));
        pl->sf_tab = (double2 *)dev_only(sizeof(double2) * (int64_t)nt * ext[0] * ext[1] * ext[2]);
    }
    std::vector<unsigned long long> tstats((size_t)5 * nt, 0);
    {
        // the pending copies as one byte range split evenly over up to four threads (one copying
        // thread on a GB300's Grace host moves ~25 GB/s: 0.25 ms for the 6 MB of T blocks of 8
        // types at lmax 10)
        int64_t tot = 0;
        for (const auto &q : pend) tot += q.n;
        auto copy_range = [&](int64_t lo, int64_t hi) {
            int64_t off = 0;
            for (const auto &q : pend) {
                const int64_t a = std::max(lo, off), b = std::min(hi, off + q.n);
                if (a < b) memcpy(q.dst + (a - off), q.src + (a - off), (size_t)(b - a));
                off += q.n;
            }
        };
        const int nth = tot >= ((int64_t)4 << 20) ? 4 : 1;
        const int64_t per = (tot + nth - 1) / nth;
        std::vector<std::thread> th;
        int started = 0;              // threads 1..started copy ranges 1..started
        try {
            for (int t = 1; t < nth; ++t) {
                th.emplace_back(copy_range, std::min(tot, t * per), std::min(tot, (t + 1) * per));
                ++started;
            }
        } catch (...) {               // a thread that cannot start leaves its ranges to this one
        }
        copy_range(0, std::min(tot, per));
        if (started + 1 < nth) copy_range(std::min(tot, (started + 1) * per), tot);
        for (auto &x : th) x.join();
    }
    const double p_staged = pms();
    cudaError_t e = cudaMemcpyAsync(pl->tables, stage, upload_bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_stats, 0, sizeof(unsigned long long) * 5 * nt, ctx->stream);
    if (e == cudaSuccess) e = launch_tfull(d_taa, d_tab, d_tbb, nt, L, pl->Tfull, d_stats, ctx->stream);
    if (e == cudaSuccess && pl->sf) e = launch_sf_phases(D.atom_pos, na, half, ext, d_ex, ctx->stream);
    if (e == cudaSuccess && pl->sf)
        e = launch_sf_table(d_ex, d_ex + (size_t)na * ext[0], d_ex + (size_t)na * (ext[0] + ext[1]), d_order,
                            d_order + na, nt, ext[0], ext[1], ext[2], pl->sf_tab, ctx->stream);
    const bool defer = defer_tcheck && ctx->staging != nullptr;
    unsigned long long *stats_host =
        defer ? reinterpret_cast<unsigned long long *>(reinterpret_cast<char *>(ctx->staging) + stats_off) : tstats.data();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(stats_host, d_stats, sizeof(unsigned long long) * 5 * nt, cudaMemcpyDeviceToHost,
                            ctx->stream);
    const double p_enq = pms();
    if (e == cudaSuccess && !defer) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        hsdla_plan_destroy(pl);
        return set_err(ctx, HSDLA_ERR_CUDA, "table upload failed: %s", cudaGetErrorString(e));
    }
    if (ptrace)
        fprintf(stderr,
                "hsdla_plan_create: validate %.3f, host tables %.3f, staging %.3f, enqueue %.3f, device wait %.3f ms "
                "(%lld bytes uploaded)\n",
                p_valid, p_tables - p_valid, p_staged - p_tables, p_enq - p_staged, pms() - p_enq,
                (long long)upload_bytes);
    if (defer) {
        pl->tcheck_pending = true;
        pl->tcheck_host = stats_host;
        if (use_classes) pl->tcheck_class_type = cls.class_type;
    } else {
        rc = check_tmats(ctx, tstats, nt, use_classes ? &cls.class_type : nullptr);
        if (rc) { hsdla_plan_destroy(pl); return rc; }
    }
    if (pl->opts.precision == HSDLA_PREC_OZAKI_FP8) {
        pl->autotune = pl->opts.num_slices == 0;
        rc = ozaki_plan_init(pl->oz, pl->opts.num_slices, pl->opts.target_rel_err);
        if (rc) { hsdla_plan_destroy(pl); return set_err(ctx, rc, "Ozaki plan set-up failed"); }
    }
    ctx->plans.insert(pl);
    *out = pl;
    return HSDLA_OK;
}

}  // namespace

namespace {

// FP64 buffers of one k-point inside a group workspace.
int64_t kpoint_fp64_bytes(const hsdla_plan *pl, int64_t G) {
    const int64_t K = pl->twoLa, ldm = 2 * (int64_t)pl->L * pl->nt;
    auto r = [](int64_t x) { return (x + 1023) / 1024 * 1024; };        // each buffer is 1 KB aligned
    // structure-factor form: M, Z and the two products of each type of a combine batch (no C, no X)
    if (pl->sf) return 2 * r(ldm * G * (int64_t)sizeof(double2)) + 2 * r(pl->tbatch * G * G * (int64_t)sizeof(double2));
    const int64_t nCX = pl->opts.precision == HSDLA_PREC_FP64 ? 2 : 1;   // FP64 keeps C and X apart
    int64_t b = nCX * r(K * G * (int64_t)sizeof(double2));
    if (pl->hoist) b += 2 * r(ldm * G * (int64_t)sizeof(double2));
    return b;
}

int64_t group_bytes(const hsdla_plan *pl, const std::vector<int> &kidx) {
    int64_t b = 0;
    std::vector<int64_t> G;
    for (int i : kidx) { b += kpoint_fp64_bytes(pl, pl->kps[i].n_g); G.push_back(pl->kps[i].n_g); }
    if (pl->opts.precision == HSDLA_PREC_OZAKI_FP8)
        b += 1024 + ozaki_group_bytes(pl->oz.num_slices, 2 * (int64_t)pl->L, pl->na, pl->nt, G, pl->panels, pl->hoist,
                                      pl->sf);
    return b;
}

int64_t group_persist_bytes(const hsdla_plan *pl, const std::vector<int> &kidx) {
    std::vector<int64_t> G;
    for (int i : kidx) G.push_back(pl->kps[i].n_g);
    if (pl->opts.precision == HSDLA_PREC_OZAKI_FP8)
        return ozaki_group_persist_bytes(pl->oz.num_slices, 2 * (int64_t)pl->L, pl->na, pl->nt, G,
                                         pl->sf ? std::max(pl->panels, pl->nt) : pl->panels);
    // the FP64 group keeps two job tables, each rounded up to 1 KiB: the T applications (one per
    // type when hoisted, else one per atom, per k-point) and the S/H products (two per type in
    // the structure-factor form, else two, per k-point)
    const int64_t nk = (int64_t)kidx.size();
    const int64_t n_t = nk * (pl->hoist ? pl->nt : pl->na);
    const int64_t n_sh = nk * 2 * (pl->sf ? pl->nt : 1);
    auto up = [](int64_t b) { return (b + 1023) / 1024 * 1024; };
    return up((int64_t)sizeof(Fp64Job) * n_t) + up((int64_t)sizeof(Fp64Job) * n_sh);
}

// Device-memory budget for one group's workspace: HSDLA_WORKSPACE_BUDGET (bytes), else 85% of
// what is free now (plus the workspace this context already holds) less 2 GiB, reduced to fit
// the context's memory cap.
int64_t workspace_budget(hsdla_context *ctx) {
    int64_t budget = 0;
    if (const char *v = getenv("HSDLA_WORKSPACE_BUDGET")) budget = strtoll(v, nullptr, 10);
    if (budget <= 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        budget = (int64_t)(0.85 * (double)(fr + (size_t)ctx->ws_bytes)) - ((int64_t)2 << 30);
        budget = std::max<int64_t>(budget, (int64_t)1 << 30);
    }
    if (ctx->mem_cap > 0) budget = std::min(budget, ctx->mem_cap - ctx->mem_used + ctx->ws_bytes);
    return budget;
}

// Atom panels of the Ozaki contraction: the fewest whose one-k-point workspace (the largest
// k-point) fits the budget; HSDLA_PANELS forces a count.  The digit planes of a panel are the
// bulk of the workspace, so P panels need about 1/P of them.
void choose_panels(hsdla_plan *pl, int64_t budget) {
    pl->panels = 1;
    if (pl->opts.precision != HSDLA_PREC_OZAKI_FP8 || pl->sf) return;   // the per-type digits are small
    const char *ev = getenv("HSDLA_PANELS");
    const int64_t forced = ev ? strtoll(ev, nullptr, 10) : 0;
    if (forced > 0) { pl->panels = (int)std::min<int64_t>(forced, pl->na); return; }
    int big = -1;
    for (int i = 0; i < (int)pl->kps.size(); ++i)
        if (pl->kps[i].n_g > 0 && (big < 0 || pl->kps[i].n_g > pl->kps[big].n_g)) big = i;
    if (big < 0) return;
    const std::vector<int> one{big};
    while (pl->panels < pl->na && group_bytes(pl, one) > budget) ++pl->panels;
}

// Structure-factor form: the most types per combine batch (each type of a batch keeps its own
// products, and the batch reads and writes S and H once) whose one-k-point workspace fits the
// budget; HSDLA_TYPE_BATCH forces a count.
void choose_type_batch(hsdla_plan *pl, int64_t budget) {
    pl->tbatch = 1;
    if (!pl->sf) return;
    const char *ev = getenv("HSDLA_TYPE_BATCH");
    const int64_t forced = ev ? strtoll(ev, nullptr, 10) : 0;
    if (forced > 0) { pl->tbatch = (int)std::min<int64_t>(forced, pl->nt); return; }
    int big = -1;
    for (int i = 0; i < (int)pl->kps.size(); ++i)
        if (pl->kps[i].n_g > 0 && (big < 0 || pl->kps[i].n_g > pl->kps[big].n_g)) big = i;
    if (big < 0) return;
    const std::vector<int> one{big};
    pl->tbatch = pl->nt;
    while (pl->tbatch > 1 && group_bytes(pl, one) > budget) --pl->tbatch;
}

// Greedy k-point groups whose workspace fits the budget (at least one k-point per group).
void form_groups(hsdla_plan *pl, int64_t budget) {
    choose_panels(pl, budget);
    choose_type_batch(pl, budget);
    pl->groups.clear();
    std::vector<int> cur;
    for (int i = 0; i < (int)pl->kps.size(); ++i) {
        if (pl->kps[i].n_g == 0) continue;
        std::vector<int> trial = cur;
        trial.push_back(i);
        if (!cur.empty() && ((int)trial.size() > kMaxGroup || group_bytes(pl, trial) > budget)) {
            hsdla_plan::Group g;
            g.kidx = cur;
            pl->groups.push_back(g);
            cur.assign(1, i);
        } else {
            cur = trial;
        }
    }
    if (!cur.empty()) {
        hsdla_plan::Group g;
        g.kidx = cur;
        pl->groups.push_back(g);
    }
    pl->group_ws_bytes = 0;
    for (auto &g : pl->groups) pl->group_ws_bytes = std::max(pl->group_ws_bytes, group_bytes(pl, g.kidx));
}

void release_groups(hsdla_plan *pl) {
    for (auto &g : pl->groups) {
        if (g.oz) ozaki_group_destroy(g.oz);
        if (g.h_jobs_sh) cudaFreeHost(g.h_jobs_sh);
        if (g.persist) ctx_free(pl->ctx, g.persist, g.persist_bytes);
        for (auto &e : g.ev_dom) if (e) cudaEventDestroy(e);
        g.ev_dom.clear();
        for (auto &e : g.ev_t) if (e) cudaEventDestroy(e);
        g.ev_t.clear();
        g.oz = nullptr;
        g.h_jobs_sh = nullptr;
        g.persist = nullptr;
    }
    if (pl->graph) cudaGraphExecDestroy(pl->graph);
    pl->graph = nullptr;
    pl->graph_outputs.clear();
    pl->prepared_ws = nullptr;
}

// Lay out every group in the workspace and build its launch tables.
int prepare_groups(hsdla_plan *pl, void *ws, cudaStream_t st) {
    hsdla_context *ctx = pl->ctx;
    const int64_t K = pl->twoLa, twoL = 2 * (int64_t)pl->L, ldm = twoL * pl->nt;
    for (auto &g : pl->groups) {
        char *p = reinterpret_cast<char *>(ws);
        auto take = [&](int64_t bytes) { char *r = p; p += (bytes + 1023) / 1024 * 1024; return r; };
        g.persist_bytes = group_persist_bytes(pl, g.kidx);
        int rcp = ctx_malloc(ctx, &g.persist, g.persist_bytes);
        if (rcp) return rcp;
        g.ev_dom.assign(pl->sf ? 2 * pl->nt : 2, nullptr);
        for (auto &e : g.ev_dom) CUDA_TRY(ctx, cudaEventCreate(&e));
        char *pp = reinterpret_cast<char *>(g.persist);
        auto keep = [&](int64_t bytes) { char *r = pp; pp += (bytes + 1023) / 1024 * 1024; return r; };
        KTable &kt = g.ktab;
        kt = KTable();
        kt.nk = (int)g.kidx.size(); kt.ldc = K; kt.ldm = ldm;
        std::vector<OzKBufs> kb;
        int64_t col = 0;
        for (int q = 0; q < kt.nk; ++q) {
            const PlanKpoint &pk = pl->kps[g.kidx[q]];
            const int64_t G = pk.n_g;
            KEntry &e = kt.e[q];
            e.kp = pk.dk;
            e.col_begin = col;
            col += G;
            if (pl->sf) {
                e.C = nullptr;            // structure-factor form: only the per-type rows
                e.X = nullptr;
            } else {
                e.C = reinterpret_cast<double2 *>(take(K * G * (int64_t)sizeof(double2)));
                e.X = pl->opts.precision == HSDLA_PREC_FP64
                          ? reinterpret_cast<double2 *>(take(K * G * (int64_t)sizeof(double2)))
                          : e.C;   // Ozaki: X reuses C once C is sliced
            }
            e.M = pl->hoist ? reinterpret_cast<double2 *>(take(ldm * G * (int64_t)sizeof(double2))) : nullptr;
            double2 *Z = pl->hoist ? reinterpret_cast<double2 *>(take(ldm * G * (int64_t)sizeof(double2))) : nullptr;
            e.Z = Z;
            if (pl->sf) {
                SfEntry &f = g.sft.e[q];
                f = SfEntry();
                f.PS = reinterpret_cast<double2 *>(take(pl->tbatch * G * G * (int64_t)sizeof(double2)));
                f.PH = reinterpret_cast<double2 *>(take(pl->tbatch * G * G * (int64_t)sizeof(double2)));
                f.ldp = G; f.n = G; f.pstride = G * G; f.g = pk.dk.g;
            }
            OzKBufs b;
            b.CX = e.C; b.M = e.M; b.Z = Z; b.G = G;
            if (pl->sf) {
                b.PS = const_cast<double2 *>(g.sft.e[q].PS);
                b.PH = const_cast<double2 *>(g.sft.e[q].PH);
                b.pstride = g.sft.e[q].pstride;
            }
            kb.push_back(b);
        }
        kt.total_cols = col;
        if (pl->sf) {
            SfTab &ft = g.sft;
            const SfTab &dm = pl->sf_dims;
            ft.nk = kt.nk;
            ft.dx = dm.dx; ft.dy = dm.dy; ft.dz = dm.dz; ft.ny = dm.ny; ft.nz = dm.nz; ft.box = dm.box;
        }
        if (pl->opts.precision == HSDLA_PREC_OZAKI_FP8) {
            OzGroupDesc d;
            d.twoL = twoL; d.na = pl->na; d.nt = pl->nt; d.hoist = pl->hoist;
            d.w = pl->w; d.Tfull = pl->Tfull; d.atom_type = pl->atom_type.data();
            d.panels = pl->panels;
            d.sf = pl->sf; d.wt = pl->wt; d.sf_tab = pl->sf_tab; d.tbatch = pl->tbatch;
            char *oz_ws = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
            int rc = ozaki_group_prepare(pl->oz, d, kb, oz_ws, g.persist, st, &g.oz);
            if (rc) return set_err(ctx, rc, "group set-up failed: %s", ozaki_last_error());
            // streamed host output runs the S/H products as one launch per column block: an event
            // pair for each, where there are more blocks than types
            const size_t nev = 2 * (size_t)ozaki_group_output_blocks(g.oz);
            while (pl->sf && g.ev_dom.size() < nev) {
                g.ev_dom.push_back(nullptr);
                CUDA_TRY(ctx, cudaEventCreate(&g.ev_dom.back()));
            }
            g.ev_t.assign(2 * ozaki_group_tapply_events(g.oz), nullptr);
            for (auto &e : g.ev_t) CUDA_TRY(ctx, cudaEventCreate(&e));
        } else {
            g.ev_t.assign(2, nullptr);
            for (auto &e : g.ev_t) CUDA_TRY(ctx, cudaEventCreate(&e));
            std::vector<Fp64Job> jt, jsh;
            for (int q = 0; q < kt.nk; ++q) {
                const KEntry &e = kt.e[q];
                const int64_t G = pl->kps[g.kidx[q]].n_g;
                if (pl->hoist) {
                    for (int t = 0; t < pl->nt; ++t) {
                        Fp64Job jb{};
                        jb.P = pl->Tfull + (int64_t)t * twoL * twoL; jb.ldp = twoL;
                        jb.Q = e.M + twoL * t; jb.ldq = ldm;
                        jb.out = const_cast<double2 *>(e.Z) + twoL * t; jb.ldo = ldm;
                        jb.m = twoL; jb.n = G; jb.k = twoL;
                        jt.push_back(jb);
                    }
                } else {
                    for (int j = 0; j < pl->na; ++j) {
                        Fp64Job jb{};
                        jb.P = pl->Tfull + (int64_t)pl->atom_type[j] * twoL * twoL; jb.ldp = twoL;
                        jb.Q = e.C + twoL * j; jb.ldq = K;
                        jb.out = e.X + twoL * j; jb.ldo = K;
                        jb.m = twoL; jb.n = G; jb.k = twoL;
                        jt.push_back(jb);
                    }
                }
                if (pl->sf) continue;
                Fp64Job js{};
                js.P = e.C; js.ldp = K; js.Q = e.C; js.ldq = K; js.w = pl->w;
                js.m = G; js.n = G; js.k = K; js.lower = 1;
                Fp64Job jh = js;
                jh.Q = e.X; jh.w = nullptr;
                jsh.push_back(js);
                jsh.push_back(jh);
            }
            g.tiles_t = assign_tiles(jt, 0);
            if (pl->sf) {
                // per type: S_t = M_t^H diag(w_t) M_t and H_t = M_t^H Z_t of every k-point into the
                // products; one launch per type (each type's jobs carry their own tile numbering)
                for (int t = 0; t < pl->nt; ++t) {
                    std::vector<Fp64Job> jt_sh;
                    for (int q = 0; q < kt.nk; ++q) {
                        const KEntry &e = kt.e[q];
                        const int64_t G = pl->kps[g.kidx[q]].n_g;
                        Fp64Job js{};
                        js.P = e.M + twoL * t; js.ldp = ldm; js.Q = e.M + twoL * t; js.ldq = ldm;
                        js.w = pl->wt + twoL * t;
                        const int64_t slot = (int64_t)(t % pl->tbatch) * g.sft.e[q].pstride;
                        js.out = const_cast<double2 *>(g.sft.e[q].PS) + slot; js.ldo = G;
                        js.m = G; js.n = G; js.k = twoL; js.lower = 1;
                        Fp64Job jh = js;
                        jh.Q = e.Z + twoL * t; jh.w = nullptr;
                        jh.out = const_cast<double2 *>(g.sft.e[q].PH) + slot;
                        jt_sh.push_back(js);
                        jt_sh.push_back(jh);
                    }
                    g.tiles_sh = assign_tiles(jt_sh, 0);
                    jsh.insert(jsh.end(), jt_sh.begin(), jt_sh.end());
                }
            } else {
                g.tiles_sh = assign_tiles(jsh, 0);
            }
            g.n_jobs_t = (int)jt.size();
            g.d_jobs_t = reinterpret_cast<Fp64Job *>(keep(sizeof(Fp64Job) * jt.size()));
            g.d_jobs_sh = reinterpret_cast<Fp64Job *>(keep(sizeof(Fp64Job) * jsh.size()));
            if (pp - reinterpret_cast<char *>(g.persist) > g.persist_bytes)
                return set_err(ctx, HSDLA_ERR_NOMEM, "job tables (%lld bytes) exceed the group's %lld persistent bytes",
                               (long long)(pp - reinterpret_cast<char *>(g.persist)), (long long)g.persist_bytes);
            if (cudaHostAlloc((void **)&g.h_jobs_sh, sizeof(Fp64Job) * jsh.size(), cudaHostAllocDefault) != cudaSuccess) {
                g.h_jobs_sh = nullptr;
                return set_err(ctx, HSDLA_ERR_NOMEM, "pinned job table allocation failed");
            }
            memcpy(g.h_jobs_sh, jsh.data(), sizeof(Fp64Job) * jsh.size());
            CUDA_TRY(ctx, cudaMemcpy(g.d_jobs_t, jt.data(), sizeof(Fp64Job) * jt.size(), cudaMemcpyHostToDevice));
            if (pl->sf)     // the products' jobs do not change between runs
                CUDA_TRY(ctx, cudaMemcpy(g.d_jobs_sh, jsh.data(), sizeof(Fp64Job) * jsh.size(), cudaMemcpyHostToDevice));
        }
    }
    pl->prepared_ws = ws;
    return HSDLA_OK;
}

// Point the groups' S/H job tables at this call's outputs (host side; copied in stream order).
void set_outputs(hsdla_plan *pl, hsdla_cx *const *dH, hsdla_cx *const *dS, const int64_t *ld) {
    for (auto &g : pl->groups) {
        const int nk = (int)g.kidx.size();
        std::vector<double2 *> S(nk), H(nk);
        std::vector<int64_t> l(nk);
        for (int q = 0; q < nk; ++q) {
            S[q] = reinterpret_cast<double2 *>(dS[g.kidx[q]]);
            H[q] = reinterpret_cast<double2 *>(dH[g.kidx[q]]);
            l[q] = ld[g.kidx[q]];
        }
        if (pl->sf) {
            for (int q = 0; q < nk; ++q) {
                g.sft.e[q].S = S[q];
                g.sft.e[q].H = H[q];
                g.sft.e[q].ldo = l[q];
            }
            if (g.oz) ozaki_group_set_sf(g.oz, g.sft);
        } else if (g.oz) {
            ozaki_group_set_outputs(g.oz, S.data(), H.data(), l.data());
        } else {
            for (int q = 0; q < nk; ++q) {
                g.h_jobs_sh[2 * q].out = S[q];
                g.h_jobs_sh[2 * q].ldo = l[q];
                g.h_jobs_sh[2 * q + 1].out = H[q];
                g.h_jobs_sh[2 * q + 1].ldo = l[q];
            }
        }
    }
}

// Event record that becomes an external event-record node under stream capture.
cudaError_t record_event(cudaEvent_t ev, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cs);
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal)
                                               : cudaEventRecord(ev, st);
}

// Device time of the S/H launches of the last execution (all groups; after it completed).
float dominant_ms(const hsdla_plan *pl) {
    float tot = 0.f;
    for (const auto &g : pl->groups) {
        float d = 0.f;
        for (size_t i = 0; i + 1 < g.ev_dom.size(); i += 2)
            if (g.ev_dom[i] && cudaEventElapsedTime(&d, g.ev_dom[i], g.ev_dom[i + 1]) == cudaSuccess) tot += d;
    }
    cudaGetLastError();
    return tot;
}

// Algorithmic flops of one group's S/H launches (FP8 digit products for Ozaki): contraction
// length 2La, or 2L per type in the structure-factor form.
void run_groups_flop_one(const hsdla_plan *pl, const hsdla_plan::Group &g, double *dom_flop) {
    const double sl = pl->oz.num_slices;
    const double Klen = pl->sf ? 2.0 * pl->L * pl->nt : (double)pl->twoLa;
    for (int q = 0; q < g.ktab.nk; ++q) {
        const double G = (double)g.ktab.e[q].kp.n_g;
        const double lower = 4.0 * G * (G + 1.0) * Klen;
        *dom_flop += 2.0 * lower * (g.oz ? sl * (sl + 1) / 2 : 1.0);
    }
}

void run_groups_flop(const hsdla_plan *pl, double *dom_flop) {
    *dom_flop = 0.0;
    for (const auto &g : pl->groups) run_groups_flop_one(pl, g, dom_flop);
}

// The combine table of a group with the caller's page-locked host H and S as its outputs (the
// device outputs become the sums of earlier batches, read when the batch is not the first).
SfTab host_output_tab(const hsdla_plan *pl, const hsdla_plan::Group &g) {
    SfTab tab = g.sft;
    for (int q = 0; q < g.ktab.nk; ++q) {
        const int i = g.kidx[q];
        tab.e[q].Si = tab.e[q].S;
        tab.e[q].Hi = tab.e[q].H;
        tab.e[q].ldi = tab.e[q].ldo;
        tab.e[q].H = reinterpret_cast<double2 *>(pl->dl->H[i]);
        tab.e[q].S = reinterpret_cast<double2 *>(pl->dl->S[i]);
        tab.e[q].ldo = pl->dl->ld[i];
    }
    return tab;
}

// The last combine batch of a group [t0, t0 + ntypes).  With a host download pending (and no graph
// capture) it runs in column blocks of kDownBlock, and after each block the copy stream downloads
// that block of every k-point's H and S lower triangle while the next block is combined.
int combine_last(hsdla_plan *pl, hsdla_plan::Group &g, int t0, int ntypes, cudaStream_t st, bool capturing) {
    hsdla_context *ctx = pl->ctx;
    SfTab tab = g.sft;
    tab.type = t0;
    tab.ntypes = ntypes;
    tab.slot0 = t0 % std::max(pl->tbatch, 1);
    if (!pl->dl || capturing) {
        CUDA_TRY(ctx, launch_sf_combine(tab, pl->sf_tab, t0 == 0, st));
        pl->launches++;
        return HSDLA_OK;
    }
    if (pl->dl->direct) {
        // the combine writes the host outputs itself (page-locked memory, addressed over the
        // CPU-GPU link), adding to the device sums of the earlier batches: no download
        SfTab ht = host_output_tab(pl, g);
        ht.type = tab.type;
        ht.ntypes = tab.ntypes;
        ht.slot0 = tab.slot0;
        CUDA_TRY(ctx, launch_sf_combine(ht, pl->sf_tab, t0 == 0, st));
        pl->launches++;
        pl->dl->done = pl->dl->in_place = true;
        return HSDLA_OK;
    }
    int64_t gmax = 0;
    for (int q = 0; q < g.ktab.nk; ++q) gmax = std::max(gmax, pl->kps[g.kidx[q]].n_g);
    for (int64_t c0 = 0; c0 < gmax; c0 += kDownBlock) {
        tab.col0 = c0;
        tab.col1 = c0 + kDownBlock;
        CUDA_TRY(ctx, launch_sf_combine(tab, pl->sf_tab, t0 == 0, st));
        pl->launches++;
        CUDA_TRY(ctx, cudaEventRecord(ctx->ev_copy, st));
        CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_copy, 0));
        for (int q = 0; q < g.ktab.nk; ++q) {
            const int i = g.kidx[q];
            const int64_t n = pl->kps[i].n_g;
            if (c0 >= n) continue;
            const int64_t w = std::min(kDownBlock, n - c0);
            const SfEntry &E = g.sft.e[q];
            const hsdla_cx *dS = reinterpret_cast<const hsdla_cx *>(E.S), *dH = reinterpret_cast<const hsdla_cx *>(E.H);
            for (int m = 0; m < 2; ++m) {
                hsdla_cx *host = m == 0 ? pl->dl->H[i] : pl->dl->S[i];
                const hsdla_cx *dev = m == 0 ? dH : dS;
                const int64_t ld = pl->dl->ld[i];
                CUDA_TRY(ctx, cudaMemcpy2DAsync(host + c0 + ld * c0, ld * sizeof(hsdla_cx), dev + c0 + E.ldo * c0,
                                                E.ldo * sizeof(hsdla_cx), (n - c0) * sizeof(hsdla_cx), w,
                                                cudaMemcpyDeviceToHost, ctx->copy_stream));
            }
        }
    }
    pl->dl->done = true;
    return HSDLA_OK;
}

// Enqueue every group's launches (no host synchronisation: capturable in a CUDA graph).
int run_groups(hsdla_plan *pl, cudaStream_t st, bool timed, float *ms_ab, float *ms_tap, double *dom_flop) {
    hsdla_context *ctx = pl->ctx;
    pl->launches = 0;
    if (dom_flop) *dom_flop = 0.0;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CUDA_TRY(ctx, cudaStreamIsCapturing(st, &cap));
    const bool capturing = cap != cudaStreamCaptureStatusNone;
    // the structure-factor form's last combine batch of a group runs here (with the download)
    const bool defer = pl->sf && pl->dl && !capturing;
    const int last_t0 = (pl->nt - 1) / std::max(pl->tbatch, 1) * std::max(pl->tbatch, 1);
    for (auto &g : pl->groups) {
        if (timed) CUDA_TRY(ctx, cudaEventRecord(ctx->evs[0], st));
        if (!pl->external) {
            CUDA_TRY(ctx, launch_construct_ab_multi(pl->dsys, g.ktab, st));
            pl->launches++;
        }
        if (timed) CUDA_TRY(ctx, cudaEventRecord(ctx->evs[1], st));
        if (dom_flop) {
            double f = 0.0;
            run_groups_flop_one(pl, g, &f);
            *dom_flop += f;
        }
        if (g.oz) {
            int nl = 0;
            // page-locked host outputs: written in column blocks while the products run, where the
            // group allows it (every type in one combine batch)
            const bool streamed = defer && pl->dl->direct && ozaki_group_streamable(g.oz);
            SfTab host_tab{};
            if (streamed) host_tab = host_output_tab(pl, g);
            const int rc = ozaki_group_run(g.oz, pl->dsys, g.ktab, st, g.ev_dom.data(), (int)g.ev_dom.size(), &nl,
                                           defer, timed ? g.ev_t.data() : nullptr, timed ? (int)g.ev_t.size() : 0,
                                           streamed ? &host_tab : nullptr);
            if (rc) return set_err(ctx, rc, "Ozaki group failed: %s", ozaki_last_error());
            pl->launches += nl;
            if (streamed) {
                pl->dl->done = pl->dl->in_place = true;
                pl->dl->blocks = ozaki_group_output_blocks(g.oz);
            } else if (defer) {
                const int t0 = ozaki_group_last_combine(g.oz);
                const int rcc = combine_last(pl, g, t0, pl->nt - t0, st, capturing);
                if (rcc) return rcc;
            }
        } else if (pl->sf) {
            if (timed) CUDA_TRY(ctx, cudaEventRecord(g.ev_t[0], st));
            CUDA_TRY(ctx, launch_fp64_jobs(g.d_jobs_t, g.n_jobs_t, g.tiles_t, st));
            if (timed) CUDA_TRY(ctx, cudaEventRecord(g.ev_t[1], st));
            pl->launches++;
            const int nj = 2 * g.ktab.nk;
            for (int t = 0; t < pl->nt; ++t) {
                CUDA_TRY(ctx, record_event(g.ev_dom[2 * t], st));
                CUDA_TRY(ctx, launch_fp64_jobs(g.d_jobs_sh + (int64_t)nj * t, nj, g.tiles_sh, st));
                CUDA_TRY(ctx, record_event(g.ev_dom[2 * t + 1], st));
                pl->launches++;
                // the batch's last type: its products into S and H
                if ((t + 1) % pl->tbatch == 0 || t + 1 == pl->nt) {
                    const int t0 = t / pl->tbatch * pl->tbatch;
                    if (t0 == last_t0) {
                        const int rcc = combine_last(pl, g, t0, t + 1 - t0, st, capturing);
                        if (rcc) return rcc;
                        continue;
                    }
                    g.sft.type = t0;
                    g.sft.ntypes = t + 1 - t0;
                    CUDA_TRY(ctx, launch_sf_combine(g.sft, pl->sf_tab, t0 == 0, st));
                    pl->launches++;
                }
            }
        } else {
            if (timed) CUDA_TRY(ctx, cudaEventRecord(g.ev_t[0], st));
            CUDA_TRY(ctx, launch_fp64_jobs(g.d_jobs_t, g.n_jobs_t, g.tiles_t, st));
            if (timed) CUDA_TRY(ctx, cudaEventRecord(g.ev_t[1], st));
            pl->launches++;
            if (pl->hoist) {
                CUDA_TRY(ctx, launch_apply_phase_multi(pl->dsys, g.ktab, st));
                pl->launches++;
            }
            CUDA_TRY(ctx, cudaMemcpyAsync(g.d_jobs_sh, g.h_jobs_sh, sizeof(Fp64Job) * 2 * g.ktab.nk,
                                          cudaMemcpyHostToDevice, st));
            CUDA_TRY(ctx, record_event(g.ev_dom[0], st));
            CUDA_TRY(ctx, launch_fp64_jobs(g.d_jobs_sh, 2 * g.ktab.nk, g.tiles_sh, st));
            CUDA_TRY(ctx, record_event(g.ev_dom[1], st));
            pl->launches++;
        }
        if (timed) {
            // stage times need the events: wait for this group (un-graphed runs only)
            CUDA_TRY(ctx, cudaEventSynchronize(g.ev_dom.back()));
            float a = 0;
            cudaEventElapsedTime(&a, ctx->evs[0], ctx->evs[1]);
            *ms_ab += a;
            for (size_t i = 0; ms_tap && i + 1 < g.ev_t.size(); i += 2) {
                float b = 0;
                if (cudaEventElapsedTime(&b, g.ev_t[i], g.ev_t[i + 1]) == cudaSuccess) *ms_tap += b;
            }
            cudaGetLastError();
        }
    }
    return HSDLA_OK;
}

// The tile tuner of the structure-factor form (after a plan's first completed run): the S/H
// tile shape and accumulation split timed on this data, or taken from the context's cache for
// this shape, then set on every group.  HSDLA_PAIR_HALVES or HSDLA_MERGE in the environment, or
// HSDLA_TILE_TUNE=0, keep the configuration the groups were prepared with.
int tune_tiles(hsdla_plan *pl, cudaStream_t st) {
    hsdla_context *ctx = pl->ctx;
    pl->tiles_done = true;
    if (pl->groups.empty() || !pl->groups[0].oz || !ozaki_group_tunable(pl->groups[0].oz)) return HSDLA_OK;
    if (getenv("HSDLA_PAIR_HALVES") || getenv("HSDLA_MERGE") || !env_flag("HSDLA_TILE_TUNE", true)) return HSDLA_OK;
    const auto &g0 = pl->groups[0];
    int64_t gmax = 0;
    for (int i : g0.kidx) gmax = std::max(gmax, pl->kps[i].n_g);
    const auto key = std::make_tuple(2 * pl->L, pl->nt, (int)g0.kidx.size(), (gmax + 511) / 512, pl->oz.num_slices);
    int h = 0, m = 0;
    auto hit = ctx->tile_cache.find(key);
    if (hit != ctx->tile_cache.end()) {
        h = hit->second.first;
        m = hit->second.second;
    } else {
        float best = 0.f;
        const int rc = ozaki_group_tune_tiles(g0.oz, st, &best);
        if (rc) return set_err(ctx, rc, "tile tuner: %s", ozaki_last_error());
        const int rce = ozaki_check_device_error(pl->oz);
        if (rce) return set_err(ctx, rce, "tile tuner: device-side error: %s", ozaki_last_error());
        ozaki_group_tiles(g0.oz, &h, &m);
        ctx->tile_cache[key] = std::make_pair(h, m);
    }
    int h0 = 0, m0 = 0;
    ozaki_group_tiles(g0.oz, &h0, &m0);
    for (auto &g : pl->groups) ozaki_group_set_tiles(g.oz, h, m);
    pl->tiles_tuned = true;
    pl->tile_h = h;
    pl->tile_m = m;
    // a captured graph holds the old launch parameters
    if ((h != h0 || m != m0) && pl->graph) {
        cudaGraphExecDestroy(pl->graph);
        pl->graph = nullptr;
        pl->graph_outputs.clear();
    }
    return HSDLA_OK;
}

}  // namespace

extern "C" {

int64_t hsdla_plan_workspace_bytes(const hsdla_plan *pl) {
    if (!pl) return 0;
    int64_t ngmax = 0;
    for (auto &k : pl->kps) ngmax = std::max(ngmax, k.n_g);
    // the slice autotuner builds the largest k-point's C at the start of the workspace
    return std::max(pl->group_ws_bytes, 2 * (int64_t)sizeof(double2) * pl->twoLa * ngmax) + 4096;
}

void hsdla_plan_destroy(hsdla_plan *pl) {
    if (!pl) return;
    hsdla_context *ctx = pl->ctx;
    cudaSetDevice(ctx->device);
    // all of the plan's work done (on any stream) before its blocks can be handed out again
    cudaDeviceSynchronize();
    release_groups(pl);
    if (pl->d_jobs) ctx_free(ctx, pl->d_jobs, pl->jobs_cap * sizeof(Fp64Job));
    if (pl->tables) ctx_free(ctx, pl->tables, pl->tables_bytes);
    ozaki_plan_release(pl->oz);
    ctx->plans.erase(pl);
    delete pl;
}

int hsdla_plan_construct_ab(hsdla_plan *pl, int32_t ik, hsdla_cx *dC, void *stream) {
    if (!pl || !dC || ik < 0 || ik >= (int)pl->kps.size()) return HSDLA_ERR_ARG;
    hsdla_context *ctx = pl->ctx;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;   // NULL = the default (legacy) stream, as in CUDA
    if (pl->kps[ik].n_g == 0) return HSDLA_OK;
    CUDA_TRY(ctx, launch_construct_ab(pl->dsys, pl->kps[ik].dk, reinterpret_cast<double2 *>(dC), pl->twoLa, st));
    return HSDLA_OK;
}

int hsdla_plan_execute(hsdla_plan *pl, hsdla_cx *const *dH, hsdla_cx *const *dS, const int64_t *ld, void *stream,
                       hsdla_report *rep) {
    if (!pl || (!pl->kps.empty() && (!dH || !dS || !ld))) return HSDLA_ERR_ARG;
    hsdla_context *ctx = pl->ctx;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;   // NULL = the default (legacy) stream, as in CUDA
    const int nk = (int)pl->kps.size();
    for (int i = 0; i < nk; ++i) {
        if (pl->kps[i].n_g == 0) continue;
        if (!dH[i] || !dS[i]) return set_err(ctx, HSDLA_ERR_ARG, "output %d is NULL", i);
        if (ld[i] < pl->kps[i].n_g) return set_err(ctx, HSDLA_ERR_ARG, "ld[%d]=%lld < n_g=%lld", i,
                                                   (long long)ld[i], (long long)pl->kps[i].n_g);
    }
    int rc;
    void *ws = nullptr;
    if (pl->autotune) {
        int64_t ngmax = 0;
        for (auto &k : pl->kps) ngmax = std::max(ngmax, k.n_g);
        rc = ctx_workspace(ctx, 2 * (int64_t)sizeof(double2) * pl->twoLa * ngmax + 4096, &ws);
        if (rc) return rc;
        rc = autotune_slices(pl, reinterpret_cast<double2 *>(ws), st);
        if (rc) return rc;
        release_groups(pl);
        pl->groups.clear();
    }
    if (pl->groups.empty()) form_groups(pl, workspace_budget(ctx));
    rc = ctx_workspace(ctx, hsdla_plan_workspace_bytes(pl), &ws);
    if (rc) return rc;
    if (pl->prepared_ws != ws) {
        const auto q0 = std::chrono::steady_clock::now();
        // groups prepared before may still be in use by queued work (a fresh plan has none)
        if (pl->prepared_ws) CUDA_TRY(ctx, cudaStreamSynchronize(st));
        release_groups(pl);
        rc = prepare_groups(pl, ws, st);
        if (rc) { release_groups(pl); return rc; }
        if (env_flag("HSDLA_TRACE", false))
            fprintf(stderr, "hsdla_plan_execute: group set-up %.3f ms (host, before the first launch)\n",
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - q0).count());
        if (pl->tiles_tuned)
            for (auto &g : pl->groups) ozaki_group_set_tiles(g.oz, pl->tile_h, pl->tile_m);
    }
    set_outputs(pl, dH, dS, ld);
    float ms_ab = 0.f, ms_tap = 0.f;
    double dom_flop = 0.0;
    const bool want_graph = pl->opts.use_graph != 0 && !pl->graph_failed;
    cudaStream_t run_st = want_graph && st == nullptr ? ctx->stream : st;   // the legacy stream cannot capture
    if (run_st != st) {
        CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, st));
        CUDA_TRY(ctx, cudaStreamWaitEvent(run_st, ctx->ev0, 0));
    }
    CUDA_TRY(ctx, cudaEventRecord(ctx->evs[2], run_st));
    if (want_graph) {
        std::vector<void *> outs;
        for (int i = 0; i < nk; ++i) { outs.push_back(dH[i]); outs.push_back(dS[i]); }
        if (pl->graph && (outs != pl->graph_outputs || pl->graph_stream != run_st)) {
            cudaGraphExecDestroy(pl->graph);
            pl->graph = nullptr;
        }
        if (!pl->graph) {
            // outputs travel through the pinned job tables, so a graph is re-captured only when the
            // output pointers or the stream change (the tables' copy nodes read them at launch)
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamBeginCapture(run_st, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                rc = run_groups(pl, run_st, false, nullptr, nullptr, &dom_flop);
                e = cudaStreamEndCapture(run_st, &graph);
                if (rc == HSDLA_OK && e == cudaSuccess) e = cudaGraphInstantiate(&pl->graph, graph, 0);
                if (graph) cudaGraphDestroy(graph);
            }
            if (rc != HSDLA_OK || e != cudaSuccess) {
                cudaGetLastError();
                pl->graph = nullptr;
                pl->graph_failed = true;     // run un-captured from now on
            } else {
                pl->graph_outputs = outs;
                pl->graph_stream = run_st;
            }
        }
        if (pl->graph) {
            CUDA_TRY(ctx, cudaGraphLaunch(pl->graph, run_st));
            if (dom_flop == 0.0) run_groups_flop(pl, &dom_flop);
        } else {
            rc = run_groups(pl, run_st, true, &ms_ab, &ms_tap, &dom_flop);
            if (rc) return rc;
        }
    } else {
        rc = run_groups(pl, run_st, true, &ms_ab, &ms_tap, &dom_flop);
        if (rc) return rc;
    }
    CUDA_TRY(ctx, cudaEventRecord(ctx->evs[3], run_st));
    if (run_st != st) {
        CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, run_st));
        CUDA_TRY(ctx, cudaStreamWaitEvent(st, ctx->ev1, 0));
    }
    CUDA_TRY(ctx, cudaEventSynchronize(ctx->evs[3]));
    rc = ozaki_check_device_error(pl->oz);
    if (rc) return set_err(ctx, rc, "device-side error: %s", ozaki_last_error());
    float ms_run = 0.f;
    cudaEventElapsedTime(&ms_run, ctx->evs[2], ctx->evs[3]);
    if (!pl->tiles_done) {
        rc = tune_tiles(pl, run_st);
        if (rc) return rc;
    }
    if (rep) {
        const float ms = ms_run;
        memset(rep, 0, sizeof(*rep));
        rep->ms_total = ms;
        rep->num_kpoints = nk;
        rep->ms_per_kpoint = nk ? ms / nk : 0.0;
        rep->flop = pl->flop;
        rep->eff_tflops = ms > 0 ? pl->flop / (ms * 1e-3) / 1e12 : 0.0;
        rep->ms_construct_ab = ms_ab;
        rep->ms_tapply = ms_tap;
        rep->ms_contract = ms - ms_ab - ms_tap;
        rep->ms_dominant = dominant_ms(pl);
        rep->dominant_flop = dom_flop;
        rep->num_slices = pl->opts.precision == HSDLA_PREC_OZAKI_FP8 ? pl->oz.num_slices : 0;
        rep->est_rel_err = pl->est_err;
        rep->kernel_launches = pl->launches;
        rep->num_panels = pl->opts.precision == HSDLA_PREC_OZAKI_FP8 ? pl->panels : 0;
        rep->num_row_sets = pl->sf ? pl->nt : 0;
        rep->rotation_classes = pl->classes > 0 ? 1 : 0;
        if (!pl->groups.empty() && pl->groups[0].oz && ozaki_group_tunable(pl->groups[0].oz)) {
            int h = 0, m = 0;
            ozaki_group_tiles(pl->groups[0].oz, &h, &m);
            rep->tile_halves = h;
            rep->merged_units = m;
            rep->tile_tuned = pl->tiles_tuned ? 1 : 0;
        }
    }
    return HSDLA_OK;
}

int hsdla_contract_ab(hsdla_context *ctx, int32_t L, int32_t a, int64_t G, const hsdla_cx *A, const hsdla_cx *B,
                      const int32_t *t_sizes, const hsdla_cx *const *t_aa, const hsdla_cx *const *t_ab,
                      const hsdla_cx *const *t_bb, const int32_t *lmaxs, int32_t max_lmax, const double *sqrt_u_norms,
                      hsdla_cx *H, hsdla_cx *S, int64_t ld, const hsdla_opts *opts, hsdla_report *rep) {
    using cx = std::complex<double>;
    if (!ctx) return HSDLA_ERR_ARG;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    if (L < 1 || a < 1 || G < 0 || max_lmax < 0 || max_lmax > kMaxLmax || (max_lmax + 1) * (max_lmax + 1) != L)
        return set_err(ctx, HSDLA_ERR_ARG, "L=%d must equal (max_lmax+1)^2 with max_lmax=%d <= %d", L, max_lmax,
                       kMaxLmax);
    if (G == 0) return HSDLA_OK;
    if (!A || !B || !t_sizes || !t_aa || !t_ab || !t_bb || !lmaxs || !sqrt_u_norms || !H || !S || ld < G)
        return set_err(ctx, HSDLA_ERR_ARG, "a required pointer is NULL or ld < n_g");
    const int nl = max_lmax + 1;
    const int64_t twoL = 2 * (int64_t)L;
    std::vector<cx> tf_all((size_t)a * twoL * twoL, 0.0);
    std::vector<double> w(twoL * a), wsq(twoL * a);
    for (int j = 0; j < a; ++j) {
        const int na_ = t_sizes[3 * j], nab = t_sizes[3 * j + 1], nb = t_sizes[3 * j + 2];
        if (na_ < 0 || nab < 0 || nb < 0 || na_ > L || nab > L || nb > L || lmaxs[j] < 0 || lmaxs[j] > max_lmax)
            return set_err(ctx, HSDLA_ERR_ARG, "atom %d: T sizes (%d, %d, %d) or lmax %d out of range", j, na_, nab, nb,
                           lmaxs[j]);
        const cx *aa = reinterpret_cast<const cx *>(t_aa[j]);
        const cx *ab = reinterpret_cast<const cx *>(t_ab[j]);
        const cx *bb = reinterpret_cast<const cx *>(t_bb[j]);
        if ((na_ && !aa) || (nab && !ab) || (nb && !bb)) return set_err(ctx, HSDLA_ERR_ARG, "atom %d: T block NULL", j);
        cx *T = tf_all.data() + (size_t)j * twoL * twoL;
        // zhemm('L') reads the lower triangles of T_AA and T_BB (h_and_s_stripped_v2.cpp:202,345);
        // zgemm('C') the whole T_AB (:209); blocks smaller than L are zero-padded, which is what
        // the reference's row compaction (X_height, :211-230) amounts to
        for (int c = 0; c < na_; ++c)
            for (int r = 0; r < na_; ++r) T[r + twoL * c] = (r >= c) ? aa[r + na_ * c] : std::conj(aa[c + na_ * r]);
        for (int c = 0; c < nb; ++c)
            for (int r = 0; r < nb; ++r)
                T[(L + r) + twoL * (L + c)] = (r >= c) ? bb[r + nb * c] : std::conj(bb[c + nb * r]);
        for (int c = 0; c < nab; ++c)
            for (int r = 0; r < nab; ++r) {
                T[r + twoL * (L + c)] = ab[r + nab * c];
                T[(L + c) + twoL * r] = std::conj(ab[r + nab * c]);
            }
        for (int l = 0; l < nl; ++l) {
            const double su = sqrt_u_norms[j * nl + l];
            for (int lm = l * l; lm < (l + 1) * (l + 1); ++lm) {
                w[twoL * j + lm] = 1.0; wsq[twoL * j + lm] = 1.0;
                // rows above the atom's lmax are left unset by apply_u_norm_s (:64-86) while B is 0 there
                const double u = (l <= lmaxs[j]) ? su * su : 0.0;
                w[twoL * j + L + lm] = u; wsq[twoL * j + L + lm] = std::sqrt(u);
            }
        }
    }
    for (const cx &v : tf_all)
        if (!std::isfinite(v.real()) || !std::isfinite(v.imag())) return set_err(ctx, HSDLA_ERR_INPUT, "T not finite");
    if (!finite_all(sqrt_u_norms, (int64_t)a * nl)) return set_err(ctx, HSDLA_ERR_INPUT, "u norms not finite");
    // ---- an external plan: every atom its own type, per-atom T application, C from the caller
    auto *pl = new hsdla_plan();
    pl->ctx = ctx;
    if (opts) pl->opts = *opts;
    if (pl->opts.precision != HSDLA_PREC_FP64 && pl->opts.precision != HSDLA_PREC_OZAKI_FP8) {
        delete pl;
        return set_err(ctx, HSDLA_ERR_ARG, "unknown precision %d", pl->opts.precision);
    }
    if (pl->opts.target_rel_err <= 0.0) pl->opts.target_rel_err = 1e-13;
    pl->L = L; pl->na = a; pl->nt = a; pl->max_lmax = max_lmax;
    pl->hoist = false;
    pl->external = true;
    pl->twoLa = twoL * a;
    pl->atom_type.resize(a);
    for (int j = 0; j < a; ++j) pl->atom_type[j] = j;
    const int64_t bytes = ((int64_t)sizeof(double2) * tf_all.size() + 255) / 256 * 256 + 2 * 8 * pl->twoLa + 512;
    int rc = ctx_malloc(ctx, &pl->tables, bytes);
    if (rc) { delete pl; return rc; }
    pl->tables_bytes = bytes;
    ctx->plans.insert(pl);
    char *dp = reinterpret_cast<char *>(pl->tables);
    pl->Tfull = reinterpret_cast<double2 *>(dp);
    pl->w = reinterpret_cast<double *>(dp + ((int64_t)sizeof(double2) * tf_all.size() + 255) / 256 * 256);
    pl->wsqrt = pl->w + pl->twoLa;
    PlanKpoint pk;
    pk.n_g = G;
    pk.dk.n_g = G;
    pl->kps.push_back(pk);
    pl->flop = 20.0 * (double)G * G * L * a + 24.0 * (double)L * L * a * G;
    cudaStream_t st = ctx->stream;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    void *dout = nullptr, *ws = nullptr;
    auto done = [&](int code) {
        cudaStreamSynchronize(st);
        hsdla_plan_destroy(pl);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return code;
    };
    cudaEventRecord(e0, st);
    if (cudaMemcpyAsync(pl->Tfull, tf_all.data(), sizeof(double2) * tf_all.size(), cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(pl->w, w.data(), 8 * pl->twoLa, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(pl->wsqrt, wsq.data(), 8 * pl->twoLa, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return done(set_err(ctx, HSDLA_ERR_CUDA, "table upload failed"));
    if (pl->opts.precision == HSDLA_PREC_OZAKI_FP8) {
        // no sampling autotune without the physics inputs: num_slices = 0 means the default
        rc = ozaki_plan_init(pl->oz, pl->opts.num_slices, pl->opts.target_rel_err);
        if (rc) return done(set_err(ctx, rc, "bad slice count"));
    }
    form_groups(pl, workspace_budget(ctx));
    rc = ctx_workspace(ctx, hsdla_plan_workspace_bytes(pl), &ws);
    if (rc) return done(rc);
    rc = prepare_groups(pl, ws, st);
    if (rc) return done(rc);
    rc = ctx_host_out(ctx, 2 * G * G * (int64_t)sizeof(double2), &dout);
    if (rc) return done(rc);
    hsdla_cx *dH = reinterpret_cast<hsdla_cx *>(dout), *dS = dH + G * G;
    const int64_t ldd = G;
    // A, B (L x a x G, column-major) straight into C's per-atom [A_a; B_a] row blocks
    const KEntry &e = pl->groups[0].ktab.e[0];
    if (cudaMemsetAsync(dout, 0, 2 * G * G * sizeof(double2), st) != cudaSuccess ||
        cudaMemcpy2DAsync(e.C, twoL * sizeof(double2), A, L * sizeof(double2), L * sizeof(double2), (size_t)a * G,
                          cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpy2DAsync(e.C + L, twoL * sizeof(double2), B, L * sizeof(double2), L * sizeof(double2), (size_t)a * G,
                          cudaMemcpyHostToDevice, st) != cudaSuccess)
        return done(set_err(ctx, HSDLA_ERR_CUDA, "A/B upload failed"));
    set_outputs(pl, &dH, &dS, &ldd);
    float ms_ab = 0.f, ms_tap = 0.f;
    double dom_flop = 0.0;
    rc = run_groups(pl, st, true, &ms_ab, &ms_tap, &dom_flop);
    if (rc) return done(rc);
    if (download_lower(H, ld, dH, G, st) != cudaSuccess || download_lower(S, ld, dS, G, st) != cudaSuccess)
        return done(set_err(ctx, HSDLA_ERR_CUDA, "H/S download failed"));
    cudaEventRecord(e1, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return done(set_err(ctx, HSDLA_ERR_CUDA, "sync failed"));
    rc = ozaki_check_device_error(pl->oz);
    if (rc) return done(set_err(ctx, rc, "device-side error: %s", ozaki_last_error()));
    if (rep) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        memset(rep, 0, sizeof(*rep));
        rep->ms_total = ms;
        rep->ms_per_kpoint = ms;
        rep->num_kpoints = 1;
        rep->flop = pl->flop;
        rep->eff_tflops = ms > 0 ? pl->flop / (ms * 1e-3) / 1e12 : 0.0;
        rep->ms_tapply = ms_tap;
        rep->ms_dominant = dominant_ms(pl);
        rep->dominant_flop = dom_flop;
        rep->num_slices = pl->opts.precision == HSDLA_PREC_OZAKI_FP8 ? pl->oz.num_slices : 0;
        rep->kernel_launches = pl->launches;
        rep->num_panels = pl->opts.precision == HSDLA_PREC_OZAKI_FP8 ? pl->panels : 0;
    }
    return done(HSDLA_OK);
}

int hsdla_create_hs(hsdla_context *ctx, const hsdla_system *s, const hsdla_kpoint *kpts, int32_t nk,
                    hsdla_cx *const *H, hsdla_cx *const *S, const int64_t *ld, const hsdla_opts *opts,
                    hsdla_report *rep) {
    if (!ctx) return HSDLA_ERR_ARG;
    if (nk > 0 && (!H || !S || !ld)) return set_err(ctx, HSDLA_ERR_ARG, "H, S or ld is NULL");
    for (int i = 0; i < nk; ++i)
        if (kpts && kpts[i].n_g > 0 && (!H[i] || !S[i] || ld[i] < kpts[i].n_g))
            return set_err(ctx, HSDLA_ERR_ARG, "k-point %d: bad output buffer or ld", i);
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    // HSDLA_TRACE=1: host-side phase times of each call on stderr
    const bool trace = env_flag("HSDLA_TRACE", false);
    using clk = std::chrono::steady_clock;
    const auto ms_since = [](clk::time_point a) { return std::chrono::duration<double, std::milli>(clk::now() - a).count(); };
    const clk::time_point t_start = clk::now();
    double t_plan = 0, t_setup = 0, t_exec = 0, t_sync = 0;
    cudaEvent_t e0, e1;
    CUDA_TRY(ctx, cudaEventCreate(&e0));
    CUDA_TRY(ctx, cudaEventCreate(&e1));
    cudaEventRecord(e0, ctx->stream);
    hsdla_plan *pl = nullptr;
    // the T blocks' check read after the launches (HSDLA_DEFER_TCHECK=0: before them)
    int rc = plan_create_impl(ctx, s, kpts, nk, opts, &pl, env_flag("HSDLA_DEFER_TCHECK", true));
    t_plan = ms_since(t_start);
    if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
    // device outputs: one buffer of the largest size, reused per k-point group
    std::vector<int64_t> ng(nk);
    int64_t out_elems = 0;
    for (int i = 0; i < nk; ++i) { ng[i] = kpts[i].n_g; out_elems += 2 * ng[i] * ng[i]; }
    void *dout = nullptr;
    rc = ctx_host_out(ctx, std::max<int64_t>(out_elems, 1) * (int64_t)sizeof(double2), &dout);
    if (rc) { hsdla_plan_destroy(pl); cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
    std::vector<hsdla_cx *> dH(nk), dS(nk);
    std::vector<int64_t> dld(nk);
    hsdla_cx *p = reinterpret_cast<hsdla_cx *>(dout);
    for (int i = 0; i < nk; ++i) {
        dH[i] = p; p += ng[i] * ng[i];
        dS[i] = p; p += ng[i] * ng[i];
        dld[i] = std::max<int64_t>(ng[i], 1);
    }
    // zero the diagonal blocks of the device outputs: the download of a column block starts at its
    // first row, so it carries the block's upper triangle, which nothing else writes
    cudaError_t e = cudaSuccess;
    for (int i = 0; e == cudaSuccess && i < nk; ++i)
        for (int m = 0; m < 2 && e == cudaSuccess; ++m)
            for (int64_t c0 = 0; c0 < ng[i] && e == cudaSuccess; c0 += kDownBlock) {
                const int64_t w = std::min(kDownBlock, ng[i] - c0);
                hsdla_cx *d = (m == 0 ? dH[i] : dS[i]) + c0 + ng[i] * c0;
                e = cudaMemset2DAsync(d, ng[i] * sizeof(hsdla_cx), 0, w * sizeof(hsdla_cx), w, ctx->stream);
            }
    // structure-factor form: the last combine downloads each column block as soon as it is done
    hsdla_plan::Download dl;
    dl.H.assign(H, H + nk);
    dl.S.assign(S, S + nk);
    dl.ld.assign(ld, ld + nk);
    // page-locked host outputs that the GPU addresses directly (unified addressing): the last
    // combine can write them in place (HSDLA_DIRECT_OUTPUT=0 keeps the download)
    dl.direct = nk > 0 && env_flag("HSDLA_DIRECT_OUTPUT", true);
    for (int i = 0; dl.direct && i < nk; ++i) {
        if (ng[i] == 0) continue;
        for (hsdla_cx *hp : {H[i], S[i]}) {
            cudaPointerAttributes pa{};
            if (cudaPointerGetAttributes(&pa, hp) != cudaSuccess || pa.type != cudaMemoryTypeHost ||
                pa.devicePointer != (void *)hp) {
                cudaGetLastError();
                dl.direct = false;
            }
        }
    }
    t_setup = ms_since(t_start) - t_plan;
    if (e == cudaSuccess) {
        pl->dl = &dl;
        rc = hsdla_plan_execute(pl, dH.data(), dS.data(), dld.data(), ctx->stream, rep);
        pl->dl = nullptr;
        t_exec = ms_since(t_start) - t_plan - t_setup;
    } else {
        rc = set_err(ctx, HSDLA_ERR_CUDA, "memset failed: %s", cudaGetErrorString(e));
    }
    if (rc == HSDLA_OK && dl.done) {
        // the end-to-end event waits for the copy stream's downloads
        e = cudaEventRecord(ctx->ev_copy, ctx->copy_stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, ctx->ev_copy, 0);
        if (e != cudaSuccess) rc = set_err(ctx, HSDLA_ERR_CUDA, "D2H copy failed: %s", cudaGetErrorString(e));
    }
    for (int i = 0; rc == HSDLA_OK && !dl.done && i < nk; ++i) {
        if (ng[i] == 0) continue;
        e = download_lower(H[i], ld[i], dH[i], ng[i], ctx->stream);
        if (e == cudaSuccess) e = download_lower(S[i], ld[i], dS[i], ng[i], ctx->stream);
        if (e != cudaSuccess) rc = set_err(ctx, HSDLA_ERR_CUDA, "D2H copy failed: %s", cudaGetErrorString(e));
    }
    cudaEventRecord(e1, ctx->stream);
    cudaError_t es = cudaStreamSynchronize(ctx->stream);
    t_sync = ms_since(t_start) - t_plan - t_setup - t_exec;
    float ms_dev = 0.f;
    if (es == cudaSuccess) cudaEventElapsedTime(&ms_dev, e0, e1);
    if (rc == HSDLA_OK && es != cudaSuccess) rc = set_err(ctx, HSDLA_ERR_CUDA, "sync failed: %s", cudaGetErrorString(es));
    if (pl->tcheck_pending && (rc == HSDLA_OK || es == cudaSuccess)) {
        // the T blocks' check, deferred past the launches (their statistics are on the host now)
        const int nt = pl->nt;
        const std::vector<unsigned long long> st(pl->tcheck_host, pl->tcheck_host + 5 * (size_t)nt);
        const int rct = check_tmats(ctx, st, nt, pl->tcheck_class_type.empty() ? nullptr : &pl->tcheck_class_type);
        if (rct) rc = rct;
    }
    if (rc == HSDLA_OK && rep) {
        rep->ms_total = ms_dev;   // end-to-end: upload, compute, download
        rep->ms_per_kpoint = nk ? ms_dev / nk : 0.0;
        rep->eff_tflops = ms_dev > 0 ? pl->flop / (ms_dev * 1e-3) / 1e12 : 0.0;
        rep->outputs_in_place = dl.in_place ? 1 : 0;
        rep->output_blocks = dl.blocks;
        rep->ms_host_setup = t_plan + t_setup;
    }
    if (trace && es == cudaSuccess) {
        // the S/H launches on the call's device timeline (ms from its start): the gaps between
        // them are the combines (and, streamed, the host writes of each block's diagonal square)
        std::string tl;
        for (const auto &g : pl->groups)
            for (size_t i = 0; i + 1 < g.ev_dom.size(); i += 2) {
                float a = 0.f, b = 0.f;
                if (cudaEventElapsedTime(&a, e0, g.ev_dom[i]) == cudaSuccess &&
                    cudaEventElapsedTime(&b, e0, g.ev_dom[i + 1]) == cudaSuccess && b > a) {
                    char buf[48];
                    snprintf(buf, sizeof(buf), " %.2f-%.2f", a, b);
                    tl += buf;
                }
            }
        cudaGetLastError();
        fprintf(stderr, "hsdla_create_hs: S/H launches at%s of %.2f ms\n", tl.c_str(), ms_dev);
    }
    const clk::time_point t_destroy = clk::now();
    hsdla_plan_destroy(pl);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (trace)
        fprintf(stderr,
                "hsdla_create_hs: plan %.2f ms, set-up %.2f ms, execute %.2f ms, sync %.2f ms, destroy %.2f ms; "
                "device %.2f ms; in place %d; context holds %lld B (%lld B kept for reuse)\n",
                t_plan, t_setup, t_exec, t_sync, ms_since(t_destroy), ms_dev, dl.in_place ? 1 : 0,
                (long long)ctx->mem_used, (long long)ctx->cached_bytes);
    return rc;
}

int hsdla_selftest_wait_timeout(hsdla_context *ctx, int32_t which, int64_t budget_cycles) {
    if (!ctx) return HSDLA_ERR_ARG;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    OzakiPlan oz{};
    int rc = ozaki_plan_init(oz, kOzDefaultSlices, 1e-13);
    if (rc) return set_err(ctx, rc, "self-test set-up failed: %s", ozaki_last_error());
    rc = ozaki_wait_selftest(oz, which, budget_cycles, ctx->stream);
    ozaki_plan_release(oz);
    if (rc) return set_err(ctx, rc, "%s", ozaki_last_error());
    return HSDLA_OK;
}

int hsdla_pack_lower(hsdla_context *ctx, int64_t n, const hsdla_cx *M, int64_t ld, hsdla_cx *packed, void *stream) {
    if (!ctx) return HSDLA_ERR_ARG;
    if (n < 0 || ld < std::max<int64_t>(n, 1) || (n > 0 && (!M || !packed)))
        return set_err(ctx, HSDLA_ERR_ARG, "pack_lower: n < 0, ld < n or a NULL buffer");
    if (n == 0) return HSDLA_OK;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const cudaError_t e = launch_pack_lower(reinterpret_cast<const double2 *>(M), ld, n,
                                            reinterpret_cast<double2 *>(packed), (cudaStream_t)stream);
    if (e != cudaSuccess) return set_err(ctx, HSDLA_ERR_CUDA, "pack_lower: %s", cudaGetErrorString(e));
    return HSDLA_OK;
}

int hsdla_zherkx_lower(hsdla_context *ctx, int32_t precision, int32_t num_slices, int64_t n, int64_t k,
                       const hsdla_cx *dP, int64_t ldp, const hsdla_cx *dQ, int64_t ldq, const double *dw,
                       hsdla_cx *dOut, int64_t ldo, void *stream) {
    if (!ctx) return HSDLA_ERR_ARG;
    if (n < 0 || k < 0 || !dP || !dQ || !dOut || ldp < k || ldq < k || ldo < n)
        return set_err(ctx, HSDLA_ERR_ARG, "bad zherkx arguments");
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;   // NULL = the default (legacy) stream, as in CUDA
    if (n == 0) return HSDLA_OK;
    if (precision == HSDLA_PREC_FP64) {
        std::vector<Fp64Job> jobs(1);
        Fp64Job &j = jobs[0];
        j.P = reinterpret_cast<const double2 *>(dP); j.ldp = ldp;
        j.Q = reinterpret_cast<const double2 *>(dQ); j.ldq = ldq;
        j.w = dw; j.out = reinterpret_cast<double2 *>(dOut); j.ldo = ldo;
        j.m = n; j.n = n; j.k = k; j.lower = 1;
        const int64_t tiles = assign_tiles(jobs, 0);
        void *dj = nullptr;
        int rc = ctx_malloc(ctx, &dj, sizeof(Fp64Job));
        if (rc) return rc;
        cudaError_t e = cudaMemcpyAsync(dj, jobs.data(), sizeof(Fp64Job), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = launch_fp64_jobs((Fp64Job *)dj, 1, tiles, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        ctx_free(ctx, dj, sizeof(Fp64Job));
        if (e != cudaSuccess) return set_err(ctx, HSDLA_ERR_CUDA, "zherkx fp64: %s", cudaGetErrorString(e));
        return HSDLA_OK;
    }
    if (precision == HSDLA_PREC_OZAKI_FP8) {
        OzakiPlan oz{};
        int rc = ozaki_plan_init(oz, num_slices, 1e-13);
        if (rc) return set_err(ctx, rc, "bad slice count");
        void *ws = nullptr;
        rc = ctx_workspace(ctx, ozaki_herkx_workspace(oz.num_slices, k, n), &ws);
        if (rc) return rc;
        int nl = 0;
        rc = ozaki_herkx(oz, reinterpret_cast<const double2 *>(dP), ldp, reinterpret_cast<const double2 *>(dQ), ldq,
                         dw, k, n, reinterpret_cast<double2 *>(dOut), ldo, ws, st, &nl);
        if (rc) { ozaki_plan_release(oz); return set_err(ctx, rc, "Ozaki zherkx failed: %s", ozaki_last_error()); }
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { ozaki_plan_release(oz); return set_err(ctx, HSDLA_ERR_CUDA, "zherkx ozaki: %s", cudaGetErrorString(e)); }
        rc = ozaki_check_device_error(oz);
        ozaki_plan_release(oz);
        if (rc) return set_err(ctx, rc, "device-side error: %s", ozaki_last_error());
        return HSDLA_OK;
    }
    return set_err(ctx, HSDLA_ERR_ARG, "unknown precision %d", precision);
}

}  // extern "C"

// =====================================================================================
// BLAS-shaped contraction plugin: the reference's dev_zherk_ / dev_zher2k_ / dev_zherkx_
// (flapw_opt/src/include/acc/wrappers.h:19-28, flapw_opt/src/wrappers.cpp:171-257) with their
// full argument semantics, on this library's lower-triangle contraction R = lower(P^H Q).
namespace {

enum PluginKind { kPluginHerk = 0, kPluginHer2k = 1, kPluginHerkx = 2 };

// True when p is host memory (pageable or page-locked): such operands are staged through device
// memory, as the reference's cuBLASXt backend does with the page-locked buffers of create_HS2.
bool host_memory(const void *p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeUnregistered;
}

int64_t r1k(int64_t b) { return (b + 1023) / 1024 * 1024; }

//   zherk : C = alpha op(A) op(A)^H + beta C                       (alpha, beta real)
//   zher2k: C = alpha op(A) op(B)^H + conj(alpha) op(B) op(A)^H + beta C
//   zherkx: C = alpha op(A) op(B)^H + beta C (the product taken as Hermitian; no diagonal rule)
// with op(X) = X (trans 'N', X n x k) or X^H (trans 'C', X k x n), on C's uplo triangle only.
// With the k x n operands X_A = op(A)^H (A itself for 'C', its conjugate transpose for 'N') and
// X_B likewise, op(A) op(B)^H = X_A^H X_B, so every product is lower(P^H Q):
//   zherk : P = Q = X_A,  zherkx: P = X_A, Q = X_B,  zher2k: P = [X_A; X_B], Q = [alpha X_B; conj(alpha) X_A].
// uplo 'U' swaps P and Q: the upper triangle of P^H Q is the conjugate transpose of the lower
// triangle of Q^H P.
int plugin_contract(hsdla_context *ctx, int kind, int32_t precision, int32_t num_slices, char uplo, char trans,
                    int64_t n, int64_t k, double2 alpha, const double2 *A, int64_t lda, const double2 *B, int64_t ldb,
                    double beta, double2 *C, int64_t ldc, cudaStream_t st) {
    static const char *names[3] = {"zherk", "zher2k", "zherkx"};
    const char *nm = names[kind];
    const char u = (char)toupper((unsigned char)uplo), tr = (char)toupper((unsigned char)trans);
    if (u != 'L' && u != 'U') return set_err(ctx, HSDLA_ERR_ARG, "%s: uplo must be 'L' or 'U'", nm);
    if (tr != 'N' && tr != 'C') return set_err(ctx, HSDLA_ERR_ARG, "%s: trans must be 'N' or 'C'", nm);
    if (precision != HSDLA_PREC_FP64 && precision != HSDLA_PREC_OZAKI_FP8)
        return set_err(ctx, HSDLA_ERR_ARG, "%s: unknown precision %d", nm, precision);
    if (n < 0 || k < 0) return set_err(ctx, HSDLA_ERR_ARG, "%s: n or k negative", nm);
    const bool two = kind != kPluginHerk;
    const int64_t rows = tr == 'N' ? n : k, cols = tr == 'N' ? k : n;   // stored shape of A (and B)
    if (lda < std::max<int64_t>(1, rows) || (two && ldb < std::max<int64_t>(1, rows)) || ldc < std::max<int64_t>(1, n))
        return set_err(ctx, HSDLA_ERR_ARG, "%s: leading dimension too small (lda, ldb >= %s, ldc >= n)", nm,
                       tr == 'N' ? "n" : "k");
    if (n == 0) return HSDLA_OK;
    const bool product = k > 0 && (alpha.x != 0.0 || alpha.y != 0.0);
    if (!C || (product && (!A || (two && !B)))) return set_err(ctx, HSDLA_ERR_ARG, "%s: NULL matrix", nm);
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const bool upper = u == 'U', herm = kind != kPluginHerkx;
    const bool hA = product && host_memory(A), hB = product && two && host_memory(B), hC = host_memory(C);
    const int64_t K = kind == kPluginHer2k ? 2 * k : k;
    // operands in place when A (and B) are already K x n: trans 'C', not zher2k
    const bool build = product && (tr == 'N' || kind == kPluginHer2k);
    // R straight into C's lower triangle when nothing is left to scale or add
    const bool direct = !upper && beta == 0.0 && (kind == kPluginHer2k || (alpha.x == 1.0 && alpha.y == 0.0));
    const int s = precision == HSDLA_PREC_OZAKI_FP8 ? (num_slices == 0 ? kOzDefaultSlices : num_slices) : 0;
    if (precision == HSDLA_PREC_OZAKI_FP8 && (s < 2 || s > kOzMaxSlices))
        return set_err(ctx, HSDLA_ERR_ARG, "%s: num_slices outside [2, 12]", nm);
    // ---- workspace: staged host operands, built operands, R, the contraction's own scratch
    const int64_t e16 = (int64_t)sizeof(double2);
    int64_t off = 0;
    auto slot = [&](bool need, int64_t bytes) { const int64_t o = off; if (need) off += r1k(bytes); return o; };
    const int64_t oA = slot(hA, rows * cols * e16), oB = slot(hB, rows * cols * e16), oC = slot(hC, n * n * e16);
    const int64_t oP = slot(build, K * n * e16), oQ = slot(build && kind != kPluginHerk, K * n * e16);
    const int64_t oR = slot(product && !direct, n * n * e16);
    const int64_t oJ = slot(product && precision == HSDLA_PREC_FP64, sizeof(Fp64Job));
    const int64_t oZ = slot(product && precision == HSDLA_PREC_OZAKI_FP8, s ? ozaki_herkx_workspace(s, K, n) : 0);
    void *wsv = nullptr;
    int rc = ctx_workspace(ctx, std::max<int64_t>(off, 1024), &wsv);
    if (rc) return rc;
    char *ws = reinterpret_cast<char *>(wsv);
    // ---- stage host memory
    const double2 *dA = A, *dB = B;
    double2 *dC = C;
    int64_t dlda = lda, dldb = ldb, dldc = ldc;
    if (hA) {
        CUDA_TRY(ctx, cudaMemcpy2DAsync(ws + oA, rows * e16, A, lda * e16, rows * e16, cols, cudaMemcpyHostToDevice, st));
        dA = reinterpret_cast<const double2 *>(ws + oA);
        dlda = rows;
    }
    if (hB) {
        CUDA_TRY(ctx, cudaMemcpy2DAsync(ws + oB, rows * e16, B, ldb * e16, rows * e16, cols, cudaMemcpyHostToDevice, st));
        dB = reinterpret_cast<const double2 *>(ws + oB);
        dldb = rows;
    }
    if (hC) {
        // the whole n x n block travels (the other triangle comes back as it went)
        CUDA_TRY(ctx, cudaMemcpy2DAsync(ws + oC, n * e16, C, ldc * e16, n * e16, n, cudaMemcpyHostToDevice, st));
        dC = reinterpret_cast<double2 *>(ws + oC);
        dldc = n;
    }
    // ---- operands and product
    const double2 one = make_double2(1.0, 0.0), calpha = make_double2(alpha.x, -alpha.y);
    double2 *R = direct ? dC : reinterpret_cast<double2 *>(ws + oR);
    const int64_t ldr = direct ? dldc : n;
    if (product) {
        const double2 *P = dA, *Q = two ? dB : dA;
        int64_t ldp = dlda, ldq = two ? dldb : dlda;
        if (build) {
            double2 *bP = reinterpret_cast<double2 *>(ws + oP);
            double2 *bQ = kind == kPluginHerk ? bP : reinterpret_cast<double2 *>(ws + oQ);
            const bool t = tr == 'N';
            cudaError_t e = launch_plugin_operand(dA, dlda, t, k, n, one, bP, K, 0, st);
            if (kind == kPluginHer2k) {
                if (e == cudaSuccess) e = launch_plugin_operand(dB, dldb, t, k, n, one, bP, K, k, st);
                if (e == cudaSuccess) e = launch_plugin_operand(dB, dldb, t, k, n, alpha, bQ, K, 0, st);
                if (e == cudaSuccess) e = launch_plugin_operand(dA, dlda, t, k, n, calpha, bQ, K, k, st);
            } else if (kind == kPluginHerkx) {
                if (e == cudaSuccess) e = launch_plugin_operand(dB, dldb, t, k, n, one, bQ, K, 0, st);
            }
            if (e != cudaSuccess) return set_err(ctx, HSDLA_ERR_CUDA, "%s: operand build: %s", nm, cudaGetErrorString(e));
            P = bP; Q = bQ; ldp = ldq = K;
        }
        if (upper) { std::swap(P, Q); std::swap(ldp, ldq); }
        if (precision == HSDLA_PREC_FP64) {
            std::vector<Fp64Job> jobs(1);
            Fp64Job &j = jobs[0];
            j.P = P; j.ldp = ldp; j.Q = Q; j.ldq = ldq; j.w = nullptr;
            j.out = R; j.ldo = ldr; j.m = n; j.n = n; j.k = K; j.lower = 1;
            const int64_t tiles = assign_tiles(jobs, 0);
            Fp64Job *dj = reinterpret_cast<Fp64Job *>(ws + oJ);
            CUDA_TRY(ctx, cudaMemcpyAsync(dj, jobs.data(), sizeof(Fp64Job), cudaMemcpyHostToDevice, st));
            CUDA_TRY(ctx, launch_fp64_jobs(dj, 1, tiles, st));
        } else {
            rc = ozaki_plan_init(ctx->plugin_oz, s, 1e-13);
            if (rc) return set_err(ctx, rc, "%s: %s", nm, ozaki_last_error());
            int nl = 0;
            rc = ozaki_herkx(ctx->plugin_oz, P, ldp, Q, ldq, nullptr, K, n, R, ldr, ws + oZ, st, &nl);
            if (rc) return set_err(ctx, rc, "%s: %s", nm, ozaki_last_error());
        }
    }
    // ---- epilogue on C's triangle (in place for the direct form: only the real diagonal)
    if (!direct || herm) {
        const double2 a = kind == kPluginHer2k ? one : alpha;
        CUDA_TRY(ctx, launch_plugin_epilogue(product ? R : nullptr, ldr, dC, dldc, n, a, beta, upper, herm, st));
    }
    if (hC) CUDA_TRY(ctx, cudaMemcpy2DAsync(C, ldc * e16, dC, n * e16, n * e16, n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if (product && precision == HSDLA_PREC_OZAKI_FP8) {
        rc = ozaki_check_device_error(ctx->plugin_oz);
        if (rc) return set_err(ctx, rc, "%s: device-side error: %s", nm, ozaki_last_error());
    }
    return HSDLA_OK;
}

// The Fortran-style entry points' library-owned context and settings (hsdla_dev_init).
std::mutex g_dev_mu;
hsdla_context *g_dev_ctx = nullptr;
int32_t g_dev_prec = HSDLA_PREC_FP64, g_dev_slices = 0;
thread_local int g_dev_status = HSDLA_OK;

hsdla_context *dev_ctx() {
    std::lock_guard<std::mutex> lock(g_dev_mu);
    if (!g_dev_ctx) {
        int dev = 0;
        if (const char *v = getenv("HSDLA_DEVICE")) dev = (int)strtol(v, nullptr, 10);
        if (hsdla_context_create(dev, &g_dev_ctx) != HSDLA_OK) g_dev_ctx = nullptr;
    }
    return g_dev_ctx;
}

void dev_call(int kind, const char *uplo, const char *trans, const int *n, const int *k, double2 alpha,
              const hsdla_cx *A, const int *lda, const hsdla_cx *B, const int *ldb, const double *beta, hsdla_cx *C,
              const int *ldc) {
    hsdla_context *ctx = dev_ctx();
    if (!ctx) { g_dev_status = HSDLA_ERR_DEVICE; return; }
    if (!uplo || !trans || !n || !k || !lda || !beta || !ldc || (kind != kPluginHerk && !ldb)) {
        g_dev_status = set_err(ctx, HSDLA_ERR_ARG, "NULL scalar argument");
        return;
    }
    std::lock_guard<std::mutex> lock(g_dev_mu);   // one context: calls are serialised
    g_dev_status = plugin_contract(ctx, kind, g_dev_prec, g_dev_slices, *uplo, *trans, *n, *k, alpha,
                                   reinterpret_cast<const double2 *>(A), *lda, reinterpret_cast<const double2 *>(B),
                                   ldb ? *ldb : 0, *beta, reinterpret_cast<double2 *>(C), *ldc, ctx->stream);
}

}  // namespace

extern "C" {

int hsdla_zherk(hsdla_context *ctx, int32_t precision, int32_t num_slices, char uplo, char trans, int64_t n, int64_t k,
                double alpha, const hsdla_cx *A, int64_t lda, double beta, hsdla_cx *C, int64_t ldc, void *stream) {
    if (!ctx) return HSDLA_ERR_ARG;
    return plugin_contract(ctx, kPluginHerk, precision, num_slices, uplo, trans, n, k, make_double2(alpha, 0.0),
                           reinterpret_cast<const double2 *>(A), lda, nullptr, 0, beta, reinterpret_cast<double2 *>(C),
                           ldc, (cudaStream_t)stream);
}

int hsdla_zher2k(hsdla_context *ctx, int32_t precision, int32_t num_slices, char uplo, char trans, int64_t n,
                 int64_t k, hsdla_cx alpha, const hsdla_cx *A, int64_t lda, const hsdla_cx *B, int64_t ldb, double beta,
                 hsdla_cx *C, int64_t ldc, void *stream) {
    if (!ctx) return HSDLA_ERR_ARG;
    return plugin_contract(ctx, kPluginHer2k, precision, num_slices, uplo, trans, n, k, make_double2(alpha.re, alpha.im),
                           reinterpret_cast<const double2 *>(A), lda, reinterpret_cast<const double2 *>(B), ldb, beta,
                           reinterpret_cast<double2 *>(C), ldc, (cudaStream_t)stream);
}

int hsdla_zherkx(hsdla_context *ctx, int32_t precision, int32_t num_slices, char uplo, char trans, int64_t n,
                 int64_t k, hsdla_cx alpha, const hsdla_cx *A, int64_t lda, const hsdla_cx *B, int64_t ldb, double beta,
                 hsdla_cx *C, int64_t ldc, void *stream) {
    if (!ctx) return HSDLA_ERR_ARG;
    return plugin_contract(ctx, kPluginHerkx, precision, num_slices, uplo, trans, n, k, make_double2(alpha.re, alpha.im),
                           reinterpret_cast<const double2 *>(A), lda, reinterpret_cast<const double2 *>(B), ldb, beta,
                           reinterpret_cast<double2 *>(C), ldc, (cudaStream_t)stream);
}

int hsdla_dev_init(int32_t device, int32_t precision, int32_t num_slices) {
    if (precision != HSDLA_PREC_FP64 && precision != HSDLA_PREC_OZAKI_FP8) return HSDLA_ERR_ARG;
    if (precision == HSDLA_PREC_OZAKI_FP8 && num_slices != 0 && (num_slices < 2 || num_slices > kOzMaxSlices))
        return HSDLA_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_dev_mu);
    if (g_dev_ctx && g_dev_ctx->device != device) {
        hsdla_context_destroy(g_dev_ctx);
        g_dev_ctx = nullptr;
    }
    if (!g_dev_ctx) {
        const int rc = hsdla_context_create(device, &g_dev_ctx);
        if (rc) { g_dev_ctx = nullptr; return rc; }
    }
    g_dev_prec = precision;
    g_dev_slices = num_slices;
    return HSDLA_OK;
}

int hsdla_dev_finalize(void) {
    std::lock_guard<std::mutex> lock(g_dev_mu);
    if (g_dev_ctx) hsdla_context_destroy(g_dev_ctx);
    g_dev_ctx = nullptr;
    return HSDLA_OK;
}

const hsdla_context *hsdla_dev_context(void) {
    std::lock_guard<std::mutex> lock(g_dev_mu);
    return g_dev_ctx;
}

int hsdla_dev_status(void) { return g_dev_status; }

void hsdla_dev_zherk_(const char *uplo, const char *trans, const int *n, const int *k, const double *alpha,
                      const hsdla_cx *A, const int *lda, const double *beta, hsdla_cx *C, const int *ldc) {
    if (!alpha) { g_dev_status = HSDLA_ERR_ARG; return; }
    dev_call(kPluginHerk, uplo, trans, n, k, make_double2(*alpha, 0.0), A, lda, nullptr, nullptr, beta, C, ldc);
}

void hsdla_dev_zher2k_(const char *uplo, const char *trans, const int *n, const int *k, const hsdla_cx *alpha,
                       const hsdla_cx *A, const int *lda, const hsdla_cx *B, const int *ldb, const double *beta,
                       hsdla_cx *C, const int *ldc) {
    if (!alpha) { g_dev_status = HSDLA_ERR_ARG; return; }
    dev_call(kPluginHer2k, uplo, trans, n, k, make_double2(alpha->re, alpha->im), A, lda, B, ldb, beta, C, ldc);
}

void hsdla_dev_zherkx_(const char *uplo, const char *trans, const int *n, const int *k, const hsdla_cx *alpha,
                       const hsdla_cx *A, const int *lda, const hsdla_cx *B, const int *ldb, const double *beta,
                       hsdla_cx *C, const int *ldc) {
    if (!alpha) { g_dev_status = HSDLA_ERR_ARG; return; }
    dev_call(kPluginHerkx, uplo, trans, n, k, make_double2(alpha->re, alpha->im), A, lda, B, ldb, beta, C, ldc);
}

}  // extern "C"
