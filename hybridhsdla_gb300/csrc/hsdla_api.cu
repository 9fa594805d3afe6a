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
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <string>
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
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evs[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    std::set<hsdla_plan *> plans;   // live plans, destroyed with the context
    // slice autotuner results: (L, atoms, types, n_G bucket, target) -> (slices, predicted error)
    std::map<std::tuple<int, int, int, int64_t, double>, std::pair<int, double>> tune_cache;
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
    bool autotune = false;           // Ozaki slice count still to be chosen from the data
    bool hoist = false;              // T application per type (no atom carries its own rotation)
    double est_err = 0.0;            // autotuner's predicted relative error
    int launches = 0;
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

int ctx_malloc(hsdla_context *ctx, void **p, int64_t bytes) {
    *p = nullptr;
    if (bytes <= 0) return HSDLA_OK;
    if (ctx->mem_cap > 0 && ctx->mem_used + bytes > ctx->mem_cap)
        return set_err(ctx, HSDLA_ERR_NOMEM, "device allocation of %lld bytes exceeds the cap (%lld used of %lld)",
                       (long long)bytes, (long long)ctx->mem_used, (long long)ctx->mem_cap);
    cudaError_t e = cudaMalloc(p, (size_t)bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return set_err(ctx, HSDLA_ERR_NOMEM, "cudaMalloc(%lld) failed: %s", (long long)bytes, cudaGetErrorString(e));
    }
    ctx->mem_used += bytes;
    return HSDLA_OK;
}

void ctx_free(hsdla_context *ctx, void *p, int64_t bytes) {
    if (!p) return;
    cudaFree(p);
    ctx->mem_used -= bytes;
}

// Workspace of at least `bytes`, owned by the context (reused across calls).
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
    const int na = s->num_atoms, nt = s->num_types, nl = s->max_lmax + 1, L = nl * nl;
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
        const hsdla_cx *T3[3] = {s->type_t_aa + (int64_t)t * L * L, s->type_t_ab + (int64_t)t * L * L,
                                 s->type_t_bb + (int64_t)t * L * L};
        for (int q = 0; q < 3; ++q)
            if (!finite_all(reinterpret_cast<const double *>(T3[q]), 2 * (int64_t)L * L))
                return set_err(ctx, HSDLA_ERR_INPUT, "T block %d of type %d not finite", q, t);
        // T_AA and T_BB must be Hermitian (AtomData.cpp:138-139 asserts it)
        for (int q = 0; q < 3; q += 2) {
            double mx = 0.0, dev = 0.0;
            for (int c = 0; c < L; ++c)
                for (int r = 0; r < L; ++r) {
                    const hsdla_cx a = T3[q][r + (int64_t)L * c], b = T3[q][c + (int64_t)L * r];
                    mx = std::max(mx, std::hypot(a.re, a.im));
                    dev = std::max(dev, std::hypot(a.re - b.re, a.im + b.im));
                }
            if (dev > 1e-12 * std::max(mx, 1e-300))
                return set_err(ctx, HSDLA_ERR_INPUT, "T_%s of type %d is not Hermitian (|T-T^H| = %.3g)",
                               q == 0 ? "AA" : "BB", t, dev);
        }
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

// Hermitian full 2L x 2L block of one type from the lower triangles of T_AA/T_BB
// (zhemm 'L' semantics, h_and_s_stripped_v2.cpp:202,345) and the full T_AB.
void build_tfull(const hsdla_system *s, int t, int L, std::vector<std::complex<double>> &out) {
    const int64_t LL = (int64_t)L * L, n = 2 * L;
    const auto *aa = reinterpret_cast<const std::complex<double> *>(s->type_t_aa) + t * LL;
    const auto *ab = reinterpret_cast<const std::complex<double> *>(s->type_t_ab) + t * LL;
    const auto *bb = reinterpret_cast<const std::complex<double> *>(s->type_t_bb) + t * LL;
    out.assign((size_t)n * n, 0.0);
    for (int c = 0; c < n; ++c)
        for (int r = 0; r < n; ++r) {
            std::complex<double> v;
            if (r < L && c < L) v = (r >= c) ? aa[r + L * c] : std::conj(aa[c + L * r]);
            else if (r < L) v = ab[r + L * (c - L)];
            else if (c < L) v = std::conj(ab[c + L * (r - L)]);
            else v = (r >= c) ? bb[(r - L) + L * (c - L)] : std::conj(bb[(c - L) + L * (r - L)]);
            out[r + (size_t)n * c] = v;
        }
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
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (auto &e : ctx->evs) if (e) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char *hsdla_last_error(const hsdla_context *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

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

int hsdla_plan_create(hsdla_context *ctx, const hsdla_system *s, const hsdla_kpoint *kpts, int32_t nk,
                      const hsdla_opts *opts, hsdla_plan **out) {
    if (!ctx || !out) return HSDLA_ERR_ARG;
    *out = nullptr;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    int rc = validate(ctx, s, kpts, nk);
    if (rc) return rc;
    auto *pl = new hsdla_plan();
    pl->ctx = ctx;
    if (opts) pl->opts = *opts;
    if (pl->opts.precision != HSDLA_PREC_FP64 && pl->opts.precision != HSDLA_PREC_OZAKI_FP8) {
        delete pl;
        return set_err(ctx, HSDLA_ERR_ARG, "unknown precision %d", pl->opts.precision);
    }
    if (pl->opts.target_rel_err <= 0.0) pl->opts.target_rel_err = 1e-13;
    const int na = s->num_atoms, nt = s->num_types, nl = s->max_lmax + 1, L = nl * nl;
    pl->L = L; pl->na = na; pl->nt = nt; pl->max_lmax = s->max_lmax;
    pl->hoist = s->atom_rotmat == nullptr;
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
    std::vector<std::complex<double>> tf_all((size_t)nt * 4 * L * L), tf;
    for (int t = 0; t < nt; ++t) {
        build_tfull(s, t, L, tf);
        std::copy(tf.begin(), tf.end(), tf_all.begin() + (size_t)t * 4 * L * L);
    }

    // ---- one device block for all tables
    int64_t bytes = 0;
    auto add = [&](int64_t b) { bytes += (b + 255) & ~int64_t(255); };
    add(sizeof(int32_t) * na); add(sizeof(double) * 3 * na); add(s->atom_rotmat ? sizeof(double) * 9 * na : 0);
    add(sizeof(double) * nt); add(sizeof(int32_t) * nt);
    for (int q = 0; q < 5; ++q) add(sizeof(double) * nt * nl);
    add(sizeof(double) * L);
    add(sizeof(double2) * tf_all.size());
    add(sizeof(double) * pl->twoLa); add(sizeof(double) * pl->twoLa);
    for (int i = 0; i < nk; ++i) add(sizeof(int32_t) * 3 * kpts[i].n_g);
    rc = ctx_malloc(ctx, &pl->tables, bytes);
    if (rc) { delete pl; return rc; }
    pl->tables_bytes = bytes;
    std::vector<char> host(bytes, 0);
    char *hp = host.data();
    char *dp = reinterpret_cast<char *>(pl->tables);
    auto put = [&](const void *src, int64_t b) -> void * {
        void *d = dp;
        if (b > 0 && src) memcpy(hp, src, b);
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
    D.type_rmt = (const double *)put(s->type_rmt, sizeof(double) * nt);
    D.type_lmax = (const int32_t *)put(s->type_lmax, sizeof(int32_t) * nt);
    D.u = (const double *)put(s->type_u, sizeof(double) * nt * nl);
    D.u_dr = (const double *)put(s->type_u_dr, sizeof(double) * nt * nl);
    D.dE_u = (const double *)put(s->type_dE_u, sizeof(double) * nt * nl);
    D.dE_u_dr = (const double *)put(s->type_dE_u_dr, sizeof(double) * nt * nl);
    D.inv_w = (const double *)put(inv_w.data(), sizeof(double) * nt * nl);
    D.ynorm = (const double *)put(yn.data(), sizeof(double) * L);
    pl->Tfull = (double2 *)put(tf_all.data(), sizeof(double2) * tf_all.size());
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
    cudaError_t e = cudaMemcpyAsync(pl->tables, host.data(), bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        hsdla_plan_destroy(pl);
        return set_err(ctx, HSDLA_ERR_CUDA, "table upload failed: %s", cudaGetErrorString(e));
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

int64_t hsdla_plan_workspace_bytes(const hsdla_plan *pl) {
    if (!pl) return 0;
    int64_t ngmax = 0;
    for (auto &k : pl->kps) ngmax = std::max(ngmax, k.n_g);
    int64_t b = 2 * (int64_t)sizeof(double2) * pl->twoLa * ngmax;   // C and X
    if (pl->hoist) b += 2 * (int64_t)sizeof(double2) * 2 * pl->L * pl->nt * ngmax + 1024;   // M and Z
    if (pl->opts.precision == HSDLA_PREC_OZAKI_FP8)
        b += 1024 + ozaki_pipeline_workspace(pl->oz.num_slices, 2 * (int64_t)pl->L, pl->na, pl->nt, ngmax);
    return b;
}

void hsdla_plan_destroy(hsdla_plan *pl) {
    if (!pl) return;
    hsdla_context *ctx = pl->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
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
    int64_t ngmax = 0;
    for (auto &k : pl->kps) ngmax = std::max(ngmax, k.n_g);
    void *ws = nullptr;
    int rc = ctx_workspace(ctx, hsdla_plan_workspace_bytes(pl), &ws);
    if (rc) return rc;
    double2 *C = reinterpret_cast<double2 *>(ws);
    if (pl->autotune) {
        rc = autotune_slices(pl, C, st);
        if (rc) return rc;
        rc = ctx_workspace(ctx, hsdla_plan_workspace_bytes(pl), &ws);
        if (rc) return rc;
        C = reinterpret_cast<double2 *>(ws);
    }
    double2 *X = C + pl->twoLa * ngmax;
    const int64_t ldm = 2 * (int64_t)pl->L * pl->nt;
    double2 *Mt = pl->hoist ? X + pl->twoLa * ngmax : nullptr;
    double2 *Zt = pl->hoist ? Mt + ldm * ngmax : nullptr;
    char *tail = reinterpret_cast<char *>(pl->hoist ? Zt + ldm * ngmax : X + pl->twoLa * ngmax);
    // the digit workspace needs 1024-byte alignment (TMA boxes, SW128 atoms)
    char *oz_ws = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(tail) + 1023) & ~uintptr_t(1023));
    const int64_t L = pl->L, twoL = 2 * L, twoLa = pl->twoLa;
    pl->launches = 0;
    float ms_ab = 0.f, ms_t = 0.f, ms_c = 0.f, ms_dom = 0.f;
    double dom_flop = 0.0;
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, st));
    for (int i = 0; i < nk; ++i) {
        const int64_t G = pl->kps[i].n_g;
        if (G == 0) continue;
        CUDA_TRY(ctx, cudaEventRecord(ctx->evs[0], st));
        CUDA_TRY(ctx, launch_construct_ab(pl->dsys, pl->kps[i].dk, C, twoLa, st, Mt, ldm));
        pl->launches++;
        CUDA_TRY(ctx, cudaEventRecord(ctx->evs[1], st));
        // (b) X_a = T_a C_a: per type (Z_t = T_t M_t, expanded by the phases) or per atom, one launch
        pl->h_jobs.clear();
        if (pl->hoist) {
            for (int t = 0; t < pl->nt; ++t) {
                Fp64Job jb{};
                jb.P = pl->Tfull + (int64_t)t * twoL * twoL; jb.ldp = twoL;
                jb.Q = Mt + twoL * t; jb.ldq = ldm;
                jb.out = Zt + twoL * t; jb.ldo = ldm;
                jb.m = twoL; jb.n = G; jb.k = twoL; jb.lower = 0;
                pl->h_jobs.push_back(jb);
            }
        } else {
            for (int j = 0; j < pl->na; ++j) {
                Fp64Job jb{};
                jb.P = pl->Tfull + (int64_t)pl->atom_type[j] * twoL * twoL; jb.ldp = twoL;
                jb.Q = C + twoL * j; jb.ldq = twoLa;
                jb.w = nullptr;
                jb.out = X + twoL * j; jb.ldo = twoLa;
                jb.m = twoL; jb.n = G; jb.k = twoL; jb.lower = 0;
                pl->h_jobs.push_back(jb);
            }
        }
        if (pl->opts.precision != HSDLA_PREC_FP64) pl->h_jobs.clear();   // the Ozaki pipeline emulates (b) too
        const int64_t nt_b = assign_tiles(pl->h_jobs, 0);
        const size_t nb = pl->h_jobs.size();
        // (c) S and H lower triangles
        if (pl->opts.precision == HSDLA_PREC_FP64) {
            Fp64Job js{};
            js.P = C; js.ldp = twoLa; js.Q = C; js.ldq = twoLa; js.w = pl->w;
            js.out = reinterpret_cast<double2 *>(dS[i]); js.ldo = ld[i];
            js.m = G; js.n = G; js.k = twoLa; js.lower = 1;
            Fp64Job jh = js;
            jh.Q = X; jh.w = nullptr; jh.out = reinterpret_cast<double2 *>(dH[i]);
            pl->h_jobs.push_back(js);
            pl->h_jobs.push_back(jh);
        }
        const int64_t nt_c = assign_tiles(pl->h_jobs, nb);
        if (!pl->h_jobs.empty()) {
            rc = upload_jobs(pl, st);
            if (rc) return rc;
        }
        if (nb > 0) {
            CUDA_TRY(ctx, launch_fp64_jobs(pl->d_jobs, (int)nb, nt_b, st));
            pl->launches++;
            if (pl->hoist) {
                CUDA_TRY(ctx, launch_apply_phase(pl->dsys, pl->kps[i].dk, Zt, ldm, X, twoLa, st));
                pl->launches++;
            }
        }
        CUDA_TRY(ctx, cudaEventRecord(ctx->evs[2], st));
        const double lower_cflop = 4.0 * (double)G * (double)(G + 1) * (double)twoLa;   // one lower triangle
        if (pl->opts.precision == HSDLA_PREC_FP64) {
            CUDA_TRY(ctx, cudaEventRecord(ctx->evs[4], st));
            CUDA_TRY(ctx, launch_fp64_jobs(pl->d_jobs + nb, (int)(pl->h_jobs.size() - nb), nt_c, st));
            CUDA_TRY(ctx, cudaEventRecord(ctx->evs[5], st));
            pl->launches++;
            dom_flop = 2.0 * lower_cflop;
        } else {
            const double s_ = pl->oz.num_slices;
            dom_flop = 2.0 * lower_cflop * s_ * (s_ + 1) / 2;
            int nl = 0;
            OzakiInputs in;
            in.C = C; in.Tfull = pl->Tfull; in.w = pl->w; in.atom_type = pl->atom_type.data(); in.X = X;
            in.twoL = twoL; in.na = pl->na; in.nt = pl->nt; in.G = G;
            in.ev_dom0 = ctx->evs[4]; in.ev_dom1 = ctx->evs[5];
            if (pl->hoist) { in.M = Mt; in.Z = Zt; in.sys = &pl->dsys; in.kp = &pl->kps[i].dk; }
            rc = ozaki_pipeline(pl->oz, in, reinterpret_cast<double2 *>(dS[i]), reinterpret_cast<double2 *>(dH[i]),
                                ld[i], oz_ws, st, &nl);
            if (rc) return set_err(ctx, rc, "Ozaki contraction failed: %s", ozaki_last_error());
            pl->launches += nl;
        }
        CUDA_TRY(ctx, cudaEventRecord(ctx->evs[3], st));
        CUDA_TRY(ctx, cudaEventSynchronize(ctx->evs[3]));
        float a = 0, b = 0, c = 0, d = 0;
        cudaEventElapsedTime(&a, ctx->evs[0], ctx->evs[1]);
        cudaEventElapsedTime(&b, ctx->evs[1], ctx->evs[2]);
        cudaEventElapsedTime(&c, ctx->evs[2], ctx->evs[3]);
        cudaEventElapsedTime(&d, ctx->evs[4], ctx->evs[5]);
        ms_ab += a; ms_t += b; ms_c += c; ms_dom = d;
    }
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, st));
    CUDA_TRY(ctx, cudaEventSynchronize(ctx->ev1));
    rc = ozaki_check_device_error(pl->oz);
    if (rc) return set_err(ctx, rc, "device-side error: %s", ozaki_last_error());
    if (rep) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        memset(rep, 0, sizeof(*rep));
        rep->ms_total = ms;
        rep->num_kpoints = nk;
        rep->ms_per_kpoint = nk ? ms / nk : 0.0;
        rep->flop = pl->flop;
        rep->eff_tflops = ms > 0 ? pl->flop / (ms * 1e-3) / 1e12 : 0.0;
        rep->ms_construct_ab = ms_ab;
        rep->ms_tapply = ms_t;
        rep->ms_contract = ms_c;
        rep->ms_dominant = ms_dom;
        rep->dominant_flop = dom_flop;
        rep->num_slices = pl->opts.precision == HSDLA_PREC_OZAKI_FP8 ? pl->oz.num_slices : 0;
        rep->est_rel_err = pl->est_err;
        rep->kernel_launches = pl->launches;
    }
    return HSDLA_OK;
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
    cudaEvent_t e0, e1;
    CUDA_TRY(ctx, cudaEventCreate(&e0));
    CUDA_TRY(ctx, cudaEventCreate(&e1));
    cudaEventRecord(e0, ctx->stream);
    hsdla_plan *pl = nullptr;
    int rc = hsdla_plan_create(ctx, s, kpts, nk, opts, &pl);
    if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
    // device outputs: one buffer of the largest size, reused per k-point group
    std::vector<int64_t> ng(nk);
    int64_t out_elems = 0;
    for (int i = 0; i < nk; ++i) { ng[i] = kpts[i].n_g; out_elems += 2 * ng[i] * ng[i]; }
    void *dout = nullptr;
    rc = ctx_malloc(ctx, &dout, out_elems * (int64_t)sizeof(double2));
    if (rc) { hsdla_plan_destroy(pl); cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
    std::vector<hsdla_cx *> dH(nk), dS(nk);
    std::vector<int64_t> dld(nk);
    hsdla_cx *p = reinterpret_cast<hsdla_cx *>(dout);
    for (int i = 0; i < nk; ++i) {
        dH[i] = p; p += ng[i] * ng[i];
        dS[i] = p; p += ng[i] * ng[i];
        dld[i] = std::max<int64_t>(ng[i], 1);
    }
    // the upper triangles of the outputs are returned as zero
    cudaError_t e = cudaMemsetAsync(dout, 0, out_elems * sizeof(double2), ctx->stream);
    if (e == cudaSuccess) {
        rc = hsdla_plan_execute(pl, dH.data(), dS.data(), dld.data(), ctx->stream, rep);
    } else {
        rc = set_err(ctx, HSDLA_ERR_CUDA, "memset failed: %s", cudaGetErrorString(e));
    }
    for (int i = 0; rc == HSDLA_OK && i < nk; ++i) {
        if (ng[i] == 0) continue;
        e = cudaMemcpy2DAsync(H[i], ld[i] * sizeof(hsdla_cx), dH[i], ng[i] * sizeof(hsdla_cx),
                              ng[i] * sizeof(hsdla_cx), ng[i], cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(S[i], ld[i] * sizeof(hsdla_cx), dS[i], ng[i] * sizeof(hsdla_cx),
                                  ng[i] * sizeof(hsdla_cx), ng[i], cudaMemcpyDeviceToHost, ctx->stream);
        if (e != cudaSuccess) rc = set_err(ctx, HSDLA_ERR_CUDA, "D2H copy failed: %s", cudaGetErrorString(e));
    }
    cudaEventRecord(e1, ctx->stream);
    cudaError_t es = cudaStreamSynchronize(ctx->stream);
    if (rc == HSDLA_OK && es != cudaSuccess) rc = set_err(ctx, HSDLA_ERR_CUDA, "sync failed: %s", cudaGetErrorString(es));
    if (rc == HSDLA_OK && rep) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        rep->ms_total = ms;   // end-to-end: upload, compute, download
        rep->ms_per_kpoint = nk ? ms / nk : 0.0;
        rep->eff_tflops = ms > 0 ? pl->flop / (ms * 1e-3) / 1e12 : 0.0;
    }
    ctx_free(ctx, dout, out_elems * (int64_t)sizeof(double2));
    hsdla_plan_destroy(pl);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
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
