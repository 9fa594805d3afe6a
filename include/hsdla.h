/*
 * hsdla.h -- C ABI of the GB300 (sm_103a) FLAPW Hamiltonian/overlap generator.
 *
 * Drop-in boundary for the H/S generation step of HybridHSDLA.  The reference
 * entry point is
 *
 *   double create_HS2(const arma::vec3& kpt, double kmax, const arma::mat33& bmat,
 *                     const arma::imat& g_mesh, const AtomData& ad, GenMethod method,
 *                     arma::cx_mat& H, arma::cx_mat& S)
 *   (flapw_opt/src/h_and_s.cpp:591-893, STRIPPED build; called once per k-point
 *    from generate_matrices, flapw_opt/src/h_and_s.cpp:919)
 *
 * which builds the matching tensors A, B (tensor_AB_match.cpp:63-129), applies
 * the per-atom T matrices and forms the lower triangles of
 *
 *   S = sum_a A_a^H A_a + B_a^H U_a B_a
 *   H = sum_a [A_a;B_a]^H [[T_AA, T_AB],[T_AB^H, T_BB]]_a [A_a;B_a]
 *
 * (h_and_s_stripped_v2.cpp:100-382).  Here the same quantities are passed as
 * plain arrays; everything runs on one GPU; there is no CPU fallback.  All
 * functions return HSDLA_OK (0) or a negative status; no function exits or
 * aborts.  Complex numbers are (re, im) pairs of doubles, layout-compatible
 * with std::complex<double> and Fortran double complex.
 *
 * Conventions (identical to the reference):
 *   - bmat: 3x3 row-major, row i = reciprocal basis vector b_i (bohr^-1, incl. 2 pi);
 *   - k-points and atom positions in fractional coordinates;
 *   - r_K = |bmat (k+G)| (types_helper.cpp:33), direction R^T (k+G) with
 *     R = mrot bmat per atom (tensor_AB_match.cpp:97, FleurData.cpp:453-455);
 *   - lm index = l(l+1)+m, L = (max_lmax+1)^2;
 *   - H, S: n_G x n_G column-major with leading dimension ld; only the lower
 *     triangle (row >= column) is defined.  Entry points with device outputs leave the
 *     strict upper triangle untouched.  The host-buffer entry points (hsdla_create_hs,
 *     hsdla_contract_ab) download 512-column blocks from their first row down, which sets
 *     the strict upper triangle of the diagonal 512 x 512 blocks to zero and leaves the rest
 *     of it untouched (the reference leaves it unset as well).  Where every H and S given to
 *     hsdla_create_hs is page-locked host memory that the GPU addresses at the same pointer
 *     (cudaHostAlloc, cudaMallocHost) and the plan takes the structure-factor form, the
 *     combine writes the lower triangles in place and the whole strict upper triangle stays
 *     untouched (HSDLA_DIRECT_OUTPUT=0 keeps the download).  With Ozaki precision and every
 *     type in one combine batch this happens in column blocks while the digit products of the
 *     next block run: each block's diagonal square is written in place, the rows below it are
 *     combined on the device and copied by the copy engine (HSDLA_STREAM_OUTPUT=0: all after
 *     the products).
 */
#ifndef HSDLA_H
#define HSDLA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hsdla_cx { double re, im; } hsdla_cx;

/* status codes */
enum {
    HSDLA_OK = 0,
    HSDLA_ERR_ARG = -1,        /* invalid argument (null pointer, bad size, bad ld) */
    HSDLA_ERR_CUDA = -2,       /* a CUDA runtime call failed */
    HSDLA_ERR_NOMEM = -3,      /* device or pinned allocation failed or exceeds the cap */
    HSDLA_ERR_INPUT = -4,      /* non-finite input, zero Wronskian, non-Hermitian T */
    HSDLA_ERR_TIMEOUT = -5,    /* a bounded device-side wait expired (kernel error word) */
    HSDLA_ERR_UNSUPPORTED = -6,/* size or option outside what this build supports */
    HSDLA_ERR_DEVICE = -7      /* no usable sm_103a device */
};

/* precision of the H/S contractions */
enum {
    HSDLA_PREC_FP64 = 0,       /* plain FP64 (DMMA) */
    HSDLA_PREC_OZAKI_FP8 = 1   /* Ozaki split: e4m3 integer digits on tcgen05, FP64 recombination */
};

/* One FLAPW cell: what the reference's AtomData holds (flapw_opt/src/include/AtomData.h:16-41),
 * stored per type with an atom->type map instead of per-atom replication
 * (FleurData.cpp:52-62 replicates per atom). */
typedef struct hsdla_system {
    int32_t num_atoms;
    int32_t num_types;
    int32_t max_lmax;            /* L = (max_lmax+1)^2 */
    int32_t reserved0;
    double vol_cell;             /* det(real basis), bohr^3 */
    double bmat[9];              /* row-major, rows = reciprocal vectors */
    const int32_t *atom_type;    /* [num_atoms], 0-based */
    const double *atom_pos;      /* [num_atoms][3] fractional */
    const double *atom_rotmat;   /* [num_atoms][9] row-major (mrot * bmat), or NULL: mrot = 1 */
    const double *type_rmt;      /* [num_types] muffin-tin radius */
    const int32_t *type_lmax;    /* [num_types] spherical cutoff, 1 <= lmax <= max_lmax */
    const double *type_u;        /* [num_types][max_lmax+1] u_l(R)      */
    const double *type_u_dr;     /* [num_types][max_lmax+1] u_l'(R)     */
    const double *type_dE_u;     /* [num_types][max_lmax+1] udot_l(R)   */
    const double *type_dE_u_dr;  /* [num_types][max_lmax+1] udot_l'(R)  */
    const double *type_dE_u_norm;/* [num_types][max_lmax+1] ||udot_l||^2 */
    const hsdla_cx *type_t_aa;   /* [num_types][L*L] augmented T_AA, column-major, Hermitian */
    const hsdla_cx *type_t_ab;   /* [num_types][L*L] augmented T_AB, column-major (T_BA = T_AB^H) */
    const hsdla_cx *type_t_bb;   /* [num_types][L*L] augmented T_BB, column-major, Hermitian */
} hsdla_system;

/* One k-point and its basis (the k_mesh of types.h:14-21; G list from the caller). */
typedef struct hsdla_kpoint {
    double k[3];                 /* fractional */
    int64_t n_g;                 /* number of G vectors (>= 1) */
    const int32_t *g;            /* [n_g][3] integer G vectors */
} hsdla_kpoint;

typedef struct hsdla_opts {
    int32_t precision;           /* HSDLA_PREC_* */
    int32_t num_slices;          /* Ozaki digit slices; 0 = autotune to the accuracy target */
    double target_rel_err;       /* Ozaki accuracy target (default 1e-13 when 0) */
    int32_t use_graph;           /* 1 = capture the whole multi-k-point pipeline in a CUDA graph */
    int32_t reserved[7];
} hsdla_opts;

typedef struct hsdla_report {
    double ms_total;             /* device time of the whole call (CUDA events) */
    double ms_per_kpoint;
    double flop;                 /* canonical 20 G^2 La + 24 L^2 a G, summed over k-points */
    double eff_tflops;           /* flop / ms_total */
    double ms_construct_ab;      /* stage times of the last un-graphed run (0 under a graph): kernel (a), */
    double ms_tapply;            /* the T-application launches (X = T C, or Z_t = T_t M_t per type), */
    double ms_contract;          /* and the rest (slicing, S/H products, combine) */
    double ms_dominant;          /* device time of the dominant launch: the S/H contraction of the last k-point */
    double dominant_flop;        /* algorithmic flops of that launch (FP8 digit products for Ozaki, FP64 for plain) */
    double est_rel_err;          /* Ozaki: relative error predicted by the slice autotuner (0 if not tuned) */
    int32_t num_slices;          /* slices used (Ozaki) */
    int32_t num_kpoints;
    int32_t kernel_launches;     /* kernels launched per execution */
    int32_t num_panels;          /* Ozaki: atom panels the contraction was streamed in (1 = resident) */
    int32_t outputs_in_place;    /* hsdla_create_hs: 1 = the GPU wrote the page-locked host H, S itself */
    int32_t num_row_sets;        /* structure-factor form: the row sets contracted (types, or (type, rotation)
                                    classes when atoms carry rotations); 0 = the per-atom form */
    int32_t rotation_classes;    /* 1: the row sets are (type, rotation) classes */
    int32_t tile_halves;         /* Ozaki, structure-factor form: S/H tiles as 256 x 256 accumulators (1) or */
                                 /* two 256 x 128 halves in alternating TMEM buffers (2); 0 otherwise */
    int32_t merged_units;        /* the same launches: 1 = adjacent digit diagonals share exact accumulation units */
    int32_t tile_tuned;          /* 1 = those two were chosen by timing on this plan's data (or a cached result) */
    int32_t output_blocks;       /* hsdla_create_hs, outputs written in place: the column blocks they were written
                                    in while the digit products of the next block ran (0 = after all products) */
    int32_t reserved[1];
    double ms_host_setup;        /* hsdla_create_hs: host time from the call's start to its first launch (plan
                                    creation and set-up; the device is idle meanwhile, and ms_total counts it) */
} hsdla_report;

typedef struct hsdla_context hsdla_context;
typedef struct hsdla_plan hsdla_plan;

/* Library / device set-up (replaces dev_init/dev_finalize, flapw_opt/src/wrappers.cpp:111-148). */
int hsdla_context_create(int device, hsdla_context **ctx);
/* Destroys the context and every plan still alive in it (plan handles become invalid). */
void hsdla_context_destroy(hsdla_context *ctx);
/* The context's last error message.  With ctx = NULL: the calling thread's last message of the
 * entry point that takes no context, hsdla_zherkx_lower_noalloc ("" after a call that succeeded). */
const char *hsdla_last_error(const hsdla_context *ctx);
/* Cap on device bytes the context may allocate (0 = no cap); exceeding it returns HSDLA_ERR_NOMEM. */
int hsdla_set_mem_cap(hsdla_context *ctx, int64_t bytes);

/* T-matrix preparation for one type: TMat::TMat + zero_nonsph + augment_tmats
 * (flapw_opt/src/types_helper.cpp:41-90, flapw_opt/src/AtomData.cpp:95-145).
 * taa, tbb, tab, tba: n x n column-major with n = (lmax+1)^2, only lower triangles
 * read (Fleur's dump convention).  Outputs: n x n column-major augmented aa, ab, bb.
 * Host-only, once per run. */
int hsdla_prepare_tmat(int32_t lmax, int32_t lmax_nonsph, const hsdla_cx *taa, const hsdla_cx *tbb,
                       const hsdla_cx *tab, const hsdla_cx *tba, const double *E_l,
                       const double *dE_u_norm, hsdla_cx *aa, hsdla_cx *ab, hsdla_cx *bb);

/* H and S for nk k-points, HOST buffers in and out (the create_HS2 drop-in; nk = 1 is
 * exactly create_HS2's contract, h_and_s.cpp:591-893).  H[i], S[i]: n_g(i) x n_g(i)
 * column-major host arrays with leading dimension ld[i] >= n_g(i).  The T blocks' check
 * (finite, Hermitian) is read after the launches: a call that returns HSDLA_ERR_INPUT for
 * it may have written H and S. */
int hsdla_create_hs(hsdla_context *ctx, const hsdla_system *sys, const hsdla_kpoint *kpts, int32_t nk,
                    hsdla_cx *const *H, hsdla_cx *const *S, const int64_t *ld,
                    const hsdla_opts *opts, hsdla_report *report);

/* Contraction-only drop-in for create_HS2_stripped_v2(L, a, G, A, B, H, S, T, l_maxs, max_lmax,
 * u_norms, method, W) (flapw_opt/src/h_and_s_stripped_v2.cpp:100-382,
 * flapw_opt/src/include/acc/h_and_s_stripped.h:24): H and S from caller-built matching tensors.
 * A, B: HOST L x a x G complex (column-major cube, element (lm, atom, g) at lm + L atom + L a g),
 * L = (max_lmax+1)^2.  Per atom j: t_sizes[3j..3j+2] = (aa_size, ab_size, bb_size) and the
 * column-major blocks t_aa[j], t_ab[j], t_bb[j] (the reference's myTMat; T_AA/T_BB through their
 * lower triangles, smaller blocks act zero-padded).  lmaxs[a], sqrt_u_norms[a][max_lmax+1] =
 * sqrt(||udot_l||^2) as the reference packs them (h_and_s.cpp:700-715).  H, S: HOST G x G,
 * leading dimension ld; lower triangles written (upper triangles: see the conventions above).  With Ozaki
 * precision, num_slices = 0 selects the default slice count (no sampling autotune here). */
int hsdla_contract_ab(hsdla_context *ctx, int32_t L, int32_t num_atoms, int64_t n_g, const hsdla_cx *A,
                      const hsdla_cx *B, const int32_t *t_sizes, const hsdla_cx *const *t_aa,
                      const hsdla_cx *const *t_ab, const hsdla_cx *const *t_bb, const int32_t *lmaxs,
                      int32_t max_lmax, const double *sqrt_u_norms, hsdla_cx *H, hsdla_cx *S, int64_t ld,
                      const hsdla_opts *opts, hsdla_report *report);

/* Device-resident execution: a plan uploads the system and the k-point lists once and owns
 * the device workspace (A/B tensors, T blocks, digit slices). */
int hsdla_plan_create(hsdla_context *ctx, const hsdla_system *sys, const hsdla_kpoint *kpts, int32_t nk,
                      const hsdla_opts *opts, hsdla_plan **plan);
/* dH[i], dS[i]: DEVICE pointers; stream: a cudaStream_t (NULL = the default stream, as in CUDA).
 * The call returns after the work on that stream has completed. */
int hsdla_plan_execute(hsdla_plan *plan, hsdla_cx *const *dH, hsdla_cx *const *dS, const int64_t *ld,
                       void *stream, hsdla_report *report);
int64_t hsdla_plan_workspace_bytes(const hsdla_plan *plan);
void hsdla_plan_destroy(hsdla_plan *plan);

/* ---- component entry points (parity tests; the fused pipeline does not call these) ---- */

/* Kernel (a): matching tensors for k-point ik of a plan into a DEVICE buffer C of
 * (2 L a) x n_g complex, column-major, rows ordered per atom as [A_a (L rows); B_a (L rows)]
 * (the reference's A(lm, a, g) is C[2 L a + lm, g], B(lm, a, g) is C[2 L a + L + lm, g]). */
int hsdla_plan_construct_ab(hsdla_plan *plan, int32_t ik, hsdla_cx *dC, void *stream);

/* Kernel (c) standalone: lower triangle of OUT = P^H diag(w) Q for K x n column-major device
 * matrices (the dev_zherk_/dev_zherkx_ plugin of flapw_opt/src/include/acc/wrappers.h:19-28
 * with uplo 'L', trans 'C', alpha 1, beta 0).  w may be NULL (all ones).  Q == P gives zherk. */
int hsdla_zherkx_lower(hsdla_context *ctx, int32_t precision, int32_t num_slices, int64_t n, int64_t k,
                       const hsdla_cx *dP, int64_t ldp, const hsdla_cx *dQ, int64_t ldq,
                       const double *dw, hsdla_cx *dOut, int64_t ldo, void *stream);

/* ---- BLAS-shaped contraction plugin: the reference's backend dev_zherk_, dev_zher2k_, dev_zherkx_
 * (flapw_opt/src/include/acc/wrappers.h:19-28, flapw_opt/src/wrappers.cpp:171-257), which
 * create_HS2_stripped_v2 calls for S = A^H A, S += W^H W, H = B^H X + X^H B and H += A^H X'
 * (flapw_opt/src/h_and_s_stripped_v2.cpp:158, 177, 300, 362).  Fortran BLAS / cuBLAS semantics,
 * column-major, on the uplo triangle of C only (the other triangle is not touched):
 *   zherk : C = alpha op(A) op(A)^H + beta C                         (alpha, beta real)
 *   zher2k: C = alpha op(A) op(B)^H + conj(alpha) op(B) op(A)^H + beta C   (beta real)
 *   zherkx: C = alpha op(A) op(B)^H + beta C, the product taken as Hermitian (cuBLAS's herkx; MKL's
 *           zgemmt in the reference's CPU build)                     (beta real)
 * op(X) = X for trans 'N' (X n x k, ld >= n), X^H for trans 'C' (X k x n, ld >= k); uplo 'L' or 'U'
 * (either case).  zherk and zher2k leave a real diagonal (its imaginary part set to zero, as BLAS
 * does); beta = 0 never reads C.  A, B, C may be device or host memory (host matrices are staged
 * through device memory, as the reference's cuBLASXt backend does with its page-locked buffers).
 * precision: HSDLA_PREC_FP64 (DMMA) or HSDLA_PREC_OZAKI_FP8 with num_slices (0 = 11) digit slices.
 * Asynchronous work runs on `stream` (NULL = the legacy default stream); the call returns after it
 * completed. */
int hsdla_zherk(hsdla_context *ctx, int32_t precision, int32_t num_slices, char uplo, char trans, int64_t n, int64_t k,
                double alpha, const hsdla_cx *A, int64_t lda, double beta, hsdla_cx *C, int64_t ldc, void *stream);
int hsdla_zher2k(hsdla_context *ctx, int32_t precision, int32_t num_slices, char uplo, char trans, int64_t n,
                 int64_t k, hsdla_cx alpha, const hsdla_cx *A, int64_t lda, const hsdla_cx *B, int64_t ldb, double beta,
                 hsdla_cx *C, int64_t ldc, void *stream);
int hsdla_zherkx(hsdla_context *ctx, int32_t precision, int32_t num_slices, char uplo, char trans, int64_t n,
                 int64_t k, hsdla_cx alpha, const hsdla_cx *A, int64_t lda, const hsdla_cx *B, int64_t ldb, double beta,
                 hsdla_cx *C, int64_t ldc, void *stream);

/* The same three with the reference's own argument lists (Fortran style: every argument by pointer,
 * void return), for a wrappers.cpp whose dev_zherk_ / dev_zher2k_ / dev_zherkx_ forward to them
 * one to one, and hsdla_dev_init / hsdla_dev_finalize in place of dev_init / dev_finalize
 * (flapw_opt/src/wrappers.cpp:111-169).  They run on a context the library owns (created by
 * hsdla_dev_init, or on first use on device HSDLA_DEVICE, default 0, in FP64), one call at a time,
 * and return after the result is in C.  hsdla_dev_status() is the status of the calling thread's
 * last hsdla_dev_* call; its message is hsdla_last_error(hsdla_dev_context()). */
int hsdla_dev_init(int32_t device, int32_t precision, int32_t num_slices);
int hsdla_dev_finalize(void);
const hsdla_context *hsdla_dev_context(void);
int hsdla_dev_status(void);
void hsdla_dev_zherk_(const char *uplo, const char *trans, const int *n, const int *k, const double *alpha,
                      const hsdla_cx *A, const int *lda, const double *beta, hsdla_cx *C, const int *ldc);
void hsdla_dev_zher2k_(const char *uplo, const char *trans, const int *n, const int *k, const hsdla_cx *alpha,
                       const hsdla_cx *A, const int *lda, const hsdla_cx *B, const int *ldb, const double *beta,
                       hsdla_cx *C, const int *ldc);
void hsdla_dev_zherkx_(const char *uplo, const char *trans, const int *n, const int *k, const hsdla_cx *alpha,
                       const hsdla_cx *A, const int *lda, const hsdla_cx *B, const int *ldb, const double *beta,
                       hsdla_cx *C, const int *ldc);

/* Matching values of one (type, l): Fleur's scalar-relativistic radial solution u_l and its energy
 * derivative udot_l at energy e for the potential r V(r) on Fleur's logarithmic mesh of n points
 * (r_i = R_MT e^{(i - n) dx}, i = 1..n), evaluated at R_MT: out = {u(R), u'(R), udot(R),
 * udot'(R), ||udot||^2}.  The quantities hsdla_system's type_u .. type_dE_u_norm hold; the
 * reference computes them in AtomData::generate_matchdata (flapw_opt/src/AtomData.cpp:72-88)
 * through radial_solve (flapw_opt/src/special_funcs.cpp:21-36) and Fleur's radfun
 * (external/compat/fleur/radfun.f, radsra.f, radsrd.F, intgr.F).  Host only, once per run;
 * n >= 7, 0 <= l <= 14. */
int hsdla_radial_match(int32_t l, double e, const double *vr, int32_t n, double rmt, double dx, double *out);

/* Hand-off to an eigensolver in Fleur's packed form: the lower triangle of the column-major
 * n x n DEVICE matrix M (leading dimension ld >= n, e.g. H or S from hsdla_plan_execute) written
 * row by row into the DEVICE array packed of n (n + 1) / 2 elements, element (r, c), c <= r, at
 * r (r + 1) / 2 + c.  That is the layout of the H and S Fleur writes per k-point
 * (fleur/src/binmat.f90:194-219) and the one the reference's checker unpacks
 * (flapw_opt/tests/flapw_verify.py:68-82).  Asynchronous on `stream` (NULL: the legacy default
 * stream); M and packed must not overlap. */
int hsdla_pack_lower(hsdla_context *ctx, int64_t n, const hsdla_cx *M, int64_t ld, hsdla_cx *packed, void *stream);

/* Failure-detection self-test (no counterpart in the reference): runs a small kernel that holds
 * TMEM like the contraction kernels and lets one of their bounded waits expire on a condition
 * that never comes true -- which = 0: an mbarrier nothing arrives on; which = 1: a grid-lockstep
 * slot that never advances -- after budget_cycles (1 .. 2e9 SM cycles).  The kernel records the
 * error word, frees TMEM and returns; the call returns HSDLA_ERR_TIMEOUT with the expired wait in
 * hsdla_last_error, and the context stays usable.  Nothing faults, traps or hangs. */
int hsdla_selftest_wait_timeout(hsdla_context *ctx, int32_t which, int64_t budget_cycles);

/* Allocation-free Ozaki form of hsdla_zherkx_lower (HSDLA_PREC_OZAKI_FP8), for callers that
 * cannot allocate device memory: code inside another framework's memory pool or under a
 * fixed memory budget, plug-ins that may only touch the buffers they are handed, processes
 * that must not call cudaMalloc after start-up.  It has no counterpart in the reference.
 *
 * All scratch (digit planes, exponents, job table, error word) lives in one static device
 * array of 128 MiB that every GPU loading this library holds until the process exits; the
 * call makes no cudaMalloc/cudaFree and no allocating library call.  Problems that need more
 * scratch than that, 2 * (2 s (roundup(n,128) + 128) (roundup(k,128) + 128) + 4 (roundup(n,128) + 128))
 * bytes plus 2 KiB (about n = 1000, k = 2432 at s = 11), are rejected with
 * HSDLA_ERR_UNSUPPORTED.  num_slices = 0 means 11.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current; make that first
 * call before any stream capture.  Every call shares the one array, so calls that overlap on
 * the GPU (other streams, other host threads) race: serialise them.  The call returns after
 * the work on `stream` (NULL = default stream) has completed.  Its error messages are read with
 * hsdla_last_error(NULL) on the calling thread. */
int hsdla_zherkx_lower_noalloc(int32_t num_slices, int64_t n, int64_t k, const hsdla_cx *dP, int64_t ldp,
                               const hsdla_cx *dQ, int64_t ldq, const double *dw, hsdla_cx *dOut,
                               int64_t ldo, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* HSDLA_H */
