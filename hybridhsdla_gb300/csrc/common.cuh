// Shared definitions of the sm_103a H/S generation library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/hsdla.h"

namespace hsdla {

constexpr int kMaxLmax = 14;                 // (14+1)^2 = 225 lm per atom
constexpr int kMaxL = (kMaxLmax + 1) * (kMaxLmax + 1);
constexpr int kMaxTypes = 64;
constexpr double kPi = 3.14159265358979323846;

// Device error word: kernels with bounded waits write a code here instead of trapping.
enum DeviceError : int {
    kDevOk = 0,
    kDevTimeout = 1,
    kDevBadInput = 2,
};

// ------------------------------------------------------------------ system
// Device-resident per-run data (uploaded once per plan).
struct DevSystem {
    int num_atoms, num_types, max_lmax, L;
    double vol_prefac;          // 4 pi / sqrt(Omega)
    double bmat[9];             // row-major rows b_i
    const int32_t *atom_type;   // [a]
    const double *atom_pos;     // [a][3]
    const double *atom_rotmat;  // [a][9] or nullptr
    const double *type_rmt;     // [t]
    const int32_t *type_lmax;   // [t]
    // per (type, l), index t*(max_lmax+1)+l
    const double *u, *u_dr, *dE_u, *dE_u_dr;
    const double *inv_w;        // 1 / (udot u' - u udot')
    const double *ynorm;        // [L] Y_lm normalisation (ylm4.f:111-137)
    // Per-type rows of (type, rotation) classes: the types are the classes, type t's atoms share
    // the rotation rots[9 type_rot[t] ..] (row-major mrot bmat).  num_rots = 0: every type's rows
    // use R = bmat (no atom carries its own rotation).
    int num_rots;
    const double *rots;         // [num_rots][9]
    const int32_t *type_rot;    // [t]
};

// Shared memory of the per-type rows kernel (construct_rows_kernel) for L lm, lmax max_lmax and
// nt types; the kernel runs only where it fits (160 KB).
inline size_t rows_kernel_smem(int L, int max_lmax, int nt) {
    const int kRowCols = 16, nl = max_lmax + 1, tnl = nt * nl;
    size_t b = sizeof(double) * 2 * kRowCols * L + sizeof(double) * (2 * kRowCols * tnl + tnl + 4 * kRowCols) + L + 16;
    return (b + 15) & ~size_t(15);
}
constexpr size_t kRowsKernelSmemMax = 160 * 1024;

struct DevKpoint {
    double k[3];
    int64_t n_g;
    const int32_t *g;           // [n_g][3]
};

// A group of k-points handled by one launch per stage (passed by value as a kernel parameter).
constexpr int kMaxGroup = 64;
struct KEntry {
    DevKpoint kp;
    double2 *C;                 // (2 L a) x n_g, ld KTable::ldc
    double2 *M;                 // (2 L nt) x n_g, ld KTable::ldm, or nullptr
    const double2 *Z;           // per-type product, ld KTable::ldm (phase expansion input)
    double2 *X;                 // per-atom output, ld KTable::ldc (phase expansion output)
    int64_t col_begin;          // first global column of this k-point
};
struct KTable {
    int nk = 0;
    int a0 = 0, a1 = -1;        // atom range of the phase expansion (a1 < 0: every atom)
    int64_t ldc = 0, ldm = 0;
    int64_t total_cols = 0;
    KEntry e[kMaxGroup];
};

// ----------------------------------------------------------- kernels (host)
// (a) for every k-point of a table in one launch (C always; M when the entries give it)
cudaError_t launch_construct_ab_multi(const DevSystem &sys, const KTable &tab, cudaStream_t st);
// X = phase Z for every k-point of a table in one launch
cudaError_t launch_apply_phase_multi(const DevSystem &sys, const KTable &tab, cudaStream_t st);
// (a) matching tensors of one k-point into C: (2 L a) x n_g column-major, per-atom [A_a; B_a]
// Optionally also the phase-free per-type rows M ((2 L nt) x n_g, ld ldm) when no atom carries
// its own rotation (M_t = C_a e^{-i 2pi K.tau_a} for every atom a of type t).
cudaError_t launch_construct_ab(const DevSystem &sys, const DevKpoint &kp, double2 *C, int64_t ldc,
                                cudaStream_t st, double2 *M = nullptr, int64_t ldm = 0);
// The Hermitian 2L x 2L blocks [[T_AA, T_AB], [T_AB^H, T_BB]] of every type (column-major, ld 2L,
// 4 L^2 apart) into tf, from the caller's lower triangles of T_AA and T_BB and all of T_AB (each
// nt x L x L, column-major per type), with the input checks per type in stats[5 t .. 5 t + 4]
// (zeroed by the caller): bit q of [0] set when block q (0 AA, 1 AB, 2 BB) holds a non-finite
// value; [1], [2] = max |T|^2 and max |T - T^H|^2 over T_AA's lower triangle, [3], [4] the same
// for T_BB (doubles as bit patterns).
cudaError_t launch_tfull(const double2 *aa, const double2 *ab, const double2 *bb, int nt, int L, double2 *tf,
                         unsigned long long *stats, cudaStream_t st);
// Per-atom structure phases along each axis, ph[o] = e^{i 2pi (i - half_c) pos[3 j + c]} with o
// running over c, then atom j, then i in [0, ext_c).
cudaError_t launch_sf_phases(const double *pos, int na, const int *half, const int *ext, double2 *ph, cudaStream_t st);
// X[2L a + r, g] = e^{i 2pi (k+g).tau_a} Z[2L t(a) + r, g]
cudaError_t launch_apply_phase(const DevSystem &sys, const DevKpoint &kp, const double2 *Z, int64_t ldz,
                               double2 *X, int64_t ldx, cudaStream_t st);

// FP64 tiled contraction OUT = P^H diag(w) Q over a batch of jobs (kernels (b) and (c) in FP64).
struct Fp64Job {
    const double2 *P; int64_t ldp;   // k x m
    const double2 *Q; int64_t ldq;   // k x n
    const double *w;                 // k weights or nullptr
    double2 *out; int64_t ldo;       // m x n
    int64_t m, n, k;
    int32_t lower;                   // 1: only elements with row >= col (m == n required)
    int32_t tiles_n;                 // tile columns of this job
    int64_t tile_begin;              // first global tile index of this job
};
constexpr int kFp64Tile = 64;
int64_t fp64_job_tiles(const Fp64Job &j);
cudaError_t launch_fp64_jobs(const Fp64Job *d_jobs, int num_jobs, int64_t total_tiles, cudaStream_t st);

// ---- structure-factor form (atoms sharing their type's rotation)
// One k-point of a combine: per-type products PS, PH (lower triangles, ld ldp) into the outputs
// S, H (ld ldo); g the k-point's G-vectors [n][3] on the device.
struct SfEntry {
    const double2 *PS = nullptr, *PH = nullptr;   // per-type products, type slot b at + b pstride
    double2 *S = nullptr, *H = nullptr;
    // what a combine that is not the first adds to (NULL: S and H themselves, ldo)
    const double2 *Si = nullptr, *Hi = nullptr;
    int64_t ldp = 0, ldo = 0, n = 0, pstride = 0, ldi = 0;
    const int32_t *g = nullptr;
    int64_t tile_begin = 0;
    // where rows < SfTab::xrow1 go instead of S and H (NULL: nowhere else), leading dimension ldx
    double2 *Sx = nullptr, *Hx = nullptr;
    int64_t ldx = 0;
};
struct SfTab {
    int nk = 0, type = 0, ntypes = 1;             // the batch: types [type, type + ntypes) in slots
    int slot0 = 0;                                // slot0, slot0 + 1, ...
    int64_t col0 = 0, col1 = INT64_MAX;           // the columns combined (of every entry)
    int64_t xrow1 = 0;                            // rows below it go to the entries' Sx, Hx when set

    int dx = 0, dy = 0, dz = 0, ny = 0, nz = 0;   // box offsets (half widths) and extents
    int64_t box = 0;                              // entries per type
    SfEntry e[kMaxGroup];
};
// SF_t(dG) = sum_{a of type t} e^{i 2pi dG.tau_a} over the box of G-vector differences, from
// per-atom factors ex[a][dGx + dx] = e^{i 2pi dGx tau_a,x} (and y, z); atoms listed by type.
cudaError_t launch_sf_table(const double2 *ex, const double2 *ey, const double2 *ez, const int32_t *order,
                            const int32_t *type_begin, int nt, int nx, int ny, int nz, double2 *sf, cudaStream_t st);
// S (+)= sum_b SF_{type+b} (.) PS_b and H (+)= sum_b SF_{type+b} (.) PH_b over the lower triangles
// of every entry, b over the batch's type slots, in columns [tab.col0, tab.col1) (multiples of 32
// but for the end); rows below tab.xrow1 into Sx, Hx instead for entries that give them.
cudaError_t launch_sf_combine(const SfTab &tab, const double2 *sf, bool first, cudaStream_t st);

// BLAS-shaped plugin (blas_plugin.cu).  Operand in the 'C' layout: dst rows [r0, r0 + k) of every
// column c < n (ld ldd) = s * src[r, c] (src k x n, transpose false) or s * conj(src[c, r]) (src
// n x k, transpose true).
cudaError_t launch_plugin_operand(const double2 *src, int64_t lds, bool transpose, int64_t k, int64_t n, double2 s,
                                  double2 *dst, int64_t ldd, int64_t r0, cudaStream_t st);
// On C's uplo triangle: C = a T(R) + beta C, T(R)[i, j] = R[i, j] (lower) or conj(R[j, i]) (upper),
// R's lower triangle read (R may be NULL: C = beta C); herm: real diagonal.
cudaError_t launch_plugin_epilogue(const double2 *R, int64_t ldr, double2 *C, int64_t ldc, int64_t n, double2 a,
                                   double beta, bool upper, bool herm, cudaStream_t st);

// Fleur's packed lower triangle (row by row) of a column-major n x n matrix (device buffers).
cudaError_t launch_pack_lower(const double2 *M, int64_t ld, int64_t n, double2 *P, cudaStream_t st);

}  // namespace hsdla
