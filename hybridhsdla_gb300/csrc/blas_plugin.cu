// Kernels of the BLAS-shaped contraction plugin: the reference's contraction backend
// dev_zherk_ / dev_zher2k_ / dev_zherkx_ (flapw_opt/src/include/acc/wrappers.h:19-28, defined at
// flapw_opt/src/wrappers.cpp:171-257) with every flag of their Fortran BLAS / cuBLAS signatures:
// uplo 'L' / 'U', trans 'N' / 'C', a scalar alpha and a real beta (beta = 1 accumulates, as
// create_HS2_stripped_v2 does for S += W^H W and H += A^H X', h_and_s_stripped_v2.cpp:177, 362).
//
// The products themselves run in the library's lower-triangle contraction OUT = P^H Q (FP64 DMMA
// or the Ozaki FP8 form), on operands in the 'C' layout (K x n, column-major).  These kernels
//   * build such an operand from the caller's matrix: a scaled copy for trans 'C', a conjugate
//     transpose (32 x 32 shared-memory tiles, coalesced on both sides) for trans 'N';
//   * apply the epilogue to the caller's C: on its uplo triangle, C = a T(R) + beta C with
//     T(R)[i, j] = R[i, j] (uplo 'L') or conj(R[j, i]) (uplo 'U', R computed from the swapped
//     operands, so that R[j, i] = (Q^H P)[j, i] = conj((P^H Q)[i, j])); for zherk and zher2k the
//     diagonal is real, as BLAS defines them: its imaginary part is set to zero and the input
//     diagonal's imaginary part is ignored.  beta = 0 never reads C (NaNs in C do not propagate).
#include <algorithm>

#include "common.cuh"

namespace hsdla {
namespace {

constexpr int kTr = 32;         // tile edge of the transposing kernels
constexpr int kTrRows = 8;      // thread rows of a tile (each thread handles kTr / kTrRows elements)

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// dst[r0 + r, c] (ld ldd) = s * src[r, c] for r < k, c < n (src k x n, ld lds)
__global__ void __launch_bounds__(256) operand_copy_kernel(const double2 *__restrict__ src, int64_t lds, int64_t k,
                                                           int64_t n, double2 s, double2 *__restrict__ dst,
                                                           int64_t ldd, int64_t r0) {
    const int64_t c = blockIdx.y;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < k; r += (int64_t)gridDim.x * blockDim.x)
        dst[r0 + r + ldd * c] = cmul(s, src[r + lds * c]);
}

// dst[r0 + r, c] (ld ldd) = s * conj(src[c, r]) for r < k, c < n (src n x k, ld lds)
__global__ void __launch_bounds__(kTr *kTrRows) operand_transpose_kernel(const double2 *__restrict__ src, int64_t lds,
                                                                         int64_t k, int64_t n, double2 s,
                                                                         double2 *__restrict__ dst, int64_t ldd,
                                                                         int64_t r0) {
    __shared__ double2 tile[kTr][kTr + 1];
    const int64_t cb = (int64_t)blockIdx.x * kTr, rb = (int64_t)blockIdx.y * kTr;
    // read: consecutive threads along c (src's contiguous index)
    for (int y = threadIdx.y; y < kTr; y += kTrRows) {
        const int64_t c = cb + threadIdx.x, r = rb + y;
        if (c < n && r < k) {
            const double2 v = src[c + lds * r];
            tile[y][threadIdx.x] = make_double2(v.x, -v.y);
        }
    }
    __syncthreads();
    // write: consecutive threads along r (dst's contiguous index)
    for (int y = threadIdx.y; y < kTr; y += kTrRows) {
        const int64_t r = rb + threadIdx.x, c = cb + y;
        if (c < n && r < k) dst[r0 + r + ldd * c] = cmul(s, tile[threadIdx.x][y]);
    }
}

// The epilogue on one 32 x 32 tile of C's uplo triangle (tiles below / above the diagonal only).
__global__ void __launch_bounds__(kTr *kTrRows) plugin_epilogue_kernel(const double2 *__restrict__ R, int64_t ldr,
                                                                       double2 *__restrict__ C, int64_t ldc, int64_t n,
                                                                       double2 a, double beta, int upper, int herm) {
    __shared__ double2 tile[kTr][kTr + 1];
    // tile (bi, bj) of the triangle: blockIdx.x enumerates the lower-triangle tiles row by row
    const int64_t x = blockIdx.x;
    int64_t ti = (int64_t)((sqrt(8.0 * (double)x + 1.0) - 1.0) * 0.5);
    while (ti * (ti + 1) / 2 > x) --ti;
    while ((ti + 1) * (ti + 2) / 2 <= x) ++ti;
    const int64_t tj = x - ti * (ti + 1) / 2;            // tj <= ti
    // C's tile: rows bi, columns bj (lower: bi = ti >= bj = tj; upper: the mirror)
    const int64_t bi = upper ? tj : ti, bj = upper ? ti : tj;
    if (upper && R) {
        // T(R)[i, j] = conj(R[j, i]): stage R's tile (rows bj, columns bi) transposed
        for (int y = threadIdx.y; y < kTr; y += kTrRows) {
            const int64_t rr = bj * kTr + threadIdx.x, rc = bi * kTr + y;   // R[rr, rc], rr >= rc where used
            if (rr < n && rc < n) tile[y][threadIdx.x] = R[rr + ldr * rc];
        }
        __syncthreads();
    }
    for (int y = threadIdx.y; y < kTr; y += kTrRows) {
        const int64_t i = bi * kTr + threadIdx.x, j = bj * kTr + y;
        if (i >= n || j >= n || (upper ? i > j : i < j)) continue;
        double2 t = make_double2(0.0, 0.0);
        if (R) {
            if (upper) {
                const double2 v = tile[threadIdx.x][y];
                t = make_double2(v.x, -v.y);
            } else {
                t = R[i + ldr * j];
            }
            t = cmul(a, t);
        }
        double2 *c = C + i + ldc * j;
        double2 o = t;
        if (beta != 0.0) {
            const double2 cv = *c;
            o.x += beta * cv.x;
            o.y += beta * cv.y;
        }
        if (herm && i == j) {
            // the diagonal of a Hermitian result is real: C_jj = a Re(R_jj) + beta Re(C_jj)
            o.y = 0.0;
        }
        *c = o;
    }
}

}  // namespace

cudaError_t launch_plugin_operand(const double2 *src, int64_t lds, bool transpose, int64_t k, int64_t n, double2 s,
                                  double2 *dst, int64_t ldd, int64_t r0, cudaStream_t st) {
    if (k <= 0 || n <= 0) return cudaSuccess;
    if (!transpose) {
        if (n > 65535) {
            // one grid row per column is at most 65535 columns: split the columns
            for (int64_t c0 = 0; c0 < n; c0 += 65535) {
                const int64_t nc = std::min<int64_t>(65535, n - c0);
                const dim3 grid((unsigned)std::min<int64_t>((k + 255) / 256, 64), (unsigned)nc);
                operand_copy_kernel<<<grid, 256, 0, st>>>(src + lds * c0, lds, k, nc, s, dst + ldd * c0, ldd, r0);
            }
        } else {
            const dim3 grid((unsigned)std::min<int64_t>((k + 255) / 256, 64), (unsigned)n);
            operand_copy_kernel<<<grid, 256, 0, st>>>(src, lds, k, n, s, dst, ldd, r0);
        }
        return cudaGetLastError();
    }
    const int64_t gy = (k + kTr - 1) / kTr;
    for (int64_t y0 = 0; y0 < gy; y0 += 65535) {
        // rows [y0 kTr, ...) of dst come from columns y0 kTr, ... of src
        const int64_t rows = std::min<int64_t>(k - y0 * kTr, (int64_t)65535 * kTr);
        const dim3 grid((unsigned)((n + kTr - 1) / kTr), (unsigned)((rows + kTr - 1) / kTr));
        operand_transpose_kernel<<<grid, dim3(kTr, kTrRows), 0, st>>>(src + lds * y0 * kTr, lds, rows, n, s, dst, ldd,
                                                                      r0 + y0 * kTr);
    }
    return cudaGetLastError();
}

cudaError_t launch_plugin_epilogue(const double2 *R, int64_t ldr, double2 *C, int64_t ldc, int64_t n, double2 a,
                                   double beta, bool upper, bool herm, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int64_t T = (n + kTr - 1) / kTr;
    const int64_t tiles = T * (T + 1) / 2;
    if (tiles > INT32_MAX) return cudaErrorInvalidValue;
    plugin_epilogue_kernel<<<(unsigned)tiles, dim3(kTr, kTrRows), 0, st>>>(R, ldr, C, ldc, n, a, beta, upper ? 1 : 0,
                                                                          herm ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace hsdla
