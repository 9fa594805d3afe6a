// Hand-off of H and S to an eigensolver in Fleur's packed form.
//
// Fleur keeps a Hermitian matrix as its lower triangle packed row by row: element (r, c),
// c <= r, at index r (r + 1) / 2 + c, n (n + 1) / 2 elements in all.  That is the layout of
// the H and S arrays Fleur writes per k-point (fleur/src/binmat.f90:194-219, write_hdf_hs) and
// the one the reference's checker unpacks (flapw_opt/tests/flapw_verify.py:68-82,
// pack_to_full).  The library's H and S are column-major with their lower triangle defined, so
// the hand-off is a transpose of the lower triangle: an HBM-bound copy (16 B read and 16 B
// written per element of the triangle).
#include "common.cuh"

namespace hsdla {

namespace {

constexpr int kPackTile = 32;
constexpr int kPackRows = 8;        // threads per tile column: 32 x 8 threads move a 32 x 32 tile

// One CTA per 32 x 32 tile of the lower triangle of tiles.  Reads walk the columns (consecutive
// threads on consecutive rows), writes walk the packed rows (consecutive threads on consecutive
// columns); the shared tile is padded to 33 columns so both directions are conflict-free.
__global__ void __launch_bounds__(kPackTile * kPackRows) pack_lower_kernel(const double2 *__restrict__ M, int64_t ld,
                                                                           int64_t n, double2 *__restrict__ P) {
    __shared__ double2 tile[kPackTile][kPackTile + 1];
    const int64_t b = blockIdx.x;
    int64_t tr = (int64_t)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
    while (tr * (tr + 1) / 2 > b) --tr;
    while ((tr + 1) * (tr + 2) / 2 <= b) ++tr;
    const int64_t tc = b - tr * (tr + 1) / 2;
    const int64_t r0 = tr * kPackTile, c0 = tc * kPackTile;
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int k = 0; k < kPackTile; k += kPackRows) {
        const int64_t r = r0 + tx, c = c0 + ty + k;
        if (r < n && c < n && c <= r) tile[ty + k][tx] = M[r + ld * c];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kPackTile; k += kPackRows) {
        const int64_t r = r0 + ty + k, c = c0 + tx;
        if (r < n && c <= r) P[r * (r + 1) / 2 + c] = tile[tx][ty + k];
    }
}

}  // namespace

cudaError_t launch_pack_lower(const double2 *M, int64_t ld, int64_t n, double2 *P, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int64_t T = (n + kPackTile - 1) / kPackTile;
    const int64_t blocks = T * (T + 1) / 2;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    pack_lower_kernel<<<(unsigned)blocks, dim3(kPackTile, kPackRows), 0, st>>>(M, ld, n, P);
    return cudaGetLastError();
}

}  // namespace hsdla
