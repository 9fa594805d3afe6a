// FP64 tensor-core contraction OUT = P^H diag(w) Q (complex128), batched over jobs.
//
// This one kernel carries the plain-FP64 form of
//   * kernel (b), the per-atom T application X_a = T_a [A_a; B_a]
//     (h_and_s_stripped_v2.cpp:193-231 zhemm+zgemm and :321-349 zhemm): P is the
//     Hermitian 2L x 2L block [[T_AA, T_AB],[T_AB^H, T_BB]], so P^H = P;
//   * kernel (c), the lower-triangle Hermitian contractions
//     S = C^H diag(1, ||udot||^2) C  (the two zherk calls, :158/:177) and
//     H = C^H X                      (zher2k + zherkx, :300/:362)
//     with C = [A_a; B_a] stacked per atom.
//
// GB300 mapping: FP64 MMA (mma.sync m16n8k4 .f64) on 64x64 complex tiles, four
// warps of 32x32, complex products as four real MMAs
//   Re += Pr Qr + Pi Qi,   Im += Pr Qi - Pi Qr,
// a two-stage cp.async pipeline over K chunks of 16, and a flat tile list over
// all jobs (lower-triangle tiles only for the Hermitian outputs) so that every
// atom / k-point of a call goes out in one launch.
#include <algorithm>

#include "common.cuh"

namespace hsdla {
namespace {

constexpr int BM = kFp64Tile, BN = kFp64Tile, BK = 16;
constexpr int SROW = 66;                       // double2 per smem row (== 2 mod 8: conflict-free fragments)
constexpr int kStageElems = 2 * BK * SROW;     // P and Q tiles of one stage (double2)
constexpr int kThreads = 128;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int sz = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void dmma(double (&d)[4], double a0, double a1, double b0) {
    asm volatile(
        "mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};\n"
        : "+d"(d[0]), "+d"(d[1]), "+d"(d[2]), "+d"(d[3])
        : "d"(a0), "d"(a1), "d"(b0));
}

__device__ __forceinline__ void tile_of(const Fp64Job &j, int64_t x, int64_t &ti, int64_t &tj) {
    if (j.lower) {
        int64_t r = (int64_t)((sqrt(8.0 * (double)x + 1.0) - 1.0) * 0.5);
        while (r * (r + 1) / 2 > x) --r;
        while ((r + 1) * (r + 2) / 2 <= x) ++r;
        ti = r;
        tj = x - r * (r + 1) / 2;
    } else {
        ti = x / j.tiles_n;
        tj = x - ti * j.tiles_n;
    }
}

__global__ void __launch_bounds__(kThreads) fp64_jobs_kernel(const Fp64Job *__restrict__ jobs, int num_jobs,
                                                            int64_t total_tiles) {
    extern __shared__ __align__(16) double2 sm[];
    for (int64_t gt = blockIdx.x; gt < total_tiles; gt += gridDim.x) {
        // job lookup (jobs sorted by tile_begin)
        int lo = 0, hi = num_jobs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (jobs[mid].tile_begin <= gt) lo = mid; else hi = mid - 1;
        }
        const Fp64Job j = jobs[lo];
        int64_t ti, tj;
        tile_of(j, gt - j.tile_begin, ti, tj);
        const int64_t m0 = ti * BM, n0 = tj * BN;

        const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
        const int gid = lane >> 2, tig = lane & 3;
        const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;

        double re[2][4][4], im[2][4][4];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b)
#pragma unroll
                for (int c = 0; c < 4; ++c) { re[a][b][c] = 0.0; im[a][b][c] = 0.0; }

        const int64_t nk = (j.k + BK - 1) / BK;
        auto load_stage = [&](int stage, int64_t kc) {
            double2 *Ps = sm + stage * kStageElems;
            double2 *Qs = Ps + BK * SROW;
            const int64_t k0 = kc * BK;
#pragma unroll
            for (int it = 0; it < (BK * BM) / kThreads; ++it) {
                const int idx = tid + it * kThreads;
                const int kk = idx % BK, c = idx / BK;
                const int64_t gk = k0 + kk;
                const bool vp = gk < j.k && (m0 + c) < j.m;
                const double2 *srcp = vp ? j.P + gk + j.ldp * (m0 + c) : j.P;
                cp_async16(Ps + kk * SROW + c, srcp, vp);
                const bool vq = gk < j.k && (n0 + c) < j.n;
                const double2 *srcq = vq ? j.Q + gk + j.ldq * (n0 + c) : j.Q;
                cp_async16(Qs + kk * SROW + c, srcq, vq);
            }
            cp_async_commit();
        };

        __syncthreads();   // previous tile's readers are done with the stages
        load_stage(0, 0);
        for (int64_t kc = 0; kc < nk; ++kc) {
            const int stage = (int)(kc & 1);
            if (kc + 1 < nk) {
                load_stage(stage ^ 1, kc + 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncthreads();
            const double2 *Ps = sm + stage * kStageElems;
            const double2 *Qs = Ps + BK * SROW;
#pragma unroll
            for (int ks = 0; ks < BK / 4; ++ks) {
                const int kk = ks * 4 + tig;
                double wk = 1.0;
                if (j.w) {
                    const int64_t gk = kc * BK + kk;
                    wk = gk < j.k ? j.w[gk] : 0.0;
                }
                double ar[2][2], ai[2][2], nai[2][2];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const double2 v = Ps[kk * SROW + wm + mt * 16 + gid + 8 * h];
                        ar[mt][h] = v.x * wk;
                        ai[mt][h] = v.y * wk;
                        nai[mt][h] = -ai[mt][h];
                    }
                double br[4], bi[4];
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    const double2 v = Qs[kk * SROW + wn + nt * 8 + gid];
                    br[nt] = v.x;
                    bi[nt] = v.y;
                }
#pragma unroll
                for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                    for (int nt = 0; nt < 4; ++nt) {
                        dmma(re[mt][nt], ar[mt][0], ar[mt][1], br[nt]);
                        dmma(re[mt][nt], ai[mt][0], ai[mt][1], bi[nt]);
                        dmma(im[mt][nt], ar[mt][0], ar[mt][1], bi[nt]);
                        dmma(im[mt][nt], nai[mt][0], nai[mt][1], br[nt]);
                    }
            }
            __syncthreads();
        }
        // epilogue: masked store (lower triangle for Hermitian outputs)
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int64_t row = m0 + wm + mt * 16 + gid + ((c >= 2) ? 8 : 0);
                    const int64_t col = n0 + wn + nt * 8 + tig * 2 + (c & 1);
                    if (row < j.m && col < j.n && (!j.lower || row >= col))
                        j.out[row + j.ldo * col] = make_double2(re[mt][nt][c], im[mt][nt][c]);
                }
    }
}

}  // namespace

int64_t fp64_job_tiles(const Fp64Job &j) {
    const int64_t tm = (j.m + BM - 1) / BM, tn = (j.n + BN - 1) / BN;
    return j.lower ? tm * (tm + 1) / 2 : tm * tn;
}

cudaError_t launch_fp64_jobs(const Fp64Job *d_jobs, int num_jobs, int64_t total_tiles, cudaStream_t st) {
    if (total_tiles <= 0) return cudaSuccess;
    const size_t smem = sizeof(double2) * 2 * kStageElems;
    cudaError_t e = cudaFuncSetAttribute(fp64_jobs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, nsm = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fp64_jobs_kernel, kThreads, smem);
    const int64_t grid = std::min<int64_t>(total_tiles, (int64_t)nsm * std::max(per_sm, 1));
    fp64_jobs_kernel<<<(unsigned)grid, kThreads, smem, st>>>(d_jobs, num_jobs, total_tiles);
    return cudaGetLastError();
}

}  // namespace hsdla
