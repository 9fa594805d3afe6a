// Ozaki-split complex FP64 contractions on the FP8 tensor cores of sm_103a.
//
// Emulates the FP64 BLAS-3 work of create_HS2_stripped_v2
// (flapw_opt/src/h_and_s_stripped_v2.cpp:155-368: zherk, zher2k, zherkx and the
// per-atom zhemm/zgemm T application) with exact integer products on tcgen05:
//
//  * slicing (oz_slice_kernel): every column g of an operand Z (K x n) gets a
//    power-of-two exponent e_g with max_k |Re,Im Z_kg| < 2^e_g, and the scaled
//    column z = Z 2^-e_g is rounded to an integer X = rint(z 2^(5s-1)) that is
//    split into s balanced base-32 digits
//        z ~= sum_i d_i 2^(1-5i),  d_1 in [-16,16],  d_i in [-16,15]  (i >= 2).
//    Every digit is an integer of magnitude <= 16, exactly representable in
//    e4m3; one byte plane per (digit, re/im).  The digit extraction runs in
//    64-bit integer arithmetic (one FP64 multiply and one conversion per value):
//    GB300's FP64 pipe delivers ~1 TFLOP/s, its integer pipes far more.
//  * products (oz_gemm_kernel): for the output tile (rows g, cols g') and each
//    diagonal t = i + j of the digit-product triangle (t = 2..s+1), the FP32
//    TMEM accumulator sums, over the contraction index and all pairs (i, t-i),
//        Re += dr_i er_j + di_i ei_j,   Im += dr_i ei_j - di_i er_j
//    as kind::f8f6f4 MMAs (e4m3 x e4m3 -> f32).  Products are integers <= 256,
//    so a K chunk of at most 2^24 / (2 * 256 * pairs) complex terms keeps every
//    partial sum an exactly representable integer; chunks are drained into the
//    FP64 output tile with weight 2^(2-5t), and the last drain applies
//    2^(e_g + e_g').
//
// GB300 mapping: persistent CTAs (one per SM, 512 TMEM columns = two 128x(128
// re + 128 im) FP32 accumulators), warp-specialised: one TMA producer warp
// (SW128 K-major 128x128-byte boxes, 64 KB per stage, 3 stages), one MMA warp
// (single elected issuer, tcgen05.commit to release stages and publish
// accumulators), eight epilogue warps (tcgen05.ld 32x32b, FP64 recombination,
// coalesced read-modify-write of the L2-resident output tile).  Every mbarrier
// wait is bounded by a clock64 budget; on expiry the kernel records an error
// word, stops issuing work, waits (bounded) for its in-flight copies and MMAs,
// frees TMEM and returns.
#include <cuda.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <type_traits>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ozaki.cuh"

namespace hsdla {

// Message of the last failed Ozaki call, per host thread: contexts driven from different threads
// never see each other's messages (each context copies it into its own message at once).
static thread_local const char *g_oz_err = "";
const char *ozaki_last_error() { return g_oz_err; }

namespace {

// ------------------------------------------------------------------ constants
constexpr int kTileM = 128;          // output rows per tile (TMEM lanes)
constexpr int kTileN = 128;          // output complex columns per tile
constexpr int kKBlock = 128;         // contraction bytes (e4m3 values) per stage
constexpr int kStages = 3;
constexpr int kStageBytes = 4 * kTileM * kKBlock;   // Ar, Ai, Br, Bi boxes
constexpr int kThreads = 320;        // warp 0 TMA, warp 1 MMA, warps 2..9 epilogue
constexpr int kEpiWarps = 8;         // two per TMEM lane quadrant, each drains half the columns
constexpr long long kWaitCycles = 2000000000LL;    // ~1 s at 2 GHz
constexpr int kExactTerms = 1 << 24;                // FP32 exact-integer bound
constexpr int kSyncEvery = 64;                      // stages per lockstep epoch (cooperative launches)
constexpr int kRetired = 0x7F7F7F7F;                // progress value of a CTA that has no work left
constexpr int kErrWords = 8;                        // error word + diagnostics of the first expired wait
constexpr int kErrAlloc = 16;                       // error words + the wait self-test's progress slots

struct OzJob {
    int32_t lmap, rmap;        // tensor-map index (0..3) of the left / right digit operand
    int32_t lower;             // 1: only tiles and elements with row >= col
    int32_t accum;             // 1: the first unit of a tile adds to the output instead of storing
    int32_t ksteps_last;       // pair tiles: K steps of 32 bytes the last k-block holds (1-4; 0: 4)
    int32_t reserved0;
    int64_t lplane, rplane;    // rows per digit plane in each map
    int64_t lrow0, rrow0;      // first operand row (output row / col 0) inside a plane
    int64_t lk0, rk0;          // first contraction byte (multiple of 128)
    int64_t nkb;               // contraction blocks of 128
    int64_t m, n;              // valid output rows / cols
    int64_t tiles_n;           // tile columns (full mode)
    int64_t tile_begin;        // first global tile index
    double2 *out;
    int64_t ldo;
    const int32_t *el;         // exponent of each output row (job-relative)
    const int32_t *er;         // exponent of each output col (job-relative)
};

// ------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait.  Returns false (and raises the CTA abort flag) when the budget expires
// or another role already aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag, int *err,
                                          int where, long long budget = kWaitCycles) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > budget) {
            *abort_flag = 1;
            atomicCAS(err, 0, kDevTimeout * 16 + where);
            return false;
        }
    }
    return true;
}
// Wait that ignores the abort flag (used only while draining in-flight work), still bounded.
__device__ __forceinline__ void mbar_drain_wait(uint64_t *bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > kWaitCycles) return;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];\n" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);          // start address
    d |= (uint64_t)1 << 16;                          // leading byte offset (unused for SW128 K-major)
    d |= (uint64_t)(1024 >> 4) << 32;                // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                          // descriptor version (sm_100 family)
    d |= (uint64_t)2 << 61;                          // SWIZZLE_128B
    return d;
}

// kind::f8f6f4, A = B = e4m3, D = f32, both K-major, M = 128, N = 128
__host__ __device__ constexpr uint32_t idesc_f8(bool negA) {
    return (1u << 4) | (0u << 7) | (0u << 10) | ((negA ? 1u : 0u) << 13) | (0u << 14) | (0u << 15) | (0u << 16) |
           ((uint32_t)(kTileN >> 3) << 17) | ((uint32_t)(kTileM >> 4) << 24);
}

__device__ __forceinline__ void mma_f8(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
        "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
template <int kN>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t (&r)[kN]) {
    if constexpr (kN == 32) tmem_ld32(taddr, r);
    else tmem_ld16(taddr, r);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// ------------------------------------------------------- work decomposition
__device__ __forceinline__ int job_of(const OzJob *jobs, int num_jobs, int64_t tile) {
    int lo = 0, hi = num_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ void tile_coords(const OzJob &j, int64_t x, int64_t &tm, int64_t &tn) {
    if (j.lower) {
        int64_t r = (int64_t)((sqrt(8.0 * (double)x + 1.0) - 1.0) * 0.5);
        while (r * (r + 1) / 2 > x) --r;
        while ((r + 1) * (r + 2) / 2 <= x) ++r;
        tm = r;
        tn = x - r * (r + 1) / 2;
    } else {
        tm = x / j.tiles_n;
        tn = x - tm * j.tiles_n;
    }
}
// Tile g of the launch: from the host-built schedule (job, tm, tn) when given, else the
// jobs' own row-major order.
__device__ __forceinline__ const OzJob &resolve_tile(const OzJob *jobs, int num_jobs, const int4 *tile_list,
                                                     int64_t tile, int64_t &tm, int64_t &tn) {
    if (tile_list) {
        const int4 e = tile_list[tile];
        tm = e.y;
        tn = e.z;
        return jobs[e.x];
    }
    const OzJob &j = jobs[job_of(jobs, num_jobs, tile)];
    tile_coords(j, tile - j.tile_begin, tm, tn);
    return j;
}

// k-blocks per exact accumulation chunk on diagonal t (pairs = t - 1 for t <= s + 1)
__host__ __device__ __forceinline__ int64_t chunk_kblocks(int pairs) {
    const int64_t terms_per_kb = (int64_t)2 * kKBlock * pairs * 256;   // re/im products x max |product|
    int64_t c = kExactTerms / terms_per_kb;
    return c < 1 ? 1 : c;
}

// Loose grid-wide lockstep for cooperative launches: every producer publishes its stage epoch in
// its slot (one per CTA, or per CTA pair), and may run at most one epoch ahead of the slowest.  All persistent CTAs walk
// identical stage sequences, so staying within an epoch keeps the operand panels they share
// resident in L2 (left to themselves, CTAs drift apart by far more than L2 can hold).
// Bounded: on expiry the CTA raises the abort flag and records the error word.
__device__ bool grid_lockstep(int *progress, int n, int epoch, volatile int *abort_flag, int *err, int slot,
                              int slack = 1, long long budget = kWaitCycles) {
    atomicExch(progress + slot, epoch);
    const long long t0 = clock64();
    while (true) {
        int mn = kRetired;
        for (int i = 0; i < n; i += 4) {
            const int4 v = __ldcg(reinterpret_cast<const int4 *>(progress + i));
            mn = min(mn, min(min(v.x, v.y), min(v.z, v.w)));
        }
        if (mn >= epoch - slack) return true;
        if (*abort_flag) return false;
        if (clock64() - t0 > budget) {
            *abort_flag = 1;
            atomicCAS(err, 0, kDevTimeout * 16 + 5);
            return false;
        }
    }
}

// x * 2^k as a double for an FP32 accumulator x (a multiple of 2^-5 below 2^25), built with
// integer operations: GB300's FP64 pipe is a small fraction of its integer pipes, and a drain
// converts 2^16 values per CTA.  (f & 0x7fffffff) >> 3 puts the FP32 exponent and the top 20
// mantissa bits exactly where the FP64 high word keeps them, so rebasing the exponent is one
// add of (1023 - 127 + k) << 20; the low word takes the last 3 mantissa bits.  Valid for
// k in [kPow2Lo, kPow2Hi] (the result stays normal); pow2_ok() checks that once per column.
constexpr int kPow2Lo = -1017, kPow2Hi = 997;
__device__ __forceinline__ bool pow2_ok(int k) { return k >= kPow2Lo && k <= kPow2Hi; }
__device__ __forceinline__ double f32_pow2_to_f64_fast(uint32_t f, uint32_t ebias) {
    const uint32_t a = f & 0x7fffffffu;
    // a signed zero keeps its bits (high word = f, low word = 0)
    const uint32_t hi = a ? ((f & 0x80000000u) | ((a >> 3) + ebias)) : f;
    const uint32_t lo = f << 29;
    return __hiloint2double((int)hi, (int)lo);
}
__device__ __noinline__ double f32_pow2_to_f64_slow(uint32_t f, int k) { return ldexp((double)__uint_as_float(f), k); }
__device__ __forceinline__ uint32_t pow2_ebias(int k) { return (uint32_t)(1023 - 127 + k) << 20; }

// Drain 32 accumulator columns of one output row: out = (out +) x 2^(kb + e_col) with kb =
// 2 - 5t + e_row (a plain store on the first unit of a tile).  Every unit carries its full scale,
// so an output that already holds an earlier panel's sum is accumulated correctly.  Loads are
// grouped kDrainBatch at a time ahead of the stores (the compiler cannot reorder a load past a
// store to a possibly aliasing column), so a drain costs a few L2 round trips per 32 columns.
constexpr int kDrainBatch = 8;
__device__ __forceinline__ void drain32(const OzJob &j, int64_t row, int64_t col0, const uint32_t (&vre)[32],
                                        const uint32_t (&vim)[32], int kb, bool first) {
#pragma unroll
    for (int h = 0; h < 32; h += kDrainBatch) {
        double2 o[kDrainBatch];
#pragma unroll
        for (int cc = 0; cc < kDrainBatch; ++cc) {
            const int64_t col = col0 + h + cc;
            const bool live = col < j.n && !(j.lower && row < col);
            o[cc] = (live && !first) ? __ldcg(j.out + row + j.ldo * col) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int cc = 0; cc < kDrainBatch; ++cc) {
            const int64_t col = col0 + h + cc;
            if (col >= j.n || (j.lower && row < col)) continue;
            const int k = kb + j.er[col];
            double re, im;
            if (pow2_ok(k)) {
                const uint32_t eb = pow2_ebias(k);
                re = f32_pow2_to_f64_fast(vre[h + cc], eb);
                im = f32_pow2_to_f64_fast(vim[h + cc], eb);
            } else {
                re = f32_pow2_to_f64_slow(vre[h + cc], k);
                im = f32_pow2_to_f64_slow(vim[h + cc], k);
            }
            j.out[row + j.ldo * col] = make_double2(re + o[cc].x, im + o[cc].y);
        }
    }
}

struct __align__(8) Barriers {
    uint64_t full[kStages];
    uint64_t empty[kStages];
    uint64_t tfull[2];
    uint64_t tempty[2];
};

__global__ void __launch_bounds__(kThreads, 1)
    oz_gemm_kernel(const __grid_constant__ CUtensorMap map0, const __grid_constant__ CUtensorMap map1,
                   const __grid_constant__ CUtensorMap map2, const __grid_constant__ CUtensorMap map3,
                   const OzJob *__restrict__ jobs, int num_jobs, int64_t total_tiles, int s, int *err,
                   const int4 *__restrict__ tile_list, int *progress) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte alignment of the stage buffers (SW128 atoms)
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ Barriers bars;
    __shared__ uint32_t tmem_base_sh;
    __shared__ volatile int abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto map_of = [&](int i) -> const CUtensorMap * {
        return i == 0 ? &map0 : i == 1 ? &map1 : i == 2 ? &map2 : &map3;
    };

    if (threadIdx.x == 0) {
        for (int i = 0; i < kStages; ++i) { mbar_init(&bars.full[i], 1); mbar_init(&bars.empty[i], 1); }
        for (int i = 0; i < 2; ++i) { mbar_init(&bars.tfull[i], 1); mbar_init(&bars.tempty[i], 32 * kEpiWarps); }
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        for (int i = 0; i < 4; ++i) asm volatile("prefetch.tensormap [%0];\n" ::"l"((uint64_t)map_of(i)) : "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(smem_u32(&tmem_base_sh))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = tmem_base_sh;

    if (warp == 0) {
        // ------------------------------------------------------------ TMA producer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            int64_t issued = 0;
            bool ok = true;
            for (int64_t tile = blockIdx.x; ok && tile < total_tiles; tile += gridDim.x) {
                int64_t tm, tn;
                const OzJob &j = resolve_tile(jobs, num_jobs, tile_list, tile, tm, tn);
                const CUtensorMap *lm = map_of(j.lmap), *rm = map_of(j.rmap);
                for (int t = 2; ok && t <= s + 1; ++t) {
                    const int ilo = max(1, t - s), ihi = min(s, t - 1);
                    const int64_t ck = chunk_kblocks(ihi - ilo + 1);
                    for (int64_t cb = 0; ok && cb < j.nkb; cb += ck) {
                        const int64_t ce = min(j.nkb, cb + ck);
                        for (int64_t kb = cb; ok && kb < ce; ++kb) {
                            for (int i = ilo; i <= ihi; ++i) {
                                const int jj = t - i;
                                if (progress && issued > 0 && issued % kSyncEvery == 0 &&
                                    !grid_lockstep(progress, (int)gridDim.x, (int)(issued / kSyncEvery), &abort_flag,
                                                   err, (int)blockIdx.x)) { ok = false; break; }
                                if (!mbar_wait(&bars.empty[stage], phase ^ 1, &abort_flag, err, 1)) { ok = false; break; }
                                unsigned char *st = smem + stage * kStageBytes;
                                mbar_expect_tx(&bars.full[stage], kStageBytes);
                                const int xl = (int)(j.lk0 + kb * kKBlock), xr = (int)(j.rk0 + kb * kKBlock);
                                const int64_t yl = j.lrow0 + tm * kTileM, yr = j.rrow0 + tn * kTileN;
                                tma_load_2d(st, lm, &bars.full[stage], xl, (int)((2 * (i - 1)) * j.lplane + yl));
                                tma_load_2d(st + 16384, lm, &bars.full[stage], xl, (int)((2 * (i - 1) + 1) * j.lplane + yl));
                                tma_load_2d(st + 32768, rm, &bars.full[stage], xr, (int)((2 * (jj - 1)) * j.rplane + yr));
                                tma_load_2d(st + 49152, rm, &bars.full[stage], xr, (int)((2 * (jj - 1) + 1) * j.rplane + yr));
                                ++issued;
                                if (++stage == kStages) { stage = 0; phase ^= 1; }
                            }
                        }
                    }
                }
            }
            if (progress) atomicExch(progress + blockIdx.x, kRetired);
            // drain: every issued stage must have landed before the CTA may exit
            if (!ok) {
                for (int q = 0; q < kStages; ++q) {
                    // the last kStages issued stages are the only ones possibly in flight
                    if (issued == 0) break;
                    if (--stage < 0) { stage = kStages - 1; phase ^= 1; }
                    mbar_drain_wait(&bars.full[stage], phase);
                    --issued;
                }
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            int64_t unit = 0;
            bool ok = true;
            const uint32_t id_pos = idesc_f8(false), id_neg = idesc_f8(true);
            const uint32_t sbase = smem_u32(smem);
            for (int64_t tile = blockIdx.x; ok && tile < total_tiles; tile += gridDim.x) {
                int64_t tm_, tn_;
                const OzJob &j = resolve_tile(jobs, num_jobs, tile_list, tile, tm_, tn_);
                for (int t = 2; ok && t <= s + 1; ++t) {
                    const int ilo = max(1, t - s), ihi = min(s, t - 1);
                    const int64_t ck = chunk_kblocks(ihi - ilo + 1);
                    for (int64_t cb = 0; ok && cb < j.nkb; cb += ck) {
                        const int64_t ce = min(j.nkb, cb + ck);
                        const int buf = (int)(unit & 1);
                        const uint32_t uphase = (uint32_t)((unit >> 1) & 1);
                        if (!mbar_wait(&bars.tempty[buf], uphase ^ 1, &abort_flag, err, 2)) { ok = false; break; }
                        tc_fence_after();
                        const uint32_t d_re = tmem_base + buf * 256, d_im = d_re + 128;
                        bool first = true;
                        for (int64_t kb = cb; ok && kb < ce; ++kb) {
                            for (int i = ilo; i <= ihi; ++i) {
                                if (!mbar_wait(&bars.full[stage], phase, &abort_flag, err, 3)) { ok = false; break; }
                                tc_fence_after();
                                const uint32_t a_re = sbase + stage * kStageBytes, a_im = a_re + 16384;
                                const uint32_t b_re = a_re + 32768, b_im = a_re + 49152;
#pragma unroll
                                for (int kk = 0; kk < kKBlock / 32; ++kk) {
                                    const uint32_t off = kk * 32;
                                    const uint32_t acc = first ? 0u : 1u;
                                    mma_f8(d_re, sw128_desc(a_re + off), sw128_desc(b_re + off), id_pos, acc);
                                    mma_f8(d_re, sw128_desc(a_im + off), sw128_desc(b_im + off), id_pos, 1u);
                                    mma_f8(d_im, sw128_desc(a_re + off), sw128_desc(b_im + off), id_pos, acc);
                                    mma_f8(d_im, sw128_desc(a_im + off), sw128_desc(b_re + off), id_neg, 1u);
                                    first = false;
                                }
                                mma_commit(&bars.empty[stage]);
                                if (++stage == kStages) { stage = 0; phase ^= 1; }
                            }
                        }
                        if (!ok) break;
                        mma_commit(&bars.tfull[buf]);
                        ++unit;
                    }
                }
            }
            // wait for the MMAs still in flight before TMEM is freed
            if (unit > 0) {
                const int64_t u = unit - 1;
                mbar_drain_wait(&bars.tfull[u & 1], (uint32_t)((u >> 1) & 1));
            }
            if (!ok) {
                // a partially issued unit may still be running: commit and wait for it too
                mma_commit(&bars.tfull[unit & 1]);
                mbar_drain_wait(&bars.tfull[unit & 1], (uint32_t)((unit >> 1) & 1));
            }
        }
    } else {
        // ------------------------------------------------------------ epilogue (warps 2..9)
        const int q = warp & 3;                      // TMEM lane quadrant of this warp
        const int cbeg = ((warp - 2) >> 2) * (kTileN / 2);   // its half of the columns
        const int r_in_tile = q * 32 + lane;
        int64_t unit = 0;
        bool ok = true;
        for (int64_t tile = blockIdx.x; ok && tile < total_tiles; tile += gridDim.x) {
            int64_t tm, tn;
            const OzJob &j = resolve_tile(jobs, num_jobs, tile_list, tile, tm, tn);
            const int64_t row = tm * kTileM + r_in_tile;
            const bool row_ok = row < j.m;
            const int erow = row_ok ? j.el[row] : 0;
            for (int t = 2; ok && t <= s + 1; ++t) {
                const int ilo = max(1, t - s), ihi = min(s, t - 1);
                const int64_t ck = chunk_kblocks(ihi - ilo + 1);
                for (int64_t cb = 0; ok && cb < j.nkb; cb += ck) {
                    const bool first = (t == 2 && cb == 0) && !j.accum;
                    const int buf = (int)(unit & 1);
                    const uint32_t uphase = (uint32_t)((unit >> 1) & 1);
                    if (!mbar_wait(&bars.tfull[buf], uphase, &abort_flag, err, 4)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t tbase = tmem_base + ((uint32_t)(q * 32) << 16) + buf * 256;
#pragma unroll 1
                    for (int c0 = cbeg; c0 < cbeg + kTileN / 2; c0 += 32) {
                        uint32_t vre[32], vim[32];
                        tmem_ld32(tbase + c0, vre);
                        tmem_ld32(tbase + 128 + c0, vim);
                        tmem_ld_wait();
                        if (c0 + 32 >= cbeg + kTileN / 2) {
                            tc_fence_before();
                            mbar_arrive(&bars.tempty[buf]);
                        }
                        if (row_ok) drain32(j, row, tn * kTileN + c0, vre, vim, 2 - 5 * t + erow, first);
                    }
                    ++unit;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem_base) : "memory");
    }
}

// ------------------------------------------------------- CTA-pair products
// The S/H launch on 2-CTA tiles: a cluster of two CTAs (one per SM) computes a 256 x 256
// output tile with tcgen05.mma.cta_group::2 (M = 256, N = 256).  Each CTA stages its own half
// of the left operand (128 rows) and its own half of the right operand (128 rows) per k-block,
// so an MMA of twice the 1-CTA tile's flops reads the same 8 KB of shared memory per SM, and TMA
// writes half the bytes per flop.  Each CTA's TMEM holds its 128 output rows x (256 re + 256 im)
// FP32 columns (single-buffered: an exact-accumulation unit runs ~10^5 cycles, its drain a few
// 10^3).  Roles:
//   leader (cluster rank 0): TMA for its halves, expect_tx for both CTAs' bytes on its full
//     barrier, the single MMA issuer, commits multicast to both CTAs' empty / tfull barriers;
//   peer (rank 1): TMA for its halves completing on the leader's full barrier (.cta_group::2);
//   both: eight epilogue warps drain their own TMEM rows and arrive on the leader's tempty.
// Every wait is bounded as in oz_gemm_kernel; both CTAs meet at a cluster barrier before TMEM
// is freed, so no CTA exits while its shared memory or TMEM can still be addressed by the other.
constexpr int kPairTile = 256;
// Epilogue warps of the pair kernel: four per TMEM lane quadrant (each drains a quarter of the
// columns) hide the drain's latencies twice as well as two; HSDLA_PAIR_EPI_WARPS=8 builds two.
#ifndef HSDLA_PAIR_EPI_WARPS
#define HSDLA_PAIR_EPI_WARPS 16
#endif
constexpr int kPairEpiWarps = HSDLA_PAIR_EPI_WARPS;
constexpr int kPairThreads = 64 + 32 * kPairEpiWarps;      // warp 0 TMA, warp 1 MMA, the rest epilogue
constexpr int kColsPerWarp = 4 * kPairTile / kPairEpiWarps;
constexpr int kChunksPerWarp = kColsPerWarp / 32;
static_assert(kChunksPerWarp >= 1 && kColsPerWarp % 32 == 0, "epilogue column split");
// TMEM columns per load (re and im each): 16 with four epilogue warps per quadrant (18 warps leave
// 96 registers a thread), 32 with two
constexpr int kLdColsPair() { return kPairEpiWarps > 8 ? 16 : 32; }
constexpr int kLdCols = kLdColsPair();
// Operand stages of the pair kernel and the drain staging that shares its shared memory (over the
// epilogue warps, kDrainBufs buffers each: a warp fills one while the bulk copies of the others
// read them).  The drain's throughput is bounded by the staging bytes in flight.
#ifndef HSDLA_PAIR_STAGES
#define HSDLA_PAIR_STAGES 3
#endif
#ifndef HSDLA_PAIR_STAGING_KB
#define HSDLA_PAIR_STAGING_KB 32
#endif
// Drain staging buffers per epilogue warp: one buffer of 4 columns (2 KB) per warp drains with
// half the proxy fences and read-waits of two 2-column buffers; c2's per-type S/H launches took
// 23.35-23.41 ms against 24.37-24.43 (two buffers) and 27.8 ms (four) on one GB300, builds alternating.
#ifndef HSDLA_DRAIN_BUFS
#define HSDLA_DRAIN_BUFS 1
#endif
constexpr int kPairStages = HSDLA_PAIR_STAGES;
constexpr int kPairStagesHalf = 4;          // 48 KB stages of the half-width tiles
constexpr int kPairStagesMax = kPairStages > kPairStagesHalf ? kPairStages : kPairStagesHalf;
constexpr int kDrainBufs = HSDLA_DRAIN_BUFS;
constexpr int kStageCols = HSDLA_PAIR_STAGING_KB * 1024 / kPairEpiWarps / kDrainBufs / 512;   // columns per buffer
constexpr int kStageWarpBytes = kDrainBufs * kStageCols * 32 * 16;   // buffers x columns x 32 rows x 16 B
static_assert(kStageCols >= 1 && kLdColsPair() % kStageCols == 0, "drain staging shape");

constexpr int kPairStageBytes = kPairEpiWarps * kStageWarpBytes;
// Bulk copies and f64 add-reductions shared memory -> global with an L2 eviction policy
// (createpolicy): an output tile stays resident through its units (evict_last) and leaves first
// after its last one (evict_first).
__device__ __forceinline__ void bulk_store_g(void *gdst, uint32_t ssrc, uint32_t bytes, uint64_t pol) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group.L2::cache_hint [%0], [%1], %2, %3;\n" ::"l"(gdst),
                 "r"(ssrc), "r"(bytes), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void bulk_add_g(void *gdst, uint32_t ssrc, uint32_t bytes, uint64_t pol) {
    asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.L2::cache_hint.add.f64 [%0], [%1], %2, %3;\n" ::"l"(
                     gdst),
                 "r"(ssrc), "r"(bytes), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ uint64_t policy_evict_last() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;\n" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(p));
    return p;
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read %0;\n" ::"n"(N) : "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_size() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;\n" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t mapa_rank(uint32_t saddr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(saddr), "r"(rank));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_remote(uint32_t cluster_addr) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];\n" ::"r"(cluster_addr) : "memory");
}
__device__ __forceinline__ void tma_load_2d_pair(void *dst, const CUtensorMap *map, uint32_t bar_cluster, int x,
                                                 int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], "
        "[%2];\n" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(bar_cluster), "r"(x), "r"(y)
        : "memory");
}
__host__ __device__ constexpr uint32_t idesc_f8_pair(bool negA) {
    return (1u << 4) | ((negA ? 1u : 0u) << 13) | ((uint32_t)(kPairTile >> 3) << 17) |
           ((uint32_t)(kPairTile >> 4) << 24);
}
__device__ __forceinline__ void mma_f8_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// The same MMA with the left operand's collector buffer: kFill reads A from shared memory and
// keeps it for the next MMA, which (kFill = false: lastuse) takes A from the buffer and frees it.
template <bool kFill>
__device__ __forceinline__ void mma_f8_pair_ca(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                               uint32_t accumulate) {
    if constexpr (kFill)
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::2.kind::f8f6f4.collector::a::fill [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
            : "memory");
    else
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::2.kind::f8f6f4.collector::a::lastuse [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
            : "memory");
}
#ifndef HSDLA_COLLECTOR_A
#define HSDLA_COLLECTOR_A 1
#endif
__device__ __forceinline__ void mma_commit_pair(uint64_t *bar) {
    const uint16_t both = 3;
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;\n" ::"r"(
            smem_u32(bar)),
        "h"(both)
        : "memory");
}

struct __align__(8) PairBarriers {
    uint64_t full[kPairStagesMax];   // leader: both CTAs' bytes of a stage landed
    uint64_t empty[kPairStagesMax];  // each CTA: the stage's MMAs completed (multicast commit)
    uint64_t tfull[2];           // each CTA: a TMEM buffer's accumulator is complete (multicast commit)
    uint64_t tempty[2];          // leader: the epilogue warps of both CTAs drained the buffer
};

// Accumulation units of a pair launch, in drain order.  Unit u sums, per K-chunk, the digit pairs
// (i, t - i) of diagonal t = t[u] into the FP32 accumulator and drains it with weight 2^(2-5t).
// A merged unit also sums the pairs (i, t + 1 - i) of the next diagonal, with the left digits
// scaled by 2^-5 (planes 2s .. 4s-1 of the left operand): the two diagonals share one drain.
constexpr int kMaxUnits = kOzMaxSlices + 1;
constexpr uint8_t kUnitMerged = 1;
struct PairUnits {
    int32_t n;
    int8_t t[kMaxUnits];
    uint8_t flags[kMaxUnits];
};

// Tile shape of a pair launch.  kHalves = 1: one 256 x 256 accumulator (re + im, all 512 TMEM
// columns), so a unit's MMAs wait while the previous unit drains.  kHalves = 2: every unit runs
// as two halves of 128 output columns (MMA N = 128) into alternating TMEM buffers, so one half
// drains while the other computes; the left operand is staged once per half (1.5x the operand
// traffic of kHalves = 1) and the right operand's stage holds 64 rows per CTA (its own tensor map).
template <int kHalves>
struct PairShape {
    static constexpr int kN = kPairTile / kHalves;             // output columns of a unit half
    static constexpr int kBRows = kN / 2;                      // right-operand rows a CTA stages
    static constexpr int kStageBytes = 2 * kTileM * kKBlock + 2 * kBRows * kKBlock;
    static constexpr int kStages = kHalves == 1 ? kPairStages : kPairStagesHalf;
    static constexpr int kBufCols = 2 * kN;                    // TMEM columns of a buffer (re + im)
    static constexpr int kColsPerWarp = 4 * kN / kPairEpiWarps;   // per quadrant: 4 warps share kN
    static constexpr int kChunks = kColsPerWarp / 32;
    static constexpr size_t kSmem = (size_t)kStages * kStageBytes + kPairStageBytes + 1024;
    static_assert(kChunks >= 1 && kColsPerWarp % 32 == 0, "epilogue column split");
    static_assert(kStages <= kPairStagesMax, "stage barriers");
    static_assert(kSmem <= 227 * 1024, "pair kernel shared memory");
};
__host__ __device__ constexpr uint32_t idesc_f8_pair_n(bool negA, int n) {
    return (1u << 4) | ((negA ? 1u : 0u) << 13) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kPairTile >> 4) << 24);
}

template <int kHalves>
__global__ void __launch_bounds__(kPairThreads, 1)
    oz_pair_kernel(const __grid_constant__ CUtensorMap map0, const __grid_constant__ CUtensorMap map1,
                   const __grid_constant__ CUtensorMap map2, const __grid_constant__ CUtensorMap map3,
                   const OzJob *__restrict__ jobs, int num_jobs, int64_t total_tiles, int s, int *err,
                   const int4 *__restrict__ tile_list, int *progress, int sync_every, int slack,
                   const __grid_constant__ PairUnits units) {
    using Shape = PairShape<kHalves>;
    constexpr int kStages = Shape::kStages;
    constexpr int kStageB = Shape::kStageBytes;
    constexpr int kN = Shape::kN;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ PairBarriers bars;
    __shared__ uint32_t tmem_base_sh;
    __shared__ volatile int abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // launched as clusters of two or not at all: nothing below (the pair TMEM allocation above
    // all) is valid otherwise
    if (cluster_size() != 2) {
        if (threadIdx.x == 0) atomicCAS(err, 0, kDevBadInput * 16 + 6);
        return;
    }
    const uint32_t rank = cluster_rank();
    const bool leader = rank == 0;
    // bounded wait that records where it expired (first failure wins)
    auto pwait = [&](uint64_t *bar, uint32_t parity, int where, int stage_, int count) -> bool {
        if (mbar_wait(bar, parity, &abort_flag, err, where)) return true;
        if (atomicCAS(err + 7, 0, 1) == 0) {
            err[1] = blockIdx.x; err[2] = (int)rank; err[3] = stage_; err[4] = (int)parity; err[5] = count;
        }
        return false;
    };
    const int64_t pair = blockIdx.x >> 1, npairs = gridDim.x >> 1;
    auto map_of = [&](int i) -> const CUtensorMap * {
        return i == 0 ? &map0 : i == 1 ? &map1 : i == 2 ? &map2 : &map3;
    };

    if (threadIdx.x == 0) {
        for (int i = 0; i < kStages; ++i) { mbar_init(&bars.full[i], 1); mbar_init(&bars.empty[i], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&bars.tfull[b], 1); mbar_init(&bars.tempty[b], 2 * kPairEpiWarps); }
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        for (int i = 0; i < 4; ++i) asm volatile("prefetch.tensormap [%0];\n" ::"l"((uint64_t)map_of(i)) : "memory");
    }
    if (warp == 1) {
        // collective over the pair: one warp of each CTA
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(smem_u32(&tmem_base_sh))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    cluster_sync_all();          // barriers of both CTAs initialised before any remote arrival
    tc_fence_after();
    const uint32_t tmem_base = tmem_base_sh;
    const uint32_t full0_leader = mapa_rank(smem_u32(&bars.full[0]), 0);
    const uint32_t tempty0_leader = mapa_rank(smem_u32(&bars.tempty[0]), 0);
    const int64_t half = (int64_t)rank * (kPairTile / 2);     // this CTA's rows of a tile
    const int64_t bhalf = (int64_t)rank * Shape::kBRows;        // this CTA's right-operand rows of a half

    if (warp == 0) {
        // ------------------------------------------------------------ TMA producers (both CTAs)
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            int64_t issued = 0;
            bool ok = true;
            for (int64_t tile = pair; ok && tile < total_tiles; tile += npairs) {
                int64_t tm, tn;
                const OzJob &j = resolve_tile(jobs, num_jobs, tile_list, tile, tm, tn);
                const CUtensorMap *lm = map_of(j.lmap), *rm = map_of(j.rmap);
                for (int u = 0; ok && u < units.n; ++u) {
                    const int t = units.t[u], merged = (units.flags[u] & kUnitMerged) ? 1 : 0;
                    const int64_t ck = merged ? j.nkb : chunk_kblocks(min(s, t - 1) - max(1, t - s) + 1);
                    for (int64_t cb = 0; ok && cb < j.nkb; cb += ck) {
                        const int64_t ce = min(j.nkb, cb + ck);
                        for (int h = 0; ok && h < kHalves; ++h) {
                            for (int64_t kb = cb; ok && kb < ce; ++kb) {
                                for (int part = 0; ok && part <= merged; ++part) {
                                    const int tt = t + part, ilo = max(1, tt - s), ihi = min(s, tt - 1);
                                    for (int i = ilo; i <= ihi; ++i) {
                                        const int jj = tt - i;
                                        const int lp = (part ? 2 * s : 0) + 2 * (i - 1);   // scaled planes of a merged part
                                        if (leader && progress && issued > 0 && issued % sync_every == 0 &&
                                            !grid_lockstep(progress, (int)npairs, (int)(issued / sync_every),
                                                           &abort_flag, err, (int)pair, slack)) { ok = false; break; }
                                        if (!pwait(&bars.empty[stage], phase ^ 1, 1, stage, (int)issued)) { ok = false; break; }
                                        unsigned char *st = smem + stage * kStageB;
                                        if (leader) mbar_expect_tx(&bars.full[stage], 2 * kStageB);
                                        const uint32_t fb = full0_leader + stage * 8;
                                        const int xl = (int)(j.lk0 + kb * kKBlock), xr = (int)(j.rk0 + kb * kKBlock);
                                        const int64_t yl = j.lrow0 + tm * kPairTile + half;
                                        const int64_t yr = j.rrow0 + tn * kPairTile + h * kN + bhalf;
                                        tma_load_2d_pair(st, lm, fb, xl, (int)(lp * j.lplane + yl));
                                        tma_load_2d_pair(st + 16384, lm, fb, xl, (int)((lp + 1) * j.lplane + yl));
                                        tma_load_2d_pair(st + 32768, rm, fb, xr, (int)((2 * (jj - 1)) * j.rplane + yr));
                                        tma_load_2d_pair(st + 32768 + Shape::kBRows * kKBlock, rm, fb, xr,
                                                         (int)((2 * (jj - 1) + 1) * j.rplane + yr));
                                        ++issued;
                                        if (++stage == kStages) { stage = 0; phase ^= 1; }
                                    }
                                }
                            }
                        }
                    }
                }
            }
            if (leader && progress) atomicExch(progress + pair, kRetired);
            // Before exit every stage this CTA issued must have been consumed: its bytes landed and
            // the MMA commit that frees it (multicast, possibly remote) arrived.  Normally these
            // waits return at once; after an abort they are bounded.
            for (int q = 0; q < kStages && issued > 0; ++q) {
                if (--stage < 0) { stage = kStages - 1; phase ^= 1; }
                mbar_drain_wait(&bars.empty[stage], phase);
                --issued;
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer (leader only)
        if (lane == 0 && leader) {
            int stage = 0;
            uint32_t phase = 0;
            int64_t unit = 0;            // unit chunks issued (each uses every buffer once)
            int hb = 0;                  // buffer of a partially issued half
            bool ok = true;
            const uint32_t id_pos = idesc_f8_pair_n(false, kN), id_neg = idesc_f8_pair_n(true, kN);
            const uint32_t sbase = smem_u32(smem);
            for (int64_t tile = pair; ok && tile < total_tiles; tile += npairs) {
                int64_t tm_, tn_;
                const OzJob &j = resolve_tile(jobs, num_jobs, tile_list, tile, tm_, tn_);
                // the job's fields in registers: the asm statements below clobber memory, and the
                // issuer must not reload them between MMAs
                const int64_t jnkb = j.nkb;
                const int jksl = j.ksteps_last > 0 ? j.ksteps_last : kKBlock / 32;
                for (int u = 0; ok && u < units.n; ++u) {
                    const int t = units.t[u], merged = (units.flags[u] & kUnitMerged) ? 1 : 0;
                    const int64_t ck = merged ? jnkb : chunk_kblocks(min(s, t - 1) - max(1, t - s) + 1);
                    for (int64_t cb = 0; ok && cb < jnkb; cb += ck) {
                        const int64_t ce = min(jnkb, cb + ck);
                        for (int h = 0; ok && h < kHalves; ++h) {
                            hb = h;
                            const uint32_t d_re = tmem_base + h * Shape::kBufCols, d_im = d_re + kN;
                            if (!pwait(&bars.tempty[h], (uint32_t)((unit & 1) ^ 1), 2, stage, (int)unit)) { ok = false; break; }
                            tc_fence_after();
                            bool first = true;
                            for (int64_t kb = cb; ok && kb < ce; ++kb) {
                                for (int part = 0; ok && part <= merged; ++part) {
                                    const int tt = t + part, ilo = max(1, tt - s), ihi = min(s, tt - 1);
                                    for (int i = ilo; i <= ihi; ++i) {
                                        if (!pwait(&bars.full[stage], phase, 3, stage, (int)unit)) { ok = false; break; }
                                        tc_fence_after();
                                        const uint32_t a_re = sbase + stage * kStageB, a_im = a_re + 16384;
                                        const uint32_t b_re = a_re + 32768, b_im = b_re + Shape::kBRows * kKBlock;
                                        // The stage's four descriptors once; a 32-byte step along K adds 2
                                        // to the start-address field (16-byte units; shared-memory
                                        // addresses stay below 2^18, so the field never carries).  The
                                        // single issuing thread has ~64 cycles per N = 128 MMA.
                                        const uint64_t dar = sw128_desc(a_re), dai = sw128_desc(a_im);
                                        const uint64_t dbr = sw128_desc(b_re), dbi = sw128_desc(b_im);
                                        auto step = [&](uint32_t kk) {
                                            const uint64_t o = 2u * kk;
                                            const uint32_t acc = first ? 0u : 1u;
#if HSDLA_COLLECTOR_A
                                            // the two MMAs of the real left plane back to back, the
                                            // second taking A from the collector buffer.  (Not for
                                            // the imaginary plane: an MMA that reads A from the
                                            // collector does not apply the negate-A bit, measured:
                                            // the -A_im B_re term came out as +A_im B_re.)
                                            mma_f8_pair_ca<true>(d_re, dar + o, dbr + o, id_pos, acc);
                                            mma_f8_pair_ca<false>(d_im, dar + o, dbi + o, id_pos, acc);
                                            mma_f8_pair(d_re, dai + o, dbi + o, id_pos, 1u);
                                            mma_f8_pair(d_im, dai + o, dbr + o, id_neg, 1u);
#else
                                            mma_f8_pair(d_re, dar + o, dbr + o, id_pos, acc);
                                            mma_f8_pair(d_re, dai + o, dbi + o, id_pos, 1u);
                                            mma_f8_pair(d_im, dar + o, dbi + o, id_pos, acc);
                                            mma_f8_pair(d_im, dai + o, dbr + o, id_neg, 1u);
#endif
                                            first = false;
                                        };
                                        // whole blocks as straight-line code (a bound in this loop slowed the
                                        // launches by 2-10%).  With 256 x 256 accumulators the job's last
                                        // k-block stops early, where the K steps past the contraction length
                                        // hold zero digits (lmax 8: 2L = 162 of 256; c1 -10%); the half-width
                                        // tiles keep whole blocks, as the check alone cost them 3-6% (c2, c3)
                                        if (kHalves == 2 || kb + 1 < jnkb || jksl == kKBlock / 32) {
#pragma unroll
                                            for (int kk = 0; kk < kKBlock / 32; ++kk) step(kk);
                                        } else {
                                            step(0);
                                            if (jksl > 1) step(1);
                                            if (jksl > 2) step(2);
                                        }
                                        mma_commit_pair(&bars.empty[stage]);
                                        if (++stage == kStages) { stage = 0; phase ^= 1; }
                                    }
                                }
                            }
                            if (!ok) break;
                            mma_commit_pair(&bars.tfull[h]);
                        }
                        if (!ok) break;
                        ++unit;
                    }
                }
            }
            if (!ok) {
                // a partially issued half may still be running: commit it and wait (bounded)
                mma_commit_pair(&bars.tfull[hb]);
                mbar_drain_wait(&bars.tfull[hb], (uint32_t)(unit & 1));
            } else if (unit > 0) {
                // the last unit's MMAs and both CTAs' drains of it
                for (int h = 0; h < kHalves; ++h) {
                    mbar_drain_wait(&bars.tfull[h], (uint32_t)((unit - 1) & 1));
                    mbar_drain_wait(&bars.tempty[h], (uint32_t)((unit - 1) & 1));
                }
            }
        }
    } else {
        // ------------------------------------------------------------ epilogue (warps 2.., both CTAs)
        // A unit's drain: TMEM -> registers -> FP64 with the full scale 2^(2-5t+e_row+e_col) (built
        // with integer operations) -> the output: a plain store for the tile's first unit,
        // fire-and-forget f64 reductions in L2 for the others.  Each lane owns one output row, so
        // successive updates of an element come from one thread and stay in program order; the
        // SM never waits on the output.  Only stored elements (row < m, col < n, lower: row >=
        // col) are written.
        constexpr int kCols = Shape::kColsPerWarp, kCh = Shape::kChunks;
        const int q = warp & 3;                      // TMEM lane quadrant of this warp
        const int cbeg = ((warp - 2) >> 2) * kCols;  // its share of a buffer's columns
        unsigned char *stg = smem + kStages * kStageB + (warp - 2) * kStageWarpBytes;
        const uint32_t stg_s = smem_u32(stg);
        const uint64_t pol_last = policy_evict_last(), pol_first = policy_evict_first();
        int64_t unit = 0;
        int rd = 0;                                  // staged buffers so far (the ring position)
        bool ok = true;
        for (int64_t tile = pair; ok && tile < total_tiles; tile += npairs) {
            int64_t tm, tn;
            const OzJob &j = resolve_tile(jobs, num_jobs, tile_list, tile, tm, tn);
            const int64_t r0 = tm * kPairTile + half + q * 32, row = r0 + lane;
            const int64_t m = j.m, n = j.n, ldo = j.ldo, nkb = j.nkb;
            const bool lower = j.lower != 0, accum = j.accum != 0;
            const int erow = row < m ? j.el[row] : 0;
            double2 *out = j.out;
            // The tile's column exponents, loaded once for all its units: lane l holds column
            // tn*256 + h*kN + cbeg + 32c + l of half h, chunk c in ex[h kCh + c], with each chunk's
            // range for the fast-path test.  The registers rotate after each chunk, so the current
            // chunk's are always in ex[0] (after a unit's chunks they are back in order).
            const int32_t *er = j.er;
            int ex[kHalves * kCh], exlo[kHalves * kCh], exhi[kHalves * kCh];
#pragma unroll
            for (int x = 0; x < kHalves * kCh; ++x) {
                const int64_t col = tn * kPairTile + (x / kCh) * kN + cbeg + 32 * (x % kCh) + lane;
                ex[x] = col < n ? __ldg(er + col) : 0;
            }
#pragma unroll
            for (int x = 0; x < kHalves * kCh; ++x) {
                exlo[x] = __reduce_min_sync(0xffffffffu, ex[x]);
                exhi[x] = __reduce_max_sync(0xffffffffu, ex[x]);
            }
            for (int u = 0; ok && u < units.n; ++u) {
                const int t = units.t[u];
                const uint8_t fl = units.flags[u];
                const int64_t ck =
                    (fl & kUnitMerged) ? nkb : chunk_kblocks(min(s, t - 1) - max(1, t - s) + 1);
                const int kb = 2 - 5 * t + erow;
                // 2^(kb + e_col) as an FP64 exponent bias: the row's part plus e_col << 20
                const uint32_t rbias = pow2_ebias(kb);
                for (int64_t cb = 0; ok && cb < nkb; cb += ck) {
                    const bool first = (u == 0 && cb == 0) && !accum;
                    const uint64_t pol = (u == units.n - 1 && cb + ck >= nkb) ? pol_first : pol_last;
#pragma unroll 1
                    for (int h = 0; h < kHalves; ++h) {
                        if (!pwait(&bars.tfull[h], (uint32_t)(unit & 1), 4, warp, (int)unit)) { ok = false; break; }
                        tc_fence_after();
                        // the previous half's copies are complete: successive updates stay in order
                        if (lane < kStageCols) bulk_wait_all();
                        const uint32_t tbase = tmem_base + ((uint32_t)(q * 32) << 16) + h * Shape::kBufCols;
#pragma unroll 1
                        for (int c = 0; c < kCh; ++c) {
                            const int64_t colb = tn * kPairTile + h * kN + cbeg + 32 * c;
                            const bool fast = __all_sync(0xffffffffu, pow2_ok(kb + exlo[0]) && pow2_ok(kb + exhi[0]));
#pragma unroll
                            for (int hh = 0; hh < 32; hh += kLdCols) {
                                uint32_t vre[kLdCols], vim[kLdCols];
                                tmem_ld<kLdCols>(tbase + cbeg + 32 * c + hh, vre);
                                tmem_ld<kLdCols>(tbase + kN + cbeg + 32 * c + hh, vim);
                                tmem_ld_wait();
                                if (c == kCh - 1 && hh + kLdCols >= 32) {
                                    tc_fence_before();
                                    __syncwarp();
                                    if (lane == 0) mbar_arrive_remote(tempty0_leader + h * 8);
                                }
#pragma unroll
                                for (int g4 = 0; g4 < kLdCols; g4 += kStageCols, ++rd) {
                                    const uint32_t buf = (uint32_t)(rd % kDrainBufs) * (kStageCols * 512);
                                    if (lane < kStageCols) bulk_wait_read<kDrainBufs - 1>();
                                    __syncwarp();
#pragma unroll
                                    for (int cc = 0; cc < kStageCols; ++cc) {
                                        const int cl = g4 + cc;
                                        const int ec = __shfl_sync(0xffffffffu, ex[0], hh + cl);
                                        double re, im;
                                        if (fast) {
                                            const uint32_t eb = rbias + ((uint32_t)ec << 20);
                                            re = f32_pow2_to_f64_fast(vre[cl], eb);
                                            im = f32_pow2_to_f64_fast(vim[cl], eb);
                                        } else {
                                            re = f32_pow2_to_f64_slow(vre[cl], kb + ec);
                                            im = f32_pow2_to_f64_slow(vim[cl], kb + ec);
                                        }
                                        *reinterpret_cast<double2 *>(stg + buf + cc * 512 + lane * 16) = make_double2(re, im);
                                    }
                                    fence_async_smem();
                                    __syncwarp();
                                    // lane cc issues the copy of the group's column cc (32 rows) and commits it
                                    if (lane < kStageCols) {
                                        const int64_t col = colb + hh + g4 + lane;
                                        const int64_t lo = lower ? max(r0, col) : r0, hi = min(r0 + 32, m);
                                        if (col < n && lo < hi) {
                                            const uint32_t src = stg_s + buf + lane * 512 + (uint32_t)(lo - r0) * 16;
                                            double2 *dst = out + lo + ldo * col;
                                            if (first) bulk_store_g(dst, src, (uint32_t)(hi - lo) * 16, pol);
                                            else bulk_add_g(dst, src, (uint32_t)(hi - lo) * 16, pol);
                                        }
                                        bulk_commit();
                                    }
                                }
                            }
                            // the next chunk's exponents into ex[0]
                            const int xe = ex[0], xl = exlo[0], xh = exhi[0];
#pragma unroll
                            for (int x = 0; x + 1 < kHalves * kCh; ++x) {
                                ex[x] = ex[x + 1];
                                exlo[x] = exlo[x + 1];
                                exhi[x] = exhi[x + 1];
                            }
                            ex[kHalves * kCh - 1] = xe;
                            exlo[kHalves * kCh - 1] = xl;
                            exhi[kHalves * kCh - 1] = xh;
                        }
                    }
                    if (!ok) break;
                    ++unit;
                }
            }
        }
        // every copy complete before the CTA may exit
        if (lane < kStageCols) bulk_wait_all();
    }
    tc_fence_before();
    __syncwarp();
    __syncthreads();
    cluster_sync_all();          // neither CTA frees TMEM or exits while the other may address it
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, 512;\n" ::"r"(tmem_base) : "memory");
    }
}

// --------------------------------------------------------------- slicing
// Digit planes of Z (Kin x ncols, column-major, ld ldz) with optional row weights v:
// padded contraction layout: source rows [b*rpb, (b+1)*rpb) land at [b*bpad, b*bpad + rpb).
//
// One CTA per plane row (= source column), 512 threads and one CTA per SM, which keeps the
// column set in flight (152 x <= 0.5 MB) inside L2: pass 1 reads the column from HBM for its
// exponent, pass 2 re-reads it from L2 and writes the digits.  Digit extraction without carries:
// with B = 16 (1 + 32 + ... + 32^(s-2)), the balanced digits d_i in [-16, 15] (i >= 2) of X are
// the 5-bit fields of U = X + B minus 16, and the top digit is U >> 5(s-1) in [-16, 16]; digits
// are encoded two at a time by the hardware f32 -> e4m3x2 conversion (exact for |d| <= 16).
// A dual table slices the same source twice in one pass (C unweighted and W = C with row
// weights), reading the source once.
constexpr int kSliceThreads = 512;
constexpr int kSliceVec = 8;       // consecutive contraction bytes per thread and plane

// One slicing launch covers an operand for every k-point of a group: the k-points' columns
// are stacked as consecutive rows of each digit plane (row0 of an entry = its first row).
struct SliceEntry {
    const double2 *Z;          // source K x ncols, column-major, ld SliceTab::ldz
    int64_t ncols;
    int64_t row0;
};
struct SliceTab {
    int nk = 0;
    int s = 0;
    int64_t ldz = 0, Kin = 0, rpb = 0, bpad = 0;
    const double *v = nullptr;          // optional per-row weights (K)
    uint8_t *digits = nullptr;
    int64_t Kpad = 0, plane_rows = 0, pitch = 0;
    int32_t *expo = nullptr;            // exponent of each plane row
    // dual: a second digit operand of the same geometry from the same source with weights v2
    const double *v2 = nullptr;
    uint8_t *digits2 = nullptr;
    int32_t *expo2 = nullptr;
    // 1: the (first) operand's digits also go, scaled by 2^-5, to planes 2s .. 4s-1 (the left
    // operand of merged accumulation units)
    int scaled = 0;
    SliceEntry e[kMaxGroup];
};

// e4m3 byte of the digit idx - 16 (idx in [0, 32]), per CTA of the slicing kernel: a digit is
// one shared-memory load instead of an integer-to-float conversion and half a packing conversion
__shared__ uint8_t g_e4m3_lut[33];
// Four e4m3 digits (|d| <= 16) times 2^-5: every nonzero digit is normal with exponent field >= 7
// (|d| >= 1), so subtracting 5 from the field (0x28 from the byte, no borrow) scales it exactly
// (d / 32 >= 2^-5 stays normal); zeros keep their bytes.
__device__ __forceinline__ uint32_t scale4_e4m3_2m5(uint32_t w) {
    return w - (0x28282828u & __vcmpne4(w & 0x7f7f7f7fu, 0u));
}

// The planes of U = X + B from the least significant: plane i (0 = most significant) holds
// ((U >> 5 (s-1-i)) & 31) - 16 for i >= 1, and the top plane the rest, U >> 5 (s-1) in
// [-16, 16].  A running arithmetic shift by 5 leaves each field in the low bits in turn (the low
// bits are the same for arithmetic and logical shifts).
// kScaled: each digit also goes, times 2^-5 (exact in e4m3 for |d| <= 16: d / 32 >= 2^-5 is
// normal), to plane 2s + 2i + part.
template <int kVec, bool kScaled>
__device__ __forceinline__ void write_part(const long long (&x)[kVec], int part, int s, uint8_t *row, int64_t plane) {
    long long u[kVec];
#pragma unroll
    for (int v = 0; v < kVec; ++v) u[v] = x[v];
#pragma unroll 1
    for (int step = 0; step < s; ++step) {
        const int i = s - 1 - step;
        uint32_t w0 = 0, w1 = 0;
#pragma unroll
        for (int v = 0; v < kVec; ++v) {
            // (the top digit of a finite row is in [-16, 16]; the clamp keeps the table read in
            // bounds for any row)
            const int idx = i == 0 ? min(max((int)u[v] + 16, 0), 32) : (int)(u[v] & 31);
            const uint32_t b = (uint32_t)g_e4m3_lut[idx] << (8 * (v & 3));
            if (v < 4) w0 |= b; else w1 |= b;
            u[v] >>= 5;
        }
        uint8_t *dst = row + (int64_t)(2 * i + part) * plane;
        if (kVec == 8) *reinterpret_cast<uint2 *>(dst) = make_uint2(w0, w1);
        else *reinterpret_cast<uint32_t *>(dst) = w0;
        if (kScaled) {
            uint8_t *dsc = row + (int64_t)(2 * s + 2 * i + part) * plane;
            if (kVec == 8) *reinterpret_cast<uint2 *>(dsc) = make_uint2(scale4_e4m3_2m5(w0), scale4_e4m3_2m5(w1));
            else *reinterpret_cast<uint32_t *>(dsc) = scale4_e4m3_2m5(w0);
        }
    }
}

template <int kVec, bool kScaled = false>
__device__ __forceinline__ void write_planes(const long long (&ur)[kVec], const long long (&ui)[kVec], int s,
                                             uint8_t *row, int64_t plane) {
    write_part<kVec, kScaled>(ur, 0, s, row, plane);
    write_part<kVec, kScaled>(ui, 1, s, row, plane);
}

// Maximum over the block of non-negative doubles given as bit patterns (which order like the
// values), with integer operations: GB300's FP64 pipe takes 16 cycles per warp instruction, and
// an FP64 max here was most of the slicing's FP64 work.
__device__ __forceinline__ unsigned long long block_max_bits(unsigned long long m, unsigned long long *red) {
    for (int o = 16; o > 0; o >>= 1) m = max(m, (unsigned long long)__shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    unsigned long long r = 0;
    for (int i = 0; i < kSliceThreads / 32; ++i) r = max(r, red[i]);
    return r;
}
// frexp's exponent of a positive finite double given as bits: x = f 2^e with f in [1/2, 1)
__device__ __forceinline__ int frexp_exp_bits(unsigned long long b) {
    const int E = (int)(b >> 52) & 0x7ff;
    if (E) return E - 1022;
    return -1010 - __clzll((long long)(b & 0xfffffffffffffull));   // subnormal: mantissa 2^-1074
}

// Integer-pipe helpers of the slicing (GB300's FP64 pipe runs ~1/64 of its integer rate).
// |x| as an ordered integer: for finite doubles the bit pattern of |x| orders like |x|.
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
// rint(x 2^k), round half to even, exactly as __double2ll_rn(x * 2^k) for |x 2^k| < 2^62: the
// mantissa shifted by the exponent, with the round bit and the sticky remainder.
__device__ __forceinline__ long long rint_pow2(double x, int k) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((b >> 52) & 0x7ff);
    const unsigned long long mant = b & 0xfffffffffffffull;
    const unsigned long long m = E ? (mant | (1ull << 52)) : mant;
    const int sh = 1075 - (E ? E : 1) - k;          // |x 2^k| = m 2^-sh
    unsigned long long q;
    if (sh <= 0) {
        q = m << (-sh);
    } else if (sh >= 54) {
        q = 0;                                      // m 2^-sh < 1/2
    } else {
        q = m >> sh;
        const unsigned long long rem = m & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        q += (rem > half) | ((rem == half) & (q & 1ull));
    }
    return (b >> 63) ? -(long long)q : (long long)q;
}
// v 2^k by an exponent add (v normal and the result normal), else ldexp
__device__ __noinline__ double ldexp_out_of_line(double v, int k) { return ldexp(v, k); }
__device__ __forceinline__ double scale_pow2(double v, int k) {
    const long long b = __double_as_longlong(v);
    const int E = (int)((b >> 52) & 0x7ff);
    if (E > 0 && E + k > 0 && E + k < 2047) return __longlong_as_double(b + ((long long)k << 52));
    return ldexp_out_of_line(v, k);    // (a call: inlined, its FP64 work was issued for every value)
}

// the weighted operand's digits of one chunk (kept out of line: inlined next to the first
// operand's, the compiler interleaves the two and spills)
template <int kV>
__device__ __noinline__ void weighted_chunk(const double2 *zc, const double *vv, int nv, int kw, long long B, int s,
                                            uint8_t *row, int64_t plane) {
    long long xr[kV], xi[kV];
#pragma unroll
    for (int u = 0; u < kV; ++u) {
        const double2 z = u < nv ? zc[u] : make_double2(0.0, 0.0);
        const double sc = u < nv ? scale_pow2(vv[u], kw) : 0.0;
        xr[u] = B + rint_pow2(z.x * sc, 0);
        xi[u] = B + rint_pow2(z.y * sc, 0);
    }
    write_planes<kV>(xr, xi, s, row, plane);
}

#ifndef HSDLA_SLICE_CTAS
#define HSDLA_SLICE_CTAS 2
#endif
template <bool kDual, bool kScaled>
__global__ void __launch_bounds__(kSliceThreads, HSDLA_SLICE_CTAS) oz_slice_kernel(const __grid_constant__ SliceTab tab) {
    // values per thread and step of the digit pass (the dual pass keeps two operands' state)
    constexpr int kV = kDual ? 4 : kSliceVec;
    const int64_t r = blockIdx.x;           // plane row
    int k = 0;
    while (k + 1 < tab.nk && tab.e[k + 1].row0 <= r) ++k;
    const int64_t g = r - tab.e[k].row0;
    const bool live = g >= 0 && g < tab.e[k].ncols;
    const double2 *Zc = tab.e[k].Z + tab.ldz * (live ? g : 0);
    const double *v = tab.v, *v2 = tab.v2;
    const int Kin = (int)tab.Kin, rpb = (int)tab.rpb, bpad = (int)tab.bpad, Kpad = (int)tab.Kpad;
    const int64_t pitch = tab.pitch, plane_rows = tab.plane_rows;
    const int s = tab.s;
    __shared__ unsigned long long red[2][kSliceThreads / 32];
    // the digit table (read in pass 2, after the barrier of the row maximum)
    if (threadIdx.x < 33) {
        const float dv = (float)((int)threadIdx.x - 16);
        g_e4m3_lut[threadIdx.x] = (uint8_t)(__nv_cvt_float2_to_fp8x2(make_float2(dv, 0.f), __NV_SATFINITE, __NV_E4M3) & 0xffu);
    }
    // pass 1: column max of max(|re|, |im|) (times the row weight; the only FP64 multiply here)
    // Each thread reads 8 consecutive values per step (all loads of a step in flight together):
    // one value per thread and step kept too few bytes in flight to cover the memory latency.
    // (the weighted and unweighted forms as separate loops: GB300 issues the FP64 multiplies of a
    // predicated-off branch all the same, at 16 cycles per warp instruction)
    unsigned long long mx = 0, mx2 = 0;
    auto pass1 = [&](auto weighted) {
        for (int k0 = threadIdx.x * kSliceVec; k0 < Kin; k0 += kSliceThreads * kSliceVec) {
            double2 z[kSliceVec];
#pragma unroll
            for (int u = 0; u < kSliceVec; ++u) z[u] = k0 + u < Kin ? Zc[k0 + u] : make_double2(0.0, 0.0);
#pragma unroll
            for (int u = 0; u < kSliceVec; ++u) {
                const unsigned long long a = max(abs_bits(z[u].x), abs_bits(z[u].y));
                if (k0 + u < Kin) {
                    if constexpr (decltype(weighted)::value) mx = max(mx, abs_bits(__longlong_as_double((long long)a) * v[k0 + u]));
                    else mx = max(mx, a);
                    if (kDual) mx2 = max(mx2, abs_bits(__longlong_as_double((long long)a) * v2[k0 + u]));
                }
            }
        }
    };
    if (live) {
        if (v) pass1(std::true_type{});
        else pass1(std::false_type{});
    }
    int e = 0, e2 = 0;
    const unsigned long long m = block_max_bits(mx, red[0]);
    if (m > 0) e = frexp_exp_bits(m);       // max < 2^e
    if (kDual) {
        const unsigned long long m2 = block_max_bits(mx2, red[1]);
        if (m2 > 0) e2 = frexp_exp_bits(m2);
    }
    if (threadIdx.x == 0) {
        tab.expo[r] = e;
        if (kDual) tab.expo2[r] = e2;
    }
    const int top = 5 * s - 1;              // X = rint(z 2^(5s-1)), |z| < 1
    const int kx = top - e, kw = top - e2;
    long long B = 0;
    for (int p = 0; p < s - 1; ++p) B |= 16ll << (5 * p);
    const int nb = Kpad / bpad;
    const int64_t plane = plane_rows * pitch;
    auto pass2 = [&](auto weighted) {
        for (int kp0 = threadIdx.x * kV; kp0 < Kpad; kp0 += kSliceThreads * kV) {
            // a chunk never straddles a contraction block (bpad is a multiple of kV)
            const int b = kp0 / bpad, rr0 = kp0 - b * bpad;
            // number of live values of this chunk (a prefix: the block tail and Kin cut it from above)
            const int nv = live && b < nb ? max(0, min(min(kV, rpb - rr0), Kin - (b * rpb + rr0))) : 0;
            const double2 *zc = Zc + b * rpb + rr0;
            long long xr[kV], xi[kV];
#pragma unroll
            for (int u = 0; u < kV; ++u) {
                const double2 z = u < nv ? zc[u] : make_double2(0.0, 0.0);
                if constexpr (decltype(weighted)::value) {
                    const double sc = u < nv ? scale_pow2(v[b * rpb + rr0 + u], kx) : 0.0;
                    xr[u] = B + rint_pow2(z.x * sc, 0);
                    xi[u] = B + rint_pow2(z.y * sc, 0);
                } else {
                    xr[u] = B + rint_pow2(z.x, kx);
                    xi[u] = B + rint_pow2(z.y, kx);
                }
            }
            write_planes<kV, kScaled>(xr, xi, s, tab.digits + r * pitch + kp0, plane);
            if (kDual)      // the chunk again (an L1 hit) for the weighted operand
                weighted_chunk<kV>(zc, v2 + b * rpb + rr0, nv, kw, B, s, tab.digits2 + r * pitch + kp0, plane);
        }
    };
    if (v) pass2(std::true_type{});
    else pass2(std::false_type{});
}

// ------------------------------------------------------------ host helpers
typedef CUresult (*PFN_encodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

PFN_encodeTiled get_encode() {
    static PFN_encodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_encodeTiled>(p);
    }
    return fn;
}

// digit operand: 2s planes of plane_rows rows; a row holds Kpad digit bytes at a row pitch of
// Kpad + pad bytes.  The pad keeps the pitch off a power of two: with a power-of-two pitch the
// 128 rows of one TMA box fall on the same L2 sets and memory channels.
struct DigitOperand {
    uint8_t *digits = nullptr;
    int32_t *expo = nullptr;
    int64_t plane_rows = 0, Kpad = 0, pitch = 0;
    CUtensorMap map;
    CUtensorMap map64;         // 64-row boxes: the right operand of half-width pair tiles
};

int64_t env_int(const char *name, int64_t dflt) {
    const char *v = getenv(name);
    if (!v || !*v) return dflt;
    char *end = nullptr;
    const long long x = strtoll(v, &end, 10);
    return (end && *end == 0) ? (int64_t)x : dflt;
}

// Row pitch pad of the digit planes (bytes, multiple of 16); HSDLA_DIGIT_PITCH_PAD overrides.
int64_t pitch_pad() {
    static const int64_t p = [] {
        int64_t x = env_int("HSDLA_DIGIT_PITCH_PAD", 128);
        if (x < 0 || x > 4096) x = 128;
        return (x + 15) / 16 * 16;
    }();
    return p;
}

// box_rows: rows of a TMA box (kTileM; 64 for the right operand of half-width pair tiles)
int make_map(DigitOperand &d, int s, int box_rows = kTileM, CUtensorMap *dst = nullptr) {
    PFN_encodeTiled enc = get_encode();
    if (!enc) { g_oz_err = "cuTensorMapEncodeTiled unavailable"; return HSDLA_ERR_CUDA; }
    if (d.Kpad % 128 != 0 || d.pitch % 16 != 0 || d.pitch < d.Kpad ||
        (reinterpret_cast<uintptr_t>(d.digits) & 255) != 0) {
        g_oz_err = "digit operand misaligned";
        return HSDLA_ERR_ARG;
    }
    const int64_t rows = d.plane_rows * 2 * s;
    if (rows > INT32_MAX || d.Kpad > INT32_MAX) { g_oz_err = "digit operand too large for TMA"; return HSDLA_ERR_UNSUPPORTED; }
    cuuint64_t dims[2] = {(cuuint64_t)d.Kpad, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)d.pitch};
    cuuint32_t box[2] = {(cuuint32_t)kKBlock, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(dst ? dst : &d.map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, d.digits, dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { g_oz_err = "cuTensorMapEncodeTiled failed"; return HSDLA_ERR_CUDA; }
    return HSDLA_OK;
}

int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

// Bump allocator over the caller's workspace.
struct Arena {
    char *p;
    int64_t used = 0;
    template <typename T>
    T *take(int64_t count) {
        T *r = reinterpret_cast<T *>(p + used);
        used += round_up((int64_t)sizeof(T) * count, 1024);
        return r;
    }
};

// planes: digit planes (2s; 4s with the 2^-5-scaled copies of a merged-unit left operand)
int64_t operand_bytes(int s, int64_t rows, int64_t Kpad, int planes = 0) {
    const int64_t pr = round_up(rows, kTileM) + kTileM;
    return round_up((planes ? planes : 2 * s) * pr * (Kpad + pitch_pad()), 1024) + round_up(4 * pr, 1024);
}

void carve_operand(Arena &a, DigitOperand &d, int s, int64_t rows, int64_t Kpad, int planes = 0) {
    d.plane_rows = round_up(rows, kTileM) + kTileM;
    d.Kpad = Kpad;
    d.pitch = Kpad + pitch_pad();
    d.digits = a.take<uint8_t>((planes ? planes : 2 * s) * d.plane_rows * d.pitch);
    d.expo = a.take<int32_t>(d.plane_rows);
}

SliceTab slice_table(const double2 *Z, int64_t ldz, const double *v, int64_t Kin, int64_t ncols, int64_t rpb,
                     int64_t bpad, int s, const DigitOperand &d) {
    SliceTab t;
    t.nk = 1; t.s = s; t.ldz = ldz; t.Kin = Kin; t.rpb = rpb; t.bpad = bpad; t.v = v;
    t.digits = d.digits; t.Kpad = d.Kpad; t.plane_rows = d.plane_rows; t.pitch = d.pitch; t.expo = d.expo;
    t.e[0] = SliceEntry{Z, ncols, 0};
    return t;
}

cudaError_t slice_launch(const SliceTab &t, cudaStream_t st) {
    if (t.digits2 && t.scaled) oz_slice_kernel<true, true><<<(unsigned)t.plane_rows, kSliceThreads, 0, st>>>(t);
    else if (t.digits2) oz_slice_kernel<true, false><<<(unsigned)t.plane_rows, kSliceThreads, 0, st>>>(t);
    else if (t.scaled) oz_slice_kernel<false, true><<<(unsigned)t.plane_rows, kSliceThreads, 0, st>>>(t);
    else oz_slice_kernel<false, false><<<(unsigned)t.plane_rows, kSliceThreads, 0, st>>>(t);
    return cudaGetLastError();
}

cudaError_t slice(const double2 *Z, int64_t ldz, const double *v, int64_t Kin, int64_t ncols, int64_t rpb,
                  int64_t bpad, int s, DigitOperand &d, cudaStream_t st) {
    return slice_launch(slice_table(Z, ldz, v, Kin, ncols, rpb, bpad, s, d), st);
}

int64_t job_tiles(const OzJob &j, int64_t tile = kTileM) {
    const int64_t tm = (j.m + tile - 1) / tile, tn = (j.n + tile - 1) / tile;
    return j.lower ? tm * (tm + 1) / 2 : tm * tn;
}

// The S/H launch runs on CTA pairs (256 x 256 tiles) unless HSDLA_PAIR=0.
bool use_pair() {
    static const bool b = env_int("HSDLA_PAIR", 1) != 0;
    return b;
}

// Accumulation units of a pair launch (see PairUnits).  Diagonals t and t + 1 share a unit when
// the left operand carries the 2^-5-scaled planes, each fits one K-chunk, and either the sum
// stays exact -- every partial sum a multiple of 2^-5 below 2^19, with |sum| <= K x 2 (re/im) x
// 256 (|product|) x (n_t + n_{t+1} / 32), K the contraction bytes that can hold nonzero digits
// (kvalid, at most nkb 128: the slicer writes zero digits past 2L in each type's k-blocks, so the
// per-type products of lmax 8 (2L = 162) count 162, not 256) -- or t >= kLooseT, where even an FP32
// rounding (2^-24 of the sum) stays far below the result's FP64 precision.  The low-order
// diagonals are not small everywhere: in a Gram element (S_gg) the products d_p(M_k) d_p(W_k) of
// rows with w_k = 1 add up with one sign, so diagonal 2p carries ~K 2^8 2^(2-10p) whatever the
// size of S_gg -- from t = 9 on below 2^-26 of S_gg, and exact here anyway (|sum| ~ 2^14).
constexpr int kLooseT = 9;
PairUnits pair_units(int s, int64_t nkb, bool merge, int64_t kvalid = 0) {
    PairUnits p;
    memset(&p, 0, sizeof(p));
    auto pairs = [&](int t) { return std::min(s, t - 1) - std::max(1, t - s) + 1; };
    const int64_t K = kvalid > 0 ? std::min(kvalid, nkb * kKBlock) : nkb * kKBlock;
    for (int t = 2; t <= s + 1;) {
        bool m = false;
        if (merge && t + 1 <= s + 1 && chunk_kblocks(pairs(t)) >= nkb && chunk_kblocks(pairs(t + 1)) >= nkb) {
            const int64_t bound = K * 2 * 256;
            m = t >= kLooseT || bound * (32 * pairs(t) + pairs(t + 1)) <= ((int64_t)1 << 24);
        }
        p.t[p.n] = (int8_t)t;
        p.flags[p.n] = m ? kUnitMerged : 0;
        ++p.n;
        t += m ? 2 : 1;
    }
    return p;
}
PairUnits pair_units_plain(int s) { return pair_units(s, 0, false); }

// Host-built tile schedule.  Persistent CTAs take tiles g, g + grid, ... so tiles that are
// close in the list run at the same time and share their operand panels in L2.  Lower-
// triangle jobs of equal size (S and H of one k-point) are walked together in square super-
// blocks of super_block() tiles, the jobs' tiles of one (tm, tn) adjacent (they share the
// left operand); full jobs (T application) go job by job, tile columns outermost.
// Super-block edge in tiles; HSDLA_SCHED_SUPERBLOCK overrides (0 = row-major over the whole
// triangle).  With the CTAs in lockstep, 8 x 8 super-blocks cut the S/H launch of the
// 8000-column FLAPW workload from 378 ms (row-major) to 355 ms: a wave then reads ~16 left and
// ~16 right panels instead of ~2 left and ~120 right ones.
// On 256 x 256 pair tiles the default edge is 4 (the same panel span).
int64_t super_block(int64_t tile) {
    static const int64_t b = env_int("HSDLA_SCHED_SUPERBLOCK", 0);
    if (b < 0) return (int64_t)1 << 30;
    if (b > 0) return b;
    return tile == kTileN ? 8 : 4;
}

void build_schedule(const std::vector<OzJob> &jobs, std::vector<int4> &list, int64_t tile = kTileN) {
    const int64_t kSuperBlock = super_block(tile);
    list.clear();
    std::vector<char> done(jobs.size(), 0);
    for (size_t a = 0; a < jobs.size(); ++a) {
        if (done[a]) continue;
        const OzJob &ja = jobs[a];
        if (ja.lower) {
            std::vector<int> group;
            for (size_t b = a; b < jobs.size(); ++b)
                if (!done[b] && jobs[b].lower && jobs[b].n == ja.n) { group.push_back((int)b); done[b] = 1; }
            const int64_t T = (ja.n + tile - 1) / tile;
            for (int64_t I = 0; I < T; I += kSuperBlock)
                for (int64_t J = 0; J <= I; J += kSuperBlock)
                    for (int64_t tm = I; tm < std::min(T, I + kSuperBlock); ++tm)
                        for (int64_t tn = J; tn < std::min(tm + 1, J + kSuperBlock); ++tn)
                            for (int g : group) list.push_back(make_int4(g, (int)tm, (int)tn, 0));
        } else {
            done[a] = 1;
            const int64_t tmn = (ja.m + tile - 1) / tile, tnn = (ja.n + tile - 1) / tile;
            for (int64_t tn = 0; tn < tnn; ++tn)
                for (int64_t tm = 0; tm < tmn; ++tm) list.push_back(make_int4((int)a, (int)tm, (int)tn, 0));
        }
    }
}

constexpr int kProgressCap = 1024;   // progress slots (>= SM count, multiple of 4)
// Streamed host output: the S/H launches of all types are cut into at most kMaxOutBlocks launches
// of whole waves of pair tiles; the tiles are ordered by kOutColumnBlocks column blocks (of about
// equal tile counts), so that the columns a launch completes are combined and sent to the host
// while the next launch runs.  Only the part completed by the last launch stays exposed.
constexpr int kMaxOutBlocks = 8;
constexpr int kOutColumnBlocks = 8;

int launch_gemm(std::vector<OzJob> &jobs, const CUtensorMap *maps, int s, int *d_err, OzJob *d_jobs,
                cudaStream_t st, cudaEvent_t ev0 = nullptr, cudaEvent_t ev1 = nullptr, int4 *d_list = nullptr,
                int *d_progress = nullptr) {
    int64_t total = 0;
    for (auto &j : jobs) {
        j.tiles_n = (j.n + kTileN - 1) / kTileN;
        j.tile_begin = total;
        total += job_tiles(j);
    }
    if (total == 0) return HSDLA_OK;
    cudaError_t e = cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(OzJob) * jobs.size(), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    std::vector<int4> list;
    if (d_list) {
        build_schedule(jobs, list);
        if ((int64_t)list.size() != total) { g_oz_err = "tile schedule size mismatch"; return HSDLA_ERR_ARG; }
        e = cudaMemcpyAsync(d_list, list.data(), sizeof(int4) * list.size(), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    }
    const size_t smem = (size_t)kStages * kStageBytes + 1024;
    e = cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t grid = std::min<int64_t>(total, nsm);
    // lockstep needs every CTA resident at once: cooperative launch, one CTA per SM
    const bool lockstep = d_progress != nullptr && grid > 1 && grid <= kProgressCap && env_int("HSDLA_LOCKSTEP", 1) != 0;
    if (lockstep) {
        const int64_t g4 = (grid + 3) / 4 * 4;
        e = cudaMemsetAsync(d_progress, 0, sizeof(int) * grid, st);
        if (e == cudaSuccess && g4 > grid) e = cudaMemsetAsync(d_progress + grid, 0x7F, sizeof(int) * (g4 - grid), st);
        if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    }
    if (ev0) cudaEventRecord(ev0, st);
    if (lockstep) {
        CUtensorMap m0 = maps[0], m1 = maps[1], m2 = maps[2], m3 = maps[3];
        const OzJob *pj = d_jobs;
        int nj = (int)jobs.size();
        int64_t tt = total;
        int ss = s;
        int *perr = d_err;
        const int4 *pl = d_list;
        int *pp = d_progress;
        void *args[] = {&m0, &m1, &m2, &m3, &pj, &nj, &tt, &ss, &perr, &pl, &pp};
        e = cudaLaunchCooperativeKernel((const void *)oz_gemm_kernel, dim3((unsigned)grid), dim3(kThreads), args, smem, st);
    } else {
        oz_gemm_kernel<<<(unsigned)grid, kThreads, smem, st>>>(maps[0], maps[1], maps[2], maps[3], d_jobs,
                                                                (int)jobs.size(), total, s, d_err, d_list, nullptr);
        e = cudaGetLastError();
    }
    if (ev1) cudaEventRecord(ev1, st);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    // the job table is read by the kernel: keep the host copy alive until it is consumed
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    return HSDLA_OK;
}

// ------------------------------------------------------------ wait self-test
// Exercises the bounded-wait and abort path of the product kernels on a condition that never
// comes true, with a short budget: the CTA holds TMEM as the product kernels do, one thread
// waits on an mbarrier nothing arrives on (which = 0) or on a lockstep slot that never advances
// (which = 1), the wait records the error word and raises the abort flag, and the CTA frees TMEM
// and returns.  Nothing faults, traps or hangs.
__global__ void __launch_bounds__(64, 1) oz_wait_probe_kernel(int *err, int *progress, long long budget, int which) {
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_sh;
    __shared__ volatile int abort_flag;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;\n" ::"r"(smem_u32(&tmem_sh))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x == 0) {
        if (which == 0) mbar_wait(&bar, 0, &abort_flag, err, 7, budget);
        else grid_lockstep(progress, 4, 3, &abort_flag, err, 0, 1, budget);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;\n" ::"r"(tmem_sh) : "memory");
    }
}

}  // namespace

int ozaki_wait_selftest(OzakiPlan &oz, int which, long long budget_cycles, cudaStream_t st) {
    if (!oz.d_error) { g_oz_err = "Ozaki plan not initialised"; return HSDLA_ERR_ARG; }
    if (which < 0 || which > 1 || budget_cycles <= 0 || budget_cycles > kWaitCycles) {
        g_oz_err = "wait self-test: which must be 0 or 1, budget in (0, 2e9] cycles";
        return HSDLA_ERR_ARG;
    }
    // progress slots for which = 1: slot 0 is this CTA, slots 1..3 stay at epoch 0
    int *progress = oz.d_error + 8;
    cudaError_t e = cudaMemsetAsync(progress, 0, 4 * sizeof(int), st);
    if (e == cudaSuccess) {
        oz_wait_probe_kernel<<<1, 64, 0, st>>>(oz.d_error, progress, budget_cycles, which);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    return ozaki_check_device_error(oz);
}

namespace {

}  // namespace

// ==================================================================== API
int ozaki_plan_init(OzakiPlan &oz, int num_slices, double target) {
    if (num_slices == 0) num_slices = kOzDefaultSlices;
    if (num_slices < 2 || num_slices > kOzMaxSlices) { g_oz_err = "num_slices outside [2, 12]"; return HSDLA_ERR_ARG; }
    oz.num_slices = num_slices;
    oz.target = target;
    if (!oz.d_error) {
        if (cudaMalloc(&oz.d_error, kErrAlloc * sizeof(int)) != cudaSuccess) { g_oz_err = "cudaMalloc"; return HSDLA_ERR_NOMEM; }
        cudaMemset(oz.d_error, 0, kErrAlloc * sizeof(int));
    }
    return HSDLA_OK;
}

void ozaki_plan_release(OzakiPlan &oz) {
    if (oz.d_error) cudaFree(oz.d_error);
    oz.d_error = nullptr;
}

int ozaki_check_device_error(OzakiPlan &oz) {
    if (!oz.d_error) return HSDLA_OK;
    int w[kErrWords] = {};
    if (cudaMemcpy(w, oz.d_error, sizeof(w), cudaMemcpyDeviceToHost) != cudaSuccess) return HSDLA_ERR_CUDA;
    const int h = w[0];
    if (h != 0) {
        static thread_local char buf[192];
        snprintf(buf, sizeof(buf),
                 "device wait expired (code %d, role %d; block %d rank %d stage %d phase %d count %d)", h / 16,
                 h % 16, w[1], w[2], w[3], w[4], w[5]);
        g_oz_err = buf;
        cudaMemset(oz.d_error, 0, sizeof(w));
        return h / 16 == kDevBadInput ? HSDLA_ERR_CUDA : HSDLA_ERR_TIMEOUT;
    }
    return HSDLA_OK;
}

int64_t schedule_capacity_lower(int64_t n) {
    const int64_t T = (n + kTileN - 1) / kTileN;
    return T * (T + 1);                                     // two lower-triangle jobs
}

int64_t ozaki_herkx_workspace(int s, int64_t K, int64_t n) {
    const int64_t Kpad = round_up(std::max<int64_t>(K, 1), kKBlock);
    return 2 * operand_bytes(s, n, Kpad) + 4096 + 4096 + round_up(sizeof(int4) * schedule_capacity_lower(n), 1024) +
           round_up(sizeof(int) * kProgressCap, 1024);
}

// ---------------------------------------------------------------- k-point groups
// A group is a set of k-points whose digit operands are resident together.  Its digit planes
// stack the k-points' columns as consecutive rows, so one tensor map per operand covers every
// k-point, one slicing launch per operand covers the group, and one oz_gemm launch runs the T
// application and one the S/H products of all k-points.  Everything but the output pointers
// is prepared once; a run only enqueues launches (it can be captured in a CUDA graph).
// One atom panel of a group: the contraction index split by atoms, each panel sliced with its own
// exponents and its S/H products accumulated into the outputs.
struct OzPanel {
    int64_t a0 = 0, a1 = 0;            // atoms [a0, a1)
    SliceTab tC, tX;                   // tC is dual: C and W
    int64_t jt_off = 0, lt_off = 0;    // this panel's T-application jobs / tiles (non-hoisted)
    int n_jobs_t = 0;
    int64_t tiles_t = 0;
};

struct OzGroup {
    int s = 0, nk = 0, panels = 1;
    bool hoist = false;
    int64_t twoL = 0, na = 0, nt = 0, K = 0, bpad = 0, rows = 0;
    std::vector<OzKBufs> kb;
    std::vector<int64_t> row0;
    std::vector<OzPanel> pan;
    DigitOperand dC, dW, dX, dM, dT;
    SliceTab tM;
    CUtensorMap maps_t[4], maps_sh[4];
    OzJob *d_jobs_t = nullptr, *d_jobs_sh = nullptr, *h_jobs_sh = nullptr;
    int n_jobs_t = 0, n_jobs_sh = 0;   // hoisted T jobs; S/H jobs per panel (2 per k-point)
    int4 *d_list_t = nullptr, *d_list_sh = nullptr;
    int64_t tiles_t = 0, tiles_sh = 0;
    int *d_progress = nullptr;
    int *d_err = nullptr;
    bool pair = false;          // S/H on CTA-pair tiles
    PairUnits units{};          // their accumulation units
    PairUnits units_t{};        // the T application's (structure-factor form on pair tiles)
    int halves = 1;             // 2: structure-factor S/H launches on half-width pair tiles
    int halves_t = 1;           // the same for the T application
    bool merged = true;         // S/H units merge adjacent digit diagonals where exact
    bool sf = false;            // structure-factor form
    int tbatch = 1;             // its types per combine batch
    // with one batch: the first side_types types are combined on a side stream while the S/H
    // launches of the others run (the combine is FP64-bound, the products tensor-bound)
    int side_types = 0;
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    SfTab sft{};                // its combine table (outputs patched per run)
    const double2 *sf_tab = nullptr;
    // Streamed host output (structure-factor form on pair tiles, every type in one combine batch):
    // the S/H products of all types in column blocks, one launch per block, each block combined
    // into the caller's page-locked outputs on blk_side while the next block's products run.
    // Block b covers tile-list entries [blk_begin[b], blk_begin[b+1]) of d_list_blk and output
    // columns [blk_col[b], blk_col[b+1]).
    int nblk = 0;
    int64_t blk_begin[kMaxOutBlocks + 1] = {};
    int64_t blk_col[kMaxOutBlocks + 1] = {};
    int4 *d_list_blk = nullptr;
    cudaStream_t blk_side = nullptr;
    cudaEvent_t ev_blk[kMaxOutBlocks] = {};
    cudaEvent_t ev_blk_join = nullptr;
};

namespace {

int64_t group_rows(const std::vector<int64_t> &G) {
    int64_t r = 0;
    for (int64_t g : G) r += round_up(std::max<int64_t>(g, 1), kTileM);
    return r + kTileM;
}

int upload_schedule(std::vector<OzJob> &jobs, OzJob *d_jobs, int4 *d_list, int64_t &tiles, int64_t tile = kTileN) {
    int64_t total = 0;
    for (auto &j : jobs) {
        j.tiles_n = (j.n + tile - 1) / tile;
        j.tile_begin = total;
        total += job_tiles(j, tile);
    }
    std::vector<int4> list;
    build_schedule(jobs, list, tile);
    if ((int64_t)list.size() != total) { g_oz_err = "tile schedule size mismatch"; return HSDLA_ERR_ARG; }
    cudaError_t e = cudaMemcpy(d_jobs, jobs.data(), sizeof(OzJob) * jobs.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && total > 0)
        e = cudaMemcpy(d_list, list.data(), sizeof(int4) * list.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    tiles = total;
    return HSDLA_OK;
}

// Launch of a prepared pair-tile job table: clusters of two CTAs, one per SM, as many pairs as
// can be resident (at most one per tile); cooperative when the lockstep slots are given.
template <int kHalves>
cudaError_t launch_pair_t(const CUtensorMap *maps, int s, int *d_err, const OzJob *d_jobs, int n_jobs, int64_t total,
                          const int4 *d_list, int *d_progress, cudaStream_t st, const PairUnits &units) {
    if (total <= 0) return cudaSuccess;
    const size_t smem = PairShape<kHalves>::kSmem;
    cudaError_t e = cudaFuncSetAttribute(oz_pair_kernel<kHalves>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kPairThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    static int max_pairs = 0;
    if (max_pairs == 0) {
        cfg.gridDim = dim3(2);
        int nc = 0;
        e = cudaOccupancyMaxActiveClusters(&nc, (const void *)oz_pair_kernel<kHalves>, &cfg);
        if (e != cudaSuccess) return e;
        if (nc < 1) return cudaErrorInvalidConfiguration;
        max_pairs = nc;
    }
    const int64_t pairs = std::min<int64_t>(total, max_pairs);
    cfg.gridDim = dim3((unsigned)(2 * pairs));
    const bool lockstep = d_progress && pairs > 1 && pairs <= kProgressCap && env_int("HSDLA_LOCKSTEP", 1) != 0;
    if (lockstep) {
        const int64_t g4 = (pairs + 3) / 4 * 4;
        e = cudaMemsetAsync(d_progress, 0, sizeof(int) * pairs, st);
        if (e == cudaSuccess && g4 > pairs) e = cudaMemsetAsync(d_progress + pairs, 0x7F, sizeof(int) * (g4 - pairs), st);
        if (e != cudaSuccess) return e;
        // cooperative: the launch waits until every pair can be resident (the lockstep needs
        // that); HSDLA_COOPERATIVE=0 drops the attribute for profilers that cannot replay a
        // cooperative cluster launch (on an otherwise idle GPU the grid is resident anyway, and
        // the lockstep waits stay bounded)
        if (env_int("HSDLA_COOPERATIVE", 1) != 0) {
            at[1].id = cudaLaunchAttributeCooperative;
            at[1].val.cooperative = 1;
            cfg.numAttrs = 2;
        }
    }
    // lockstep epoch (stages) and how many epochs a pair may lead the slowest one
    static const int sync_every = (int)std::max<int64_t>(8, env_int("HSDLA_SYNC_EVERY", kSyncEvery));
    static const int slack = (int)std::max<int64_t>(1, env_int("HSDLA_SYNC_SLACK", 1));
    return cudaLaunchKernelEx(&cfg, oz_pair_kernel<kHalves>, maps[0], maps[1], maps[2], maps[3], d_jobs, n_jobs, total,
                              s, d_err, d_list, lockstep ? d_progress : (int *)nullptr, sync_every, slack, units);
}

// halves = 2: the half-width tiles, whose right-operand maps (maps[j.rmap] of every job) must have
// 64-row boxes (make_map(.., kPairTile / 4)); 1: 128-row boxes.
cudaError_t launch_pair(const CUtensorMap *maps, int s, int *d_err, const OzJob *d_jobs, int n_jobs, int64_t total,
                        const int4 *d_list, int *d_progress, cudaStream_t st, const PairUnits &units, int halves = 1) {
    return halves == 2 ? launch_pair_t<2>(maps, s, d_err, d_jobs, n_jobs, total, d_list, d_progress, st, units)
                       : launch_pair_t<1>(maps, s, d_err, d_jobs, n_jobs, total, d_list, d_progress, st, units);
}

// Launch of a prepared job table (no host synchronisation; capturable).
cudaError_t launch_prepared(const CUtensorMap *maps, int s, int *d_err, const OzJob *d_jobs, int n_jobs,
                            int64_t total, const int4 *d_list, int *d_progress, cudaStream_t st) {
    if (total <= 0) return cudaSuccess;
    const size_t smem = (size_t)kStages * kStageBytes + 1024;
    cudaError_t e = cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t grid = std::min<int64_t>(total, nsm);
    const bool lockstep = d_progress && grid > 1 && grid <= kProgressCap && env_int("HSDLA_LOCKSTEP", 1) != 0;
    if (lockstep) {
        const int64_t g4 = (grid + 3) / 4 * 4;
        e = cudaMemsetAsync(d_progress, 0, sizeof(int) * grid, st);
        if (e == cudaSuccess && g4 > grid) e = cudaMemsetAsync(d_progress + grid, 0x7F, sizeof(int) * (g4 - grid), st);
        if (e != cudaSuccess) return e;
        CUtensorMap m0 = maps[0], m1 = maps[1], m2 = maps[2], m3 = maps[3];
        const OzJob *pj = d_jobs;
        int nj = n_jobs;
        int64_t tt = total;
        int ss = s;
        int *perr = d_err;
        const int4 *pl = d_list;
        int *pp = d_progress;
        void *args[] = {&m0, &m1, &m2, &m3, &pj, &nj, &tt, &ss, &perr, &pl, &pp};
        return cudaLaunchCooperativeKernel((const void *)oz_gemm_kernel, dim3((unsigned)grid), dim3(kThreads), args,
                                           smem, st);
    }
    oz_gemm_kernel<<<(unsigned)grid, kThreads, smem, st>>>(maps[0], maps[1], maps[2], maps[3], d_jobs, n_jobs, total,
                                                            s, d_err, d_list, nullptr);
    return cudaGetLastError();
}

}  // namespace

// P^H diag(w) Q (lower triangle) for one pair of K x n operands: the contraction behind
// hsdla_zherkx_lower and the BLAS-shaped plugin.
int ozaki_herkx(OzakiPlan &oz, const double2 *P, int64_t ldp, const double2 *Q, int64_t ldq, const double *w,
                int64_t K, int64_t n, double2 *out, int64_t ldo, void *ws, cudaStream_t st, int *launches) {
    const int s = oz.num_slices;
    const int64_t Kpad = round_up(std::max<int64_t>(K, 1), kKBlock);
    Arena ar{reinterpret_cast<char *>(ws)};
    DigitOperand dp, dq;
    carve_operand(ar, dp, s, n, Kpad);
    carve_operand(ar, dq, s, n, Kpad);
    OzJob *d_jobs = ar.take<OzJob>(4);
    int4 *d_list = ar.take<int4>(schedule_capacity_lower(n));
    cudaError_t e = slice(P, ldp, nullptr, K, n, Kpad, Kpad, s, dp, st);
    if (e == cudaSuccess) e = slice(Q, ldq, w, K, n, Kpad, Kpad, s, dq, st);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    int rc = make_map(dp, s);
    if (!rc) rc = make_map(dq, s);
    if (rc) return rc;
    CUtensorMap maps[4] = {dp.map, dq.map, dp.map, dp.map};
    std::vector<OzJob> jobs(1);
    OzJob &j = jobs[0];
    memset(&j, 0, sizeof(j));
    j.lmap = 0; j.rmap = 1; j.lower = 1;
    j.lplane = dp.plane_rows; j.rplane = dq.plane_rows;
    j.nkb = Kpad / kKBlock; j.m = n; j.n = n;
    j.out = out; j.ldo = ldo; j.el = dp.expo; j.er = dq.expo;
    if (use_pair()) {
        // CTA-pair 256 x 256 tiles with 256 x 256 accumulators, one exact unit per diagonal and
        // K chunk (no merged units: the left operand has no scaled planes), pairs in lockstep
        int *d_progress = ar.take<int>(kProgressCap);
        int64_t tiles = 0;
        rc = upload_schedule(jobs, d_jobs, d_list, tiles, kPairTile);
        if (rc) return rc;
        const cudaError_t el = launch_pair(maps, s, oz.d_error, d_jobs, 1, tiles, d_list, d_progress, st,
                                           pair_units(s, j.nkb, false), 1);
        if (el != cudaSuccess) { g_oz_err = cudaGetErrorString(el); return HSDLA_ERR_CUDA; }
    } else {
        rc = launch_gemm(jobs, maps, s, oz.d_error, d_jobs, st, nullptr, nullptr, d_list);
    }
    if (launches) *launches = 3;
    return rc;
}

// Run-time scratch of a group (digit planes and exponents, rewritten by every run; groups of a
// plan share it) and its persistent part (T digits, job tables, tile schedules, lockstep slots).
static int64_t panel_atoms(int64_t na, int panels) { return (na + panels - 1) / panels; }
// Stride of one atom's 2L rows along the contraction index of the digit planes: 16 bytes keeps
// every atom's block on a TMA boundary (the T application starts its loads there).  A T job reads
// ceil(2L / 128) k-blocks from that start; the rows past 2L it covers (padding and the next atoms)
// meet T digits that are exactly zero, and reads past the operand's extent are zero-filled.
static int64_t atom_stride(int64_t twoL) { return round_up(twoL, 16); }

int64_t ozaki_group_bytes(int s, int64_t twoL, int64_t na, int64_t nt, const std::vector<int64_t> &G, int panels,
                          bool hoist, bool sf) {
    const int64_t bpad = atom_stride(twoL), rows = group_rows(G);
    if (sf) {      // M (with its scaled copy on pair tiles), M diag(w_t) and Z digits: each
                   // type's rows on whole k-blocks
        const int64_t KT = round_up(twoL, kKBlock) * nt;
        auto dig = [&](int64_t planes) {
            return round_up(planes * rows * (KT + pitch_pad()), 1024) + round_up(4 * rows, 1024);
        };
        return dig((use_pair() ? 4 : 2) * s) + 2 * dig(2 * s) + 4096;
    }
    const int64_t Kp = round_up(bpad * panel_atoms(na, panels), kKBlock);
    const int64_t Kx = hoist ? std::max(Kp, round_up(bpad * nt, kKBlock)) : Kp;
    auto dig = [&](int64_t K) { return round_up(2 * s * rows * (K + pitch_pad()), 1024) + round_up(4 * rows, 1024); };
    return 2 * dig(Kp) + dig(Kx) + 4096;
}

int64_t ozaki_group_persist_bytes(int s, int64_t twoL, int64_t na, int64_t nt, const std::vector<int64_t> &G,
                                  int panels) {
    const int64_t bpad = round_up(atom_stride(twoL), kKBlock);    // T operand: one atom's rows per plane row
    const int64_t nk = (int64_t)G.size();
    int64_t tiles_t = 0, tiles_sh = 0, tiles_blk = 0;
    for (int64_t g : G) {
        const int64_t T = (g + kTileN - 1) / kTileN, Tp = (g + kPairTile - 1) / kPairTile;
        tiles_t += std::max(na, nt) * ((twoL + kTileM - 1) / kTileM) * T;
        tiles_sh += T * (T + 1);
        tiles_blk += Tp * (Tp + 1);
    }
    return operand_bytes(s, nt * twoL, bpad, use_pair() ? 4 * s : 2 * s) +
           round_up(sizeof(OzJob) * nk * (std::max(na, nt) + 2), 1024) +
           round_up(sizeof(OzJob) * 2 * nk * panels, 1024) + round_up(sizeof(int4) * (tiles_t + panels), 1024) +
           round_up(sizeof(int4) * (tiles_sh + 1), 1024) + round_up(sizeof(int) * kProgressCap, 1024) +
           round_up(sizeof(int4) * (nt * tiles_blk + 1), 1024) + 8192;
}

// The streamed host output's launches (pair tiles).  The tile columns are split into
// kOutColumnBlocks ranges of about equal lower-triangle tile counts; the tile list runs through
// them in order, and within a range type by type, each type in the per-type schedule's order (so
// that the pairs working at a time share few types' operands in L2).  The list is then cut into
// launches of whole waves (one tile per cluster pair of the GPU); launch b leaves columns
// [blk_col[b], blk_col[b+1]) complete (possibly none).  jobs0: the first type's S/H jobs.
static int build_output_blocks(OzGroup *g, const std::vector<OzJob> &jobs0, int64_t tile) {
    std::vector<int4> l0;
    build_schedule(jobs0, l0, tile);
    int64_t T = 0;
    for (const auto &j : jobs0) T = std::max<int64_t>(T, (j.n + tile - 1) / tile);
    g->nblk = 0;
    if (T < 2) return HSDLA_OK;
    const int C = (int)std::min<int64_t>(kOutColumnBlocks, T);
    const int64_t total = T * (T + 1) / 2;
    std::vector<int64_t> cb(C + 1, T);
    cb[0] = 0;
    int64_t acc = 0, c = 0;
    for (int b = 1; b < C; ++b) {
        while (c < T && acc < total * b / C) { acc += T - c; ++c; }
        cb[b] = c;
    }
    std::vector<int4> lb;
    lb.reserve(l0.size() * g->nt);
    for (int b = 0; b < C; ++b)
        for (int t = 0; t < g->nt; ++t)
            for (const int4 &e : l0)
                if (e.z >= cb[b] && e.z < cb[b + 1]) lb.push_back(make_int4(t * g->n_jobs_sh + e.x, e.y, e.z, 0));
    const int64_t N = (int64_t)lb.size();
    if (N != (int64_t)l0.size() * g->nt) { g_oz_err = "output block schedule size mismatch"; return HSDLA_ERR_ARG; }
    // first incomplete tile column after list position i: suffix minimum of the tile columns
    std::vector<int64_t> open(N + 1, T);
    for (int64_t i = N - 1; i >= 0; --i) open[i] = std::min<int64_t>(open[i + 1], lb[i].z);
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t wave = std::max(1, nsm / 2);
    const int64_t waves = (N + wave - 1) / wave;
    const int64_t per = std::max<int64_t>(1, (waves + kMaxOutBlocks - 1) / kMaxOutBlocks) * wave;
    g->blk_begin[0] = 0;
    g->blk_col[0] = 0;
    for (int64_t i0 = 0; i0 < N && g->nblk < kMaxOutBlocks; ++g->nblk) {
        const int64_t i1 = g->nblk + 1 == kMaxOutBlocks ? N : std::min(N, i0 + per);
        g->blk_begin[g->nblk + 1] = i1;
        g->blk_col[g->nblk + 1] = std::max(g->blk_col[g->nblk], open[i1] * tile);
        i0 = i1;
    }
    g->blk_col[g->nblk] = T * tile;
    const cudaError_t e = cudaMemcpy(g->d_list_blk, lb.data(), sizeof(int4) * N, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    return HSDLA_OK;
}

// Structure-factor form of a group: digit planes of M, M diag(w_t) and Z (2L rows per type, each
// type's rows starting on a k-block so that the per-type products never mix types), the T
// application Z_t = T_t M_t, and per type one S/H launch into the products PS, PH followed by the
// combine into S and H.
static int group_prepare_sf(OzakiPlan &oz, const OzGroupDesc &d, const std::vector<OzKBufs> &kb, void *ws,
                            void *persist, cudaStream_t st, OzGroup **out) {
    auto *g = new OzGroup();
    g->sf = true;
    g->s = oz.num_slices;
    g->nk = (int)kb.size();
    g->hoist = true;
    g->twoL = d.twoL; g->na = d.na; g->nt = d.nt;
    // type stride along the contraction: whole 128-byte k-blocks (TMA boxes aligned to them; a
    // 32-byte stride for lmax 8 put every other type's boxes across 128-byte lines: c3 10.3 -> 12.4 ms)
    g->pair = use_pair();
    g->bpad = round_up(d.twoL, kKBlock);
    const int64_t tkb = g->bpad / kKBlock, KT = g->bpad * d.nt;
    // K steps of 32 bytes in a type's last k-block (the contraction length is 2L per type)
    const int ksl = (int)((d.twoL - (tkb - 1) * kKBlock + 31) / 32);
    g->kb = kb;
    g->d_err = oz.d_error;
    g->sf_tab = d.sf_tab;
    g->tbatch = std::max(1, d.tbatch);
    // HSDLA_COMBINE_OVERLAP=1: the first half of the combine on a side stream, next to the S/H
    // launches of the other types.  Off by default: on the 8000-column workload the co-running
    // combine slowed the S/H launches by more than it saved (31.7 against 31.4 ms per k-point).
    if (g->tbatch >= d.nt && d.nt >= 2 && env_int("HSDLA_COMBINE_OVERLAP", 0) != 0) {
        g->side_types = (int)(d.nt / 2);
        if (cudaStreamCreateWithFlags(&g->side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&g->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&g->ev_join, cudaEventDisableTiming) != cudaSuccess) {
            g_oz_err = "side stream creation failed";
            ozaki_group_destroy(g);
            return HSDLA_ERR_CUDA;
        }
    }
    std::vector<int64_t> G;
    for (auto &k : kb) G.push_back(k.G);
    g->rows = group_rows(G);
    int64_t r0 = 0;
    for (int64_t x : G) { g->row0.push_back(r0); r0 += round_up(std::max<int64_t>(x, 1), kTileM); }
    const int s = g->s;
    Arena ar{reinterpret_cast<char *>(ws)};
    Arena keep{reinterpret_cast<char *>(persist)};
    auto carve_rows = [&](DigitOperand &o, int planes) {
        o.plane_rows = g->rows;
        o.Kpad = KT;
        o.pitch = KT + pitch_pad();
        o.digits = ar.take<uint8_t>(planes * o.plane_rows * o.pitch);
        o.expo = ar.take<int32_t>(o.plane_rows);
    };
    // M: the S/H products' left operand; on pair tiles with its digits scaled by 2^-5 as well
    // (planes 2s .. 4s-1), the merged accumulation units' left digits
    carve_rows(g->dM, g->pair ? 4 * s : 2 * s);
    carve_rows(g->dW, 2 * s);    // M diag(w_t)
    carve_rows(g->dX, 2 * s);    // Z
    // T: the left operand of the T application, with its scaled copy on pair tiles
    carve_operand(keep, g->dT, s, d.nt * d.twoL, tkb * kKBlock, g->pair ? 4 * s : 2 * s);
    const int64_t nk = g->nk;
    int64_t tiles_t = 0, tiles_sh = 0;
    for (int64_t x : G) {
        const int64_t T = (x + kTileN - 1) / kTileN;
        tiles_t += d.nt * ((d.twoL + kTileM - 1) / kTileM) * T;
        tiles_sh += T * (T + 1);
    }
    g->d_jobs_t = keep.take<OzJob>(nk * (d.nt + 2));
    g->d_jobs_sh = keep.take<OzJob>(2 * nk * d.nt);
    g->d_list_t = keep.take<int4>(tiles_t + 1);
    g->d_list_sh = keep.take<int4>(tiles_sh + 1);
    g->d_progress = keep.take<int>(kProgressCap);
    int64_t tiles_blk = 0;
    for (int64_t x : G) {
        const int64_t Tp = (x + kPairTile - 1) / kPairTile;
        tiles_blk += Tp * (Tp + 1);
    }
    g->d_list_blk = keep.take<int4>(d.nt * tiles_blk + 1);
    auto fail = [&](int code) { ozaki_group_destroy(g); return code; };
    auto table = [&](const DigitOperand &o, int which) {
        SliceTab t;
        t.nk = g->nk; t.s = s; t.ldz = d.twoL * d.nt; t.Kin = d.twoL * d.nt; t.rpb = d.twoL; t.bpad = g->bpad;
        t.digits = o.digits; t.Kpad = KT; t.plane_rows = o.plane_rows; t.pitch = o.pitch; t.expo = o.expo;
        for (int k = 0; k < g->nk; ++k) t.e[k] = SliceEntry{which == 0 ? kb[k].M : kb[k].Z, kb[k].G, g->row0[k]};
        return t;
    };
    g->tM = table(g->dM, 0);              // dual: M and M diag(w_t)
    g->tM.scaled = g->pair ? 1 : 0;
    g->tM.v2 = d.wt;
    g->tM.digits2 = g->dW.digits;
    g->tM.expo2 = g->dW.expo;
    OzPanel p;                            // one "panel" carries the Z slicing table
    p.a0 = 0; p.a1 = d.na;
    p.tX = table(g->dX, 1);
    g->pan.push_back(p);
    g->panels = 1;
    SliceTab tT = slice_table(d.Tfull, d.twoL, nullptr, d.twoL, d.nt * d.twoL, d.twoL, g->bpad, s, g->dT);
    tT.scaled = g->pair ? 1 : 0;
    cudaError_t e = slice_launch(tT, st);    // stream-ordered before every use of the T digits
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return fail(HSDLA_ERR_CUDA); }
    int rc = make_map(g->dM, g->pair ? 2 * s : s);
    if (!rc) rc = make_map(g->dW, s);
    if (!rc) rc = make_map(g->dX, s);
    if (!rc) rc = make_map(g->dT, g->pair ? 2 * s : s);
    // half-width pair tiles (HSDLA_PAIR_HALVES=1: full width; the tile tuner may switch the S/H
    // launches): the right operands' 64-row maps, made for both shapes
    g->halves = g->pair && env_int("HSDLA_PAIR_HALVES", 2) == 2 ? 2 : 1;
    g->halves_t = g->halves;
    if (!rc && g->pair) rc = make_map(g->dM, 2 * s, kPairTile / 4, &g->dM.map64);
    if (!rc && g->pair) rc = make_map(g->dW, s, kPairTile / 4, &g->dW.map64);
    if (!rc && g->pair) rc = make_map(g->dX, s, kPairTile / 4, &g->dX.map64);
    if (rc) return fail(rc);
    // T application per type: Z_t = T_t M_t
    std::vector<OzJob> jt;
    for (int k = 0; k < g->nk; ++k)
        for (int64_t t = 0; t < d.nt; ++t) {
            OzJob j;
            memset(&j, 0, sizeof(j));
            j.lmap = 3; j.rmap = 0;
            j.lplane = g->dT.plane_rows; j.rplane = g->dM.plane_rows;
            j.lrow0 = t * d.twoL; j.rrow0 = g->row0[k];
            j.rk0 = t * g->bpad;
            j.nkb = tkb;
            j.ksteps_last = ksl;
            j.m = d.twoL; j.n = kb[k].G;
            j.out = kb[k].Z + d.twoL * t; j.ldo = d.twoL * d.nt;
            j.el = g->dT.expo + t * d.twoL; j.er = g->dM.expo + g->row0[k];
            jt.push_back(j);
        }
    g->n_jobs_t = (int)jt.size();
    // on pair tiles (256 x 256: one tile row per type) in merged accumulation units
    rc = upload_schedule(jt, g->d_jobs_t, g->d_list_t, g->tiles_t, g->pair ? kPairTile : kTileN);
    g->units_t = g->pair ? pair_units(s, tkb, env_int("HSDLA_MERGE", 1) != 0, d.twoL) : pair_units_plain(s);
    if (rc) return fail(rc);
    g->maps_t[0] = g->halves_t == 2 ? g->dM.map64 : g->dM.map;  // right operand
    g->maps_t[1] = g->dM.map; g->maps_t[2] = g->dM.map; g->maps_t[3] = g->dT.map;
    // per type: S_t = M_t^H diag(w_t) M_t and H_t = M_t^H Z_t into the products; on pair tiles
    // with merged accumulation units (HSDLA_MERGE=0: one per diagonal)
    g->merged = env_int("HSDLA_MERGE", 1) != 0;
    g->units = g->pair ? pair_units(s, tkb, g->merged, d.twoL) : pair_units_plain(s);
    const int64_t tile = g->pair ? kPairTile : kTileN;
    g->n_jobs_sh = 2 * g->nk;
    std::vector<OzJob> all;
    for (int64_t t = 0; t < d.nt; ++t) {
        std::vector<OzJob> jsh;
        for (int k = 0; k < g->nk; ++k)
            for (int which = 0; which < 2; ++which) {
                OzJob j;
                memset(&j, 0, sizeof(j));
                j.lmap = 0; j.rmap = which == 0 ? 1 : 2; j.lower = 1;
                j.lplane = g->rows; j.rplane = g->rows;
                j.lrow0 = g->row0[k]; j.rrow0 = g->row0[k];
                j.lk0 = t * g->bpad; j.rk0 = t * g->bpad;
                j.nkb = tkb;
                j.ksteps_last = ksl;
                j.m = kb[k].G; j.n = kb[k].G;
                j.out = (which == 0 ? kb[k].PS : kb[k].PH) + (t % g->tbatch) * kb[k].pstride;
                j.ldo = kb[k].G;
                j.el = g->dM.expo + g->row0[k];
                j.er = (which == 0 ? g->dW.expo : g->dX.expo) + g->row0[k];
                jsh.push_back(j);
            }
        if (t == 0) {
            rc = upload_schedule(jsh, g->d_jobs_sh, g->d_list_sh, g->tiles_sh, tile);
            if (rc) return fail(rc);
        } else {
            int64_t total = 0;
            for (auto &j : jsh) {
                j.tiles_n = (j.n + tile - 1) / tile;
                j.tile_begin = total;
                total += job_tiles(j, tile);
            }
        }
        all.insert(all.end(), jsh.begin(), jsh.end());
    }
    e = cudaMemcpy(g->d_jobs_sh, all.data(), sizeof(OzJob) * all.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return fail(HSDLA_ERR_CUDA); }
    if (g->pair) {
        rc = build_output_blocks(g, std::vector<OzJob>(all.begin(), all.begin() + g->n_jobs_sh), tile);
        if (rc) return fail(rc);
    }
    g->maps_sh[0] = g->dM.map;
    g->maps_sh[1] = g->halves == 2 ? g->dW.map64 : g->dW.map;   // right operands
    g->maps_sh[2] = g->halves == 2 ? g->dX.map64 : g->dX.map;
    g->maps_sh[3] = g->dM.map;
    *out = g;
    return HSDLA_OK;
}

int ozaki_group_prepare(OzakiPlan &oz, const OzGroupDesc &d, const std::vector<OzKBufs> &kb, void *ws,
                        void *persist, cudaStream_t st, OzGroup **out) {
    *out = nullptr;
    if (kb.empty() || (int)kb.size() > kMaxGroup) { g_oz_err = "group size out of range"; return HSDLA_ERR_ARG; }
    if (d.panels < 1 || d.panels > d.na) { g_oz_err = "panel count out of range"; return HSDLA_ERR_ARG; }
    if (d.sf) return group_prepare_sf(oz, d, kb, ws, persist, st, out);
    auto *g = new OzGroup();
    g->s = oz.num_slices;
    g->nk = (int)kb.size();
    g->hoist = d.hoist;
    g->twoL = d.twoL; g->na = d.na; g->nt = d.nt;
    g->K = d.twoL * d.na;
    g->bpad = atom_stride(d.twoL);
    const int64_t tkb = (d.twoL + kKBlock - 1) / kKBlock;      // k-blocks of one T application
    g->kb = kb;
    g->d_err = oz.d_error;
    // atom panels: equal sizes but the last
    const int64_t pa = panel_atoms(d.na, d.panels);
    for (int64_t a0 = 0; a0 < d.na; a0 += pa) {
        OzPanel p;
        p.a0 = a0;
        p.a1 = std::min(d.na, a0 + pa);
        g->pan.push_back(p);
    }
    g->panels = (int)g->pan.size();
    std::vector<int64_t> G;
    for (auto &k : kb) G.push_back(k.G);
    g->rows = group_rows(G);
    int64_t r0 = 0;
    for (int64_t x : G) { g->row0.push_back(r0); r0 += round_up(std::max<int64_t>(x, 1), kTileM); }
    const int s = g->s;
    Arena ar{reinterpret_cast<char *>(ws)};
    Arena keep{reinterpret_cast<char *>(persist)};
    auto carve_rows = [&](DigitOperand &o, int64_t kpad) {
        o.plane_rows = g->rows;
        o.Kpad = kpad;
        o.pitch = kpad + pitch_pad();
        o.digits = ar.take<uint8_t>(2 * s * o.plane_rows * o.pitch);
        o.expo = ar.take<int32_t>(o.plane_rows);
    };
    const int64_t Kp = round_up(g->bpad * pa, kKBlock), Km = round_up(g->bpad * d.nt, kKBlock);
    carve_rows(g->dC, Kp);
    carve_rows(g->dW, Kp);
    carve_rows(g->dX, d.hoist ? std::max(Kp, Km) : Kp);
    carve_operand(keep, g->dT, s, d.nt * d.twoL, tkb * kKBlock);
    // the M digits (per-type rows, K = bpad nt) borrow the X digit region: they are consumed by the
    // T application, which runs before any panel's X is sliced
    g->dM.plane_rows = g->rows;
    g->dM.Kpad = Km;
    g->dM.pitch = g->dM.Kpad + pitch_pad();
    g->dM.digits = g->dX.digits;
    g->dM.expo = g->dX.expo;
    const int64_t nk = g->nk;
    int64_t tiles_t = 0, tiles_sh = 0;
    for (int64_t x : G) {
        const int64_t T = (x + kTileN - 1) / kTileN;
        tiles_t += std::max(d.na, d.nt) * ((d.twoL + kTileM - 1) / kTileM) * T;
        tiles_sh += T * (T + 1);
    }
    g->d_jobs_t = keep.take<OzJob>(nk * (std::max(d.na, d.nt) + 2));
    g->d_jobs_sh = keep.take<OzJob>(2 * nk * g->panels);
    g->d_list_t = keep.take<int4>(tiles_t + g->panels);
    g->d_list_sh = keep.take<int4>(tiles_sh + 1);
    g->d_progress = keep.take<int>(kProgressCap);
    int rc = HSDLA_OK;
    auto fail = [&](int code) { ozaki_group_destroy(g); return code; };
    if (cudaHostAlloc((void **)&g->h_jobs_sh, sizeof(OzJob) * 2 * nk * g->panels, cudaHostAllocDefault) !=
        cudaSuccess) {
        g->h_jobs_sh = nullptr;
        g_oz_err = "pinned job table allocation failed";
        return fail(HSDLA_ERR_NOMEM);
    }
    // slicing tables: source rows [a0 2L, a1 2L) of every k-point's column
    auto table = [&](const DigitOperand &o, int64_t ldz, const double *v, int64_t row_off, int64_t Kin, int64_t kpad,
                     int which) {
        SliceTab t;
        t.nk = g->nk; t.s = s; t.ldz = ldz; t.Kin = Kin; t.rpb = d.twoL; t.bpad = g->bpad; t.v = v;
        t.digits = o.digits; t.Kpad = kpad; t.plane_rows = o.plane_rows; t.pitch = o.pitch; t.expo = o.expo;
        for (int k = 0; k < g->nk; ++k) {
            const double2 *src = which == 1 ? kb[k].M : kb[k].CX + row_off;
            t.e[k] = SliceEntry{src, kb[k].G, g->row0[k]};
        }
        return t;
    };
    for (OzPanel &p : g->pan) {
        const int64_t off = p.a0 * d.twoL, Kin = (p.a1 - p.a0) * d.twoL;
        const int64_t kpad = round_up((p.a1 - p.a0) * g->bpad, kKBlock);
        p.tC = table(g->dC, g->K, nullptr, off, Kin, kpad, 0);
        p.tC.v2 = d.w + off;
        p.tC.digits2 = g->dW.digits;
        p.tC.expo2 = g->dW.expo;
        p.tX = table(g->dX, g->K, nullptr, off, Kin, kpad, 0);
    }
    if (d.hoist) g->tM = table(g->dM, d.twoL * d.nt, nullptr, 0, d.twoL * d.nt, Km, 1);
    // T digits once: they do not change between runs
    cudaError_t e = slice(d.Tfull, d.twoL, nullptr, d.twoL, d.nt * d.twoL, d.twoL, g->bpad, s, g->dT, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return fail(HSDLA_ERR_CUDA); }
    rc = make_map(g->dC, s);
    if (!rc) rc = make_map(g->dW, s);
    if (!rc) rc = make_map(g->dX, s);
    if (!rc) rc = make_map(g->dT, s);
    if (!rc && d.hoist) rc = make_map(g->dM, s);
    if (rc) return fail(rc);
    // (b) T application: per type once (hoisted), or per atom of each panel
    if (d.hoist) {
        std::vector<OzJob> jt;
        for (int k = 0; k < g->nk; ++k)
            for (int64_t t = 0; t < d.nt; ++t) {
                OzJob j;
                memset(&j, 0, sizeof(j));
                j.lmap = 3; j.rmap = 0;
                j.lplane = g->dT.plane_rows; j.rplane = g->dM.plane_rows;
                j.lrow0 = t * d.twoL; j.rrow0 = g->row0[k];
                j.rk0 = t * g->bpad;
                j.nkb = tkb;
                j.m = d.twoL; j.n = kb[k].G;
                j.out = kb[k].Z + d.twoL * t; j.ldo = d.twoL * d.nt;
                j.el = g->dT.expo + t * d.twoL; j.er = g->dM.expo + g->row0[k];
                jt.push_back(j);
            }
        g->n_jobs_t = (int)jt.size();
        rc = upload_schedule(jt, g->d_jobs_t, g->d_list_t, g->tiles_t);
        if (rc) return fail(rc);
    } else {
        int64_t joff = 0, loff = 0;
        for (OzPanel &p : g->pan) {
            std::vector<OzJob> jt;
            for (int k = 0; k < g->nk; ++k)
                for (int64_t a = p.a0; a < p.a1; ++a) {
                    const int64_t t = d.atom_type[a];
                    OzJob j;
                    memset(&j, 0, sizeof(j));
                    j.lmap = 3; j.rmap = 0;
                    j.lplane = g->dT.plane_rows; j.rplane = g->dC.plane_rows;
                    j.lrow0 = t * d.twoL; j.rrow0 = g->row0[k];
                    j.rk0 = (a - p.a0) * g->bpad;
                    j.nkb = tkb;
                    j.m = d.twoL; j.n = kb[k].G;
                    j.out = kb[k].CX + d.twoL * a; j.ldo = g->K;
                    j.el = g->dT.expo + t * d.twoL; j.er = g->dC.expo + g->row0[k];
                    jt.push_back(j);
                }
            p.jt_off = joff;
            p.lt_off = loff;
            p.n_jobs_t = (int)jt.size();
            rc = upload_schedule(jt, g->d_jobs_t + joff, g->d_list_t + loff, p.tiles_t);
            if (rc) return fail(rc);
            joff += p.n_jobs_t;
            loff += p.tiles_t;
        }
    }
    g->maps_t[0] = d.hoist ? g->dM.map : g->dC.map;
    g->maps_t[1] = g->maps_t[0]; g->maps_t[2] = g->maps_t[0]; g->maps_t[3] = g->dT.map;
    // (c) S and H jobs of every panel; outputs are patched per run, later panels accumulate
    g->pair = use_pair();
    g->units = pair_units_plain(g->s);
    const int64_t tile = g->pair ? kPairTile : kTileN;
    g->n_jobs_sh = 2 * g->nk;
    for (int pi = 0; pi < g->panels; ++pi) {
        const OzPanel &p = g->pan[pi];
        std::vector<OzJob> jsh;
        for (int k = 0; k < g->nk; ++k)
            for (int which = 0; which < 2; ++which) {
                OzJob j;
                memset(&j, 0, sizeof(j));
                j.lmap = 0; j.rmap = which == 0 ? 1 : 2; j.lower = 1;
                j.accum = pi > 0;
                j.lplane = g->dC.plane_rows; j.rplane = which == 0 ? g->dW.plane_rows : g->dX.plane_rows;
                j.lrow0 = g->row0[k]; j.rrow0 = g->row0[k];
                j.nkb = round_up((p.a1 - p.a0) * g->bpad, kKBlock) / kKBlock;
                j.m = kb[k].G; j.n = kb[k].G;
                j.el = g->dC.expo + g->row0[k];
                j.er = (which == 0 ? g->dW.expo : g->dX.expo) + g->row0[k];
                jsh.push_back(j);
            }
        // the tile list is the same for every panel: upload it once
        if (pi == 0) {
            rc = upload_schedule(jsh, g->d_jobs_sh, g->d_list_sh, g->tiles_sh, tile);
            if (rc) return fail(rc);
        } else {
            int64_t total = 0;
            for (auto &j : jsh) {
                j.tiles_n = (j.n + tile - 1) / tile;
                j.tile_begin = total;
                total += job_tiles(j, tile);
            }
        }
        memcpy(g->h_jobs_sh + 2 * g->nk * pi, jsh.data(), sizeof(OzJob) * jsh.size());
    }
    g->maps_sh[0] = g->dC.map; g->maps_sh[1] = g->dW.map; g->maps_sh[2] = g->dX.map; g->maps_sh[3] = g->dC.map;
    *out = g;
    return HSDLA_OK;
}

void ozaki_group_set_sf(OzGroup *g, const SfTab &t) { g->sft = t; }
int ozaki_group_last_combine(const OzGroup *g) {
    if (g->side_types > 0) return g->side_types;
    return (g->nt - 1) / g->tbatch * g->tbatch;
}

void ozaki_group_set_outputs(OzGroup *g, double2 *const *S, double2 *const *H, const int64_t *ld) {
    for (int pi = 0; pi < g->panels; ++pi) {
        OzJob *j = g->h_jobs_sh + 2 * g->nk * pi;
        for (int k = 0; k < g->nk; ++k) {
            j[2 * k].out = S[k];
            j[2 * k].ldo = ld[k];
            j[2 * k + 1].out = H[k];
            j[2 * k + 1].ldo = ld[k];
        }
    }
}

// Events around the S/H launch; under stream capture they become external event-record nodes
// so that a replayed graph still times the launch.
static cudaError_t record(cudaEvent_t ev, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cs);
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal)
                                               : cudaEventRecord(ev, st);
}

// One run: [hoisted: M digits, Z_t = T_t M_t], then per atom panel: C and W digits, the panel's
// T application (or phase expansion), X digits, the S/H products (accumulating after the first
// panel).  With several panels the events span the panels' S/H launches and the slicing between
// them.
int ozaki_group_tapply_events(const OzGroup *g) { return (g->sf || g->hoist) ? 1 : g->panels; }

bool ozaki_group_streamable(const OzGroup *g) {
    return g && g->sf && g->pair && g->nblk > 1 && g->tbatch >= g->nt && g->side_types == 0 &&
           env_int("HSDLA_STREAM_OUTPUT", 1) != 0;
}

int ozaki_group_output_blocks(const OzGroup *g) { return g ? g->nblk : 0; }

// The streamed host output's S/H part.  Per column block: one pair launch over every type's tiles
// of the block, then the block's combine on the main stream, which writes the block's diagonal
// square (rows < the block's end) into the caller's page-locked outputs in place and the rows
// below it into the device outputs; the copy engine then downloads those rows (side stream)
// while the next block's products run.  The last block's combine writes everything in place.
// The main stream waits for the last download at the end.  No SM work runs beside the products.
static cudaError_t run_sh_streamed(OzGroup *g, cudaStream_t st, const cudaEvent_t *ev, int nev, const SfTab &out,
                                   int *nl) {
    cudaError_t e = cudaSuccess;
    if (!g->blk_side) {
        e = cudaStreamCreateWithFlags(&g->blk_side, cudaStreamNonBlocking);
        for (int b = 0; b < g->nblk && e == cudaSuccess; ++b)
            e = cudaEventCreateWithFlags(&g->ev_blk[b], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->ev_blk_join, cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
    }
    // the dominant-launch event pairs: pair b spans block b's S/H launch where there are enough of
    // them (the rest, and a shortfall, span nothing)
    const int npair = nev / 2;
    for (int b = 0; b < g->nblk && e == cudaSuccess; ++b) {
        const int64_t c0 = g->blk_col[b], c1 = g->blk_col[b + 1];
        const bool last = b + 1 == g->nblk;
        if (b < npair) e = record(ev[2 * b], st);
        if (e == cudaSuccess)
            e = launch_pair(g->maps_sh, g->s, g->d_err, g->d_jobs_sh, g->n_jobs_sh * g->nt,
                            g->blk_begin[b + 1] - g->blk_begin[b], g->d_list_blk + g->blk_begin[b], nullptr, st,
                            g->units, g->halves);
        if (e == cudaSuccess && b < npair) e = record(ev[2 * b + 1], st);
        SfTab tab = out;
        tab.type = 0;
        tab.ntypes = g->nt;
        tab.slot0 = 0;
        tab.col0 = c0;
        tab.col1 = c1;
        if (!last) {
            // rows below the block's diagonal square into the device outputs (the sums Si, Hi of an
            // earlier batch are the device outputs themselves; this is the only batch)
            tab.xrow1 = c1;
            for (int q = 0; q < tab.nk; ++q) {
                SfEntry &E = tab.e[q];
                E.Sx = E.S;
                E.Hx = E.H;
                E.ldx = E.ldo;
                E.S = const_cast<double2 *>(E.Si);
                E.H = const_cast<double2 *>(E.Hi);
                E.ldo = E.ldi;
            }
        }
        if (c1 <= c0) { *nl += 1; continue; }       // no column completed by this launch
        if (e == cudaSuccess) e = launch_sf_combine(tab, g->sf_tab, true, st);
        *nl += 2;
        if (last || e != cudaSuccess) continue;
        e = cudaEventRecord(g->ev_blk[b], st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(g->blk_side, g->ev_blk[b], 0);
        for (int q = 0; q < tab.nk && e == cudaSuccess; ++q) {
            const SfEntry &E = tab.e[q];
            if (c1 >= E.n) continue;
            const int64_t w = std::min(c1, E.n) - c0;
            for (int m = 0; m < 2 && e == cudaSuccess; ++m) {
                double2 *host = (m == 0 ? E.Sx : E.Hx) + c1 + E.ldx * c0;
                const double2 *dev = (m == 0 ? E.S : E.H) + c1 + E.ldo * c0;
                e = cudaMemcpy2DAsync(host, E.ldx * sizeof(double2), dev, E.ldo * sizeof(double2),
                                      (E.n - c1) * sizeof(double2), w, cudaMemcpyDeviceToHost, g->blk_side);
            }
        }
    }
    for (int p = g->nblk; p < npair && e == cudaSuccess; ++p) {
        e = record(ev[2 * p], st);
        if (e == cudaSuccess) e = record(ev[2 * p + 1], st);
    }
    if (e == cudaSuccess) e = cudaEventRecord(g->ev_blk_join, g->blk_side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, g->ev_blk_join, 0);
    return e;
}

int ozaki_group_run(OzGroup *g, const DevSystem &sys, const KTable &ktab, cudaStream_t st, const cudaEvent_t *ev,
                    int nev, int *launches, bool defer_last_combine, const cudaEvent_t *ev_t, int nev_t,
                    const SfTab *host_out) {
    const cudaEvent_t ev0 = nev >= 2 ? ev[0] : nullptr, ev1 = nev >= 2 ? ev[nev - 1] : nullptr;
    // T-application events: pair q around the q-th T launch (when the caller gave enough of them)
    const bool tev = ev_t && nev_t >= 2 * ozaki_group_tapply_events(g);
    int nl = 0;
    cudaError_t e = cudaSuccess;
    if (g->sf) {
        e = slice_launch(g->tM, st);                      // M and M diag(w_t)
        if (e == cudaSuccess && tev) e = cudaEventRecord(ev_t[0], st);
        if (e == cudaSuccess)
            e = g->pair ? launch_pair(g->maps_t, g->s, g->d_err, g->d_jobs_t, g->n_jobs_t, g->tiles_t, g->d_list_t,
                                      nullptr, st, g->units_t, g->halves_t)
                        : launch_prepared(g->maps_t, g->s, g->d_err, g->d_jobs_t, g->n_jobs_t, g->tiles_t,
                                          g->d_list_t, nullptr, st);
        if (e == cudaSuccess && tev) e = cudaEventRecord(ev_t[1], st);
        if (e == cudaSuccess) e = slice_launch(g->pan[0].tX, st);    // Z
        nl += 3;
        if (host_out && ozaki_group_streamable(g)) {
            if (e == cudaSuccess) e = run_sh_streamed(g, st, ev, nev, *host_out, &nl);
            if (launches) *launches = nl;
            if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
            return HSDLA_OK;
        }
        for (int t = 0; t < g->nt && e == cudaSuccess; ++t) {
            const OzJob *jobs = g->d_jobs_sh + (int64_t)g->n_jobs_sh * t;
            if (nev >= 2 * g->nt) e = record(ev[2 * t], st);
            // no grid lockstep here: the per-type operands are small enough for L2 without it, and
            // pairs that drift apart spread their drains over the MMA phases of the others (c2
            // 34.5 -> 33.8 ms, c3 11.7 -> 11.4 ms, c4 461 -> 442 ms per k-point)
            if (e == cudaSuccess)
                e = g->pair ? launch_pair(g->maps_sh, g->s, g->d_err, jobs, g->n_jobs_sh, g->tiles_sh, g->d_list_sh,
                                          nullptr, st, g->units, g->halves)
                            : launch_prepared(g->maps_sh, g->s, g->d_err, jobs, g->n_jobs_sh, g->tiles_sh,
                                              g->d_list_sh, g->d_progress, st);
            if (e == cudaSuccess && nev >= 2 * g->nt) e = record(ev[2 * t + 1], st);
            nl += 1;
            if (g->side_types > 0) {
                // the first side_types types' products into S and H on the side stream, then the
                // rest (the caller's when it defers the last combine)
                if (e == cudaSuccess && t + 1 == g->side_types) {
                    SfTab tab = g->sft;
                    tab.type = 0;
                    tab.ntypes = g->side_types;
                    tab.slot0 = 0;
                    // plain records: under graph capture they fork the side stream into the graph
                    // and join it back
                    e = cudaEventRecord(g->ev_fork, st);
                    if (e == cudaSuccess) e = cudaStreamWaitEvent(g->side, g->ev_fork, 0);
                    if (e == cudaSuccess) e = launch_sf_combine(tab, g->sf_tab, true, g->side);
                    if (e == cudaSuccess) e = cudaEventRecord(g->ev_join, g->side);
                    nl += 1;
                }
                if (e == cudaSuccess && t + 1 == g->nt) {
                    e = cudaStreamWaitEvent(st, g->ev_join, 0);
                    if (e == cudaSuccess && !defer_last_combine) {
                        SfTab tab = g->sft;
                        tab.type = g->side_types;
                        tab.ntypes = g->nt - g->side_types;
                        tab.slot0 = g->side_types;
                        e = launch_sf_combine(tab, g->sf_tab, false, st);
                        nl += 1;
                    }
                }
                continue;
            }
            // the batch's last type: its products into S and H (the caller combines the group's last
            // batch when it defers it)
            if (e == cudaSuccess && ((t + 1) % g->tbatch == 0 || t + 1 == g->nt) &&
                !(defer_last_combine && t + 1 == g->nt)) {
                const int t0 = t / g->tbatch * g->tbatch;
                g->sft.type = t0;
                g->sft.ntypes = t + 1 - t0;
                e = launch_sf_combine(g->sft, g->sf_tab, t0 == 0, st);
                nl += 1;
            }
        }
        // event pairs past the types (kept for the streamed form's column blocks) span nothing,
        // after the S/H launches (the last event closes the group's products)
        for (int p = g->nt; nev >= 2 * g->nt && p < nev / 2 && e == cudaSuccess; ++p) {
            e = record(ev[2 * p], st);
            if (e == cudaSuccess) e = record(ev[2 * p + 1], st);
        }
        if (launches) *launches = nl;
        if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
        return HSDLA_OK;
    }
    if (g->hoist) {
        e = slice_launch(g->tM, st);
        if (e == cudaSuccess && tev) e = cudaEventRecord(ev_t[0], st);
        if (e == cudaSuccess)
            e = launch_prepared(g->maps_t, g->s, g->d_err, g->d_jobs_t, g->n_jobs_t, g->tiles_t, g->d_list_t, nullptr,
                                st);
        if (e == cudaSuccess && tev) e = cudaEventRecord(ev_t[1], st);
        nl += 2;
    }
    // the S/H job tables travel from pinned memory in stream order (a graph replays the copy)
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(g->d_jobs_sh, g->h_jobs_sh, sizeof(OzJob) * g->n_jobs_sh * g->panels,
                            cudaMemcpyHostToDevice, st);
    for (int pi = 0; pi < g->panels && e == cudaSuccess; ++pi) {
        const OzPanel &p = g->pan[pi];
        e = slice_launch(p.tC, st);           // C and W = C diag(w) in one pass over C
        nl += 1;
        if (e == cudaSuccess) {
            if (g->hoist) {
                KTable kt = ktab;
                kt.a0 = (int)p.a0;
                kt.a1 = (int)p.a1;
                e = launch_apply_phase_multi(sys, kt, st);
            } else {
                if (tev) e = cudaEventRecord(ev_t[2 * pi], st);
                if (e == cudaSuccess)
                    e = launch_prepared(g->maps_t, g->s, g->d_err, g->d_jobs_t + p.jt_off, p.n_jobs_t, p.tiles_t,
                                        g->d_list_t + p.lt_off, nullptr, st);
                if (e == cudaSuccess && tev) e = cudaEventRecord(ev_t[2 * pi + 1], st);
            }
            nl += 1;
        }
        if (e == cudaSuccess) { e = slice_launch(p.tX, st); nl += 1; }
        if (e == cudaSuccess && pi == 0 && ev0) e = record(ev0, st);
        const OzJob *jobs = g->d_jobs_sh + (int64_t)g->n_jobs_sh * pi;
        if (e == cudaSuccess)
            e = g->pair ? launch_pair(g->maps_sh, g->s, g->d_err, jobs, g->n_jobs_sh, g->tiles_sh, g->d_list_sh,
                                      g->d_progress, st, g->units)
                        : launch_prepared(g->maps_sh, g->s, g->d_err, jobs, g->n_jobs_sh, g->tiles_sh, g->d_list_sh,
                                          g->d_progress, st);
        nl += 1;
    }
    if (e == cudaSuccess && ev1) e = record(ev1, st);
    if (launches) *launches = nl;
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    return HSDLA_OK;
}

// The structure-factor form's S/H tile configuration: tile shape (halves 1: 256 x 256
// accumulators; 2: two 256 x 128 halves in alternating TMEM buffers) and accumulation split
// (merged: adjacent digit diagonals share an exact FP32 unit; else one unit per diagonal).
static void set_sh_tiles(OzGroup *g, int halves, bool merged) {
    g->halves = halves;
    g->merged = merged;
    g->units = pair_units(g->s, g->bpad / kKBlock, merged, g->twoL);
    g->maps_sh[1] = halves == 2 ? g->dW.map64 : g->dW.map;
    g->maps_sh[2] = halves == 2 ? g->dX.map64 : g->dX.map;
}

bool ozaki_group_tunable(const OzGroup *g) { return g && g->sf && g->pair; }

void ozaki_group_tiles(const OzGroup *g, int *halves, int *merged) {
    *halves = g->halves;
    *merged = g->merged ? 1 : 0;
}

void ozaki_group_set_tiles(OzGroup *g, int halves, int merged) {
    if (ozaki_group_tunable(g)) set_sh_tiles(g, halves == 1 ? 1 : 2, merged != 0);
}

// Times the first type's S/H launch (every k-point of the group) in each configuration and keeps
// the fastest.  The digit planes must hold a completed run's data (the launches only rewrite that
// type's product slot, which the run has combined already).  Each configuration runs twice, the
// second timed.
int ozaki_group_tune_tiles(OzGroup *g, cudaStream_t st, float *ms_best) {
    if (!ozaki_group_tunable(g)) return HSDLA_OK;
    const int cfg[4][2] = {{2, 1}, {1, 1}, {2, 0}, {1, 0}};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        g_oz_err = "tile tuner: event creation failed";
        return HSDLA_ERR_CUDA;
    }
    const int h0 = g->halves;
    const bool m0 = g->merged;
    // a prefix of the tile list is enough to rank the configurations (a batched group's launch
    // covers every k-point): at most 16 waves of pair tiles
    const int64_t tiles = std::min<int64_t>(g->tiles_sh, 16 * 76);
    float best = -1.f;
    int bi = 0;
    cudaError_t e = cudaSuccess;
    for (int c = 0; c < 4 && e == cudaSuccess; ++c) {
        set_sh_tiles(g, cfg[c][0], cfg[c][1] != 0);
        // one untimed launch, then the faster of two timed ones (a launch slowed by something
        // else on the machine would otherwise fix a worse configuration for the plan)
        float ms = -1.f;
        for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
            if (rep > 0) e = cudaEventRecord(e0, st);
            if (e == cudaSuccess)
                e = launch_pair(g->maps_sh, g->s, g->d_err, g->d_jobs_sh, g->n_jobs_sh, tiles, g->d_list_sh, nullptr,
                                st, g->units, g->halves);
            if (e == cudaSuccess && rep > 0) e = cudaEventRecord(e1, st);
            if (e == cudaSuccess && rep > 0) e = cudaEventSynchronize(e1);
            float t = 0.f;
            if (e == cudaSuccess && rep > 0) e = cudaEventElapsedTime(&t, e0, e1);
            if (e == cudaSuccess && rep > 0 && (ms < 0.f || t < ms)) ms = t;
        }
        if (e == cudaSuccess && (best < 0.f || ms < best)) { best = ms; bi = c; }
        if (e == cudaSuccess && env_int("HSDLA_TRACE", 0))
            fprintf(stderr, "tile tuner: halves %d, %s units: %.3f ms\n", cfg[c][0], cfg[c][1] ? "merged" : "single-diagonal",
                    ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        set_sh_tiles(g, h0, m0);
        g_oz_err = cudaGetErrorString(e);
        return HSDLA_ERR_CUDA;
    }
    set_sh_tiles(g, cfg[bi][0], cfg[bi][1] != 0);
    if (ms_best) *ms_best = best;
    return HSDLA_OK;
}

void ozaki_group_destroy(OzGroup *g) {
    if (!g) return;
    if (g->h_jobs_sh) cudaFreeHost(g->h_jobs_sh);
    if (g->ev_fork) cudaEventDestroy(g->ev_fork);
    if (g->ev_join) cudaEventDestroy(g->ev_join);
    if (g->side) cudaStreamDestroy(g->side);
    for (auto &ev : g->ev_blk)
        if (ev) cudaEventDestroy(ev);
    if (g->ev_blk_join) cudaEventDestroy(g->ev_blk_join);
    if (g->blk_side) cudaStreamDestroy(g->blk_side);
    delete g;
}

// One k-point through a temporary group (the slice autotuner's probe).
int64_t ozaki_pipeline_workspace(int s, int64_t twoL, int64_t na, int64_t nt, int64_t G) {
    const std::vector<int64_t> g{G};
    return ozaki_group_bytes(s, twoL, na, nt, g, 1, true, false) + ozaki_group_persist_bytes(s, twoL, na, nt, g, 1) +
           2048;
}

int ozaki_pipeline(OzakiPlan &oz, const OzakiInputs &in, double2 *S, double2 *H, int64_t ldo, void *ws,
                   cudaStream_t st, int *launches) {
    OzGroupDesc d;
    d.twoL = in.twoL; d.na = in.na; d.nt = in.nt; d.hoist = in.M != nullptr;
    d.w = in.w; d.Tfull = in.Tfull; d.atom_type = in.atom_type;
    std::vector<OzKBufs> kb(1);
    // the probe keeps C and X apart: C is its input, X is written by the T application
    kb[0].CX = const_cast<double2 *>(in.C);
    kb[0].M = const_cast<double2 *>(in.M);
    kb[0].Z = in.Z;
    kb[0].G = in.G;
    OzGroup *g = nullptr;
    const int64_t scratch = ozaki_group_bytes(oz.num_slices, in.twoL, in.na, in.nt, std::vector<int64_t>{in.G}, 1,
                                              d.hoist, false);
    char *persist = reinterpret_cast<char *>(ws) + (scratch + 1023) / 1024 * 1024;
    int rc = ozaki_group_prepare(oz, d, kb, ws, persist, st, &g);
    if (rc) return rc;
    double2 *Sp[1] = {S}, *Hp[1] = {H};
    int64_t ld[1] = {ldo};
    ozaki_group_set_outputs(g, Sp, Hp, ld);
    KTable kt;
    kt.nk = 1; kt.ldc = in.twoL * in.na; kt.ldm = in.twoL * in.nt; kt.total_cols = in.G;
    if (in.kp) kt.e[0] = KEntry{*in.kp, nullptr, nullptr, in.Z, kb[0].CX, 0};
    const cudaEvent_t evs[2] = {in.ev_dom0, in.ev_dom1};
    rc = ozaki_group_run(g, in.sys ? *in.sys : DevSystem{}, kt, st, evs, in.ev_dom0 ? 2 : 0, launches);
    if (rc == HSDLA_OK && cudaStreamSynchronize(st) != cudaSuccess) rc = HSDLA_ERR_CUDA;
    ozaki_group_destroy(g);
    return rc;
}

}  // namespace hsdla

// ======================================================================
// Allocation-free variant of the Ozaki lower-triangle contraction.
//
// Some callers cannot allocate device memory: code running inside another
// framework's memory pool or under a fixed memory budget, plug-ins that may only
// touch the buffers they are handed, and processes that must not call cudaMalloc
// once their steady state has begun.  For them, hsdla_zherkx_lower_noalloc keeps
// every scratch byte of the Ozaki contraction (digit planes, exponents, the job
// table and the device error word) in one file-scope device array of
// kNoAllocScratchBytes.  That array exists on every GPU that loads this library
// and stays resident until the process exits.  The caller still passes the
// inputs and the output.
#include <mutex>

namespace hsdla {
namespace {

constexpr int64_t kNoAllocScratchBytes = int64_t(128) << 20;   // 128 MiB
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Host-side cache of the array's device address, per device.  In host code the
// symbol g_noalloc_scratch is only a stand-in for the device array, so its address
// must come from cudaGetSymbolAddress with that device current.
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_ptr[kNoAllocMaxDevices] = {};

int noalloc_scratch(unsigned char **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        g_oz_err = "no current CUDA device";
        return HSDLA_ERR_DEVICE;
    }
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        g_oz_err = "device index beyond the 64 devices the static scratch table covers";
        return HSDLA_ERR_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            g_oz_err = "cudaGetSymbolAddress of the static scratch failed";
            return HSDLA_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = reinterpret_cast<unsigned char *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return HSDLA_OK;
}

// Bytes of static scratch one call needs: two digit operands, their exponents, the
// job table and the error word.
int64_t noalloc_bytes(int s, int64_t n, int64_t Kpad) {
    return 2 * operand_bytes(s, n, Kpad) + round_up(sizeof(OzJob), 1024) + 1024;
}

}  // namespace
}  // namespace hsdla

extern "C" int hsdla_zherkx_lower_noalloc(int32_t num_slices, int64_t n, int64_t k, const hsdla_cx *dP, int64_t ldp,
                                          const hsdla_cx *dQ, int64_t ldq, const double *dw, hsdla_cx *dOut,
                                          int64_t ldo, void *stream) {
    using namespace hsdla;
    const int s = num_slices == 0 ? kOzDefaultSlices : num_slices;
    if (s < 2 || s > kOzMaxSlices) {
        g_oz_err = "num_slices outside [2, 12] (0 selects 11)";
        return HSDLA_ERR_ARG;
    }
    if (n < 0 || k < 0 || !dP || !dQ || !dOut || ldp < k || ldq < k || ldo < n) {
        g_oz_err = "bad arguments: n or k negative, a NULL buffer, or a leading dimension below k (inputs) or n "
                   "(output)";
        return HSDLA_ERR_ARG;
    }
    g_oz_err = "";
    if (n == 0) return HSDLA_OK;
    const int64_t Kpad = round_up(std::max<int64_t>(k, 1), kKBlock);
    if (noalloc_bytes(s, n, Kpad) > kNoAllocScratchBytes) {
        g_oz_err = "problem exceeds the 128 MiB static scratch of hsdla_zherkx_lower_noalloc";
        return HSDLA_ERR_UNSUPPORTED;
    }
    unsigned char *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Arena ar{reinterpret_cast<char *>(scratch)};
    DigitOperand dp, dq;
    carve_operand(ar, dp, s, n, Kpad);
    carve_operand(ar, dq, s, n, Kpad);
    OzJob *d_job = ar.take<OzJob>(1);
    int *d_err = ar.take<int>(1);
    // the array keeps the previous call's contents: the error word must start at zero
    // (digit planes and exponents are rewritten in full by the slicing kernel)
    cudaError_t e = cudaMemsetAsync(d_err, 0, sizeof(int), st);
    if (e == cudaSuccess) e = slice(reinterpret_cast<const double2 *>(dP), ldp, nullptr, k, n, Kpad, Kpad, s, dp, st);
    if (e == cudaSuccess) e = slice(reinterpret_cast<const double2 *>(dQ), ldq, dw, k, n, Kpad, Kpad, s, dq, st);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    rc = make_map(dp, s);
    if (!rc) rc = make_map(dq, s);
    if (rc) return rc;
    OzJob j;
    memset(&j, 0, sizeof(j));
    j.lmap = 0; j.rmap = 1; j.lower = 1;
    j.lplane = dp.plane_rows; j.rplane = dq.plane_rows;
    j.nkb = Kpad / kKBlock; j.m = n; j.n = n;
    j.tiles_n = (n + kTileN - 1) / kTileN;
    j.tile_begin = 0;
    j.out = reinterpret_cast<double2 *>(dOut); j.ldo = ldo;
    j.el = dp.expo; j.er = dq.expo;
    const int64_t tiles = job_tiles(j);
    e = cudaMemcpyAsync(d_job, &j, sizeof(OzJob), cudaMemcpyHostToDevice, st);
    const size_t smem = (size_t)kStages * kStageBytes + 1024;
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int dev = 0, nsm = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    const int64_t grid = std::min<int64_t>(tiles, nsm);
    oz_gemm_kernel<<<(unsigned)grid, kThreads, smem, st>>>(dp.map, dq.map, dp.map, dp.map, d_job, 1, tiles, s, d_err,
                                                            nullptr, nullptr);
    e = cudaGetLastError();
    int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { g_oz_err = cudaGetErrorString(e); return HSDLA_ERR_CUDA; }
    if (herr != 0) {
        // the error word: code * 16 + the role whose bounded wait expired (1 TMA producer, 2 MMA
        // issuer waiting for a drained accumulator, 3 MMA issuer waiting for operands, 4 epilogue)
        static thread_local char buf[160];
        snprintf(buf, sizeof(buf), "device wait expired in hsdla_zherkx_lower_noalloc (code %d, role %d)", herr / 16,
                 herr % 16);
        g_oz_err = buf;
        return herr / 16 == kDevBadInput ? HSDLA_ERR_CUDA : HSDLA_ERR_TIMEOUT;
    }
    return HSDLA_OK;
}
