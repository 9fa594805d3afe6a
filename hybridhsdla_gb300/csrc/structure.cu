// Structure-factor form of S and H for plans whose atoms share their type's rotation.
//
// With C_a = phi_a (.) M_t(a) and X_a = phi_a (.) Z_t(a), phi_a(g) = e^{i 2pi (k+g).tau_a} (the
// per-type rows M_t and Z_t = T_t M_t of the hoisted T application), the per-atom sums of
// create_HS2_stripped_v2 (flapw_opt/src/h_and_s_stripped_v2.cpp:155-368) regroup by type:
//     S[g, g'] = sum_t SF_t(g' - g) (M_t^H diag(w_t) M_t)[g, g'],
//     H[g, g'] = sum_t SF_t(g' - g) (M_t^H Z_t)[g, g'],
//     SF_t(dG) = sum_{a of type t} e^{i 2pi dG.tau_a}          (k cancels),
// so the contractions run over 2L rows per type instead of 2L rows per atom (a factor of atoms
// per type fewer products), and the structure factors enter once per element and type.
#include "common.cuh"

namespace hsdla {

namespace {

__device__ __forceinline__ double2 cmul_d(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}


// sf[t][(ix ny + iy) nz + iz] = sum over the atoms of type t of ex[a][ix] ey[a][iy] ez[a][iz],
// the atoms listed type by type (order[type_begin[t] .. type_begin[t+1])).  One CTA per (ix, t):
// the products ex ey of a chunk of atoms go to shared memory once per block of entries, and each
// entry then costs one complex FMA per atom (FP64, the pipe that bounds this table).
constexpr int kSfChunk = 16, kSfTabThreads = 256, kSfSmem = 48 * 1024;
__global__ void __launch_bounds__(kSfTabThreads) sf_table_kernel(const double2 *__restrict__ ex,
                                                                 const double2 *__restrict__ ey,
                                                                 const double2 *__restrict__ ez,
                                                                 const int32_t *__restrict__ order,
                                                                 const int32_t *__restrict__ type_begin, int nx,
                                                                 int ny, int nz, int chunk, double2 *__restrict__ sf) {
    extern __shared__ double2 pxy[];            // [chunk][ny]
    const int ix = blockIdx.x, t = blockIdx.y;
    const int64_t nyz = (int64_t)ny * nz;
    const int a0 = type_begin[t], a1 = type_begin[t + 1];
    double2 *out = sf + ((int64_t)t * nx + ix) * nyz;
    for (int64_t e0 = 0; e0 < nyz; e0 += blockDim.x) {
        const int64_t e = e0 + threadIdx.x;
        const int iy = (int)(e / nz), iz = (int)(e % nz);
        double2 acc = make_double2(0.0, 0.0);
        for (int c0 = a0; c0 < a1; c0 += chunk) {
            const int nc = min(chunk, a1 - c0);
            __syncthreads();
            for (int w = threadIdx.x; w < nc * ny; w += blockDim.x) {
                const int k = w / ny, y = w - k * ny;
                const int a = order[c0 + k];
                pxy[k * ny + y] = cmul_d(ex[(int64_t)a * nx + ix], ey[(int64_t)a * ny + y]);
            }
            __syncthreads();
            if (e < nyz)
                for (int k = 0; k < nc; ++k) {
                    const double2 p = pxy[k * ny + iy], z = ez[(int64_t)order[c0 + k] * nz + iz];
                    acc.x = fma(p.x, z.x, fma(-p.y, z.y, acc.x));
                    acc.y = fma(p.x, z.y, fma(p.y, z.x, acc.y));
                }
        }
        if (e < nyz) out[e] = acc;
    }
}

// 128-thread CTAs (32 rows x 4 column lanes): small enough to share an SM with a pair launch
constexpr int kSfTile = 32, kSfRows = 4;

// out (+)= sum over the batch's types t of SF_t(g_col - g_row) * P_t over the lower triangle of
// every entry (S and H together), one CTA per 32 x 32 tile; consecutive threads take consecutive
// rows of a column.  A batch of several types reads and writes S and H once.  The tiles of an
// entry are its tile columns [tc0, tc1) (a column range of the launch), each from the diagonal
// tile down.
__global__ void __launch_bounds__(kSfTile * kSfRows) sf_combine_kernel(const __grid_constant__ SfTab tab,
                                                                       const double2 *__restrict__ sf, int first) {
    const int64_t tile = blockIdx.x;
    int k = 0;
    while (k + 1 < tab.nk && tab.e[k + 1].tile_begin <= tile) ++k;
    const SfEntry &E = tab.e[k];
    const int64_t b = tile - E.tile_begin;
    // tile column tc: the last one whose first tile is at or before b (tiles before tile column
    // c: sum_{c'=tc0}^{c-1} (T - c'))
    const int64_t T = (E.n + kSfTile - 1) / kSfTile, tc0 = tab.col0 / kSfTile;
    auto before = [&](int64_t c) { return (c - tc0) * T - (c * (c - 1) - tc0 * (tc0 - 1)) / 2; };
    int64_t lo = tc0, hi = (min(E.n, tab.col1) + kSfTile - 1) / kSfTile - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) / 2;
        if (before(mid) <= b) lo = mid;
        else hi = mid - 1;
    }
    const int64_t tc = lo, tr = tc + (b - before(tc));
    const int64_t row = tr * kSfTile + threadIdx.x;
    if (row >= E.n) return;
    const int32_t *gr = E.g + 3 * row;
    const int gr0 = gr[0], gr1 = gr[1], gr2 = gr[2];
    const double2 *sft = sf + (int64_t)tab.type * tab.box;
#pragma unroll
    for (int q = 0; q < kSfTile; q += kSfRows) {
        const int64_t col = tc * kSfTile + threadIdx.y + q;
        if (col > row) continue;
        const int32_t *gc = E.g + 3 * col;
        const int64_t idx = ((int64_t)(gc[0] - gr0 + tab.dx) * tab.ny + (gc[1] - gr1 + tab.dy)) * tab.nz +
                            (gc[2] - gr2 + tab.dz);
        const int64_t off = row + E.ldp * col;
        double2 vs = make_double2(0.0, 0.0), vh = make_double2(0.0, 0.0);
        for (int b = 0; b < tab.ntypes; ++b) {
            const double2 f = sft[idx + b * tab.box];
            const double2 ps = E.PS[off + (tab.slot0 + b) * E.pstride], ph = E.PH[off + (tab.slot0 + b) * E.pstride];
            vs.x = fma(f.x, ps.x, fma(-f.y, ps.y, vs.x));
            vs.y = fma(f.x, ps.y, fma(f.y, ps.x, vs.y));
            vh.x = fma(f.x, ph.x, fma(-f.y, ph.y, vh.x));
            vh.y = fma(f.x, ph.y, fma(f.y, ph.x, vh.y));
        }
        const bool x = E.Sx && row < tab.xrow1;
        double2 *so = x ? E.Sx + row + E.ldx * col : E.S + row + E.ldo * col;
        double2 *ho = x ? E.Hx + row + E.ldx * col : E.H + row + E.ldo * col;
        if (!first) {
            const double2 s0 = E.Si[row + E.ldi * col], h0 = E.Hi[row + E.ldi * col];
            vs.x += s0.x; vs.y += s0.y;
            vh.x += h0.x; vh.y += h0.y;
        }
        *so = vs;
        *ho = vh;
    }
}

}  // namespace

cudaError_t launch_sf_table(const double2 *ex, const double2 *ey, const double2 *ez, const int32_t *order,
                            const int32_t *type_begin, int nt, int nx, int ny, int nz, double2 *sf, cudaStream_t st) {
    const int64_t n = (int64_t)nx * ny * nz * nt;
    if (n <= 0) return cudaSuccess;
    // atoms per shared-memory chunk: kSfChunk, fewer for a long y extent
    const int chunk = std::min<int>(kSfChunk, kSfSmem / (int)sizeof(double2) / std::max(ny, 1));
    if (nx > 65535 || nt > 65535 || chunk < 1) return cudaErrorInvalidValue;
    const size_t smem = sizeof(double2) * (size_t)chunk * ny;
    sf_table_kernel<<<dim3((unsigned)nx, (unsigned)nt), kSfTabThreads, smem, st>>>(ex, ey, ez, order, type_begin, nx,
                                                                                 ny, nz, chunk, sf);
    return cudaGetLastError();
}

int64_t sf_tab_tiles(SfTab &tab) {
    int64_t total = 0;
    const int64_t tc0 = tab.col0 / kSfTile;
    for (int k = 0; k < tab.nk; ++k) {
        const int64_t T = (tab.e[k].n + kSfTile - 1) / kSfTile;
        const int64_t tc1 = (std::min(tab.e[k].n, tab.col1) + kSfTile - 1) / kSfTile;   // (col1 may be INT64_MAX)
        tab.e[k].tile_begin = total;
        // tile columns [tc0, tc1), T - c tiles each
        if (tc1 > tc0) total += (tc1 - tc0) * T - (tc1 * (tc1 - 1) - tc0 * (tc0 - 1)) / 2;
    }
    return total;
}

cudaError_t launch_sf_combine(const SfTab &tab, const double2 *sf, bool first, cudaStream_t st) {
    SfTab t = tab;
    for (int k = 0; k < t.nk; ++k)
        if (!t.e[k].Si) {
            t.e[k].Si = t.e[k].S;
            t.e[k].Hi = t.e[k].H;
            t.e[k].ldi = t.e[k].ldo;
        }
    const int64_t tiles = sf_tab_tiles(t);
    if (tiles <= 0) return cudaSuccess;
    if (tiles > 0x7fffffffLL) return cudaErrorInvalidValue;
    sf_combine_kernel<<<(unsigned)tiles, dim3(kSfTile, kSfRows), 0, st>>>(t, sf, first ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace hsdla
