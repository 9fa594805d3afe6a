// Kernel (a): FLAPW matching tensors A, B on the GPU in FP64.
//
// Restates construct_AB (flapw_opt/src/tensor_AB_match.cpp:63-129): for every
// G vector, atom j, l, m
//
//   A = conj(Y_lm(R_j^T K^)) 4pi/sqrt(Omega) e^{i 2pi K.tau_j} / W_lj [udot_l |K| j_l'(|K|R) - udot'_l j_l(|K|R)]
//   B = (same prefactor)                                              [-u_l |K| j_l'(|K|R) + u'_l j_l(|K|R)]
//
// with K = k + G, |K| = |bmat K| (types_helper.cpp:33) and j_l, j_l' from the
// sphbes/dsphbs recurrences (external/compat/fleur/sphbes.f:19-76,
// dsphbs.f:24-42), Y_lm from ylm4 (external/compat/fleur/ylm4.f:4-139).
//
// GB300 mapping: one CTA per G column (grid-strided).  Everything that does not
// depend on the atom is hoisted out of the per-atom loop (Bessel values per
// type, Y_lm per G when no atom carries its own rotation, the phase per atom),
// then the whole 2*L*a column is written with consecutive threads on
// consecutive 16-byte elements (coalesced, full 32-byte sectors).  Output
// layout: rows ordered per atom as [A_a (L rows); B_a (L rows)], so that the
// stacked contraction operand [A;B] is one column-major matrix.
#include <algorithm>

#include "common.cuh"

namespace hsdla {
namespace {

// sphbes.f:19-76 (REAL = double).  fj[0..lmax].
__device__ void sphbes_dev(int lmax, double x, double *fj) {
    const double small = 1.0e-3;
    const double xx = x * x;
    if (x >= small) {
        const double xinv = 1.0 / x;
        double sn, cs;
        sincos(x, &sn, &cs);
        fj[0] = sn * xinv;
        fj[1] = (fj[0] - cs) * xinv;
        if ((double)lmax < x) {
            for (int l = 2; l <= lmax; ++l) fj[l] = (2 * l - 1) * xinv * fj[l - 1] - fj[l - 2];
        } else if (lmax >= 2) {
            // Miller's downward recursion from n = int(lmax + 10 + x); only aux[0..lmax] is kept
            const int n = (int)(lmax + 10 + x);
            double aux[kMaxLmax + 1];
            double a_next = 0.0;   // aux(i+1)
            double a_cur = 1.0;    // aux(i), i = n-1
            for (int i = n - 1; i >= 1; --i) {
                const double a_prev = (2 * i + 1) * xinv * a_cur - a_next;
                if (i - 1 <= lmax) aux[i - 1] = a_prev;
                a_next = a_cur;
                a_cur = a_prev;
            }
            const int mn = (fabs(fj[0]) < fabs(fj[1])) ? 1 : 0;
            const double quot = fj[mn] / aux[mn];
            for (int l = 2; l <= lmax; ++l) fj[l] = aux[l] * quot;
        }
    } else {
        fj[0] = 1.0 - xx / 6.0 * (1.0 - xx / 20.0 * (1.0 - xx / 42.0));
        fj[1] = (x / 3.0) * (1.0 - xx / 10.0 * (1.0 - xx / 28.0));
        double fac = xx / 15.0;
        for (int l = 2; l <= lmax; ++l) {
            fj[l] = fac * (1.0 - xx / (4 * l + 6));
            fac = x * fac / (2 * l + 3);
        }
    }
}

// dsphbs.f:24-42
__device__ void dsphbs_dev(int lmax, double x, const double *fj, double *dfj) {
    const double xlim = 1.0e-4;
    dfj[0] = -fj[1];
    if (x < xlim) {
        const double x2 = 0.5 * x * x;
        double fac = 1.0 / 3.0;
        for (int l = 1; l <= lmax; ++l) {
            dfj[l] = fac * (l - x2 * (l + 2) / (2 * l + 3));
            fac = x * fac / (2 * l + 3);
        }
    } else {
        for (int l = 1; l <= lmax; ++l) dfj[l] = fj[l - 1] - (l + 1) * fj[l] / x;
    }
}

// ylm4.f:45-105 for one m (called by thread m = 0..lmax); writes ylm[l(l+1) +- m].
__device__ void ylm_column_dev(int lmax, int m, const double *v, const double *ynorm, double2 *ylm) {
    const double small = 1.0e-12;
    const double x = v[0], y = v[1], z = v[2];
    const double xy = x * x + y * y;
    const double r = sqrt(xy + z * z);
    const double rxy = sqrt(xy);
    double cth, sth, cph, sph;
    if (r > small) { cth = z / r; sth = rxy / r; } else { sth = 0.0; cth = 1.0; }
    if (rxy > small) { cph = x / rxy; sph = y / rxy; } else { cph = 1.0; sph = 0.0; }
    // the reference runs one sequential fac recursion over m; thread m replays its prefix
    double fac = 1.0;
    for (int mm = 0; mm < m; ++mm) {
        fac = (double)(-(mm + mm - 1)) * fac;
        fac = fac * sth;
    }
    double p[kMaxLmax + 1];   // p(l, m) for l = m..lmax
    if (m < lmax) {
        fac = (double)(-(m + m - 1)) * fac;
        p[m] = fac;
        p[m + 1] = (m + m + 1) * cth * fac;
        for (int l = m + 2; l <= lmax; ++l)
            p[l] = ((l + l - 1) * cth * p[l - 1] - (l + m - 1) * p[l - 2]) / (l - m);
    } else {
        p[m] = (double)(-(lmax + lmax - 1)) * fac;
    }
    // cos(m phi), sin(m phi) by the reference's recursion
    double c0 = 1.0, s0 = 0.0, c1 = cph, s1 = sph;
    double cm = (m == 0) ? c0 : c1, sm = (m == 0) ? s0 : s1;
    const double cph2 = cph + cph;
    for (int mm = 2; mm <= m; ++mm) {
        const double s2 = cph2 * s1 - s0, c2 = cph2 * c1 - c0;
        s0 = s1; c0 = c1; s1 = s2; c1 = c2;
        sm = s2; cm = c2;
    }
    for (int l = m; l <= lmax; ++l) {
        const int lm0 = l * (l + 1);
        if (m == 0) {
            ylm[lm0] = make_double2(ynorm[lm0] * p[l], 0.0);
        } else {
            const double yr = p[l] * cm, yi = p[l] * sm;
            ylm[lm0 + m] = make_double2(ynorm[lm0 + m] * yr, ynorm[lm0 + m] * yi);
            ylm[lm0 - m] = make_double2(yr * ynorm[lm0 - m], -yi * ynorm[lm0 - m]);
        }
    }
}

constexpr int kThreads = 256;
constexpr int kRotChunk = 16;   // atoms whose Y_lm sets are staged together when atoms carry rotations

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ int entry_of(const KTable &tab, int64_t gc) {
    int k = 0;
    while (k + 1 < tab.nk && tab.e[k + 1].col_begin <= gc) ++k;
    return k;
}

template <bool kRot>
__global__ void __launch_bounds__(kThreads) construct_ab_kernel(DevSystem sys, const __grid_constant__ KTable tab) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = sys.L, nl = sys.max_lmax + 1, na = sys.num_atoms, nt = sys.num_types;
    const int twoL = 2 * L;
    double *au = reinterpret_cast<double *>(smem_raw);           // [nt*nl]
    double *bu = au + nt * nl;                                     // [nt*nl]
    double2 *vph = reinterpret_cast<double2 *>(bu + nt * nl);     // [na] vol_prefac * phase
    double2 *ylm = vph + na;                                       // [L] or [kRotChunk*L]
    unsigned char *l_of = reinterpret_cast<unsigned char *>(ylm + (kRot ? kRotChunk : 1) * L);  // [L]
    __shared__ double kvec[3];
    __shared__ double knorm;

    for (int lm = threadIdx.x; lm < L; lm += blockDim.x) {
        int l = (int)sqrt((double)lm);
        while (l * l > lm) --l;
        while ((l + 1) * (l + 1) <= lm) ++l;
        l_of[lm] = (unsigned char)l;
    }
    const int64_t ldc = tab.ldc, ldm = tab.ldm;
    for (int64_t gc = blockIdx.x; gc < tab.total_cols; gc += gridDim.x) {
        const KEntry &ent = tab.e[entry_of(tab, gc)];
        const DevKpoint &kp = ent.kp;
        const int64_t gi = gc - ent.col_begin;
        double2 *C = ent.C;
        double2 *M = ent.M;
        __syncthreads();
        if (threadIdx.x == 0) {
            const int32_t *gv = kp.g + 3 * gi;
            double K[3] = {kp.k[0] + gv[0], kp.k[1] + gv[1], kp.k[2] + gv[2]};
            double s = 0.0;
            for (int r = 0; r < 3; ++r) {
                const double t = sys.bmat[3 * r] * K[0] + sys.bmat[3 * r + 1] * K[1] + sys.bmat[3 * r + 2] * K[2];
                s += t * t;
            }
            kvec[0] = K[0]; kvec[1] = K[1]; kvec[2] = K[2];
            knorm = sqrt(s);
        }
        __syncthreads();
        const double K0 = kvec[0], K1 = kvec[1], K2 = kvec[2], kn = knorm;
        // Bessel values per type (calc_bessel at R_t |K| for max_lmax, tensor_AB_match.cpp:104)
        for (int t = threadIdx.x; t < nt; t += blockDim.x) {
            double fj[kMaxLmax + 1], dfj[kMaxLmax + 1];
            const double x = sys.type_rmt[t] * kn;
            sphbes_dev(sys.max_lmax, x, fj);
            dsphbs_dev(sys.max_lmax, x, fj, dfj);
            for (int l = 0; l < nl; ++l) {
                const int tl = t * nl + l;
                au[tl] = sys.dE_u[tl] * kn * dfj[l] - sys.dE_u_dr[tl] * fj[l];
                bu[tl] = -sys.u[tl] * kn * dfj[l] + sys.u_dr[tl] * fj[l];
            }
        }
        // structure phase per atom, premultiplied by 4 pi / sqrt(Omega) (only the per-atom rows C
        // carry it)
        for (int j = threadIdx.x; C && j < na; j += blockDim.x) {
            const double *p = sys.atom_pos + 3 * j;
            const double arg = 2 * kPi * (K0 * p[0] + K1 * p[1] + K2 * p[2]);
            double sn, cs;
            sincos(arg, &sn, &cs);
            vph[j] = make_double2(sys.vol_prefac * cs, sys.vol_prefac * sn);
        }
        if (!kRot) {
            // K_base = normalise(bmat^T K): every atom shares R = bmat
            if (threadIdx.x <= sys.max_lmax) {
                double v[3];
                for (int c = 0; c < 3; ++c)
                    v[c] = sys.bmat[c] * K0 + sys.bmat[3 + c] * K1 + sys.bmat[6 + c] * K2;
                const double nrm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                if (nrm > 0.0) { v[0] /= nrm; v[1] /= nrm; v[2] /= nrm; }
                ylm_column_dev(sys.max_lmax, threadIdx.x, v, sys.ynorm, ylm);
            }
            __syncthreads();
            double2 *col = C + ldc * gi;
            // C may be absent: the structure-factor form needs only the per-type rows M
            const int64_t nrow = C ? (int64_t)twoL * na : 0;
            for (int64_t idx = threadIdx.x; idx < nrow; idx += blockDim.x) {
                const int j = (int)(idx / twoL);
                const int r = (int)(idx - (int64_t)j * twoL);
                const bool isB = r >= L;
                const int lm = isB ? r - L : r;
                const int l = l_of[lm];
                const int t = sys.atom_type[j];
                double2 out = make_double2(0.0, 0.0);
                if (l <= sys.type_lmax[t]) {
                    const int tl = t * nl + l;
                    const double2 common = make_double2(vph[j].x * sys.inv_w[tl], vph[j].y * sys.inv_w[tl]);
                    const double2 y = ylm[lm];
                    const double2 yc = make_double2(y.x, -y.y);
                    const double2 ycc = cmul(yc, common);
                    const double f = isB ? bu[tl] : au[tl];
                    out = make_double2(ycc.x * f, ycc.y * f);
                }
                col[idx] = out;
            }
            // phase-free per-type rows M_t = [A_t; B_t] / e^{i 2pi K.tau} (shared by every atom of type t)
            if (M) {
                double2 *mcol = M + ldm * gi;
                const int nrm = twoL * nt;
                for (int idx = threadIdx.x; idx < nrm; idx += blockDim.x) {
                    const int t = idx / twoL;
                    const int r = idx - t * twoL;
                    const bool isB = r >= L;
                    const int lm = isB ? r - L : r;
                    const int l = l_of[lm];
                    double2 out = make_double2(0.0, 0.0);
                    if (l <= sys.type_lmax[t]) {
                        // conj(Y_lm) times the real prefactor, then the radial factor: the complex
                        // product with a zero imaginary part, without its FP64 work on zeros
                        const int tl = t * nl + l;
                        const double c = sys.vol_prefac * sys.inv_w[tl];
                        const double2 y = ylm[lm];
                        const double f = isB ? bu[tl] : au[tl];
                        out = make_double2((y.x * c) * f, (-y.y * c) * f);
                    }
                    mcol[idx] = out;
                }
            }
        } else {
            for (int j0 = 0; j0 < na; j0 += kRotChunk) {
                const int nj = min(kRotChunk, na - j0);
                __syncthreads();
                for (int w = threadIdx.x; w < nj * nl; w += blockDim.x) {
                    const int jj = w / nl, m = w - jj * nl;
                    const double *R = sys.atom_rotmat + 9 * (j0 + jj);
                    double v[3];
                    for (int c = 0; c < 3; ++c) v[c] = R[c] * K0 + R[3 + c] * K1 + R[6 + c] * K2;
                    const double nrm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                    if (nrm > 0.0) { v[0] /= nrm; v[1] /= nrm; v[2] /= nrm; }
                    ylm_column_dev(sys.max_lmax, m, v, sys.ynorm, ylm + jj * L);
                }
                __syncthreads();
                double2 *col = C + ldc * gi + (int64_t)twoL * j0;
                const int nrow = twoL * nj;
                for (int idx = threadIdx.x; idx < nrow; idx += blockDim.x) {
                    const int jj = idx / twoL;
                    const int r = idx - jj * twoL;
                    const int j = j0 + jj;
                    const bool isB = r >= L;
                    const int lm = isB ? r - L : r;
                    const int l = l_of[lm];
                    const int t = sys.atom_type[j];
                    double2 out = make_double2(0.0, 0.0);
                    if (l <= sys.type_lmax[t]) {
                        const int tl = t * nl + l;
                        const double2 common = make_double2(vph[j].x * sys.inv_w[tl], vph[j].y * sys.inv_w[tl]);
                        const double2 y = ylm[jj * L + lm];
                        const double2 yc = make_double2(y.x, -y.y);
                        const double2 ycc = cmul(yc, common);
                        const double f = isB ? bu[tl] : au[tl];
                        out = make_double2(ycc.x * f, ycc.y * f);
                    }
                    col[idx] = out;
                }
            }
        }
    }
}

// Per-type rows M only (atoms sharing their type's rotation, no per-atom rows), kRowCols G columns
// per CTA.  The per-column scalar work -- the Bessel recursions per type and the Y_lm sets, FP64
// code with data-dependent loops -- runs one column per lane, as work items (column, type) and
// (column, m), instead of on a few lanes of one warp per column: GB300 issues an FP64 warp
// instruction in 16 cycles however few of its lanes are active.  The same formulas in the same
// order as construct_ab_kernel, so M is the same to the bit.
constexpr int kRowCols = 16;
__global__ void __launch_bounds__(kThreads) construct_rows_kernel(DevSystem sys, const __grid_constant__ KTable tab) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = sys.L, nl = sys.max_lmax + 1, nt = sys.num_types, twoL = 2 * L, tnl = nt * nl;
    double2 *ylm = reinterpret_cast<double2 *>(smem_raw);          // [kRowCols][L]
    double *au = reinterpret_cast<double *>(ylm + kRowCols * L);    // [kRowCols][nt nl]
    double *bu = au + kRowCols * tnl;                               // [kRowCols][nt nl]
    double *cf = bu + kRowCols * tnl;                               // [nt nl] 4 pi / sqrt(Omega) / W
    double *kv = cf + tnl;                                          // [kRowCols][4]: K, |bmat K|
    unsigned char *l_of = reinterpret_cast<unsigned char *>(kv + 4 * kRowCols);   // [L]
    for (int lm = threadIdx.x; lm < L; lm += blockDim.x) {
        int l = (int)sqrt((double)lm);
        while (l * l > lm) --l;
        while ((l + 1) * (l + 1) <= lm) ++l;
        l_of[lm] = (unsigned char)l;
    }
    for (int i = threadIdx.x; i < tnl; i += blockDim.x) cf[i] = sys.vol_prefac * sys.inv_w[i];
    const int64_t ldm = tab.ldm;
    for (int64_t col0 = blockIdx.x * (int64_t)kRowCols; col0 < tab.total_cols; col0 += (int64_t)gridDim.x * kRowCols) {
        const int ncols = (int)(tab.total_cols - col0 < kRowCols ? tab.total_cols - col0 : kRowCols);
        __syncthreads();
        if (threadIdx.x < ncols) {
            const int64_t gc = col0 + threadIdx.x;
            const KEntry &ent = tab.e[entry_of(tab, gc)];
            const int32_t *gv = ent.kp.g + 3 * (gc - ent.col_begin);
            const double K[3] = {ent.kp.k[0] + gv[0], ent.kp.k[1] + gv[1], ent.kp.k[2] + gv[2]};
            double s = 0.0;
            for (int r = 0; r < 3; ++r) {
                const double t = sys.bmat[3 * r] * K[0] + sys.bmat[3 * r + 1] * K[1] + sys.bmat[3 * r + 2] * K[2];
                s += t * t;
            }
            double *k4 = kv + 4 * threadIdx.x;
            k4[0] = K[0]; k4[1] = K[1]; k4[2] = K[2]; k4[3] = sqrt(s);
        }
        __syncthreads();
        // the columns' Bessel values per type, then their Y_lm sets (one warp per kind, mostly);
        // with (type, rotation) classes the Y_lm sets come once per rotation, each followed by the
        // rows of the types (classes) that carry it
        const int nrot = sys.num_rots > 0 ? sys.num_rots : 1;
        for (int rho = 0; rho < nrot; ++rho) {
            // R^T K with R = mrot bmat of this rotation (tensor_AB_match.cpp:97), bmat without one
            const double *R = sys.num_rots > 0 ? sys.rots + 9 * rho : sys.bmat;
            const int nb = rho == 0 ? ncols * nt : 0, ny = ncols * nl;
            if (rho > 0) __syncthreads();     // the previous rotation's rows have read ylm
            for (int w = threadIdx.x; w < nb + ny; w += blockDim.x) {
                if (w < nb) {
                    const int c = w / nt, t = w - c * nt;
                    const double kn = kv[4 * c + 3];
                    double fj[kMaxLmax + 1], dfj[kMaxLmax + 1];
                    const double x = sys.type_rmt[t] * kn;
                    sphbes_dev(sys.max_lmax, x, fj);
                    dsphbs_dev(sys.max_lmax, x, fj, dfj);
                    for (int l = 0; l < nl; ++l) {
                        const int tl = t * nl + l;
                        au[c * tnl + tl] = sys.dE_u[tl] * kn * dfj[l] - sys.dE_u_dr[tl] * fj[l];
                        bu[c * tnl + tl] = -sys.u[tl] * kn * dfj[l] + sys.u_dr[tl] * fj[l];
                    }
                } else {
                    const int q = w - nb, c = q / nl, m = q - c * nl;
                    const double *k4 = kv + 4 * c;
                    double v[3];
                    for (int d = 0; d < 3; ++d) v[d] = R[d] * k4[0] + R[3 + d] * k4[1] + R[6 + d] * k4[2];
                    const double nrm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                    if (nrm > 0.0) { v[0] /= nrm; v[1] /= nrm; v[2] /= nrm; }
                    ylm_column_dev(sys.max_lmax, m, v, sys.ynorm, ylm + c * L);
                }
            }
            __syncthreads();
            // the rows M_t = [A_t; B_t] / e^{i 2pi K.tau} of each column (types with this rotation)
            for (int c = 0; c < ncols; ++c) {
                const int64_t gc = col0 + c;
                const KEntry &ent = tab.e[entry_of(tab, gc)];
                if (!ent.M) continue;
                double2 *mcol = ent.M + ldm * (gc - ent.col_begin);
                for (int idx = threadIdx.x; idx < twoL * nt; idx += blockDim.x) {
                    const int t = idx / twoL;
                    if (sys.num_rots > 0 && sys.type_rot[t] != rho) continue;
                    const int r = idx - t * twoL;
                    const bool isB = r >= L;
                    const int lm = isB ? r - L : r;
                    const int l = l_of[lm];
                    double2 out = make_double2(0.0, 0.0);
                    if (l <= sys.type_lmax[t]) {
                        const int tl = t * nl + l;
                        const double cc = cf[tl];
                        const double2 y = ylm[c * L + lm];
                        const double f = isB ? bu[c * tnl + tl] : au[c * tnl + tl];
                        out = make_double2((y.x * cc) * f, (-y.y * cc) * f);
                    }
                    mcol[idx] = out;
                }
            }
        }
    }
}

}  // namespace

// X[2L a + r, g] = e^{i 2pi (k+g).tau_a} Z[2L t(a) + r, g]: the per-atom T application rebuilt
// from the per-type product Z_t = T_t M_t, for the atoms [a0, a1) of the table.
__global__ void __launch_bounds__(kThreads) apply_phase_kernel(DevSystem sys, const __grid_constant__ KTable tab) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *ph = reinterpret_cast<double2 *>(smem_raw);       // [na]
    const int twoL = 2 * sys.L, na = sys.num_atoms;
    const int64_t ldz = tab.ldm, ldx = tab.ldc;
    for (int64_t gc = blockIdx.x; gc < tab.total_cols; gc += gridDim.x) {
        const KEntry &ent = tab.e[entry_of(tab, gc)];
        const DevKpoint &kp = ent.kp;
        const int64_t gi = gc - ent.col_begin;
        const double2 *Z = ent.Z;
        double2 *X = ent.X;
        __syncthreads();
        const int32_t *gv = kp.g + 3 * gi;
        const double K0 = kp.k[0] + gv[0], K1 = kp.k[1] + gv[1], K2 = kp.k[2] + gv[2];
        for (int j = threadIdx.x; j < na; j += blockDim.x) {
            const double *p = sys.atom_pos + 3 * j;
            double sn, cs;
            sincos(2 * kPi * (K0 * p[0] + K1 * p[1] + K2 * p[2]), &sn, &cs);
            ph[j] = make_double2(cs, sn);
        }
        __syncthreads();
        const double2 *zc = Z + ldz * gi;
        double2 *xc = X + ldx * gi;
        const int a0 = tab.a0, a1 = tab.a1 < 0 ? na : tab.a1;
        const int64_t r0 = (int64_t)twoL * a0, nrow = (int64_t)twoL * (a1 - a0);
        for (int64_t i = threadIdx.x; i < nrow; i += blockDim.x) {
            const int64_t idx = r0 + i;
            const int j = (int)(idx / twoL);
            const int r = (int)(idx - (int64_t)j * twoL);
            xc[idx] = cmul(ph[j], zc[(int64_t)twoL * sys.atom_type[j] + r]);
        }
    }
}

// The full Hermitian T block of a type, as the reference's zhemm('L') calls read it from the lower
// triangles (h_and_s_stripped_v2.cpp:202,345).  One CTA column per type (blockIdx.y), threads over
// the L x L entries (r fastest): each writes the four quadrant entries at (r, c) and folds its
// checks into the CTA's, then one atomic each.
constexpr int kTfThreads = 256;
__global__ void __launch_bounds__(kTfThreads) tfull_kernel(const double2 *__restrict__ aa_all,
                                                           const double2 *__restrict__ ab_all,
                                                           const double2 *__restrict__ bb_all, int L, double2 *tf,
                                                           unsigned long long *stats) {
    const int t = blockIdx.y;
    const int64_t LL = (int64_t)L * L, n = 2 * (int64_t)L;
    const double2 *aa = aa_all + t * LL, *ab = ab_all + t * LL, *bb = bb_all + t * LL;
    double2 *out = tf + t * 4 * LL;
    unsigned int flags = 0;
    unsigned long long st[4] = {0, 0, 0, 0};
    auto bits = [](double v) { return (unsigned long long)__double_as_longlong(v); };
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < LL; e += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % L), c = (int)(e / L);
        const int64_t i = r + (int64_t)L * c, iT = c + (int64_t)L * r;
        const double2 a = aa[i], aT = aa[iT], b = bb[i], bT = bb[iT], x = ab[i], xT = ab[iT];
        if (!isfinite(a.x) || !isfinite(a.y)) flags |= 1u;
        if (!isfinite(x.x) || !isfinite(x.y)) flags |= 2u;
        if (!isfinite(b.x) || !isfinite(b.y)) flags |= 4u;
        const bool low = r >= c;
        // a non-finite entry is flagged above and assembled as zero, so that nothing downstream
        // (the digit slicing above all) meets it before the flag is read
        auto fin = [](double2 v) { return (isfinite(v.x) && isfinite(v.y)) ? v : make_double2(0.0, 0.0); };
        out[r + n * c] = fin(low ? a : make_double2(aT.x, -aT.y));
        out[(L + r) + n * (L + c)] = fin(low ? b : make_double2(bT.x, -bT.y));
        out[r + n * (L + c)] = fin(x);
        out[(L + r) + n * c] = fin(make_double2(xT.x, -xT.y));
        if (low) {
            // |T|^2 of the pair and |T - T^H|^2 (the mirror element is the pair's other half)
            st[0] = max(st[0], bits(fmax(a.x * a.x + a.y * a.y, aT.x * aT.x + aT.y * aT.y)));
            st[1] = max(st[1], bits((a.x - aT.x) * (a.x - aT.x) + (a.y + aT.y) * (a.y + aT.y)));
            st[2] = max(st[2], bits(fmax(b.x * b.x + b.y * b.y, bT.x * bT.x + bT.y * bT.y)));
            st[3] = max(st[3], bits((b.x - bT.x) * (b.x - bT.x) + (b.y + bT.y) * (b.y + bT.y)));
        }
    }
    __shared__ unsigned long long red[kTfThreads / 32][4];
    __shared__ unsigned int fl[kTfThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        flags |= __shfl_xor_sync(0xffffffffu, flags, o);
        for (int q = 0; q < 4; ++q) st[q] = max(st[q], (unsigned long long)__shfl_xor_sync(0xffffffffu, st[q], o));
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        fl[w] = flags;
        for (int q = 0; q < 4; ++q) red[w][q] = st[q];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kTfThreads / 32; ++k) {
            flags |= fl[k];
            for (int q = 0; q < 4; ++q) st[q] = max(st[q], red[k][q]);
        }
        if (flags) atomicOr(stats + 5 * t, (unsigned long long)flags);
        for (int q = 0; q < 4; ++q)
            if (st[q]) atomicMax(stats + 5 * t + 1 + q, st[q]);
    }
}

__global__ void sf_phase_kernel(const double *pos, int na, int h0, int h1, int h2, int e0, int e1, int e2,
                                double2 *ph) {
    const int64_t n0 = (int64_t)na * e0, n1 = (int64_t)na * e1, total = n0 + n1 + (int64_t)na * e2;
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total; o += (int64_t)gridDim.x * blockDim.x) {
        int c, e, h;
        int64_t q = o;
        if (q < n0) { c = 0; e = e0; h = h0; }
        else if (q < n0 + n1) { q -= n0; c = 1; e = e1; h = h1; }
        else { q -= n0 + n1; c = 2; e = e2; h = h2; }
        const int j = (int)(q / e), i = (int)(q % e);
        double sn, cs;
        sincos(2 * kPi * (double)(i - h) * pos[3 * j + c], &sn, &cs);
        ph[o] = make_double2(cs, sn);
    }
}

int sm_count() {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    return nsm;
}

cudaError_t launch_tfull(const double2 *aa, const double2 *ab, const double2 *bb, int nt, int L, double2 *tf,
                         unsigned long long *stats, cudaStream_t st) {
    if (nt <= 0 || L <= 0) return cudaSuccess;
    const int64_t LL = (int64_t)L * L;
    const dim3 grid((unsigned)std::min<int64_t>((LL + kTfThreads - 1) / kTfThreads, 64), (unsigned)nt);
    tfull_kernel<<<grid, kTfThreads, 0, st>>>(aa, ab, bb, L, tf, stats);
    return cudaGetLastError();
}

cudaError_t launch_sf_phases(const double *pos, int na, const int *half, const int *ext, double2 *ph, cudaStream_t st) {
    const int64_t total = (int64_t)na * (ext[0] + ext[1] + ext[2]);
    if (total <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((total + 255) / 256, 4096);
    sf_phase_kernel<<<(unsigned)blocks, 256, 0, st>>>(pos, na, half[0], half[1], half[2], ext[0], ext[1], ext[2], ph);
    return cudaGetLastError();
}

cudaError_t launch_apply_phase_multi(const DevSystem &sys, const KTable &tab, cudaStream_t st) {
    if (tab.total_cols <= 0) return cudaSuccess;
    const int64_t grid = std::min<int64_t>(tab.total_cols, (int64_t)sm_count() * 8);
    const size_t smem = sizeof(double2) * sys.num_atoms;
    apply_phase_kernel<<<(unsigned)grid, kThreads, smem, st>>>(sys, tab);
    return cudaGetLastError();
}

cudaError_t launch_apply_phase(const DevSystem &sys, const DevKpoint &kp, const double2 *Z, int64_t ldz,
                               double2 *X, int64_t ldx, cudaStream_t st) {
    KTable tab;
    tab.nk = 1; tab.ldc = ldx; tab.ldm = ldz; tab.total_cols = kp.n_g;
    tab.e[0] = KEntry{kp, nullptr, nullptr, Z, X, 0};
    return launch_apply_phase_multi(sys, tab, st);
}

cudaError_t launch_construct_ab(const DevSystem &sys, const DevKpoint &kp, double2 *C, int64_t ldc,
                                cudaStream_t st, double2 *M, int64_t ldm) {
    KTable tab;
    tab.nk = 1; tab.ldc = ldc; tab.ldm = ldm; tab.total_cols = kp.n_g;
    tab.e[0] = KEntry{kp, C, M, nullptr, nullptr, 0};
    return launch_construct_ab_multi(sys, tab, st);
}

cudaError_t launch_construct_ab_multi(const DevSystem &sys, const KTable &tab, cudaStream_t st) {
    if (tab.total_cols <= 0) return cudaSuccess;
    bool anyM = false, anyC = false;
    for (int k = 0; k < tab.nk; ++k) { anyM = anyM || tab.e[k].M; anyC = anyC || tab.e[k].C; }
    const bool rot = sys.atom_rotmat != nullptr;
    const size_t smem_rows = rows_kernel_smem(sys.L, sys.max_lmax, sys.num_types);
    // (the column-per-CTA kernel below for many types at a high lmax, whose tables do not fit;
    // per-type rows of (type, rotation) classes come only from this kernel)
    if ((!rot || sys.num_rots > 0) && anyM && !anyC && smem_rows <= kRowsKernelSmemMax) {
        const size_t smem = smem_rows;
        cudaError_t e = cudaFuncSetAttribute(construct_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        const int64_t grid = std::min<int64_t>((tab.total_cols + kRowCols - 1) / kRowCols, (int64_t)sm_count() * 4);
        construct_rows_kernel<<<(unsigned)grid, kThreads, smem, st>>>(sys, tab);
        return cudaGetLastError();
    }
    const int nl = sys.max_lmax + 1;
    size_t smem = sizeof(double) * 2 * sys.num_types * nl + sizeof(double2) * sys.num_atoms +
                  sizeof(double2) * (rot ? kRotChunk : 1) * sys.L + sys.L + 16;
    smem = (smem + 15) & ~size_t(15);
    const int64_t grid = std::min<int64_t>(tab.total_cols, (int64_t)sm_count() * 8);
    if (rot) {
        if (anyM) return cudaErrorInvalidValue;  // per-type rows exist only when atoms share the rotation
        cudaFuncSetAttribute(construct_ab_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        construct_ab_kernel<true><<<(unsigned)grid, kThreads, smem, st>>>(sys, tab);
    } else {
        cudaFuncSetAttribute(construct_ab_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        construct_ab_kernel<false><<<(unsigned)grid, kThreads, smem, st>>>(sys, tab);
    }
    return cudaGetLastError();
}

}  // namespace hsdla
