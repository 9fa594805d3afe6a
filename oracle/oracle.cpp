// CPU oracle for the FLAPW H/S generation path -- TEST INFRASTRUCTURE ONLY.
//
// This file is the checker against which the GPU library is compared.  Only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it; the
// library never calls it.  It restates, in plain C++ loops, the reference's
// algorithm for the path (file:line citations are relative to the reference
// project root):
//
//   sphbes      flapw_opt/external/compat/fleur/sphbes.f:19-76
//   dsphbs      flapw_opt/external/compat/fleur/dsphbs.f:24-42
//   ylm4        flapw_opt/external/compat/fleur/ylm4.f:4-139
//   kmesh       flapw_opt/src/types_helper.cpp:20-37   (r_K = |bmat (k+G)|)
//   construct_AB flapw_opt/src/tensor_AB_match.cpp:63-129
//   TMat / zero_nonsph / augment_tmats
//               flapw_opt/src/types_helper.cpp:41-90, flapw_opt/src/AtomData.cpp:95-145
//   naive S, H  flapw_opt/src/h_and_s.cpp:88-162
//   radfun      flapw_opt/external/compat/fleur/radfun.f:3-58, radsra.f:10-139,
//               radsrd.F:31-169, intgr.F:68-126 (intgr0), constants.f:15-25;
//               the call convention of flapw_opt/external/compat/libflerp.f90:50-90
//               (r0 = R_MT exp(dx (1 - n))).  Only the Fleur-dump golden test uses it:
//               the GPU library takes the boundary values as inputs.
//
// The reference's Fortran is compiled with -fdefault-real-8 / -r8, so every
// REAL is a double and every COMPLEX a double complex; these restatements use
// double throughout and call the C library's sin/cos/sqrt.
//
// Layouts: complex numbers are interleaved (re, im) doubles.  A and B are the
// reference's cubes (L, a, G) in column-major order, i.e. element
// (lm, atom, g) sits at lm + L*atom + L*a*g.  bmat and rotation matrices are
// 3x3 row-major with row i = reciprocal basis vector b_i.  T matrices are L x L
// column-major.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

typedef std::complex<double> cxd;

static const double kPi = 3.14159265358979323846;

extern "C" {

// sphbes.f:19-76 -- spherical Bessel j_l(x), l = 0..lmax (lmax >= 1, x >= 0).
int oracle_sphbes(int lmax, double x, double *fj) {
    if (lmax < 1 || x < 0.0) return -1;
    const double small = 1.0e-3;
    double xx = x * x;
    double xinv = 0.0;
    if (x >= small) {
        xinv = 1.0 / x;
        fj[0] = std::sin(x) * xinv;
        fj[1] = (fj[0] - std::cos(x)) * xinv;
    } else {
        fj[0] = 1.0 - xx / 6.0 * (1.0 - xx / 20.0 * (1.0 - xx / 42.0));
        fj[1] = (x / 3.0) * (1.0 - xx / 10.0 * (1.0 - xx / 28.0));
        double fac = xx / 15.0;
        for (int l = 2; l <= lmax; ++l) {
            fj[l] = fac * (1.0 - xx / (4 * l + 6));
            fac = x * fac / (2 * l + 3);
        }
        return 0;
    }
    if ((double)lmax < x) {
        for (int l = 2; l <= lmax; ++l) fj[l] = (2 * l - 1) * xinv * fj[l - 1] - fj[l - 2];
    } else if (lmax >= 2) {
        int n = (int)(lmax + 10 + x);
        std::vector<double> aux(n + 1);
        aux[n] = 0.0;
        aux[n - 1] = 1.0;
        for (int i = n - 1; i >= 1; --i) aux[i - 1] = (2 * i + 1) * xinv * aux[i] - aux[i + 1];
        int mn = 0;
        if (std::fabs(fj[0]) < std::fabs(fj[1])) mn = 1;
        double quot = fj[mn] / aux[mn];
        for (int l = 2; l <= lmax; ++l) fj[l] = aux[l] * quot;
    }
    return 0;
}

// dsphbs.f:24-42 -- d j_l / dx from the j_l values.
void oracle_dsphbs(int lmax, double x, const double *fj, double *dfj) {
    const double xlim = 1.0e-4;
    dfj[0] = -fj[1];
    if (x < xlim) {
        double x2 = 0.5 * x * x;
        double fac = 1.0 / 3.0;
        for (int l = 1; l <= lmax; ++l) {
            dfj[l] = fac * (l - x2 * (l + 2) / (2 * l + 3));
            fac = x * fac / (2 * l + 3);
        }
    } else {
        for (int l = 1; l <= lmax; ++l) dfj[l] = fj[l - 1] - (l + 1) * fj[l] / x;
    }
}

// ylm4.f:4-139 -- complex Y_lm(v) for l <= lmax at index l(l+1)+m.
void oracle_ylm4(int lmax, const double *v, double *ylm_out) {
    const double small = 1.0e-12;
    const int n1 = lmax + 1;
    std::vector<double> ynorm(n1 * n1), p(n1 * n1), c(n1), s(n1);
    // ylmnorm (ylm4.f:111-137); pimach() = 3.1415926535897932
    const double fpi = 4.0 * 3.1415926535897932;
    for (int l = 0; l <= lmax; ++l) {
        int lm0 = l * (l + 1);
        double cd = 1.0;
        double a = std::sqrt((2 * l + 1) / fpi);
        ynorm[lm0] = a;
        for (int m = 1; m <= l; ++m) {
            cd = cd / ((l + 1 - m) * (l + m));
            ynorm[lm0 + m] = a * std::sqrt(cd);
            ynorm[lm0 - m] = ((m & 1) ? -1.0 : 1.0) * ynorm[lm0 + m];
        }
    }
    double x = v[0], y = v[1], z = v[2];
    double xy = x * x + y * y;
    double r = std::sqrt(xy + z * z);
    double rxy = std::sqrt(xy);
    double cth, sth, cph, sph;
    if (r > small) { cth = z / r; sth = rxy / r; } else { sth = 0.0; cth = 1.0; }
    if (rxy > small) { cph = x / rxy; sph = y / rxy; } else { cph = 1.0; sph = 0.0; }
#define P(l, m) p[(l) * n1 + (m)]
    double fac = 1.0;
    for (int m = 0; m <= lmax - 1; ++m) {
        fac = -(m + m - 1) * fac;
        P(m, m) = fac;
        P(m + 1, m) = (m + m + 1) * cth * fac;
        for (int l = m + 2; l <= lmax; ++l)
            P(l, m) = ((l + l - 1) * cth * P(l - 1, m) - (l + m - 1) * P(l - 2, m)) / (l - m);
        fac = fac * sth;
    }
    P(lmax, lmax) = -(lmax + lmax - 1) * fac;
    s[0] = 0.0; c[0] = 1.0;
    if (lmax >= 1) { s[1] = sph; c[1] = cph; }
    double cph2 = cph + cph;
    for (int m = 2; m <= lmax; ++m) {
        s[m] = cph2 * s[m - 1] - s[m - 2];
        c[m] = cph2 * c[m - 1] - c[m - 2];
    }
    for (int l = 0; l <= lmax; ++l) {
        int lm = l * (l + 1);
        ylm_out[2 * lm] = ynorm[lm] * P(l, 0);
        ylm_out[2 * lm + 1] = 0.0;
    }
    for (int m = 1; m <= lmax; ++m) {
        for (int l = m; l <= lmax; ++l) {
            int lm0 = l * (l + 1);
            double yr = P(l, m) * c[m], yi = P(l, m) * s[m];
            ylm_out[2 * (lm0 + m)] = ynorm[lm0 + m] * yr;
            ylm_out[2 * (lm0 + m) + 1] = ynorm[lm0 + m] * yi;
            ylm_out[2 * (lm0 - m)] = yr * ynorm[lm0 - m];
            ylm_out[2 * (lm0 - m) + 1] = -yi * ynorm[lm0 - m];
        }
    }
#undef P
}

// types_helper.cpp:20-37 -- r_K(i) = || bmat * (k + g_i) || (bmat rows = b_i).
void oracle_kmesh(const double *k, const double *bmat, const int32_t *g, int64_t n, double *rK) {
    for (int64_t i = 0; i < n; ++i) {
        double K[3] = {k[0] + g[3 * i], k[1] + g[3 * i + 1], k[2] + g[3 * i + 2]};
        double s = 0.0;
        for (int r = 0; r < 3; ++r) {
            double t = bmat[3 * r] * K[0] + bmat[3 * r + 1] * K[1] + bmat[3 * r + 2] * K[2];
            s += t * t;
        }
        rK[i] = std::sqrt(s);
    }
}

// tensor_AB_match.cpp:63-129.  Per-atom quantities are indexed per type via
// atom_type (the reference replicates them per atom, FleurData.cpp:52-62).
// rotmat: [a][9] row-major (mrot * bmat) or NULL for identity mrot (rotmat = bmat).
// u_* arrays: [types][max_lmax+1].  A, B: interleaved complex (L, a, G).
int oracle_construct_ab(int num_atoms, int max_lmax, double vol_cell, const double *bmat,
                        const int32_t *atom_type, const double *atom_pos, const double *rotmat,
                        const double *type_rmt, const int32_t *type_lmax,
                        const double *u, const double *u_dr, const double *dE_u,
                        const double *dE_u_dr,
                        const double *kpt, const int32_t *g, int64_t n_g,
                        double *A_out, double *B_out, int nthreads) {
    const int L = (max_lmax + 1) * (max_lmax + 1);
    const int nl = max_lmax + 1;
    const int64_t La = (int64_t)L * num_atoms;
    std::vector<double> rK(n_g);
    oracle_kmesh(kpt, bmat, g, n_g, rK.data());
    const double vol_prefac = 4 * kPi / std::sqrt(vol_cell);
    cxd *A = reinterpret_cast<cxd *>(A_out);
    cxd *B = reinterpret_cast<cxd *>(B_out);
    std::memset(A_out, 0, sizeof(cxd) * La * n_g);
    std::memset(B_out, 0, sizeof(cxd) * La * n_g);
    int status = 0;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t i = 0; i < n_g; ++i) {
        std::vector<double> fj(nl), dfj(nl), ylm(2 * L);
        double K[3] = {kpt[0] + g[3 * i], kpt[1] + g[3 * i + 1], kpt[2] + g[3 * i + 2]};
        double K_norm = rK[i];
        for (int j = 0; j < num_atoms; ++j) {
            const int t = atom_type[j];
            const double *R = rotmat ? rotmat + 9 * j : bmat;
            // K_base = normalise(R^T K)
            double kb[3];
            for (int c = 0; c < 3; ++c) kb[c] = R[c] * K[0] + R[3 + c] * K[1] + R[6 + c] * K[2];
            double nrm = std::sqrt(kb[0] * kb[0] + kb[1] * kb[1] + kb[2] * kb[2]);
            if (nrm > 0.0) for (int c = 0; c < 3; ++c) kb[c] /= nrm;
            const double *p = atom_pos + 3 * j;
            double arg = 2 * kPi * (K[0] * p[0] + K[1] * p[1] + K[2] * p[2]);
            cxd phase = std::exp(cxd(0.0, arg));
            if (oracle_sphbes(max_lmax, type_rmt[t] * K_norm, fj.data()) != 0) {
                status = -1;
                continue;
            }
            oracle_dsphbs(max_lmax, type_rmt[t] * K_norm, fj.data(), dfj.data());
            oracle_ylm4(max_lmax, kb, ylm.data());
            for (int l = 0; l <= type_lmax[t]; ++l) {
                const int tl = t * nl + l;
                double A_u = dE_u[tl] * K_norm * dfj[l] - dE_u_dr[tl] * fj[l];
                double B_u = -u[tl] * K_norm * dfj[l] + u_dr[tl] * fj[l];
                double inv_w = 1. / (dE_u[tl] * u_dr[tl] - u[tl] * dE_u_dr[tl]);
                cxd common = vol_prefac * phase * inv_w;
                for (int m = -l; m <= l; ++m) {
                    int lm = l * (l + 1) + m;
                    cxd yc(ylm[2 * lm], -ylm[2 * lm + 1]);
                    A[lm + (int64_t)L * j + La * i] = yc * common * A_u;
                    B[lm + (int64_t)L * j + La * i] = yc * common * B_u;
                }
            }
        }
    }
    return status;
}

// types_helper.cpp:41-90 and AtomData.cpp:95-145 for one type.
// Inputs are Fleur's blocks (only the lower triangles are read): taa, tbb,
// tab, tba, each n x n column-major with n = (lmax+1)^2.  Output: augmented
// full aa, ab, bb (n x n column-major); ba = ab^H is implied.
int oracle_prepare_tmat(int lmax, int lmax_nonsph, const double *taa_in, const double *tbb_in,
                        const double *tab_in, const double *tba_in, const double *E_l,
                        const double *dE_u_norm, double *aa_out, double *ab_out, double *bb_out) {
    const int n = (lmax + 1) * (lmax + 1);
    const cxd *taa = reinterpret_cast<const cxd *>(taa_in);
    const cxd *tbb = reinterpret_cast<const cxd *>(tbb_in);
    const cxd *tab = reinterpret_cast<const cxd *>(tab_in);
    const cxd *tba = reinterpret_cast<const cxd *>(tba_in);
    cxd *aa = reinterpret_cast<cxd *>(aa_out);
    cxd *ab = reinterpret_cast<cxd *>(ab_out);
    cxd *bb = reinterpret_cast<cxd *>(bb_out);
    for (int c = 0; c < n; ++c)
        for (int r = 0; r < n; ++r) {
            // symmatl: lower triangle mirrored with conjugation
            aa[r + n * c] = (r >= c) ? taa[r + n * c] : std::conj(taa[c + n * r]);
            bb[r + n * c] = (r >= c) ? tbb[r + n * c] : std::conj(tbb[c + n * r]);
            // trimatl(tab) + trimatu(tba^H), diagonal from tab
            ab[r + n * c] = (r >= c) ? tab[r + n * c] : std::conj(tba[c + n * r]);
        }
    for (int r = 0; r < n; ++r)
        if (std::fabs(std::abs(tab[r + n * r] - tba[r + n * r])) >= 1e-15) return -2;
    // zero_nonsph: rows/cols >= (lmax_nonsph+1)^2 cleared
    const int s0 = (lmax_nonsph + 1) * (lmax_nonsph + 1);
    if (s0 < n) {
        for (int c = 0; c < n; ++c)
            for (int r = 0; r < n; ++r)
                if (r >= s0 || c >= s0) {
                    aa[r + n * c] = 0.0; ab[r + n * c] = 0.0; bb[r + n * c] = 0.0;
                }
    }
    for (int l = 0; l <= lmax; ++l)
        for (int m = -l; m <= l; ++m) {
            int lm = l * (l + 1) + m;
            aa[lm + n * lm] += E_l[l];
            bb[lm + n * lm] += E_l[l] * dE_u_norm[l];
            ab[lm + n * lm] += 0.5;
        }
    return 0;
}

// h_and_s.cpp:88-162 -- direct-formula S and H (all n_g x n_g entries).
// aa, ab, bb: per atom, L x L column-major (ba = ab^H).  dE_u_norm: per atom,
// max_lmax+1 values.  H and S column-major G x G.
void oracle_hs_naive(int L, int num_atoms, int max_lmax, int64_t n_g, const double *A_in,
                     const double *B_in, const double *aa_in, const double *ab_in,
                     const double *bb_in, const double *dE_u_norm, double *H_out,
                     double *S_out, int nthreads) {
    const cxd *A = reinterpret_cast<const cxd *>(A_in);
    const cxd *B = reinterpret_cast<const cxd *>(B_in);
    const cxd *aa = reinterpret_cast<const cxd *>(aa_in);
    const cxd *ab = reinterpret_cast<const cxd *>(ab_in);
    const cxd *bb = reinterpret_cast<const cxd *>(bb_in);
    cxd *H = reinterpret_cast<cxd *>(H_out);
    cxd *S = reinterpret_cast<cxd *>(S_out);
    const int64_t La = (int64_t)L * num_atoms;
    const int64_t LL = (int64_t)L * L;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t G = 0; G < n_g; ++G) {
        for (int64_t Gp = 0; Gp < n_g; ++Gp) {
            cxd s = 0.0;
            for (int at = 0; at < num_atoms; ++at)
                for (int l = 0; l <= max_lmax; ++l) {
                    double un = dE_u_norm[at * (max_lmax + 1) + l];
                    for (int m = -l; m <= l; ++m) {
                        int lm = l * (l + 1) + m;
                        s += std::conj(A[lm + L * at + La * Gp]) * A[lm + L * at + La * G] +
                             std::conj(B[lm + L * at + La * Gp]) * B[lm + L * at + La * G] * un;
                    }
                }
            S[Gp + n_g * G] = s;
            cxd h = 0.0;
            for (int at = 0; at < num_atoms; ++at) {
                const cxd *Aa = A + L * at, *Ba = B + L * at;
                const cxd *taa = aa + LL * at, *tab = ab + LL * at, *tbb = bb + LL * at;
                for (int lm = 0; lm < L; ++lm)
                    for (int lmp = 0; lmp < L; ++lmp) {
                        cxd cA = std::conj(Aa[lmp + La * G]), cB = std::conj(Ba[lmp + La * G]);
                        h += cA * taa[lmp + L * lm] * Aa[lm + La * Gp];
                        h += cB * tbb[lmp + L * lm] * Ba[lm + La * Gp];
                        h += cA * tab[lmp + L * lm] * Ba[lm + La * Gp];
                        h += cB * std::conj(tab[lm + L * lmp]) * Aa[lm + La * Gp];
                    }
            }
            H[G + n_g * Gp] = h;
        }
    }
}

// ---------------------------------------------------------------- radial solver
// intgr0 (intgr.F:68-126): definite integral of y on the logarithmic mesh r_i = r0 e^{h(i-1)},
// a power-law start on [0, r0], 7-point Lagrange steps up to the point n0 where the
// Simpson-type 7-point rule (weights 41,216,27,272,27,216,41 / 140) takes over.
static double intgr0(const double *y, double r0, double h, int jri) {
    static const double lag[5][7] = {
        {19087., 65112., -46461., 37504., -20211., 6312., -863.},
        {-863., 25128., 46989., -16256., 7299., -2088., 271.},
        {271., -2760., 30819., 37504., -6771., 1608., -191.},
        {-191., 1608., -6771., 37504., 30819., -2760., 271.},
        {271., -2088., 7299., -16256., 46989., 25128., -863.}};
    static const double w7[7] = {41., 216., 27., 272., 27., 216., 41.};
    double z = 0.0;
    if (y[0] * y[1] > 0.0) {
        const double alpha = 1.0 + std::log(y[1] / y[0]) / h;
        if (alpha > 0.0) z = r0 * y[0] / alpha;
    }
    const int nsteps = (jri - 1) / 6;
    int n0 = jri - 6 * nsteps;           // 1-based start of the 7-point rule
    const double dr = std::exp(h);
    double r[7];
    r[0] = r0;
    for (int i = 1; i < 7; ++i) r[i] = dr * r[i - 1];
    if (n0 > 1) {
        double yr[7];
        for (int i = 0; i < 7; ++i) yr[i] = r[i] * y[i];
        for (int j = 0; j < n0 - 1; ++j) {
            double d = 0.0;
            for (int i = 0; i < 7; ++i) d += lag[j][i] * yr[i];
            z += h * d / 60480.;
        }
    }
    r[0] = r[n0 - 1];
    for (int m = 0; m < nsteps; ++m) {
        for (int i = 1; i < 7; ++i) r[i] = dr * r[i - 1];
        double d = 0.0;
        for (int i = 0; i < 7; ++i) d += (h * w7[i] * r[i] / 140.) * y[n0 - 1 + i];
        z += d;
        n0 += 6;
        r[0] = r[6];
    }
    return z;
}

// Scalar-relativistic outward integration of (p, q) = (r u, c^-1 r u_small) at energy e
// (radsra.f:10-139) and of its energy derivative (pe, qe) (radsrd.F:31-169, with the
// relativistic correction factor (1 + fl1/(c rm)^2) of the RELATIVISTIC_CORRECTIONS build):
// 4th-order Runge-Kutta for the first five steps, then the 6-step Adams-Bashforth
// predictor / Adams-Moulton corrector (at most five corrector sweeps, relative tolerance 1e-6).
// vr = r V(r) on the n-point mesh ending at rmt.  out = {u(R), u'(R), udot(R), udot'(R),
// <udot|udot>} (the rad_match fields u, u_dr, dE_u, dE_u_dr, dE_u_norm).
int oracle_radfun(int l, double e, const double *vr, int n, double rmt, double h, double *out) {
    if (n < 13 || !(h > 0.0) || !(rmt > 0.0)) return -1;
    const double c = 137.0359895;          // constants.f:22, Hartree units
    const double cin = 1.0 / c, cin2 = cin * cin;
    const double r0 = rmt * std::exp(h * (1 - n));
    const double fl1 = (double)l * (l + 1);
    const double dr = std::exp(h), drh = std::sqrt(dr);
    const double eps = 1e-6;
    std::vector<double> p(n), q(n), pp(n), qp(n), pe(n), qe(n);
    // ---- u at e
    double s = std::sqrt(fl1 + 1 - cin2 * vr[0] * vr[0]) - 1.;
    double rm = 2. * r0 + cin2 * (r0 * e - vr[0]);
    p[0] = std::pow(r0, l + 1);
    q[0] = s * p[0] / rm;
    pp[0] = rm * q[0] + p[0];
    qp[0] = (fl1 / rm + vr[0] - r0 * e) * p[0] - q[0];
    double r = r0;
    for (int i = 0; i < 5; ++i) {
        const double rh2 = drh * r, rh = dr * r;
        const double sk1 = h * pp[i], sl1 = h * qp[i];
        double rve = 0.5 * (vr[i] + vr[i + 1]) - rh2 * e;
        rm = 2. * rh2 - cin2 * rve;
        double yn = p[i] + 0.5 * sk1, zn = q[i] + 0.5 * sl1;
        const double sk2 = h * (rm * zn + yn), sl2 = h * ((fl1 / rm + rve) * yn - zn);
        yn = p[i] + 0.5 * sk2; zn = q[i] + 0.5 * sl2;
        const double sk3 = h * (rm * zn + yn), sl3 = h * ((fl1 / rm + rve) * yn - zn);
        rve = vr[i + 1] - rh * e;
        rm = 2. * rh - cin2 * rve;
        yn = p[i] + sk3; zn = q[i] + sl3;
        const double sk4 = h * (rm * zn + yn), sl4 = h * ((fl1 / rm + rve) * yn - zn);
        p[i + 1] = p[i] + (sk1 + 2. * sk2 + 2. * sk3 + sk4) / 6.;
        q[i + 1] = q[i] + (sl1 + 2. * sl2 + 2. * sl3 + sl4) / 6.;
        pp[i + 1] = rm * q[i + 1] + p[i + 1];
        qp[i + 1] = (fl1 / rm + rve) * p[i + 1] - q[i + 1];
        r = rh;
    }
    for (int i = 5; i < n - 1; ++i) {
        r = r * dr;
        double p0 = p[i] + h * (4277. * pp[i] - 7923. * pp[i - 1] + 9982. * pp[i - 2] - 7298. * pp[i - 3] +
                                2877. * pp[i - 4] - 475. * pp[i - 5]) / 1440.;
        double q0 = q[i] + h * (4277. * qp[i] - 7923. * qp[i - 1] + 9982. * qp[i - 2] - 7298. * qp[i - 3] +
                                2877. * qp[i - 4] - 475. * qp[i - 5]) / 1440.;
        const double rve = vr[i + 1] - r * e;
        rm = 2. * r - cin2 * rve;
        double p1p = rm * q0 + p0, q1p = (fl1 / rm + rve) * p0 - q0, p1 = p0, q1 = q0;
        for (int it = 0; it < 5; ++it) {
            p1 = p[i] + h * (475. * p1p + 1427. * pp[i] - 798. * pp[i - 1] + 482. * pp[i - 2] - 173. * pp[i - 3] +
                             27. * pp[i - 4]) / 1440.;
            q1 = q[i] + h * (475. * q1p + 1427. * qp[i] - 798. * qp[i - 1] + 482. * qp[i - 2] - 173. * qp[i - 3] +
                             27. * qp[i - 4]) / 1440.;
            p1p = rm * q1 + p1;
            q1p = (fl1 / rm + rve) * p1 - q1;
            const double erp = std::fabs(p1 - p0) / (std::fabs(p1) + std::fabs(h * p1p));
            const double erq = std::fabs(q1 - q0) / (std::fabs(q1) + std::fabs(h * p1p));
            if (erp < eps && erq < eps) break;
            p0 = p1;
            q0 = q1;
        }
        p[i + 1] = p1; q[i + 1] = q1; pp[i + 1] = p1p; qp[i + 1] = q1p;
    }
    for (int i = 0; i < n; ++i) q[i] = cin * q[i];
    std::vector<double> y(n);
    for (int i = 0; i < n; ++i) y[i] = p[i] * p[i] + q[i] * q[i];
    double t = 1.0 / std::sqrt(intgr0(y.data(), r0, h, n));
    const double us = t * p[n - 1] / r;
    const double dus = t * (pp[n - 1] - p[n - 1]) / (r * r);
    for (int i = 0; i < n; ++i) { p[i] *= t; q[i] *= t; }
    // ---- udot at e (orthogonalised to u)
    auto corr = [&](double rmv) { return 1. + cin2 * fl1 / (rmv * rmv); };
    rm = 2. * r0 + cin2 * (r0 * e - vr[0]);
    pe[0] = 0; qe[0] = 0;
    pp[0] = r0 * cin * q[0];
    qp[0] = -r0 * p[0] * corr(rm);
    r = r0;
    for (int i = 0; i < 5; ++i) {
        const double rh2 = drh * r, rh = dr * r;
        const double sk1 = h * pp[i], sl1 = h * qp[i];
        double rve = 0.5 * (vr[i] + vr[i + 1]) - rh2 * e;
        rm = 2. * rh2 - cin2 * rve;
        double yn = pe[i] + 0.5 * sk1, zn = qe[i] + 0.5 * sl1;
        const double t1 = 0.5 * rh2 * cin * (q[i] + q[i + 1]);
        const double t2 = 0.5 * rh2 * (p[i] + p[i + 1]) * corr(rm);
        const double sk2 = h * (rm * zn + yn + t1), sl2 = h * ((fl1 / rm + rve) * yn - zn - t2);
        yn = pe[i] + 0.5 * sk2; zn = qe[i] + 0.5 * sl2;
        const double sk3 = h * (rm * zn + yn + t1), sl3 = h * ((fl1 / rm + rve) * yn - zn - t2);
        rve = vr[i + 1] - rh * e;
        rm = 2. * rh - cin2 * rve;
        yn = pe[i] + sk3; zn = qe[i] + sl3;
        const double sk4 = h * (rm * zn + yn + rh * cin * q[i + 1]);
        const double sl4 = h * ((fl1 / rm + rve) * yn - zn - rh * p[i + 1] * corr(rm));
        pe[i + 1] = pe[i] + (sk1 + 2. * sk2 + 2. * sk3 + sk4) / 6.;
        qe[i + 1] = qe[i] + (sl1 + 2. * sl2 + 2. * sl3 + sl4) / 6.;
        pp[i + 1] = rm * qe[i + 1] + pe[i + 1] + rh * cin * q[i + 1];
        qp[i + 1] = (fl1 / rm + rve) * pe[i + 1] - qe[i + 1] - rh * p[i + 1] * corr(rm);
        r = rh;
    }
    for (int i = 5; i < n - 1; ++i) {
        r = r * dr;
        double p0 = pe[i] + h * (4277. * pp[i] - 7923. * pp[i - 1] + 9982. * pp[i - 2] - 7298. * pp[i - 3] +
                                 2877. * pp[i - 4] - 475. * pp[i - 5]) / 1440.;
        double q0 = qe[i] + h * (4277. * qp[i] - 7923. * qp[i - 1] + 9982. * qp[i - 2] - 7298. * qp[i - 3] +
                                 2877. * qp[i - 4] - 475. * qp[i - 5]) / 1440.;
        const double rve = vr[i + 1] - r * e;
        rm = 2. * r - cin2 * rve;
        const double t1 = cin * r * q[i + 1];
        const double t2 = r * p[i + 1] * corr(rm);
        double p1p = rm * q0 + p0 + t1, q1p = (fl1 / rm + rve) * p0 - q0 - t2, p1 = p0, q1 = q0;
        for (int it = 0; it < 5; ++it) {
            p1 = pe[i] + h * (475. * p1p + 1427. * pp[i] - 798. * pp[i - 1] + 482. * pp[i - 2] - 173. * pp[i - 3] +
                              27. * pp[i - 4]) / 1440.;
            q1 = qe[i] + h * (475. * q1p + 1427. * qp[i] - 798. * qp[i - 1] + 482. * qp[i - 2] - 173. * qp[i - 3] +
                              27. * qp[i - 4]) / 1440.;
            p1p = rm * q1 + p1 + t1;
            q1p = (fl1 / rm + rve) * p1 - q1 - t2;
            const double erp = std::fabs(p1 - p0) / (std::fabs(p1) + std::fabs(h * p1p));
            const double erq = std::fabs(q1 - q0) / (std::fabs(q1) + std::fabs(h * p1p));
            if (erp < eps && erq < eps) break;
            p0 = p1;
            q0 = q1;
        }
        pe[i + 1] = p1; qe[i + 1] = q1; pp[i + 1] = p1p; qp[i + 1] = q1p;
    }
    for (int i = 0; i < n; ++i) qe[i] = cin * qe[i];
    for (int i = 0; i < n; ++i) y[i] = p[i] * pe[i] + q[i] * qe[i];
    t = intgr0(y.data(), r0, h, n);
    double dud = (pp[n - 1] - pe[n - 1]) / (r * r);
    for (int i = 0; i < n; ++i) { pe[i] -= t * p[i]; qe[i] -= t * q[i]; }
    const double ud = pe[n - 1] / r;
    dud = dud - t * dus;
    for (int i = 0; i < n; ++i) y[i] = pe[i] * pe[i] + qe[i] * qe[i];
    const double ddn = intgr0(y.data(), r0, h, n);
    out[0] = us; out[1] = dus; out[2] = ud; out[3] = dud; out[4] = ddn;
    return 0;
}

}  // extern "C"
