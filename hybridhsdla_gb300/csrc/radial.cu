// Boundary values of Fleur's scalar-relativistic radial solutions: the inputs of the matching
// step (AtomData::generate_matchdata, flapw_opt/src/AtomData.cpp:72-88, through radial_solve,
// flapw_opt/src/special_funcs.cpp:21-36, and libflerp's wrap_radfun, external/compat/libflerp.f90:50-93).
//
// For angular momentum l, energy e and the potential r V(r) on Fleur's logarithmic mesh
// r_i = r_0 e^{(i-1) h}, r_n = R_MT, the large and small components (p, q) of r u(r) are
// integrated outward (radsra.f): a fourth-order Runge-Kutta start over five steps, then the
// sixth-order Adams-Bashforth predictor with an Adams-Moulton corrector iterated to a relative
// change of 1e-6 (at most five times), normalised with intgr0.  The energy derivative (pe, qe)
// solves the inhomogeneous equation (radsrd.F, with its relativistic correction factor
// 1 + fl1 / (c rm)^2 on the inhomogeneous term) and is made orthogonal to (p, q).  intgr0
// integrates on the mesh: the power-series start below r_0, the 7-point Lagrange rule on the
// first points and the 7-point Simpson-like rule after them.  c is Fleur's speed of light in
// Hartree units, 137.0359895.  Host code, run once per (type, l) of a run, as in the reference.
#include <cmath>
#include <vector>

#include "common.cuh"

namespace hsdla {
namespace {

constexpr double kLight = 137.0359895;
constexpr double kCorrEps = 1.0e-6;

// The 7-point Lagrange weights of intgr.F (divided by 60480) for the integrals over the first
// mesh intervals, and the 7-point rule of the rest (weights / 140 per 6 intervals).
constexpr double kLagrange[5][7] = {
    {19087., 65112., -46461., 37504., -20211., 6312., -863.},
    {-863., 25128., 46989., -16256., 7299., -2088., 271.},
    {271., -2760., 30819., 37504., -6771., 1608., -191.},
    {-191., 1608., -6771., 37504., 30819., -2760., 271.},
    {271., -2088., 7299., -16256., 46989., 25128., -863.}};
constexpr double kRule[7] = {41., 216., 27., 272., 27., 216., 41.};

// Integral of y over the mesh (intgr0): y[0 .. n-1] at r0 e^{i h}.
double integrate(const std::vector<double> &y, double r0, double h, int n) {
    double z = 0.0;
    if (y[0] * y[1] > 0.0) {
        // below r0: the leading power y ~ r^(alpha - 1)
        const double alpha = 1.0 + std::log(y[1] / y[0]) / h;
        if (alpha > 0.0) z = r0 * y[0] / alpha;
    }
    const int steps = (n - 1) / 6;
    int n0 = n - 6 * steps;           // first point of the 6-interval blocks (1-based)
    const double dr = std::exp(h);
    double r[7];
    r[0] = r0;
    for (int i = 1; i < 7; ++i) r[i] = dr * r[i - 1];
    if (n0 > 1) {
        double yr[7];
        for (int i = 0; i < 7; ++i) yr[i] = r[i] * y[i];
        for (int j = 0; j < n0 - 1; ++j) {
            double dot = 0.0;
            for (int i = 0; i < 7; ++i) dot += kLagrange[j][i] * yr[i];
            z += h * dot / 60480.0;
        }
    }
    r[0] = r[n0 - 1];
    for (int m = 0; m < steps; ++m) {
        for (int i = 1; i < 7; ++i) r[i] = dr * r[i - 1];
        double dot = 0.0;
        for (int i = 0; i < 7; ++i) dot += (h * kRule[i] * r[i] / 140.0) * y[n0 - 1 + i];
        z += dot;
        n0 += 6;
        r[0] = r[6];
    }
    return z;
}

// The 6-step Adams-Bashforth predictor and Adams-Moulton corrector weights (/1440).
inline double predict(const std::vector<double> &d, int i) {
    return (4277. * d[i] - 7923. * d[i - 1] + 9982. * d[i - 2] - 7298. * d[i - 3] + 2877. * d[i - 4] -
            475. * d[i - 5]) / 1440.;
}
inline double correct(double dnext, const std::vector<double> &d, int i) {
    return (475. * dnext + 1427. * d[i] - 798. * d[i - 1] + 482. * d[i - 2] - 173. * d[i - 3] + 27. * d[i - 4]) /
           1440.;
}

struct RadialSolution {
    std::vector<double> p, q;   // normalised large and small components on the mesh
    double us = 0, dus = 0;     // u(R), u'(R)
    double r_end = 0;           // the last mesh radius as the integration reached it
};

// radsra.f: u at energy e.
RadialSolution solve_u(int l, double e, const double *vr, int n, double r0, double h) {
    const double cin = 1.0 / kLight, cin2 = cin * cin, fl1 = (double)l * (l + 1);
    RadialSolution s;
    std::vector<double> &p = s.p, &q = s.q, pp(n), qp(n);
    p.assign(n, 0.0);
    q.assign(n, 0.0);
    const double sq = std::sqrt(fl1 + 1 - cin2 * vr[0] * vr[0]) - 1.;
    double rm = 2. * r0 + cin2 * (r0 * e - vr[0]);
    p[0] = std::pow(r0, l + 1);
    q[0] = sq * p[0] / rm;
    pp[0] = rm * q[0] + p[0];
    qp[0] = (fl1 / rm + vr[0] - r0 * e) * p[0] - q[0];
    const double dr = std::exp(h), drh = std::sqrt(dr);
    double r = r0;
    for (int i = 0; i < 5; ++i) {
        const double rh2 = drh * r, rh = dr * r;
        const double k1 = h * pp[i], l1 = h * qp[i];
        double rve = 0.5 * (vr[i] + vr[i + 1]) - rh2 * e;
        rm = 2. * rh2 - cin2 * rve;
        double yn = p[i] + 0.5 * k1, zn = q[i] + 0.5 * l1;
        const double k2 = h * (rm * zn + yn), l2 = h * ((fl1 / rm + rve) * yn - zn);
        yn = p[i] + 0.5 * k2;
        zn = q[i] + 0.5 * l2;
        const double k3 = h * (rm * zn + yn), l3 = h * ((fl1 / rm + rve) * yn - zn);
        rve = vr[i + 1] - rh * e;
        rm = 2. * rh - cin2 * rve;
        yn = p[i] + k3;
        zn = q[i] + l3;
        const double k4 = h * (rm * zn + yn), l4 = h * ((fl1 / rm + rve) * yn - zn);
        p[i + 1] = p[i] + (k1 + 2. * k2 + 2. * k3 + k4) / 6.;
        q[i + 1] = q[i] + (l1 + 2. * l2 + 2. * l3 + l4) / 6.;
        pp[i + 1] = rm * q[i + 1] + p[i + 1];
        qp[i + 1] = (fl1 / rm + rve) * p[i + 1] - q[i + 1];
        r = rh;
    }
    for (int i = 5; i < n - 1; ++i) {
        r = r * dr;
        double p0 = p[i] + h * predict(pp, i), q0 = q[i] + h * predict(qp, i);
        const double rve = vr[i + 1] - r * e;
        rm = 2. * r - cin2 * rve;
        double p1p = rm * q0 + p0, q1p = (fl1 / rm + rve) * p0 - q0;
        double p1 = p0, q1 = q0;
        for (int it = 0; it < 5; ++it) {
            p1 = p[i] + h * correct(p1p, pp, i);
            q1 = q[i] + h * correct(q1p, qp, i);
            p1p = rm * q1 + p1;
            q1p = (fl1 / rm + rve) * p1 - q1;
            const double erp = std::fabs(p1 - p0) / (std::fabs(p1) + std::fabs(h * p1p));
            const double erq = std::fabs(q1 - q0) / (std::fabs(q1) + std::fabs(h * p1p));
            if (erp < kCorrEps && erq < kCorrEps) break;
            p0 = p1;
            q0 = q1;
        }
        p[i + 1] = p1;
        q[i + 1] = q1;
        pp[i + 1] = p1p;
        qp[i + 1] = q1p;
    }
    std::vector<double> rho(n);
    for (int i = 0; i < n; ++i) q[i] *= cin;
    for (int i = 0; i < n; ++i) rho[i] = p[i] * p[i] + q[i] * q[i];
    const double t = 1.0 / std::sqrt(integrate(rho, r0, h, n));
    s.us = t * p[n - 1] / r;
    s.dus = t * (pp[n - 1] - p[n - 1]) / (r * r);
    for (int i = 0; i < n; ++i) { p[i] *= t; q[i] *= t; }
    s.r_end = r;
    return s;
}

// radsrd.F: u-dot at energy e, orthogonal to u; returns (udot(R), udot'(R), ||udot||^2).
void solve_udot(int l, double e, const double *vr, int n, double r0, double h, const RadialSolution &u, double *ud,
                double *dud, double *ddn) {
    const double cin = 1.0 / kLight, cin2 = cin * cin, fl1 = (double)l * (l + 1);
    const std::vector<double> &p = u.p, &q = u.q;
    std::vector<double> pe(n, 0.0), qe(n, 0.0), pp(n), qp(n);
    // the relativistic correction of the inhomogeneous term
    auto corr = [&](double rm_) { return 1. + cin2 * fl1 / (rm_ * rm_); };
    double rm = 2. * r0 + cin2 * (r0 * e - vr[0]);
    pp[0] = r0 * cin * q[0];
    qp[0] = -r0 * p[0] * corr(rm);
    const double dr = std::exp(h), drh = std::sqrt(dr);
    double r = r0;
    for (int i = 0; i < 5; ++i) {
        const double rh2 = drh * r, rh = dr * r;
        const double k1 = h * pp[i], l1 = h * qp[i];
        double rve = 0.5 * (vr[i] + vr[i + 1]) - rh2 * e;
        rm = 2. * rh2 - cin2 * rve;
        double yn = pe[i] + 0.5 * k1, zn = qe[i] + 0.5 * l1;
        const double t1 = 0.5 * rh2 * cin * (q[i] + q[i + 1]);
        const double t2 = 0.5 * rh2 * (p[i] + p[i + 1]) * corr(rm);
        const double k2 = h * (rm * zn + yn + t1), l2 = h * ((fl1 / rm + rve) * yn - zn - t2);
        yn = pe[i] + 0.5 * k2;
        zn = qe[i] + 0.5 * l2;
        const double k3 = h * (rm * zn + yn + t1), l3 = h * ((fl1 / rm + rve) * yn - zn - t2);
        rve = vr[i + 1] - rh * e;
        rm = 2. * rh - cin2 * rve;
        yn = pe[i] + k3;
        zn = qe[i] + l3;
        const double k4 = h * (rm * zn + yn + rh * cin * q[i + 1]);
        const double l4 = h * ((fl1 / rm + rve) * yn - zn - rh * p[i + 1] * corr(rm));
        pe[i + 1] = pe[i] + (k1 + 2. * k2 + 2. * k3 + k4) / 6.;
        qe[i + 1] = qe[i] + (l1 + 2. * l2 + 2. * l3 + l4) / 6.;
        pp[i + 1] = rm * qe[i + 1] + pe[i + 1] + rh * cin * q[i + 1];
        qp[i + 1] = (fl1 / rm + rve) * pe[i + 1] - qe[i + 1] - rh * p[i + 1] * corr(rm);
        r = rh;
    }
    for (int i = 5; i < n - 1; ++i) {
        r = r * dr;
        double p0 = pe[i] + h * predict(pp, i), q0 = qe[i] + h * predict(qp, i);
        const double rve = vr[i + 1] - r * e;
        rm = 2. * r - cin2 * rve;
        const double t1 = cin * r * q[i + 1], t2 = r * p[i + 1] * corr(rm);
        double p1p = rm * q0 + p0 + t1, q1p = (fl1 / rm + rve) * p0 - q0 - t2;
        double p1 = p0, q1 = q0;
        for (int it = 0; it < 5; ++it) {
            p1 = pe[i] + h * correct(p1p, pp, i);
            q1 = qe[i] + h * correct(q1p, qp, i);
            p1p = rm * q1 + p1 + t1;
            q1p = (fl1 / rm + rve) * p1 - q1 - t2;
            const double erp = std::fabs(p1 - p0) / (std::fabs(p1) + std::fabs(h * p1p));
            const double erq = std::fabs(q1 - q0) / (std::fabs(q1) + std::fabs(h * p1p));
            if (erp < kCorrEps && erq < kCorrEps) break;
            p0 = p1;
            q0 = q1;
        }
        pe[i + 1] = p1;
        qe[i + 1] = q1;
        pp[i + 1] = p1p;
        qp[i + 1] = q1p;
    }
    std::vector<double> y(n);
    for (int i = 0; i < n; ++i) qe[i] *= cin;
    for (int i = 0; i < n; ++i) y[i] = p[i] * pe[i] + q[i] * qe[i];
    const double ov = integrate(y, r0, h, n);
    double d = (pp[n - 1] - pe[n - 1]) / (r * r);
    for (int i = 0; i < n; ++i) { pe[i] -= ov * p[i]; qe[i] -= ov * q[i]; }
    *ud = pe[n - 1] / r;
    *dud = d - ov * u.dus;
    for (int i = 0; i < n; ++i) y[i] = pe[i] * pe[i] + qe[i] * qe[i];
    *ddn = integrate(y, r0, h, n);
}

}  // namespace
}  // namespace hsdla

extern "C" int hsdla_radial_match(int32_t l, double e, const double *vr, int32_t n, double rmt, double dx,
                                  double *out) {
    using namespace hsdla;
    // the Runge-Kutta start needs 6 points and intgr0's first rule 7
    if (l < 0 || l > kMaxLmax || !vr || !out || n < 7 || !(rmt > 0.0) || !(dx > 0.0) || !std::isfinite(e))
        return HSDLA_ERR_ARG;
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(vr[i])) return HSDLA_ERR_INPUT;
    const double r0 = rmt * std::exp(dx * (1 - n));    // first mesh point (libflerp.f90:70)
    const RadialSolution u = solve_u(l, e, vr, n, r0, dx);
    double ud = 0, dud = 0, ddn = 0;
    solve_udot(l, e, vr, n, r0, dx, u, &ud, &dud, &ddn);
    out[0] = u.us;
    out[1] = u.dus;
    out[2] = ud;
    out[3] = dud;
    out[4] = ddn;
    for (int k = 0; k < 5; ++k)
        if (!std::isfinite(out[k])) return HSDLA_ERR_INPUT;
    return HSDLA_OK;
}
