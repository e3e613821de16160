// pbsm3d_oracle.cpp -- CPU oracle of CHM's PBSM3D step.
//
// TEST INFRASTRUCTURE ONLY: the checker for libpbsm3d_cuda and the timed
// CPU baseline.  Nothing in the product links or calls this file.
//
// Restates Chrismarsh/CHM src/modules/PBSM3D.cpp loop by loop (file:line
// cited at each block) with the default-branch physics, the extruded
// nearest-neighbour system of src/math/LinearAlgebra.cpp and its solver
// settings.  Third-party arithmetic restated from published algorithms:
//  - Trilinos 15.0.0 (spack.yaml:31): Belos block GMRES with block size 1
//    (restarted GMRES(m), right preconditioning, residual scaled by the
//    initial residual) and Ifpack2 ILUT (Saad's dual-threshold ILU(p,tau));
//  - MeteoIO (version unpinned, spack.yaml:29): Atmosphere::stdDryAirDensity
//    = standard-atmosphere pressure / (R_dry * T).
// Compiled with -ffp-contract=off so x86 and Arm give the same bits.

#include "pbsm3d_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- constants
// PhysConst.h:31, PhysConst.h:39, Snow.h:31, Atmosphere.h:31
const double kKappa = 0.4;
const double kRhoIce = 917;
const double kZ0Snow = 0.01;
const double kZUR = 50.0;

// ---------------------------------------------------------------- helpers
// module_base.hpp:471-479
inline bool is_nan(double v) {
    if (std::fabs(v - -9999.0) < 1e-5) return true;
    if (std::isnan(v)) return true;
    return false;
}
// std::max(a, b) is (a < b) ? b : a; keeping that form keeps its NaN behaviour.
inline double smax(double a, double b) { return (a < b) ? b : a; }

// Atmosphere.cpp:32-38
double log_scale_wind(double u, double Z_in, double Z_out, double snowdepthavg, double z0) {
    u = u * std::log((Z_out - (snowdepthavg + z0)) / z0) / std::log((Z_in - (snowdepthavg + z0)) / z0);
    return u;
}

// Atmosphere.cpp:62-80.  T is in K but compared with Tfreeze = 0, so the
// over-water branch is always taken for T > 0 K.
double saturated_vapour_pressure(double T) {
    const double TA = T - 273.15;
    const double Aw = 611.21, Bw = 17.502, Cw = 240.97;
    const double Ai = 611.15, Bi = 22.452, Ci = 272.55;
    const double Tfreeze = 0.;
    if (T >= Tfreeze) return Aw * std::exp((Bw * TA) / (Cw + TA));
    return Ai * std::exp((Bi * TA) / (Ci + TA));
}

// coordinates.cpp:112-131: bearing (deg, CW from north) -> polar (rad) -> (cos, sin)
void bearing_to_cartesian(double bearing, double& x, double& y) {
    double h = 450. - bearing;
    if (h > 360.) h = h - 360.;
    const double theta = h * M_PI / 180.;
    x = std::cos(theta);
    y = std::sin(theta);
}

// MeteoIO Atmosphere::stdAirPressure / stdDryAirDensity (called at
// PBSM3D.cpp:785).  Standard atmosphere: p0 = 101325 Pa, T0 = 288.15 K,
// lapse rate 0.0065 K/m, g = 9.80665, R_dry = 287.058, geopotential
// height with R0 = 6356766 m.  rho = p(z) / (R_dry * T).
double std_air_pressure(double altitude) {
    const double p0 = 101325.;
    const double lapse_rate = 0.0065;
    const double sea_level_temp = 288.15;
    const double R_dry = 287.058;
    const double g = 9.80665;
    const double R0 = 6356766.0;
    const double expo = g / (lapse_rate * R_dry);
    return p0 * std::pow(1. - ((lapse_rate * R0 * altitude) / (sea_level_temp * (R0 + altitude))), expo);
}
double std_dry_air_density(double altitude, double temperature) {
    return std_air_pressure(altitude) / (287.058 * temperature);
}

inline int sgn(double v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }

// The root finder of the reference's two bracket_and_solve_root calls
// (PBSM3D.cpp:557, 708): Boost 1.85.0's (spack.yaml) bracket_and_solve_root(
// f, guess, factor 1, rising, |a - b| < 1e-8, 500 evaluations), which walks
// from the guess until f changes sign and then runs TOMS 748 on the bracket,
// returning the bracket whose midpoint the reference takes; when no bracket
// is found it throws and the caller keeps its default.
//
// Restated: the same walk -- away from zero (b *= factor) when f(guess) has
// the sign that puts the root there ((f < 0) == (guess < 0 ? !rising :
// rising)), else towards it (a /= factor), by a factor that is 1 at first and
// doubles at the 32nd move, then after 16, 8, 4, 2 more moves and at every
// move after that; a walk towards zero that passes below DBL_MIN returns the
// bracket (a, 0) -- and the root of the bracket refined to full precision by
// Newton-Raphson with a bisection fallback (rtsafe, Press et al., Numerical
// Recipes, section 9.4) in place of TOMS 748: the reference's midpoint lies
// within 5e-9 of that root.  Returns false when the walk fails.
//
// Each call gets the full budget of 500 evaluations.  In the reference the
// budget is an in/out argument shared by all faces of one OpenMP thread
// (PBSM3D.cpp:422): Boost documents that it returns the evaluations used, so
// later faces inherit a shrinking budget and the results depend on the thread
// count.  That is not restated.
template <class F, class DF>
bool bracket_solve(F f, DF df, double guess, bool rising, double& root) {
    const int budget = 500;
    double a = guess, b = guess;
    double fa = f(a), fb = fa;
    const bool away = (fa < 0) == (guess < 0 ? !rising : rising);
    double factor = 1.0;
    int every = 32;
    for (int s = 1; sgn(fa) == sgn(fb); ++s) {
        if (!away && std::fabs(a) < 2.2250738585072014e-308) {
            root = a / 2.0;
            return true;
        }
        if (s >= budget) return false;
        if (s % every == 0) {
            factor *= 2;
            if (every > 1) every /= 2;
        }
        if (away) {
            a = b;
            fa = fb;
            b *= factor;
            fb = f(b);
        } else {
            b = a;
            fb = fa;
            a /= factor;
            fa = f(a);
        }
    }
    if (fa == 0) { root = a; return true; }
    if (fb == 0) { root = b; return true; }
    double lo = std::min(a, b), hi = std::max(a, b);
    double flo = lo == a ? fa : fb;
    double x = 0.5 * (lo + hi);
    for (int it = 0; it < 100; ++it) {
        const double fx = f(x);
        if (fx == 0) break;
        if (sgn(fx) == sgn(flo)) {
            lo = x;
            flo = fx;
        } else {
            hi = x;
        }
        double xn = x - fx / df(x);
        if (!(xn > lo && xn < hi)) xn = 0.5 * (lo + hi);
        const bool done = std::fabs(xn - x) <= 1e-15 * std::fabs(xn);
        x = xn;
        if (done) break;
    }
    root = x;
    return true;
}

// z0_ustar_coupling (PBSM3D.cpp:691-712): the friction velocity over snow
// with partly buried vegetation is the root of Li and Pomeroy (2000) eqn 5,
//     g(u) = u2 kappa / log(2 / (c u^2 + lambda/2)) - u,  c = 0.6131702345e-2,
// which falls with u, found from guess 1.  false: no bracket (u* keeps its
// 1.3 placeholder).
bool coupled_ustar(double u2, double lambda, double& ustar) {
    const double c = 0.6131702345e-2;
    auto g = [&](double u) { return u2 * kKappa / std::log(2.0 / (c * u * u + .5 * lambda)) - u; };
    auto dg = [&](double u) {
        const double q = c * u * u + .5 * lambda;
        const double ell = std::log(2.0 / q);
        return u2 * kKappa * (2.0 * c * u) / (q * ell * ell) - 1.0;
    };
    return bracket_solve(g, dg, 1.0, false, ustar);
}

// ----------------------------------------------------------- wind inputs
// Atmosphere.cpp:41-46
double exp_scale_wind(double u, double Z_in, double Z_out, double alpha) { return u * std::exp(alpha * (Z_out / Z_in - 1)); }

// Exponential integral E1(x), x > 0 (gsl_sf_expint_E1 in the reference; GSL
// version unpinned): the power series for x <= 1, the continued fraction
// (modified Lentz) above (Press et al., Numerical Recipes, section 6.3).
double expint_e1(double x) {
    const double euler = 0.57721566490153286061;
    if (x <= 1.0) {
        double sum = 0, term = 1;
        for (int k = 1; k < 200; ++k) {
            term *= -x / k;
            const double d = -term / k;
            sum += d;
            if (std::fabs(d) < std::fabs(sum) * 1e-17) break;
        }
        return -euler - std::log(x) + sum;
    }
    const double tiny = 1e-300;
    double b = x + 1.0, cc = 1.0 / tiny, d = 1.0 / b, h = d;
    for (int i = 1; i < 10000; ++i) {
        const double an = -(double)i * i;
        b += 2.0;
        d = 1.0 / (an * d + b);
        cc = b + an / cc;
        const double del = cc * d;
        h *= del;
        if (std::fabs(del - 1.0) < 1e-17) break;
    }
    return h * std::exp(-x);
}

// thin_plate_spline::operator() (interpolation/TPSpline.cpp:55-157) for n <= 16
// samples: the (n+1)x(n+1) system [1, R(x_i, x_j)] / [0, 1 ... 1] with the
// basis R(d) = -(log(q) + c + E1(q)), q = (d weight / 2)^2, weight 0.01 and
// the reference's c = 0.577215; solved by Gaussian elimination with full
// pivoting (Eigen::FullPivLU in the reference) for nz right-hand sides (the
// same samples carry several fields), evaluated at the query.
void tps_interp_multi(const double* sx, const double* sy, const double* const* sz, int nz, int n, double qx,
                      double qy, double* out) {
    const double weight = 0.01, c = 0.577215;
    auto basis = [&](double dx, double dy) {
        double d = std::sqrt(dx * dx + dy * dy);
        d = (d * weight / 2.0) * (d * weight / 2.0);
        return -(std::log(d) + c + expint_e1(d));
    };
    const int m = n + 1;
    double A[17][17] = {}, b[2][17] = {}, y[17] = {}, x[17] = {};
    for (int i = 0; i < n; ++i)
        for (int j = i; j < n; ++j) {
            const double xd = sx[i] - sx[j], yd = sy[i] - sy[j];
            if (xd == 0. && yd == 0.) continue;
            const double Rd = j == i ? 0.0 : basis(xd, yd);
            A[i][j + 1] = Rd;
            A[j][i + 1] = Rd;
        }
    for (int i = 0; i < m; ++i) {
        A[i][0] = 1;
        A[m - 1][i] = 1;
    }
    A[m - 1][0] = 0;
    for (int f = 0; f < nz; ++f) {
        for (int i = 0; i < n; ++i) b[f][i] = sz[f][i];
        b[f][m - 1] = 0.0;
    }
    int colp[17];
    for (int k = 0; k < m; ++k) colp[k] = k;
    for (int k = 0; k < m; ++k) {
        int pr = k, pc = k;
        double best = -1;
        for (int i = k; i < m; ++i)
            for (int j = k; j < m; ++j)
                if (std::fabs(A[i][j]) > best) {
                    best = std::fabs(A[i][j]);
                    pr = i;
                    pc = j;
                }
        if (best == 0) break;
        for (int j = 0; j < m; ++j) std::swap(A[k][j], A[pr][j]);
        for (int f = 0; f < nz; ++f) std::swap(b[f][k], b[f][pr]);
        for (int i = 0; i < m; ++i) std::swap(A[i][k], A[i][pc]);
        std::swap(colp[k], colp[pc]);
        for (int i = k + 1; i < m; ++i) {
            const double g = A[i][k] / A[k][k];
            for (int j = k; j < m; ++j) A[i][j] -= g * A[k][j];
            for (int f = 0; f < nz; ++f) b[f][i] -= g * b[f][k];
        }
    }
    for (int f = 0; f < nz; ++f) {
        for (int k = m - 1; k >= 0; --k) {
            double v = b[f][k];
            for (int j = k + 1; j < m; ++j) v -= A[k][j] * y[j];
            y[k] = A[k][k] != 0 ? v / A[k][k] : 0.0;
        }
        for (int k = 0; k < m; ++k) x[colp[k]] = y[k];
        double z0 = x[0];
        for (int i = 1; i < m; ++i) z0 += x[i] * basis(sx[i - 1] - qx, sy[i - 1] - qy);
        out[f] = z0;
    }
}
double tps_interp(const double* sx, const double* sy, const double* sz, int n, double qx, double qy) {
    double out;
    const double* z[1] = {sz};
    tps_interp_multi(sx, sy, z, 1, n, qx, qy, &out);
    return out;
}

// inv_dist::operator() (interpolation/inv_dist.cpp:36-78): weights 1/d^2; a
// sample at the query resets the sums to it and the later samples still add.
double idw_interp(const double* sx, const double* sy, const double* sz, int n, double qx, double qy) {
    double numerator = 0.0, denominator = 0.0;
    for (int i = 0; i < n; ++i) {
        const double xdiff = sx[i] - qx, ydiff = sy[i] - qy;
        const double di = std::pow(std::sqrt(std::pow(xdiff, 2.0) + std::pow(ydiff, 2.0)), 2.0);
        if (di == 0) {
            numerator = sz[i];
            denominator = 1.0;
        } else {
            numerator += sz[i] / di;
            denominator += 1 / di;
        }
    }
    return numerator / denominator;
}

// ---------------------------------------------------- subgrid topography
inline double smin(double a, double b) { return (b < a) ? b : a; }  // std::min

// gsl_ran_gaussian_pdf(x, sigma) and gsl_cdf_gaussian_Q(x, sigma): the
// normal density and upper tail.
double gauss_pdf(double x, double sigma) {
    const double u = x / sigma;
    return std::exp(-u * u / 2.0) / (std::sqrt(2.0 * M_PI) * sigma);
}
double gauss_Q(double x, double sigma) { return 0.5 * std::erfc(x / (sigma * std::sqrt(2.0))); }

// Regularised incomplete gamma functions P(a, x) and Q(a, x): the series for
// x < a + 1 and the continued fraction (modified Lentz) otherwise (Press et
// al., Numerical Recipes, section 6.2).
void incomplete_gamma(double a, double x, double& P, double& Q) {
    if (!(x > 0)) {
        P = 0;
        Q = 1;
        return;
    }
    const double lpre = -x + a * std::log(x) - std::lgamma(a);
    if (x < a + 1) {
        double ap = a, del = 1.0 / a, sum = del;
        for (int n = 0; n < 100000; ++n) {
            ap += 1;
            del *= x / ap;
            sum += del;
            if (std::fabs(del) < std::fabs(sum) * 1e-17) break;
        }
        P = sum * std::exp(lpre);
        Q = 1.0 - P;
    } else {
        const double tiny = 1e-300;
        double b = x + 1 - a, cc = 1 / tiny, d = 1 / b, h = d;
        for (int i = 1; i < 100000; ++i) {
            const double an = -i * (i - a);
            b += 2;
            d = an * d + b;
            if (std::fabs(d) < tiny) d = tiny;
            cc = b + an / cc;
            if (std::fabs(cc) < tiny) cc = tiny;
            d = 1 / d;
            const double del = d * cc;
            h *= del;
            if (std::fabs(del - 1) < 1e-17) break;
        }
        Q = std::exp(lpre) * h;
        P = 1.0 - Q;
    }
}
// gsl_cdf_gamma_P / _Q (x, shape a, scale b) and gsl_ran_gamma_pdf
double gamma_P(double x, double a, double b) {
    double P, Q;
    incomplete_gamma(a, x / b, P, Q);
    return P;
}
double gamma_Q(double x, double a, double b) {
    double P, Q;
    incomplete_gamma(a, x / b, P, Q);
    return Q;
}
double gamma_pdf(double x, double a, double b) {
    if (x < 0) return 0;
    if (x == 0) return a == 1 ? 1 / b : (a > 1 ? 0 : INFINITY);
    return std::exp((a - 1) * std::log(x / b) - x / b - std::lgamma(a)) / b;
}

// Gauss-Legendre nodes and weights on [-1, 1] (Newton on P_n, Press et al.,
// Numerical Recipes, section 4.5).
struct GaussLegendre {
    double x[20], w[20];
    GaussLegendre() {
        const int n = 20;
        for (int i = 0; i < n; ++i) {
            long double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0;
            for (int it = 0; it < 100; ++it) {
                long double p1 = 1, p2 = 0;
                for (int j = 0; j < n; ++j) {
                    const long double p3 = p2;
                    p2 = p1;
                    p1 = ((2 * j + 1) * z * p2 - j * p3) / (j + 1);
                }
                pp = n * (z * p1 - p2) / (z * z - 1);
                const long double z1 = z;
                z = z1 - p1 / pp;
                if (std::fabs((double)(z - z1)) < 1e-19) break;
            }
            x[i] = (double)z;
            w[i] = (double)(2 / ((1 - z * z) * pp * pp));
        }
    }
};
const GaussLegendre kGL20;

template <class F>
double gl20(F f, double a, double b) {
    const double c = 0.5 * (a + b), h = 0.5 * (b - a);
    double s = 0;
    for (int i = 0; i < 20; ++i) s += kGL20.w[i] * f(c + h * kGL20.x[i]);
    return s * h;
}
template <class F>
double adapt(F f, double a, double b, double whole, double floor, int depth) {
    const double m = 0.5 * (a + b);
    const double l = gl20(f, a, m), r = gl20(f, m, b);
    if (depth >= 40 || std::fabs(l + r - whole) <= std::max(1e-14 * (std::fabs(l) + std::fabs(r)), floor))
        return l + r;
    return adapt(f, a, m, l, floor, depth + 1) + adapt(f, m, b, r, floor, depth + 1);
}
// The reference integrates with gsl_integration_qags (GSL, version unpinned in
// spack.yaml; QUADPACK's QAGS) to relative 1e-7.  Here: 20-point
// Gauss-Legendre on 64 panels, each bisected until its two halves agree with
// it to relative 1e-14 (or absolute 1e-17 times the integrand's scale); the
// panels keep a narrow Gaussian from falling between the nodes.  The QAGS
// result lies within its tolerance of this.
template <class F>
double integrate(F f, double a, double b, double scale) {
    const int panels = 64;
    double s = 0;
    for (int k = 0; k < panels; ++k) {
        const double x0 = a + (b - a) * k / panels, x1 = a + (b - a) * (k + 1) / panels;
        s += adapt(f, x0, x1, gl20(f, x0, x1), 1e-17 * scale, 0);
    }
    return s;
}

struct SubgridFace {
    double min_sd_trans_avg, frac_contrib, frac_contrib_nosnw, tpi_lim, test_int;
    bool have_test_int;
};

// PBSM3D.cpp:486-645: subgrid topographic holding capacity and contributing
// fraction of one face.
SubgridFace subgrid_face(const pbsm3d_config& cfg, double snow_depth, const double tpi[5]) {
    SubgridFace o{cfg.min_sd_trans, 1.0, 1.0, 0.0, 0.0, false};
    const double min_sd_trans = cfg.min_sd_trans;
    if (cfg.use_subgrid_topo_V2) {  // :486-597
        const double fac_fill = 0.8;
        double tpi_lim = -min_sd_trans;
        if (!is_nan(tpi[1])) {
            const double moy_tpi = smax(-5.0, smin(5.0, tpi[0]));
            const double std_tpi = smin(5.0, smax(0.1, tpi[1]));
            if (snow_depth > min_sd_trans) {
                // the depth-dependent coefficients of :509-537 are declared in
                // inner scopes and never reach the integrals
                const double a1 = 1.5, b1 = 0.3, a2 = 0.6, b2 = 0.55;
                auto fill = [&](double x) {
                    const double x2 = x + 0.25;
                    if (x2 <= 0) return (1. - a1 * std::tanh(b1 * x2)) * gauss_pdf(x - moy_tpi, std_tpi);
                    return (1. - a2 * std::tanh(b2 * x2)) * gauss_pdf(x - moy_tpi, std_tpi);
                };
                const double result = integrate(fill, -50, 50, 1.0);
                o.test_int = result;
                o.have_test_int = true;
                auto froot = [&](double xx) {
                    return (1 - a1 * std::tanh(b1 * (xx + 0.25))) * snow_depth / result + fac_fill * xx;
                };
                auto dfroot = [&](double xx) {
                    const double th = std::tanh(b1 * (xx + 0.25));
                    return -a1 * b1 * (1 - th * th) * snow_depth / result + fac_fill;
                };
                double r;
                if (bracket_solve(froot, dfroot, -1.0, true, r)) tpi_lim = r;
                auto fill2 = [&](double x) {
                    const double x2 = x + 0.25;
                    if (x2 <= 0) return (1. - a1 * std::tanh(b1 * x2)) * snow_depth / result * gauss_pdf(x - moy_tpi, std_tpi);
                    return (1. - a2 * std::tanh(b2 * x2)) * snow_depth / result * gauss_pdf(x - moy_tpi, std_tpi);
                };
                const double h1 = integrate(fill2, -50, tpi_lim, snow_depth);
                auto fill3 = [&](double x) { return -fac_fill * x * gauss_pdf(x - moy_tpi, std_tpi); };
                const double h2 = integrate(fill3, tpi_lim, -min_sd_trans / fac_fill, 5.0);
                const double h3 = min_sd_trans * gauss_Q(-min_sd_trans / fac_fill - moy_tpi, std_tpi);
                o.min_sd_trans_avg = smin(h1 + h2 + h3, snow_depth);
            }
            o.frac_contrib = gauss_Q(tpi_lim - moy_tpi, std_tpi);
        }
        o.tpi_lim = tpi_lim;
    }
    if (cfg.use_subgrid_topo) {  // :604-645
        if (!is_nan(tpi[2])) {
            const double frac_neg = tpi[2];
            if (frac_neg > 0.) {
                const double moy_tpi_neg = smax(-10.0, smin(-0.05, tpi[3]));
                const double std_tpi_neg = smin(5.0, smax(0.1, tpi[4]));
                const double shape_gam = std::pow(moy_tpi_neg, 2.0) / std::pow(std_tpi_neg, 2.0);
                const double scale_gam = -std::pow(std_tpi_neg, 2.0) / moy_tpi_neg;
                o.frac_contrib = (1. - frac_neg) + frac_neg * gamma_P(snow_depth, shape_gam, scale_gam);
                o.frac_contrib_nosnw = (1. - frac_neg);
                if (snow_depth > min_sd_trans) {
                    const double hint =
                        shape_gam * scale_gam -
                        scale_gam * (snow_depth * gamma_pdf(snow_depth, shape_gam, scale_gam) -
                                     min_sd_trans * gamma_pdf(min_sd_trans, shape_gam, scale_gam) +
                                     shape_gam * gamma_P(min_sd_trans, shape_gam, scale_gam) +
                                     shape_gam * gamma_Q(snow_depth, shape_gam, scale_gam));
                    o.min_sd_trans_avg =
                        (1. - frac_neg) * min_sd_trans +
                        frac_neg * (min_sd_trans * gamma_P(min_sd_trans, shape_gam, scale_gam) + hint +
                                    snow_depth * gamma_Q(snow_depth, shape_gam, scale_gam));
                }
            }
        }
    }
    return o;
}

// iterative_subl (PBSM3D.cpp:1062-1096): the ice-bulb temperature Ti (C) of
// Pomeroy and Li (2000) / Harder (2013) A.5, the root of
//     f(Ti) = T + D L (rho/1000 - .611 mw exp(17.3 Ti/(237.3+Ti)) / (R (Ti+273.15) 1000)) / lambda_t - Ti
// by Boost's newton_raphson_iterate(f, guess T, min -50, max 0, 6 digits).
// Restated as the Newton iteration that the call documents: start at T, stop
// after the first step no larger than |Ti| 2^(1-6), return the iterate after
// that step.  A step that would land on or beyond a bound is replaced by half
// the way to that bound, and after each step the bound on the side the step
// left from moves to the point it left.  f is concave with f' < -1, so every
// iterate after the first lies at or above the root and they descend onto
// it; a bound is met only when the root lies close to 0 C.
double ice_bulb_temperature(double T, double t, double ea, double D, double lambda_t, double L) {
    const double mw = 0.01801528 * 1000.0;
    const double R = 8.31441 / 1000.0;
    const double rho = (mw * ea) / (R * t);
    const double tol = std::ldexp(1.0, 1 - 6);
    double lo = -50, hi = 0;
    double x = T;
    for (int it = 0; it < 100; ++it) {
        const double e = std::exp(17.3 * x / (237.3 + x));
        const double f = T + D * L * (rho / 1000.0 - .611 * mw * e / (R * (x + 273.15) * 1000.0)) / lambda_t - x;
        if (f == 0) break;
        const double df =
            D * L *
                (-0.6110000000e-3 * mw * (17.3 / (237.3 + x) - 17.3 * x / ((237.3 + x) * (237.3 + x))) * e /
                     (R * (x + 273.15)) +
                 0.6110000000e-3 * mw * e / (R * (x + 273.15) * (x + 273.15))) /
                lambda_t -
            1;
        const double from = x;
        double step = f / df;
        x = from - step;
        if (x <= lo) {
            step = 0.5 * (from - lo);
            x = from - step;
        } else if (x >= hi) {
            step = 0.5 * (from - hi);
            x = from - step;
        }
        if (step > 0)
            hi = from;
        else
            lo = from;
        if (!(std::fabs(x * tol) < std::fabs(step))) break;
    }
    return x;
}

// armadillo's direct dot of two 3-vectors: two accumulators (0,2) and (1).
inline double dot3(const double* a, const double* b) {
    double v1 = 0, v2 = 0;
    v1 += a[0] * b[0];
    v2 += a[1] * b[1];
    v1 += a[2] * b[2];
    return v1 + v2;
}

// ---------------------------------------------------------------- CSR system
struct System {
    int64_t rows = 0;
    std::vector<int64_t> rowptr;
    std::vector<int32_t> cols;
    std::vector<double> vals, rhs, x;

    void zero() {  // LinearAlgebra.cpp:199-206
        std::fill(vals.begin(), vals.end(), 0.0);
        std::fill(rhs.begin(), rhs.end(), 0.0);
        std::fill(x.begin(), x.end(), 0.0);
    }
    // sumIntoGlobalValues: a column missing from the row's graph is ignored.
    inline void sum_into(int64_t r, int64_t c, double v) {
        for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
            if (cols[k] == c) {
                vals[k] += v;
                return;
            }
    }
    inline void replace(int64_t r, int64_t c, double v) {
        for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
            if (cols[k] == c) {
                vals[k] = v;
                return;
            }
    }
    double rhs_max() const {  // normInf, LinearAlgebra.cpp:264-270
        double m = 0;
        for (double v : rhs) m = std::max(m, std::fabs(v));
        return m;
    }
};

// ---------------------------------------------------------------- ILUT
// Saad's ILUT(p, tau) (Iterative Methods for Sparse Linear Systems, alg. 10.6),
// the algorithm of Ifpack2::ILUT: drop |w_k| < tau*||a_i||_2, keep at most p
// off-diagonals in each of L and U per row, with
// p = ceil(level_of_fill * nnz(A_local) / (2 * rows_local)).
// The factor covers one block of rows; couplings to other blocks are dropped
// (Ifpack2 factors the rank-local matrix only).
struct ILUT {
    int64_t r0 = 0, n = 0;  // global rows [r0, r0+n) handled via the row list
    std::vector<int64_t> rows;  // global row ids in this block, ascending local order
    std::vector<int64_t> lp, up;  // row pointers
    std::vector<int32_t> lc, uc;  // local column ids
    std::vector<double> lv, uv, udiag_inv;
};

void ilut_factor(const System& A, const std::vector<int64_t>& rows, double tau, double lof, ILUT& F) {
    const int64_t n = (int64_t)rows.size();
    F.rows = rows;
    F.n = n;
    std::unordered_map<int64_t, int32_t> g2l;
    g2l.reserve(n * 2);
    for (int64_t i = 0; i < n; ++i) g2l[rows[i]] = (int32_t)i;
    int64_t nnz_local = 0;
    for (int64_t i = 0; i < n; ++i) nnz_local += A.rowptr[rows[i] + 1] - A.rowptr[rows[i]];
    int64_t p = (int64_t)std::ceil(lof * (double)nnz_local / (2.0 * (double)std::max<int64_t>(n, 1)));
    if (p < 1) p = 1;
    F.lp.assign(1, 0);
    F.up.assign(1, 0);
    F.lc.clear(); F.uc.clear(); F.lv.clear(); F.uv.clear();
    F.udiag_inv.assign(n, 0.0);
    std::vector<double> w(n, 0.0);
    std::vector<char> used(n, 0);
    std::vector<int32_t> pat;
    for (int64_t i = 0; i < n; ++i) {
        const int64_t gr = rows[i];
        pat.clear();
        double nrm = 0;
        for (int64_t k = A.rowptr[gr]; k < A.rowptr[gr + 1]; ++k) {
            auto it = g2l.find(A.cols[k]);
            nrm += A.vals[k] * A.vals[k];
            if (it == g2l.end()) continue;
            int32_t j = it->second;
            if (!used[j]) { used[j] = 1; pat.push_back(j); w[j] = 0; }
            w[j] += A.vals[k];
        }
        if (!used[i]) { used[i] = 1; pat.push_back((int32_t)i); w[i] = 0; }
        const double tol_i = tau * std::sqrt(nrm);
        // eliminate lower entries in increasing column order
        int32_t last = -1;
        while (true) {
            int32_t k = -1;
            for (int32_t j : pat)
                if (j < i && j > last && (k < 0 || j < k)) k = j;
            if (k < 0) break;
            last = k;
            double wk = w[k] * F.udiag_inv[k];
            if (std::fabs(wk) < tol_i) { w[k] = 0; continue; }
            w[k] = wk;
            for (int64_t q = F.up[k]; q < F.up[k + 1]; ++q) {
                int32_t j = F.uc[q];
                if (!used[j]) { used[j] = 1; pat.push_back(j); w[j] = 0; }
                w[j] -= wk * F.uv[q];
            }
        }
        // split, drop, keep p largest
        std::vector<std::pair<double, int32_t>> L, U;
        double diag = w[i];
        for (int32_t j : pat) {
            if (j == i) continue;
            double v = w[j];
            if (v == 0 || std::fabs(v) < tol_i) continue;
            if (j < i) L.push_back({v, j}); else U.push_back({v, j});
        }
        auto keep = [p](std::vector<std::pair<double, int32_t>>& v) {
            if ((int64_t)v.size() > p) {
                std::nth_element(v.begin(), v.begin() + p, v.end(),
                                 [](auto& a, auto& b) { return std::fabs(a.first) > std::fabs(b.first); });
                v.resize(p);
            }
            std::sort(v.begin(), v.end(), [](auto& a, auto& b) { return a.second < b.second; });
        };
        keep(L);
        keep(U);
        for (auto& e : L) { F.lc.push_back(e.second); F.lv.push_back(e.first); }
        for (auto& e : U) { F.uc.push_back(e.second); F.uv.push_back(e.first); }
        F.lp.push_back((int64_t)F.lc.size());
        F.up.push_back((int64_t)F.uc.size());
        if (diag == 0) diag = (tol_i > 0 ? tol_i : 1e-300);
        F.udiag_inv[i] = 1.0 / diag;
        for (int32_t j : pat) { used[j] = 0; w[j] = 0; }
    }
}

// z = (LU)^{-1} r on the block's rows (global indexing of r and z)
void ilut_apply(const ILUT& F, const double* r, double* z, std::vector<double>& tmp) {
    const int64_t n = F.n;
    tmp.resize(n);
    for (int64_t i = 0; i < n; ++i) {
        double s = r[F.rows[i]];
        for (int64_t q = F.lp[i]; q < F.lp[i + 1]; ++q) s -= F.lv[q] * tmp[F.lc[q]];
        tmp[i] = s;
    }
    for (int64_t i = n - 1; i >= 0; --i) {
        double s = tmp[i];
        for (int64_t q = F.up[i]; q < F.up[i + 1]; ++q) s -= F.uv[q] * tmp[F.uc[q]];
        tmp[i] = s * F.udiag_inv[i];
    }
    for (int64_t i = 0; i < n; ++i) z[F.rows[i]] = tmp[i];
}

struct Precond {
    std::vector<ILUT> blocks;
    void build(const System& A, int64_t n_faces, int nLayer, int nblocks, double tau, double lof) {
        if (nblocks < 1) nblocks = 1;
        if (nblocks > n_faces) nblocks = (int)std::max<int64_t>(1, n_faces);
        blocks.assign(nblocks, ILUT());
#pragma omp parallel for schedule(dynamic, 1)
        for (int b = 0; b < nblocks; ++b) {
            int64_t f0 = n_faces * b / nblocks, f1 = n_faces * (b + 1) / nblocks;
            std::vector<int64_t> rows;
            rows.reserve((f1 - f0) * nLayer);
            // a rank's local rows: its faces, layer by layer (LinearAlgebra.cpp:39-55)
            for (int z = 0; z < nLayer; ++z)
                for (int64_t f = f0; f < f1; ++f) rows.push_back((int64_t)z * n_faces + f);
            ilut_factor(A, rows, tau, lof, blocks[b]);
        }
    }
    void apply(const double* r, double* z) const {
#pragma omp parallel for schedule(dynamic, 1)
        for (int b = 0; b < (int)blocks.size(); ++b) {
            std::vector<double> tmp;
            ilut_apply(blocks[b], r, z, tmp);
        }
    }
};

void spmv(const System& A, const double* x, double* y) {
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < A.rows; ++r) {
        double s = 0;
        for (int64_t k = A.rowptr[r]; k < A.rowptr[r + 1]; ++k) s += A.vals[k] * x[A.cols[k]];
        y[r] = s;
    }
}
double dotv(const double* a, const double* b, int64_t n) {
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

// Restarted GMRES(m), right preconditioned, modified Gram-Schmidt, Givens
// rotations; convergence when the residual norm <= tol * ||r0|| (Belos'
// default scaling; r0 = b for x0 = 0), confirmed on the explicit residual.
// Returns 0 converged, 1 not converged.
int gmres(const System& A, const Precond& M, const double* b, double* x, int m, int maxit, double tol, int& iters,
          double& relres) {
    const int64_t n = A.rows;
    std::vector<double> r(n), z(n), w(n);
    std::vector<std::vector<double>> V(m + 1, std::vector<double>(n));
    std::vector<double> H((m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    spmv(A, x, w.data());
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - w[i];
    const double r0 = std::sqrt(dotv(r.data(), r.data(), n));
    iters = 0;
    if (r0 == 0) { relres = 0; return 0; }
    double beta = r0;
    const double target = tol * r0;
    while (true) {
#pragma omp parallel for
        for (int64_t i = 0; i < n; ++i) V[0][i] = r[i] / beta;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int j = 0;
        double res = beta;
        for (; j < m && iters < maxit; ++j) {
            M.apply(V[j].data(), z.data());
            spmv(A, z.data(), w.data());
            for (int i = 0; i <= j; ++i) {
                double h = dotv(w.data(), V[i].data(), n);
                H[i * m + j] = h;
                double* vi = V[i].data();
#pragma omp parallel for
                for (int64_t k = 0; k < n; ++k) w[k] -= h * vi[k];
            }
            double hn = std::sqrt(dotv(w.data(), w.data(), n));
            H[(j + 1) * m + j] = hn;
            if (hn != 0) {
                double* vj = V[j + 1].data();
#pragma omp parallel for
                for (int64_t k = 0; k < n; ++k) vj[k] = w[k] / hn;
            }
            for (int i = 0; i < j; ++i) {
                double a = H[i * m + j], c = H[(i + 1) * m + j];
                H[i * m + j] = cs[i] * a + sn[i] * c;
                H[(i + 1) * m + j] = -sn[i] * a + cs[i] * c;
            }
            double a = H[j * m + j], c = H[(j + 1) * m + j];
            double d = std::hypot(a, c);
            cs[j] = d == 0 ? 1 : a / d;
            sn[j] = d == 0 ? 0 : c / d;
            H[j * m + j] = d;
            H[(j + 1) * m + j] = 0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            res = std::fabs(g[j + 1]);
            ++iters;
            if (res <= target || hn == 0) { ++j; break; }
        }
        // y = H^{-1} g, x += M^{-1} V y
        for (int i = j - 1; i >= 0; --i) {
            double s = g[i];
            for (int k = i + 1; k < j; ++k) s -= H[i * m + k] * y[k];
            y[i] = s / H[i * m + i];
        }
        std::fill(w.begin(), w.end(), 0.0);
        for (int i = 0; i < j; ++i) {
            double yi = y[i];
            double* vi = V[i].data();
#pragma omp parallel for
            for (int64_t k = 0; k < n; ++k) w[k] += yi * vi[k];
        }
        M.apply(w.data(), z.data());
#pragma omp parallel for
        for (int64_t k = 0; k < n; ++k) x[k] += z[k];
        spmv(A, x, w.data());
#pragma omp parallel for
        for (int64_t k = 0; k < n; ++k) r[k] = b[k] - w[k];
        beta = std::sqrt(dotv(r.data(), r.data(), n));
        relres = beta / r0;
        if (beta <= target) return 0;
        if (iters >= maxit) return 1;
    }
}

}  // namespace

// ================================================================ context
struct oracle_ctx {
    pbsm3d_config cfg;
    oracle_solver_cfg scfg;
    int64_t T = 0;
    int L = 0;
    double dz = 0, susp_depth = 5, l_max = 40;
    bool enable_veg = true;
    // mesh
    std::vector<int32_t> nbr;
    std::vector<double> E, m, area, center;
    std::vector<double> canopy, lai, stalkN, stalkD;
    std::vector<uint8_t> water;
    // PBSM3D::data (PBSM3D.hpp:367-408)
    std::vector<double> A5;  // [5*T]
    std::vector<uint8_t> face_neigh;
    std::vector<uint8_t> saltation;
    std::vector<double> hs, z0, ustar, c_salt, ustar_th, u_z, csubl;
    // forcing of the current step
    std::vector<double> f_UR, f_U2, f_dir, f_swe, f_t, f_rh, f_sd, f_fetch, f_psh;
    double dt = 0;
    // face variables
    std::vector<double> Qsalt, Qsusp, Qsubl, Qsubl_mass, sum_subl, drift_mass, sum_drift, more_than_avail, bsp;
    // raw vegetation (the wind modules read it whatever PBSM3D's enable_veg says)
    std::vector<uint8_t> has_veg;
    std::vector<double> canopy_raw, lai_raw;
    // subgrid TPI parameters [5][T] (NaN = undefined) and the subgrid outputs
    std::vector<double> tpi, frac_contrib, frac_contrib_nosnw, hold_topo, tpi_lim, test_int;
    System susp, dep;
    bool suspension_present = false, deposition_present = false;
    double susp_rhs_max = 0, dep_rhs_max = 0;
    int susp_iters = 0, dep_iters = 0;
    double susp_relres = 0, dep_relres = 0;
    double ms_susp_solve = 0, ms_dep_solve = 0, ms_assembly = 0;
    std::string err;
};

static thread_local std::string g_create_error;

extern "C" {

double oracle_log_scale_wind(double u, double z_in, double z_out, double sd, double z0) {
    return log_scale_wind(u, z_in, z_out, sd, z0);
}
double oracle_saturated_vapour_pressure(double T) { return saturated_vapour_pressure(T); }
void oracle_bearing_to_cartesian(double b, double* xy) { bearing_to_cartesian(b, xy[0], xy[1]); }
double oracle_std_dry_air_density(double z, double T) { return std_dry_air_density(z, T); }
int oracle_coupled_ustar(double u2, double lambda, double* ustar) { return coupled_ustar(u2, lambda, *ustar) ? 1 : 0; }
double oracle_ice_bulb_temperature(double T, double t, double ea, double D, double lambda_t, double L) {
    return ice_bulb_temperature(T, t, ea, D, lambda_t, L);
}
void oracle_incomplete_gamma(double a, double x, double* P, double* Q) { incomplete_gamma(a, x, *P, *Q); }
double oracle_gamma_pdf(double x, double a, double b) { return gamma_pdf(x, a, b); }
void oracle_subgrid_face(const pbsm3d_config* cfg, double snow_depth, const double* tpi, double* out) {
    const SubgridFace o = subgrid_face(*cfg, snow_depth, tpi);
    out[0] = o.min_sd_trans_avg;
    out[1] = o.frac_contrib;
    out[2] = o.frac_contrib_nosnw;
    out[3] = o.tpi_lim;
    out[4] = o.have_test_int ? o.test_int : -9999.0;
}

// triangulation.hpp:1466-1475 edge(i) = v[cw(i)] - v[ccw(i)], ccw(i)=(i+1)%3, cw(i)=(i+2)%3
// triangulation.hpp:1443-1463 edge_unit_normal, :1493-1498 edge_length,
// :1577-1589 center (centroid), :1830-1856 get_area (2-D area when no "area" parameter)
void oracle_face_geometry(int64_t nv, const double* xyz, int64_t nt, const int32_t* tri, double* E, double* M,
                          double* area, double* center) {
    (void)nv;
    for (int64_t f = 0; f < nt; ++f) {
        const double* p[3];
        for (int k = 0; k < 3; ++k) p[k] = xyz + 3 * (int64_t)tri[3 * f + k];
        double ex[3], ey[3];
        for (int i = 0; i < 3; ++i) {
            const double* a = p[(i + 1) % 3];
            const double* b = p[(i + 2) % 3];
            ex[i] = b[0] - a[0];
            ey[i] = b[1] - a[1];
        }
        for (int i = 0; i < 3; ++i) {
            double nx = ey[i], ny = -ex[i];
            int i1 = (i + 1) % 3;
            double D = ex[i1] * nx + ey[i1] * ny;
            if (D > 0) { nx = -nx; ny = -ny; }
            double len = std::sqrt(nx * nx + ny * ny);
            M[6 * f + 2 * i] = nx / len;
            M[6 * f + 2 * i + 1] = ny / len;
            E[3 * f + i] = std::sqrt(ex[i] * ex[i] + ey[i] * ey[i]);
        }
        area[f] = ((p[1][0] - p[0][0]) * (p[2][1] - p[0][1]) - (p[1][1] - p[0][1]) * (p[2][0] - p[0][0])) / 2.0;
        for (int c = 0; c < 3; ++c) center[3 * f + c] = (p[0][c] + p[1][c] + p[2][c]) / 3.0;
    }
}

int oracle_face_neighbors(int64_t nv, int64_t nt, const int32_t* tri, int32_t* neigh) {
    std::unordered_map<uint64_t, std::pair<int64_t, int>> open;
    open.reserve(nt * 2);
    for (int64_t i = 0; i < 3 * nt; ++i) neigh[i] = -1;
    for (int64_t f = 0; f < nt; ++f)
        for (int j = 0; j < 3; ++j) {
            uint64_t a = (uint64_t)tri[3 * f + (j + 1) % 3], b = (uint64_t)tri[3 * f + (j + 2) % 3];
            if (a >= (uint64_t)nv || b >= (uint64_t)nv) return PBSM3D_ERR_BAD_MESH;
            uint64_t key = std::min(a, b) * (uint64_t)nv + std::max(a, b);
            auto it = open.find(key);
            if (it == open.end()) {
                open.emplace(key, std::make_pair(f, j));
            } else {
                neigh[3 * f + j] = (int32_t)it->second.first;
                neigh[3 * it->second.first + it->second.second] = (int32_t)f;
                open.erase(it);
            }
        }
    return 0;
}

int oracle_set_threads(int n) {
    const int prev = omp_get_max_threads();
    if (n > 0) omp_set_num_threads(n);
    return prev;
}

void oracle_solver_defaults(oracle_solver_cfg* s) {
    s->restart = 30;
    s->maxit = 1000;
    s->tol = 1e-8;
    s->ilut_drop = 1e-4;
    s->ilut_fill = 3.0;
    s->nblocks = 1;
    s->dep_maxit = 1000;
    s->dep_tol = 1e-8;
}

const char* oracle_last_error(const oracle_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

int oracle_set_solver(oracle_ctx* ctx, const oracle_solver_cfg* s) {
    ctx->scfg = *s;
    return 0;
}

// PBSM3D::PBSM3D (PBSM3D.cpp:103-219) + PBSM3D::init (PBSM3D.cpp:221-398)
// + the two NearestNeighborProblem graphs (LinearAlgebra.cpp:31-116).
int oracle_create(const pbsm3d_mesh_desc* mesh, const pbsm3d_config* cfg, oracle_ctx** out) {
    *out = nullptr;
    if (!mesh || !cfg || mesh->n_faces <= 0 || !mesh->neighbor || !mesh->edge_length || !mesh->edge_normal ||
        !mesh->area || !mesh->center) {
        g_create_error = "invalid mesh description";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (cfg->use_exp_fetch && cfg->use_tanh_fetch) {  // PBSM3D.cpp:132-135
        g_create_error = "PBSM3d: Cannot specify both exp_fetch and tanh_fetch";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (cfg->settling_velocity < 0) {  // PBSM3D.cpp:237-240
        g_create_error = "PBSM3D settling velocity must be positive";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (cfg->nLayer < 1) {
        g_create_error = "nLayer must be >= 1";
        return PBSM3D_ERR_INVALID_ARG;
    }
    auto* c = new oracle_ctx();
    c->cfg = *cfg;
    oracle_solver_defaults(&c->scfg);
    const int64_t T = mesh->n_faces;
    const int L = cfg->nLayer;
    c->T = T;
    c->L = L;
    c->susp_depth = 5;
    c->dz = c->susp_depth / (double)L;  // v_edge_height, PBSM3D.cpp:225-226
    c->l_max = 40;
    c->nbr.assign(mesh->neighbor, mesh->neighbor + 3 * T);
    c->E.assign(mesh->edge_length, mesh->edge_length + 3 * T);
    c->m.assign(mesh->edge_normal, mesh->edge_normal + 6 * T);
    c->area.assign(mesh->area, mesh->area + T);
    c->center.assign(mesh->center, mesh->center + 3 * T);
    for (int64_t i = 0; i < 3 * T; ++i)
        if (c->nbr[i] < -1 || c->nbr[i] >= T) {
            g_create_error = "neighbour index out of range";
            delete c;
            return PBSM3D_ERR_BAD_MESH;
        }
    // Vegetation (PBSM3D.cpp:278-325): any face without vegetation clears
    // enable_veg for the whole module.
    bool all_veg = mesh->canopy_height != nullptr;
    if (all_veg && mesh->has_vegetation)
        for (int64_t i = 0; i < T; ++i) all_veg = all_veg && mesh->has_vegetation[i];
    c->enable_veg = cfg->enable_veg && all_veg;
    c->canopy.assign(T, 0);
    c->lai.assign(T, 0);
    c->stalkN.assign(T, 0);
    c->stalkD.assign(T, 0);
    if (c->enable_veg) {
        for (int64_t i = 0; i < T; ++i) {
            c->canopy[i] = mesh->canopy_height[i];
            if (cfg->use_R94_lambda) {
                c->lai[i] = mesh->lai ? mesh->lai[i] : 0;
            } else {
                c->stalkN[i] = mesh->stalk_number ? mesh->stalk_number[i] : 1;
                c->stalkD[i] = mesh->stalk_diameter ? mesh->stalk_diameter[i] : 0.8;
            }
        }
    }
    c->has_veg.assign(T, 0);
    c->canopy_raw.assign(T, 0);
    c->lai_raw.assign(T, 0);
    if (mesh->canopy_height)
        for (int64_t i = 0; i < T; ++i) {
            c->has_veg[i] = mesh->has_vegetation ? mesh->has_vegetation[i] : 1;
            c->canopy_raw[i] = mesh->canopy_height[i];
            c->lai_raw[i] = mesh->lai ? mesh->lai[i] : 0.0;
        }
    c->water.assign(T, 0);
    if (mesh->is_water) c->water.assign(mesh->is_water, mesh->is_water + T);
    // prism areas and neighbour flags (PBSM3D.cpp:362-392)
    c->A5.assign(5 * T, 0);
    c->face_neigh.assign(3 * T, 0);
    for (int64_t i = 0; i < T; ++i) {
        for (int j = 0; j < 3; ++j) c->A5[5 * i + j] = c->E[3 * i + j] * c->dz;
        c->A5[5 * i + 3] = c->A5[5 * i + 4] = c->area[i];
        for (int j = 0; j < 3; ++j) c->face_neigh[3 * i + j] = c->nbr[3 * i + j] >= 0;
    }
    c->saltation.assign(T, 0);
    c->hs.assign(T, 0);
    c->z0.assign(T, 0);
    c->ustar.assign(T, 0);
    c->c_salt.assign(T, 0);
    c->ustar_th.assign(T, 0);
    c->u_z.assign((int64_t)L * T, 0);
    c->csubl.assign((int64_t)L * T, 0);
    const double nanv = -9999.0;  // variablestorage default
    c->Qsalt.assign(T, nanv);
    c->Qsusp.assign(T, nanv);
    c->Qsubl.assign(T, nanv);
    c->Qsubl_mass.assign(T, nanv);
    c->sum_subl.assign(T, 0);
    c->drift_mass.assign(T, nanv);
    c->sum_drift.assign(T, 0);  // PBSM3D.cpp:392
    c->more_than_avail.assign(T, nanv);
    c->bsp.assign(T, nanv);
    c->tpi.assign(5 * T, NAN);
    {
        const double* src[5] = {mesh->tpi_mean, mesh->tpi_std, mesh->tpi_neg_frac, mesh->tpi_neg_mean,
                                mesh->tpi_neg_std};
        for (int k = 0; k < 5; ++k)
            if (src[k]) std::copy(src[k], src[k] + T, c->tpi.begin() + k * T);
    }
    c->frac_contrib.assign(T, nanv);
    c->frac_contrib_nosnw.assign(T, nanv);
    c->hold_topo.assign(T, nanv);
    c->tpi_lim.assign(T, nanv);
    c->test_int.assign(T, nanv);
    // Suspension graph: row z*T+i = self, lateral (same layer, face order),
    // below, above (LinearAlgebra.cpp:67-116).
    {
        System& S = c->susp;
        S.rows = T * L;
        S.rowptr.assign(S.rows + 1, 0);
        for (int z = 0; z < L; ++z)
            for (int64_t i = 0; i < T; ++i) {
                int64_t r = (int64_t)z * T + i;
                int n = 1;
                for (int f = 0; f < 3; ++f) n += c->nbr[3 * i + f] >= 0;
                n += (z > 0) + (z < L - 1);
                S.rowptr[r + 1] = n;
            }
        for (int64_t r = 0; r < S.rows; ++r) S.rowptr[r + 1] += S.rowptr[r];
        S.cols.assign(S.rowptr[S.rows], 0);
        for (int z = 0; z < L; ++z)
            for (int64_t i = 0; i < T; ++i) {
                int64_t r = (int64_t)z * T + i;
                int64_t k = S.rowptr[r];
                S.cols[k++] = (int32_t)r;
                for (int f = 0; f < 3; ++f)
                    if (c->nbr[3 * i + f] >= 0) S.cols[k++] = (int32_t)((int64_t)z * T + c->nbr[3 * i + f]);
                if (z > 0) S.cols[k++] = (int32_t)((int64_t)(z - 1) * T + i);
                if (z < L - 1) S.cols[k++] = (int32_t)((int64_t)(z + 1) * T + i);
            }
        S.vals.assign(S.cols.size(), 0);
        S.rhs.assign(S.rows, 0);
        S.x.assign(S.rows, 0);
    }
    {
        System& D = c->dep;
        D.rows = T;
        D.rowptr.assign(T + 1, 0);
        for (int64_t i = 0; i < T; ++i) {
            int n = 1;
            for (int f = 0; f < 3; ++f) n += c->nbr[3 * i + f] >= 0;
            D.rowptr[i + 1] = D.rowptr[i] + n;
        }
        D.cols.assign(D.rowptr[T], 0);
        for (int64_t i = 0; i < T; ++i) {
            int64_t k = D.rowptr[i];
            D.cols[k++] = (int32_t)i;
            for (int f = 0; f < 3; ++f)
                if (c->nbr[3 * i + f] >= 0) D.cols[k++] = c->nbr[3 * i + f];
        }
        D.vals.assign(D.cols.size(), 0);
        D.rhs.assign(T, 0);
        D.x.assign(T, 0);
    }
    *out = c;
    return 0;
}

void oracle_destroy(oracle_ctx* ctx) { delete ctx; }

// PBSM3D.cpp:400-1406: zero both systems, per-face saltation, layer
// coefficients and suspension row assembly.
int oracle_stage_assemble_suspension(oracle_ctx* c, const pbsm3d_forcing* F, double dt) {
    auto t0 = std::chrono::steady_clock::now();
    const int64_t T = c->T;
    const int L = c->L;
    const pbsm3d_config& cfg = c->cfg;
    if (!F || !F->U_R || !F->U_2m_above_srf || !F->vw_dir || !F->swe || !F->t || !F->rh || !F->snowdepthavg) {
        c->err = "missing forcing";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if ((cfg.use_exp_fetch || cfg.use_tanh_fetch) && !F->fetch) {
        c->err = "fetch forcing required";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (cfg.use_PomLi_probability && !F->p_snow_hours) {
        c->err = "p_snow_hours forcing required";
        return PBSM3D_ERR_INVALID_ARG;
    }
    c->dt = dt;
    c->f_UR.assign(F->U_R, F->U_R + T);
    c->f_U2.assign(F->U_2m_above_srf, F->U_2m_above_srf + T);
    c->f_dir.assign(F->vw_dir, F->vw_dir + T);
    c->f_swe.assign(F->swe, F->swe + T);
    c->f_t.assign(F->t, F->t + T);
    c->f_rh.assign(F->rh, F->rh + T);
    c->f_sd.assign(F->snowdepthavg, F->snowdepthavg + T);
    if (F->fetch) c->f_fetch.assign(F->fetch, F->fetch + T); else c->f_fetch.assign(T, 1000);
    if (F->p_snow_hours) c->f_psh.assign(F->p_snow_hours, F->p_snow_hours + T); else c->f_psh.assign(T, 0);

    c->susp.zero();
    c->dep.zero();
    c->suspension_present = false;
    c->deposition_present = false;

    const double dz = c->dz;
    const double z0_snow = cfg.z0_snow;
    const double cos_pi_4 = std::cos(M_PI / 4.0);
    System& S = c->susp;

#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < T; ++i) {
        const double* m = &c->m[6 * i];
        const double* A = &c->A5[5 * i];
        double mm5[5][3] = {{m[0], m[1], 0}, {m[2], m[3], 0}, {m[4], m[5], 0}, {0, 0, 1}, {0, 0, -1}};
        // PBSM3D.cpp:436-470
        double fetch = 1000;
        if (cfg.use_exp_fetch || cfg.use_tanh_fetch) fetch = c->f_fetch[i];
        double frac_contrib = 1.;
        double min_sd_trans_avg = cfg.min_sd_trans;
        double uref = c->f_UR[i];
        double snow_depth = c->f_sd[i];
        snow_depth = is_nan(snow_depth) ? 0 : snow_depth;
        if (cfg.use_subgrid_topo || cfg.use_subgrid_topo_V2) {  // PBSM3D.cpp:480-645
            const double tpi[5] = {c->tpi[i], c->tpi[T + i], c->tpi[2 * T + i], c->tpi[3 * T + i], c->tpi[4 * T + i]};
            const SubgridFace sg = subgrid_face(cfg, snow_depth, tpi);
            frac_contrib = sg.frac_contrib;
            min_sd_trans_avg = sg.min_sd_trans_avg;
            c->frac_contrib[i] = sg.frac_contrib;
            c->hold_topo[i] = sg.min_sd_trans_avg;
            if (cfg.use_subgrid_topo) c->frac_contrib_nosnw[i] = sg.frac_contrib_nosnw;
            if (cfg.use_subgrid_topo_V2) {
                c->tpi_lim[i] = sg.tpi_lim;
                if (sg.have_test_int) c->test_int[i] = sg.test_int;
            }
        }
        double u2 = c->f_U2[i];
        double z10 = 10. + snow_depth;
        double u10;
        if (z10 < kZUR)
            u10 = log_scale_wind(uref, kZUR, z10, snow_depth, z0_snow);
        else
            u10 = uref;
        double swe = c->f_swe[i];
        swe = is_nan(swe) ? 0 : swe;
        double height_diff = smax(0.0, c->canopy[i] - snow_depth);
        if (!c->enable_veg) height_diff = 0;
        // PBSM3D.cpp:649-760
        double ustar = 1.3;
        double lambda = 0;
        bool saltation = false;
        double z0 = 0;
        double T_c = c->f_t[i];
        double u_star_saltation_threshold = 0.35 + (1.0 / 150.0) * T_c + (1.0 / 8200.0) * T_c * T_c;
        u_star_saltation_threshold = u_star_saltation_threshold * cfg.ustar_th_scale;
        if (height_diff <= cfg.cutoff && snow_depth >= min_sd_trans_avg && !c->water[i]) {
            if (cfg.use_R94_lambda)
                lambda = 0.5 * c->lai[i] * height_diff;
            else
                lambda = c->stalkN[i] * c->stalkD[i] * height_diff;
            if (cfg.z0_ustar_coupling) {
                double u = 0;
                if (coupled_ustar(u2, lambda, u)) ustar = u;  // no bracket: u* stays 1.3 (:710-713)
            } else {
                ustar = u2 * kKappa / std::log(2.0 / 0.0002);
            }
            if (ustar >= u_star_saltation_threshold) {
                saltation = true;
                if (cfg.z0_ustar_coupling)
                    z0 = 0.6131702345e-2 * ustar * ustar + .5 * lambda;  // Li and Pomeroy 2000 eqn 4 (:736)
                else
                    z0 = z0_snow;
            }
        }
        if (!saltation) {
            z0 = z0_snow;
            ustar = smax(0.01, kKappa * uref / std::log(kZUR / z0));
        }
        z0 = smax(z0_snow, z0);
        ustar = smax(0.01, ustar);
        // PBSM3D.cpp:761-925
        double hs = 0;
        if (saltation) hs = 0.08436 * std::pow(ustar, 1.27);
        double Qsalt = 0;
        double c_salt = 0;
        double t = c->f_t[i] + 273.15;
        if (saltation) {
            double rho_f = std_dry_air_density(c->center[3 * i + 2], t);
            double Beta = 202.0;
            double mB = 0.16;
            double tau_n_ratio = (mB * Beta * lambda) / (1.0 + mB * Beta * lambda);
            c_salt = rho_f / (3.29 * ustar) *
                     (1.0 - tau_n_ratio - (u_star_saltation_threshold * u_star_saltation_threshold) / (ustar * ustar));
            if (c_salt < 0 || std::isnan(c_salt)) {
                c_salt = 0;
                saltation = false;
            }
            if (cfg.use_exp_fetch && fetch < 500) {
                double fetch_ref = 500;
                double mu = 3.0;
                c_salt *= 1.0 - std::exp(-mu * fetch / fetch_ref);
            } else if (cfg.use_tanh_fetch && fetch <= 300.) {
                double fetch_ref = 300;  // quirk: Lc uses fetch_ref, not fetch
                double Lc = 0.5 * std::tanh(0.1333333333e-1 * fetch_ref - 2.0) + 0.5;
                c_salt *= Lc;
            }
            if (cfg.use_PomLi_probability) {  // PBSM3D.cpp:848-865
                double Ah = c->f_psh[i];
                double u_mean = 11.2 + 0.365 * T_c + 0.00706 * T_c * T_c + 0.9 * std::log(Ah);
                double delta = 0.145 * T_c + 0.00196 * T_c * T_c + 4.3;
                double z0v = (c->stalkN[i] * c->stalkD[i] * height_diff) / 2.0;
                double us = u10 / std::sqrt((1 + 340.0 * z0v));
                double Pu10 = 1.0 / (1.0 + std::exp((std::sqrt(M_PI) * (u_mean - us)) / delta));
                c->bsp[i] = Pu10;
                c_salt *= Pu10;
            }
            if (cfg.use_subgrid_topo || cfg.use_subgrid_topo_V2) c_salt *= frac_contrib;  // :867-870
            double uhs = 2.8 * u_star_saltation_threshold;
            Qsalt = c_salt * uhs * hs;
            double mass = 0;
            double vx, vy;
            bearing_to_cartesian(c->f_dir[i], vx, vy);
            double uvw[3] = {-vx, -vy, 0};
            double V = c->area[i];
            for (int j = 0; j < 3; ++j) {
                double udotm = dot3(uvw, mm5[j]);
                double Ej = c->E[3 * i + j];
                mass += -Ej * Qsalt * udotm;
            }
            mass = mass / V * dt;
            if (mass < 0 && std::fabs(mass) > swe) {
                c_salt = 0;
                Qsalt = c_salt * uhs * hs;
            }
        }
        c->Qsalt[i] = Qsalt;
        c->saltation[i] = saltation;
        c->hs[i] = hs;
        c->z0[i] = z0;
        c->ustar[i] = ustar;
        c->c_salt[i] = c_salt;
        c->ustar_th[i] = u_star_saltation_threshold;

        // PBSM3D.cpp:927-1233 layer coefficients
        double rh = c->f_rh[i] / 100.;
        double es = saturated_vapour_pressure(t);
        double ea = rh * es / 1000.;
        // PBSM3D.cpp:1062-1096: with iterative_subl the ice-bulb temperature is
        // a per-face value; the rate uses it below
        double Ti = 0;
        if (cfg.iterative_subl) {
            double D = 2.06e-5 * std::pow(t / 273.15, 1.75);
            double lambda_t = 0.000063 * t + 0.00673;
            Ti = ice_bulb_temperature(T_c, t, ea, D, lambda_t, 2.838e6);
        }
        double vwx, vwy;
        bearing_to_cartesian(c->f_dir[i], vwx, vwy);
        for (int z = 0; z < L; ++z) {
            double cz = z * dz + hs + dz / 2.;
            double u_z = 0;
            double hz = cz + snow_depth;
            if (saltation && cz < height_diff)
                u_z = 2.8 * u_star_saltation_threshold;
            else if (cz < height_diff)
                u_z = 0.01;
            else {
                if (hz < kZUR)
                    u_z = smax(0.01, log_scale_wind(uref, kZUR, hz, snow_depth, z0));
                else
                    u_z = smax(0.01, uref);
            }
            c->u_z[(int64_t)z * T + i] = u_z;
            double rm = 4.6e-5 * std::pow(cz, -0.258);
            double mm_alpha = 4.08 + 12.6 * cz;
            double mm = 4. / 3. * M_PI * kRhoIce * rm * rm * rm * (1.0 + 3.0 / mm_alpha + 2. / (mm_alpha * mm_alpha));
            double r_z = std::pow((3.0 * mm) / (4 * M_PI * kRhoIce), 0.3333333);
            double xrz = 0.005 * std::pow(u_z, 1.36);
            double omega = cfg.settling_velocity;
            if (!cfg.do_fixed_settling) omega = 1.1e7 * std::pow(r_z, 1.8);
            omega = omega * cfg.settling_scale;
            double Vr = omega + 3.0 * xrz * cos_pi_4;
            double v = 1.88e-5;
            double Re = 2.0 * r_z * Vr / v;
            double Nu, Sh;
            Nu = Sh = 1.79 + 0.606 * std::pow(Re, 0.5);
            double D = 2.06e-5 * std::pow(t / 273.15, 1.75);
            double lambda_t = 0.000063 * t + 0.00673;
            double Ls = 2.838e6;
            double M = 18.01;
            double R = 8313;
            double sigma = (rh - 1.0) * (1.019 + 0.027 * std::log(cz));
            double rho = (M * es) / (R * t);
            double Qr = 0.9 * M_PI * rm * rm * 120.0;
            double dmdtz;
            if (cfg.iterative_subl) {
                // eqn 13 of Pomeroy and Li 2000 as PBSM3D.cpp:1099 writes it: Ts in K
                // against t + 273.15 with t already in K
                double Ts = Ti + 273.15;
                dmdtz = 2.0 * M_PI * rm * lambda_t / Ls * Nu * (Ts - (t + 273.15));
            } else {
                dmdtz = Sh * rho * D * (6.283185308 * Nu * R * r_z * sigma * t * t * lambda_t - Ls * M * Qr + Qr * R * t) /
                        (D * Ls * Sh * (Ls * M - R * t) * rho + lambda_t * t * t * Nu * R);
            }
            double csubl = dmdtz / mm;
            double K[5] = {0, 0, 0, 0, 0};
            double alpha[5] = {0, 0, 0, 0, 0};
            if (cfg.do_lateral_diff)
                for (int a = 0; a < 3; ++a) {
                    alpha[a] = A[a];
                    K[a] = 0.00001;
                    alpha[a] *= K[a];
                }
            double l = kKappa * (cz + z0) * c->l_max / (kKappa * (cz + z0) + c->l_max);
            double w = omega;
            double diffusion_coeff = cfg.snow_diffusion_const;
            if (cfg.rouault_diffusion_coef) {
                double c2 = 1.0;
                double dc = 1.0 / (1.0 + (c2 * w * w) / (1.56 * ustar * ustar));
                diffusion_coeff = dc;
            }
            K[3] = K[4] = diffusion_coeff * ustar * l;
            alpha[3] = A[3] * K[3] / dz;
            alpha[4] = A[4] * K[4] / dz;
            double uvw[3] = {-vwx, -vwy, 0};
            {
                double v1 = 0, v2 = 0;  // armadillo norm2 of a 3-vector
                v1 += uvw[0] * uvw[0];
                v2 += uvw[1] * uvw[1];
                v1 += uvw[2] * uvw[2];
                double nrm = std::sqrt(v1 + v2);
                double s = u_z / nrm;
                uvw[0] *= s;
                uvw[1] *= s;
                uvw[2] *= s;
            }
            uvw[2] = -w;
            double udotm[5];
            for (int j = 0; j < 5; ++j) udotm[j] = dot3(uvw, mm5[j]);
            int64_t idx = (int64_t)T * z + i;
            double V = c->area[i] * dz;
            V /= 5.0;
            if (!cfg.do_sublimation) csubl = 0.0;
            c->csubl[idx] = csubl;
            // PBSM3D.cpp:1236-1279 lateral faces
            for (int f = 0; f < 3; ++f) {
                bool has = c->face_neigh[3 * i + f];
                int64_t nidx = has ? (int64_t)T * z + c->nbr[3 * i + f] : -1;
                if (udotm[f] > 0) {
                    if (has) {
                        S.sum_into(idx, idx, (V * csubl - A[f] * udotm[f] - alpha[f]));
                        S.sum_into(idx, nidx, (alpha[f]));
                    } else {
                        S.sum_into(idx, idx, (-0.1e-1 * alpha[f] - 1. * A[f] * udotm[f] + csubl * V));
                    }
                } else {
                    if (has) {
                        S.sum_into(idx, idx, V * csubl - alpha[f]);
                        S.sum_into(idx, nidx, -A[f] * udotm[f] + alpha[f]);
                    } else {
                        S.sum_into(idx, idx, -0.1e-1 * alpha[f] - .99 * A[f] * udotm[f] + csubl * V);
                    }
                }
            }
            // PBSM3D.cpp:1282-1404 vertical faces
            if (z == 0) {
                double alpha4 = A[4] * K[4] / (hs / 2.0 + dz / 2.0);
                S.sum_into(idx, idx, V * csubl - A[4] * udotm[4] - alpha4);
                double val = -alpha4 * c_salt;
                S.rhs[idx] += val;
                int64_t nidx = (int64_t)T * (z + 1) + i;
                if (udotm[3] > 0) {
                    S.sum_into(idx, idx, V * csubl - A[3] * udotm[3] - alpha[3]);
                    S.sum_into(idx, nidx, alpha[3]);
                } else {
                    S.sum_into(idx, idx, V * csubl - alpha[3]);
                    S.sum_into(idx, nidx, -A[3] * udotm[3] + alpha[3]);
                }
            } else if (z == L - 1) {
                double cprecip = 0;
                if (udotm[3] > 0) {
                    S.sum_into(idx, idx, V * csubl - A[3] * udotm[3] - alpha[3]);
                    double val = -alpha[3] * cprecip;
                    S.rhs[idx] += val;
                } else {
                    S.sum_into(idx, idx, V * csubl - alpha[3]);
                    double val = A[3] * cprecip * udotm[3] - alpha[3] * cprecip;
                    S.rhs[idx] += val;
                }
                int64_t nidx = (int64_t)T * (z - 1) + i;
                if (udotm[4] > 0) {
                    S.sum_into(idx, idx, V * csubl - A[4] * udotm[4] - alpha[4]);
                    S.sum_into(idx, nidx, alpha[4]);
                } else {
                    S.sum_into(idx, idx, V * csubl - alpha[4]);
                    S.sum_into(idx, nidx, -A[4] * udotm[4] + alpha[4]);
                }
            } else {
                int64_t nidx = (int64_t)T * (z + 1) + i;
                if (udotm[3] > 0) {
                    S.sum_into(idx, idx, V * csubl - A[3] * udotm[3] - alpha[3]);
                    S.sum_into(idx, nidx, alpha[3]);
                } else {
                    S.sum_into(idx, idx, V * csubl - alpha[3]);
                    S.sum_into(idx, nidx, -A[3] * udotm[3] + alpha[3]);
                }
                nidx = (int64_t)T * (z - 1) + i;
                if (udotm[4] > 0) {
                    S.sum_into(idx, idx, V * csubl - A[4] * udotm[4] - alpha[4]);
                    S.sum_into(idx, nidx, alpha[4]);
                } else {
                    S.sum_into(idx, idx, V * csubl - alpha[4]);
                    S.sum_into(idx, nidx, -A[4] * udotm[4] + alpha[4]);
                }
            }
        }
    }
    // PBSM3D.cpp:1424-1427
    c->susp_rhs_max = S.rhs_max();
    c->suspension_present = c->susp_rhs_max > 1e-12;
    auto t1 = std::chrono::steady_clock::now();
    c->ms_assembly = std::chrono::duration<double, std::milli>(t1 - t0).count();
    for (double v : S.vals)
        if (std::isnan(v)) { c->err = "NaN in the assembled suspension system"; return PBSM3D_ERR_NAN_INPUT; }
    for (double v : S.rhs)
        if (std::isnan(v)) { c->err = "NaN in the suspension right-hand side"; return PBSM3D_ERR_NAN_INPUT; }
    return 0;
}

// PBSM3D.cpp:1429-1459 (Solve only when suspension is present)
int oracle_stage_solve_suspension(oracle_ctx* c) {
    c->susp_iters = 0;
    c->susp_relres = 0;
    c->ms_susp_solve = 0;
    if (!c->suspension_present) return 0;
    auto t0 = std::chrono::steady_clock::now();
    Precond M;
    M.build(c->susp, c->T, c->L, c->scfg.nblocks, c->scfg.ilut_drop, c->scfg.ilut_fill);
    std::fill(c->susp.x.begin(), c->susp.x.end(), 0.0);
    int rc = gmres(c->susp, M, c->susp.rhs.data(), c->susp.x.data(), c->scfg.restart, c->scfg.maxit, c->scfg.tol,
                   c->susp_iters, c->susp_relres);
    c->ms_susp_solve = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (rc) {
        c->err = "Belos solver failed to converge";
        return PBSM3D_ERR_NOT_CONVERGED;
    }
    return 0;
}

int oracle_stage_set_suspension_solution(oracle_ctx* c, const double* x) {
    std::copy(x, x + c->susp.rows, c->susp.x.begin());
    return 0;
}

// PBSM3D.cpp:1467-1503 (column post) and :1516-1663 (deposition assembly)
int oracle_stage_post_and_assemble_deposition(oracle_ctx* c) {
    const int64_t T = c->T;
    const int L = c->L;
    const double dz = c->dz;
    const double* x = c->susp.x.data();
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < T; ++i) {
        double Qsusp = 0;
        double Qsubl = 0;
        for (int z = 0; z < L; ++z) {
            double cc = x[T * z + i];
            cc = cc < 0 || is_nan(cc) ? 0 : cc;
            double u_z = c->u_z[(int64_t)z * T + i];
            Qsusp += cc * u_z * dz;
            Qsubl += c->csubl[(int64_t)z * T + i] * cc * dz;
        }
        c->Qsusp[i] = Qsusp;
        c->Qsubl[i] = Qsubl;
        c->Qsubl_mass[i] = Qsubl * c->dt;
        c->sum_subl[i] += c->Qsubl_mass[i];
    }
    System& D = c->dep;
    const double eps = c->cfg.smooth_coeff;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < T; ++i) {
        double vx, vy;
        bearing_to_cartesian(c->f_dir[i], vx, vy);
        double uvw[3] = {-vx, -vy, 0};
        double V = c->area[i];
        D.replace(i, i, V);
        for (int j = 0; j < 3; ++j) {
            double mj[3] = {c->m[6 * i + 2 * j], c->m[6 * i + 2 * j + 1], 0};
            double udotm = dot3(uvw, mj);
            double Ej = c->E[3 * i + j];
            double Qtj = 0, Qsj = 0;
            int32_t nb = c->nbr[3 * i + j];
            if (udotm > 0) {
                Qtj = c->Qsusp[i];
                Qsj = c->Qsalt[i];
            } else {
                if (nb >= 0) {
                    Qtj = c->Qsusp[nb];
                    Qsj = c->Qsalt[nb];
                    if (is_nan(Qsj)) Qsj = 0;
                } else {
                    Qtj = c->Qsusp[i];
                    Qsj = c->Qsalt[i];
                }
            }
            if (nb >= 0) {
                double ddx = c->center[3 * i] - c->center[3 * nb];
                double ddy = c->center[3 * i + 1] - c->center[3 * nb + 1];
                double dxj = std::sqrt(ddx * ddx + ddy * ddy);  // distance_UTM, coordinates.cpp:100-106
                D.sum_into(i, i, eps * Ej / dxj);
                D.sum_into(i, nb, -eps * Ej / dxj);
            }
            double val = -Ej * (Qtj + Qsj) * udotm;
            D.rhs[i] += val;
        }
    }
    c->dep_rhs_max = D.rhs_max();
    c->deposition_present = c->suspension_present && c->dep_rhs_max > 1e-12;
    for (double v : D.vals)
        if (std::isnan(v)) { c->err = "NaN in the assembled deposition system"; return PBSM3D_ERR_NAN_INPUT; }
    return 0;
}

int oracle_stage_solve_deposition(oracle_ctx* c) {
    c->dep_iters = 0;
    c->dep_relres = 0;
    c->ms_dep_solve = 0;
    if (!c->deposition_present) return 0;
    auto t0 = std::chrono::steady_clock::now();
    Precond M;
    M.build(c->dep, c->T, 1, c->scfg.nblocks, c->scfg.ilut_drop, c->scfg.ilut_fill);
    std::fill(c->dep.x.begin(), c->dep.x.end(), 0.0);
    int rc = gmres(c->dep, M, c->dep.rhs.data(), c->dep.x.data(), c->scfg.restart, c->scfg.dep_maxit,
                   c->scfg.dep_tol, c->dep_iters, c->dep_relres);
    c->ms_dep_solve = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (rc) {
        c->err = "Belos solver failed to converge";
        return PBSM3D_ERR_NOT_CONVERGED;
    }
    return 0;
}

int oracle_stage_set_deposition_solution(oracle_ctx* c, const double* q) {
    std::copy(q, q + c->T, c->dep.x.begin());
    return 0;
}

static void copy_out(double* dst, const std::vector<double>& src) {
    if (dst) std::memcpy(dst, src.data(), src.size() * sizeof(double));
}

// PBSM3D.cpp:1710-1740 erosion/deposition update (skipped without deposition)
int oracle_stage_update(oracle_ctx* c, const pbsm3d_outputs* out, pbsm3d_stats* st) {
    const int64_t T = c->T;
    double led_div = 0, led_dep = 0, led_clip = 0, led_snow = 0, led_res = 0;
    for (int64_t i = 0; i < T; ++i) {
        double swe = c->f_swe[i];
        swe = is_nan(swe) ? 0 : swe;
        led_snow += c->area[i] * swe;
    }
    if (c->deposition_present) {
        const double* q = c->dep.x.data();
        std::vector<double> Aq(T);
        spmv(c->dep, q, Aq.data());
        for (int64_t i = 0; i < T; ++i) {
            double qdep = is_nan(q[i]) ? 0 : q[i];
            double mass = 0;
            mass = qdep * c->dt;
            double swe = c->f_swe[i];
            swe = is_nan(swe) ? 0 : swe;
            if (mass < 0 && std::fabs(mass) > swe) {
                c->more_than_avail[i] = 1;
                mass = -swe;
            }
            if (mass < 0 && !c->saltation[i]) mass = 0;
            c->drift_mass[i] = mass;
            c->sum_drift[i] += mass;
            led_div += c->dt * c->dep.rhs[i];
            led_dep += c->dt * c->area[i] * q[i];
            led_clip += c->area[i] * (mass - q[i] * c->dt);
            led_res += c->dt * (c->dep.rhs[i] - Aq[i]);
        }
    }
    if (out) {
        copy_out(out->Qsalt, c->Qsalt);
        copy_out(out->Qsusp, c->Qsusp);
        copy_out(out->Qsubl, c->Qsubl);
        copy_out(out->Qsubl_mass, c->Qsubl_mass);
        copy_out(out->sum_subl, c->sum_subl);
        copy_out(out->drift_mass, c->drift_mass);
        copy_out(out->sum_drift, c->sum_drift);
        copy_out(out->pbsm_more_than_avail, c->more_than_avail);
        copy_out(out->blowingsnow_probability, c->bsp);
        copy_out(out->frac_contrib, c->frac_contrib);
        copy_out(out->frac_contrib_nosnw, c->frac_contrib_nosnw);
        copy_out(out->hold_topo, c->hold_topo);
        copy_out(out->tpi_lim, c->tpi_lim);
        copy_out(out->test_int, c->test_int);
        copy_out(out->c, c->susp.x);
    }
    if (st) {
        std::memset(st, 0, sizeof(*st));
        st->suspension_present = c->suspension_present;
        st->deposition_present = c->deposition_present;
        st->susp_iters = c->susp_iters;
        st->susp_matvecs = c->susp_iters;
        st->dep_iters = c->dep_iters;
        st->susp_rel_residual = c->susp_relres;
        st->dep_rel_residual = c->dep_relres;
        st->susp_rhs_max = c->susp_rhs_max;
        st->dep_rhs_max = c->dep_rhs_max;
        st->ms_coefficients = c->ms_assembly;
        st->ms_susp_solve = c->ms_susp_solve;
        st->ms_dep_solve = c->ms_dep_solve;
        st->ledger_divergence = led_div;
        st->ledger_deposited = led_dep;
        st->ledger_clipped = led_clip;
        st->ledger_snow_mass = led_snow;
        st->ledger_residual = led_res;
    }
    return 0;
}

int oracle_step(oracle_ctx* c, const pbsm3d_forcing* f, double dt, const pbsm3d_outputs* out, pbsm3d_stats* st) {
    auto t0 = std::chrono::steady_clock::now();
    int rc = oracle_stage_assemble_suspension(c, f, dt);
    if (rc) return rc;
    if ((rc = oracle_stage_solve_suspension(c))) return rc;
    if ((rc = oracle_stage_post_and_assemble_deposition(c))) return rc;
    if ((rc = oracle_stage_solve_deposition(c))) return rc;
    rc = oracle_stage_update(c, out, st);
    if (st) st->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

int64_t oracle_rows(const oracle_ctx* c, int32_t which) { return which ? c->dep.rows : c->susp.rows; }
int64_t oracle_nnz(const oracle_ctx* c, int32_t which) {
    return which ? (int64_t)c->dep.cols.size() : (int64_t)c->susp.cols.size();
}
int oracle_get_system(const oracle_ctx* c, int32_t which, int64_t* rowptr, int32_t* cols, double* vals,
                      double* rhs, double* x) {
    const System& S = which ? c->dep : c->susp;
    if (rowptr) std::memcpy(rowptr, S.rowptr.data(), S.rowptr.size() * sizeof(int64_t));
    if (cols) std::memcpy(cols, S.cols.data(), S.cols.size() * sizeof(int32_t));
    if (vals) std::memcpy(vals, S.vals.data(), S.vals.size() * sizeof(double));
    if (rhs) std::memcpy(rhs, S.rhs.data(), S.rhs.size() * sizeof(double));
    if (x) std::memcpy(x, S.x.data(), S.x.size() * sizeof(double));
    return 0;
}
// scale_wind_vert::run(mesh&) (scale_wind_vert.cpp:53-227): per face the
// wind 2 m above the snow from U_R through the canopy profile (point_scale),
// then the thin plate spline of the neighbours' values at the face centre,
// clamped at 0.1 m/s.
int oracle_scale_wind_vert(const oracle_ctx* c, int ignore_canopy, const double* U_R, const double* snowdepthavg,
                           double* u2m) {
    const int64_t T = c->T;
    std::vector<double> pt(T);
    for (int64_t i = 0; i < T; ++i) {
        const double U = U_R[i];
        const double Z_R = kZUR;
        double Z_CanTop = 0;
        if (!ignore_canopy && c->has_veg[i]) Z_CanTop = c->canopy_raw[i];
        const double Z_CanBot = Z_CanTop / 2.0;
        double sd = snowdepthavg ? snowdepthavg[i] : 0.0;
        if (is_nan(sd)) sd = 0.0;
        const double Z_2m = sd + 2.0;
        if (Z_2m >= Z_R) {
            pt[i] = U;
            continue;
        }
        double u;
        if (!ignore_canopy && (Z_CanTop > 0.0) && (Z_2m < Z_CanTop)) {
            const double alpha = c->lai_raw[i];
            if (sd < Z_CanTop) {
                const double U_CanTop = log_scale_wind(U, Z_R, Z_CanTop, sd, kZ0Snow);
                const double U_CanBot = exp_scale_wind(U_CanTop, Z_CanTop, Z_CanBot, alpha);
                if (Z_2m < Z_CanBot)
                    u = log_scale_wind(U_CanBot, Z_CanBot, Z_2m, sd, kZ0Snow);
                else
                    u = exp_scale_wind(U_CanTop, Z_CanTop, Z_2m, alpha);
            } else {
                u = log_scale_wind(U, Z_R, Z_2m, sd, kZ0Snow);
            }
        } else {
            u = log_scale_wind(U, Z_R, Z_2m, sd, kZ0Snow);
        }
        pt[i] = smax(0.1, u);
    }
    for (int64_t i = 0; i < T; ++i) {
        double sx[3], sy[3], sz[3];
        int n = 0;
        for (int j = 0; j < 3; ++j) {
            const int32_t nb = c->nbr[3 * i + j];
            if (nb < 0) continue;
            sx[n] = c->center[3 * nb];
            sy[n] = c->center[3 * nb + 1];
            sz[n] = pt[nb];
            ++n;
        }
        if (n > 0)
            u2m[i] = smax(0.1, tps_interp(sx, sy, sz, n, c->center[3 * i], c->center[3 * i + 1]));
        else
            u2m[i] = smax(0.1, pt[i]);
    }
    return 0;
}

// fetchr::run (fetchr.cpp:55-117): upwind search along vw_dir in `steps`
// steps of max_distance/steps; each step takes the face whose centre is
// nearest the point at that distance (brute force here; a kd-tree of face
// centres in the reference, triangulation.cpp:170-178; the lowest index wins
// a tie) and stops at the first that is higher than the rising line of slope
// I, or (incl_veg) within the internal-boundary-layer recovery length.
int oracle_fetchr(const oracle_ctx* c, int steps, double max_distance, double I, int incl_veg, const double* vw_dir,
                  double* fetch) {
    const int64_t T = c->T;
    const double size_of_step = max_distance / steps;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < T; ++i) {
        fetch[i] = max_distance;
        if (incl_veg && c->has_veg[i] && c->canopy_raw[i] > 1) {
            fetch[i] = 0;
            continue;
        }
        const double br = vw_dir[i] * (M_PI / 180.0);
        const double cx = c->center[3 * i], cy = c->center[3 * i + 1], cz = c->center[3 * i + 2];
        for (int j = 1; j <= steps; ++j) {
            const double distance = j * size_of_step;
            const double qx = cx + distance * std::sin(br), qy = cy + distance * std::cos(br);
            int64_t f = 0;
            double best = INFINITY;
            for (int64_t k = 0; k < T; ++k) {
                const double dx = c->center[3 * k] - qx, dy = c->center[3 * k + 1] - qy;
                const double d2 = dx * dx + dy * dy;
                if (d2 < best) {
                    best = d2;
                    f = k;
                }
            }
            double Z_CanTop = 0;
            if (incl_veg && c->has_veg[f]) Z_CanTop = c->canopy_raw[f];
            const double Z_test = c->center[3 * f + 2] + Z_CanTop;
            const double Z_core = cz + distance * I;
            const double z0_1 = 0.12 * Z_CanTop, z0_2 = 0.001, n = 1.0 / 0.8, h = 5;
            const double x_sss = std::pow(((33.33333333 * h - 25. * z0_2) / (std::log(z0_1 / z0_2) * z0_2)), n) * z0_2;
            if (Z_test >= Z_core || (incl_veg && distance < x_sss)) {
                fetch[i] = distance;
                break;
            }
        }
    }
    return 0;
}

// The face -> station lists of CHM's core (core.cpp:168-205, metdata.cpp:
// 591-622): the n_nearest nearest stations (nearest first, the lower index on a
// tie), or every station within radius (ascending index).  Returns the count.
int oracle_select_stations(const oracle_ctx* c, int64_t face, int64_t ns, const double* sx, const double* sy,
                           int n_nearest, double radius, int32_t* out) {
    const double qx = c->center[3 * face], qy = c->center[3 * face + 1];
    std::vector<std::pair<double, int>> d(ns);
    for (int64_t k = 0; k < ns; ++k) {
        const double dx = sx[k] - qx, dy = sy[k] - qy;
        d[k] = {dx * dx + dy * dy, (int)k};
    }
    int n = 0;
    if (n_nearest > 0) {
        std::sort(d.begin(), d.end());
        for (int k = 0; k < n_nearest && k < (int)ns; ++k) out[n++] = d[k].second;
    } else {
        for (int64_t k = 0; k < ns; ++k)
            if (d[k].first <= radius * radius) out[n++] = (int)k;
    }
    return n;
}

// uniform_wind::run (interp_met/uniform_wind.cpp:58-127): per face, the
// stations' winds as zonal components (speed at least 0.1 m/s; stations
// with a missing speed or direction are skipped), interpolated to the face
// centre (interp 0 = thin plate spline, 1 = IDW, 2 = nearest), back to
// speed (at least 0.1) and bearing.  Returns -1 when a face has no valid
// station.
int oracle_uniform_wind(const oracle_ctx* c, int64_t ns, const double* sx, const double* sy, int n_nearest,
                        double radius, int interp, const double* st_U, const double* st_dir, double* U_R,
                        double* vw_dir) {
    const int64_t T = c->T;
    int bad = 0;
    std::vector<int32_t> sel(ns);
    for (int64_t i = 0; i < T; ++i) {
        const int n = oracle_select_stations(c, i, ns, sx, sy, n_nearest, radius, sel.data());
        double px[16], py[16], pu[16], pv[16];
        int m = 0;
        for (int k = 0; k < n && m < 16; ++k) {
            const int s = sel[k];
            if (is_nan(st_U[s]) || is_nan(st_dir[s])) continue;
            double W = st_U[s];
            W = smax(W, 0.1);
            const double theta = st_dir[s] * M_PI / 180.;
            px[m] = sx[s];
            py[m] = sy[s];
            pu[m] = -W * std::sin(theta);
            pv[m] = -W * std::cos(theta);
            ++m;
        }
        if (m == 0) {
            bad = 1;
            continue;
        }
        const double qx = c->center[3 * i], qy = c->center[3 * i + 1];
        double zu, zv;
        if (interp == 0) {
            const double* z[2] = {pu, pv};
            double o[2];
            tps_interp_multi(px, py, z, 2, m, qx, qy, o);
            zu = o[0];
            zv = o[1];
        } else if (interp == 1) {
            zu = idw_interp(px, py, pu, m, qx, qy);
            zv = idw_interp(px, py, pv, m, qx, qy);
        } else {
            zu = pu[0];
            zv = pv[0];
        }
        double theta = 3.0 * M_PI * 0.5 - std::atan2(zv, zu);
        if (theta > 2 * M_PI) theta = theta - 2 * M_PI;
        double W = std::sqrt(zu * zu + zv * zv);
        W = smax(W, 0.1);
        U_R[i] = W;
        vw_dir[i] = theta * 180.0 / M_PI;
    }
    return bad ? -1 : 0;
}

double oracle_expint_e1(double x) { return expint_e1(x); }
double oracle_tps(const double* sx, const double* sy, const double* sz, int n, double qx, double qy) {
    return tps_interp(sx, sy, sz, n, qx, qy);
}

int oracle_get_face_fields(const oracle_ctx* c, double* saltation, double* hs, double* z0, double* ustar,
                           double* c_salt, double* ustar_th, double* u_z, double* csubl) {
    if (saltation)
        for (int64_t i = 0; i < c->T; ++i) saltation[i] = c->saltation[i];
    copy_out(hs, c->hs);
    copy_out(z0, c->z0);
    copy_out(ustar, c->ustar);
    copy_out(c_salt, c->c_salt);
    copy_out(ustar_th, c->ustar_th);
    copy_out(u_z, c->u_z);
    copy_out(csubl, c->csubl);
    return 0;
}
int oracle_get_state(const oracle_ctx* c, double* sum_drift, double* sum_subl, double* drift_mass,
                     double* more_than_avail) {
    copy_out(sum_drift, c->sum_drift);
    copy_out(sum_subl, c->sum_subl);
    copy_out(drift_mass, c->drift_mass);
    copy_out(more_than_avail, c->more_than_avail);
    return 0;
}
int oracle_set_state(oracle_ctx* c, const double* sum_drift, const double* sum_subl, const double* drift_mass,
                     const double* more_than_avail) {
    const int64_t T = c->T;
    if (sum_drift) c->sum_drift.assign(sum_drift, sum_drift + T);
    if (sum_subl) c->sum_subl.assign(sum_subl, sum_subl + T);
    if (drift_mass) c->drift_mass.assign(drift_mass, drift_mass + T);
    if (more_than_avail) c->more_than_avail.assign(more_than_avail, more_than_avail + T);
    return 0;
}

// FP64 MLP 14 -> 128 -> 128 -> 128 -> 1 with ReLU, loss 0.5*mean((y-t)^2).
double oracle_mlp_loss_grad(int64_t n, const float* x, const float* target, const float* w0, const float* b0,
                            const float* w1, const float* b1, const float* w2, const float* b2, const float* w3,
                            const float* b3, double* gw0, double* gb0, double* gw1, double* gb1, double* gw2,
                            double* gb2, double* gw3, double* gb3, double* y_out) {
    const int I = 14, H = 128;
    const float* W[4] = {w0, w1, w2, w3};
    const float* B[4] = {b0, b1, b2, b3};
    double* GW[4] = {gw0, gw1, gw2, gw3};
    double* GB[4] = {gb0, gb1, gb2, gb3};
    const int din[4] = {I, H, H, H}, dout[4] = {H, H, H, 1};
    for (int l = 0; l < 4; ++l) {
        if (GW[l]) std::fill(GW[l], GW[l] + din[l] * dout[l], 0.0);
        if (GB[l]) std::fill(GB[l], GB[l] + dout[l], 0.0);
    }
    double loss = 0;
    std::vector<double> a[5], g[5];
    for (int64_t r = 0; r < n; ++r) {
        a[0].assign(x + r * I, x + r * I + I);
        for (int l = 0; l < 4; ++l) {
            a[l + 1].assign(dout[l], 0.0);
            for (int o = 0; o < dout[l]; ++o) {
                double s = B[l][o];
                for (int k = 0; k < din[l]; ++k) s += (double)W[l][o * din[l] + k] * a[l][k];
                a[l + 1][o] = (l < 3 && s < 0) ? 0 : s;
            }
        }
        double y = a[4][0];
        if (y_out) y_out[r] = y;
        double d = y - (double)target[r];
        loss += 0.5 * d * d;
        g[4].assign(1, d / (double)n);
        for (int l = 3; l >= 0; --l) {
            g[l].assign(din[l], 0.0);
            for (int o = 0; o < dout[l]; ++o) {
                double go = g[l + 1][o];
                if (l < 3 && a[l + 1][o] <= 0) go = 0;
                if (GB[l]) GB[l][o] += go;
                for (int k = 0; k < din[l]; ++k) {
                    if (GW[l]) GW[l][o * din[l] + k] += go * a[l][k];
                    g[l][k] += go * (double)W[l][o * din[l] + k];
                }
            }
        }
    }
    return loss / (double)n;
}

}  // extern "C"
