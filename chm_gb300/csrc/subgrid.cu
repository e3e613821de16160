// subgrid.cu -- subgrid topography branches of the PBSM3D step
// (use_subgrid_topo and use_subgrid_topo_V2, PBSM3D.cpp:480-645, 866-870).
//
// One thread per face computes the holding capacity min_sd_trans_avg that
// gates saltation and the contributing fraction frac_contrib that scales
// c_salt, from the face's subgrid topographic-position-index statistics,
// before the saltation pass reads them.  Per-face scalar work, off the
// default path: the kernel runs only when a branch is on.
//
//  * use_subgrid_topo: TPI < 0 over a fraction of the face, gamma-distributed;
//    closed forms in the regularised incomplete gamma functions, evaluated by
//    the series (x < a + 1) or the continued fraction (modified Lentz) of
//    Press et al., Numerical Recipes, section 6.2.
//  * use_subgrid_topo_V2: Gaussian TPI and a filling function; the reference
//    integrates with gsl_integration_qags to relative 1e-7.  Here:
//    - the normalisation integral depends only on the face's static TPI
//      statistics (the depth-dependent filling coefficients of
//      PBSM3D.cpp:509-537 are declared in inner scopes and never reach it), so
//      it is evaluated once per face at create;
//    - the gully integral up to the filled-gully threshold by composite
//      16-point Gauss-Legendre over the Gaussian's +-12 sigma support, split at
//      the filling function's kink x = -0.25, panels at most 2 sigma and 2
//      wide (accurate to ~1e-15; the QAGS result lies within its tolerance);
//    - the linear-times-Gaussian integral in closed form;
//    - the threshold by the bracketing walk and refinement of roots.cuh.
#include <math.h>

#include "pbsm3d_internal.cuh"
#include "roots.cuh"

namespace pbsm {
namespace {

constexpr int kGL = 16;
__constant__ double c_gl_x[kGL];  // Gauss-Legendre nodes on [-1, 1]
__constant__ double c_gl_w[kGL];  // and weights

// std::min / std::max with their NaN behaviour: (b < a) ? b : a, (a < b) ? b : a
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ bool is_nan_chm(double v) { return fabs(v - -9999.0) < 1e-5 || isnan(v); }

// gsl_ran_gaussian_pdf(x, sigma), gsl_cdf_gaussian_Q(x, sigma)
__device__ __forceinline__ double gauss_pdf(double x, double sigma) {
    const double u = x / sigma;
    return exp(-0.5 * u * u) / (2.5066282746310002 * sigma);
}
__device__ __forceinline__ double gauss_Q(double x, double sigma) { return 0.5 * erfc(x / (sigma * M_SQRT2)); }

// The filling function's coefficients (PBSM3D.cpp:505-509)
constexpr double kA1 = 1.5, kB1 = 0.3, kA2 = 0.6, kB2 = 0.55, kFacFill = 0.8;

// my_fill_topo (PBSM3D.cpp:38-52): normalised snow depth of TPI x times the
// Gaussian TPI density
__device__ __forceinline__ double fill(double x, double m, double s) {
    const double x2 = x + 0.25;
    const double f = x2 <= 0 ? 1. - kA1 * tanh(kB1 * x2) : 1. - kA2 * tanh(kB2 * x2);
    return f * gauss_pdf(x - m, s);
}

// integral of fill over [lo, hi], composite Gauss-Legendre on the support
__device__ double fill_integral(double lo, double hi, double m, double s) {
    lo = fmax(lo, m - 12.0 * s);
    hi = fmin(hi, m + 12.0 * s);
    if (!(hi > lo)) return 0.0;
    const double hmax = fmin(2.0 * s, 2.0);
    double total = 0.0;
    // two pieces, split at the kink
    const double cuts[3] = {lo, fmin(fmax(-0.25, lo), hi), hi};
    for (int p = 0; p < 2; ++p) {
        const double a = cuts[p], b = cuts[p + 1];
        if (!(b > a)) continue;
        const int n = (int)ceil((b - a) / hmax);
        const double w = (b - a) / n;
        for (int k = 0; k < n; ++k) {
            const double c = a + (k + 0.5) * w, h = 0.5 * w;
            double acc = 0.0;
#pragma unroll 4
            for (int q = 0; q < kGL; ++q) acc += c_gl_w[q] * fill(c + h * c_gl_x[q], m, s);
            total += acc * h;
        }
    }
    return total;
}

// Regularised incomplete gamma P(a, x), Q(a, x) (Numerical Recipes 6.2)
__device__ void incomplete_gamma(double a, double x, double& P, double& Q) {
    if (!(x > 0)) {
        P = 0;
        Q = 1;
        return;
    }
    const double lpre = -x + a * log(x) - lgamma(a);
    if (x < a + 1) {
        double ap = a, del = 1.0 / a, sum = del;
        for (int n = 0; n < 100000; ++n) {
            ap += 1;
            del *= x / ap;
            sum += del;
            if (fabs(del) < fabs(sum) * 1e-17) break;
        }
        P = sum * exp(lpre);
        Q = 1.0 - P;
    } else {
        const double tiny = 1e-300;
        double b = x + 1 - a, cc = 1 / tiny, d = 1 / b, h = d;
        for (int i = 1; i < 100000; ++i) {
            const double an = -i * (i - a);
            b += 2;
            d = an * d + b;
            if (fabs(d) < tiny) d = tiny;
            cc = b + an / cc;
            if (fabs(cc) < tiny) cc = tiny;
            d = 1 / d;
            const double del = d * cc;
            h *= del;
            if (fabs(del - 1) < 1e-17) break;
        }
        Q = exp(lpre) * h;
        P = 1.0 - Q;
    }
}
// gsl_ran_gamma_pdf (x, shape a, scale b)
__device__ double gamma_pdf(double x, double a, double b) {
    if (x < 0) return 0;
    if (x == 0) return a == 1 ? 1 / b : (a > 1 ? 0 : INFINITY);
    return exp((a - 1) * log(x / b) - x / b - lgamma(a)) / b;
}

__global__ void k_subgrid_init(Params P, Subgrid g) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.T; i += (int64_t)gridDim.x * blockDim.x) {
        const double sd_raw = g.tpi[P.Tp + i];
        if (is_nan_chm(sd_raw)) {
            g.I0[i] = 0.0;
            continue;
        }
        const double m = smax(-5.0, smin(5.0, g.tpi[i]));
        const double s = smin(5.0, smax(0.1, sd_raw));
        g.I0[i] = fill_integral(-50, 50, m, s);
    }
}

__global__ void k_subgrid(Params P, Subgrid g, Forcing F, FaceState S) {
    const int64_t Tp = P.Tp;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.T; i += (int64_t)gridDim.x * blockDim.x) {
        double snow_depth = F.sd[i];
        snow_depth = is_nan_chm(snow_depth) ? 0 : snow_depth;
        const double min_sd_trans = P.min_sd_trans;
        double frac_contrib = 1.0, min_sd_trans_avg = min_sd_trans;
        double* out = S.sub;
        if (P.subgrid & 2) {  // use_subgrid_topo_V2, PBSM3D.cpp:486-597
            double tpi_lim = -min_sd_trans;
            if (!is_nan_chm(g.tpi[Tp + i])) {
                const double m = smax(-5.0, smin(5.0, g.tpi[i]));
                const double s = smin(5.0, smax(0.1, g.tpi[Tp + i]));
                if (snow_depth > min_sd_trans) {
                    const double result = g.I0[i];
                    out[SG_TESTINT * Tp + i] = result;
                    const double k = snow_depth / result;
                    // filled-gully threshold: (1 - a1 tanh(b1 (x + .25))) hs / I0 + fac x = 0
                    auto fr = [&](double x) { return (1 - kA1 * tanh(kB1 * (x + 0.25))) * k + kFacFill * x; };
                    auto dfr = [&](double x) {
                        const double th = tanh(kB1 * (x + 0.25));
                        return -kA1 * kB1 * (1 - th * th) * k + kFacFill;
                    };
                    double r;
                    if (bracket_solve(fr, dfr, -1.0, true, r)) tpi_lim = r;
                    // snow held in the unfilled gullies (my_fill_topo2, :566-572)
                    const double h1 = k * fill_integral(-50, tpi_lim, m, s);
                    // and in the filled ones, -fac x over [tpi_lim, -min_sd/fac] (my_fill_topo3,
                    // :575-582): with z = (x - m)/s, -fac (m (Phi(zu) - Phi(zl)) + s (phi(zl) - phi(zu)))
                    const double zl = (tpi_lim - m) / s, zu = (-min_sd_trans / kFacFill - m) / s;
                    const double dPhi = 0.5 * (erfc(zl * M_SQRT1_2) - erfc(zu * M_SQRT1_2));
                    const double dphi = (exp(-0.5 * zl * zl) - exp(-0.5 * zu * zu)) * 0.3989422804014327;
                    const double h2 = -kFacFill * (m * dPhi + s * dphi);
                    // and on positive TPI (:585)
                    const double h3 = min_sd_trans * gauss_Q(-min_sd_trans / kFacFill - m, s);
                    min_sd_trans_avg = smin(h1 + h2 + h3, snow_depth);
                }
                frac_contrib = gauss_Q(tpi_lim - m, s);
            }
            out[SG_TPILIM * Tp + i] = tpi_lim;
        }
        if (P.subgrid & 1) {  // use_subgrid_topo, PBSM3D.cpp:604-645
            double nosnw = 1.0;
            const double frac_neg = g.tpi[2 * Tp + i];
            if (!is_nan_chm(frac_neg) && frac_neg > 0.) {
                const double mn = smax(-10.0, smin(-0.05, g.tpi[3 * Tp + i]));
                const double sn = smin(5.0, smax(0.1, g.tpi[4 * Tp + i]));
                const double shape = (mn * mn) / (sn * sn);
                const double scale = -(sn * sn) / mn;
                double Pd, Qd;
                incomplete_gamma(shape, snow_depth / scale, Pd, Qd);
                frac_contrib = (1. - frac_neg) + frac_neg * Pd;
                nosnw = 1. - frac_neg;
                if (snow_depth > min_sd_trans) {
                    double Pm, Qm;
                    incomplete_gamma(shape, min_sd_trans / scale, Pm, Qm);
                    const double hint = shape * scale - scale * (snow_depth * gamma_pdf(snow_depth, shape, scale) -
                                                                 min_sd_trans * gamma_pdf(min_sd_trans, shape, scale) +
                                                                 shape * Pm + shape * Qd);
                    min_sd_trans_avg = (1. - frac_neg) * min_sd_trans + frac_neg * (min_sd_trans * Pm + hint + snow_depth * Qd);
                }
            }
            out[SG_NOSNW * Tp + i] = nosnw;
        }
        out[SG_HOLD * Tp + i] = min_sd_trans_avg;
        out[SG_FRAC * Tp + i] = frac_contrib;
    }
}

}  // namespace

void launch_subgrid(Ctx& c, cudaStream_t s) {
    k_subgrid<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.sg, c.Fo, c.S);
}

// Gauss-Legendre nodes and weights (Newton on P_n from Tricomi's initial
// guesses), the V2 normalisation integrals, and the outputs' initial -9999.
int subgrid_init(Ctx& c, cudaStream_t s) {
    double x[kGL], w[kGL];
    for (int i = 0; i < kGL; ++i) {
        long double z = cosl(3.14159265358979323846264338327950288L * (i + 0.75L) / (kGL + 0.5L)), pp = 0;
        for (int it = 0; it < 100; ++it) {
            long double p1 = 1, p2 = 0;
            for (int j = 0; j < kGL; ++j) {
                const long double p3 = p2;
                p2 = p1;
                p1 = ((2 * j + 1) * z * p2 - j * p3) / (j + 1);
            }
            pp = kGL * (z * p1 - p2) / (z * z - 1);
            const long double z1 = z;
            z = z1 - p1 / pp;
            if (fabsl(z - z1) < 1e-19L) break;
        }
        x[i] = (double)z;
        w[i] = (double)(2 / ((1 - z * z) * pp * pp));
    }
    if (cudaMemcpyToSymbolAsync(c_gl_x, x, sizeof(x), 0, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyToSymbolAsync(c_gl_w, w, sizeof(w), 0, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return 1;
    if (c.P.subgrid & 2) k_subgrid_init<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.sg);
    return cudaGetLastError() != cudaSuccess;
}

}  // namespace pbsm
