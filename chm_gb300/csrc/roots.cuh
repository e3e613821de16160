// roots.cuh -- the scalar root finder of the per-face PBSM3D branches.
//
// The reference calls Boost's bracket_and_solve_root(f, guess, factor 1,
// rising, |a - b| < 1e-8, 500 evaluations) for the coupled friction velocity
// (PBSM3D.cpp:708) and the filled-gully TPI threshold (PBSM3D.cpp:557) and
// takes the midpoint of the bracket it returns.  Here the bracket comes from
// the same walk: away from zero (b *= factor) when f(guess) has the sign that
// puts the root there, else towards zero (a /= factor), by a factor that is 1
// for the first 31 moves, doubles at the 32nd and then after 16, 8, 4, 2 more
// moves and at every move after that; a walk towards zero that passes below
// DBL_MIN brackets the root 0.  The first 31 moves leave the bracket where it
// is, so the walk starts at the 32nd (guesses are +-1, far from the DBL_MIN
// test).  The root of the bracket is then refined to full precision by Newton
// steps kept inside it, bisecting when a step leaves it (the reference's
// TOMS 748 stops at a bracket narrower than 1e-8; its midpoint lies within
// 5e-9 of this root).  At most 500 evaluations in the walk and 100 refinement
// steps.  Returns false when no bracket is found.
#pragma once

#include <math.h>

namespace pbsm {

__device__ __forceinline__ int sgn(double v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }

template <class F, class DF>
__device__ bool bracket_solve(F f, DF df, double guess, bool rising, double& root) {
    double a = guess, b = guess;
    double fa = f(a), fb = fa;
    const bool away = (fa < 0) == (guess < 0 ? !rising : rising);
    double factor = 2.0;
    int every = 16;
    for (int s = 32; sgn(fa) == sgn(fb); ++s) {
        if (!away && fabs(a) < 2.2250738585072014e-308) {
            root = a / 2.0;
            return true;
        }
        if (s >= 500) return false;
        if (s > 32 && s % every == 0) {
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
    double lo = fmin(a, b), hi = fmax(a, b);
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
        const bool done = fabs(xn - x) <= 1e-15 * fabs(xn);
        x = xn;
        if (done) break;
    }
    root = x;
    return true;
}

}  // namespace pbsm
