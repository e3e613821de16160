// fp64_math.cuh -- FP64 exp / log / reciprocal with few FP64-pipe instructions.
//
// GB300 issues FP64 at 2 thread-instructions per cycle per SM, so the PBSM3D
// assembly (several transcendental functions per row) is bound by the FP64
// pipe.  These routines move range reduction, special-case screening and
// exponent reconstruction to the integer pipe and shorten the polynomials
// with shared-memory tables:
//
//  * exp: Tang's table-driven method (P. T. P. Tang, "Table-driven
//    implementation of the exponential function in IEEE floating-point
//    arithmetic", ACM TOMS 15(2), 1989) with 256 table points:
//    x = (256 n + j) ln2/256 + r, |r| <= ln2/512, exp(x) = 2^n 2^(j/256) e^r,
//    e^r - 1 by its degree-4 Taylor polynomial (truncation < 4e-17).
//  * log: Tang's table-driven logarithm (ACM TOMS 16(4), 1990) with 256
//    table points: x = 2^e m, m in [1, 2), c_j ~ 1/m for the top 8 mantissa
//    bits, r = m c_j - 1 (one FMA, |r| < 2^-8), log x = e ln2 - log c_j +
//    log1p(r), log1p by its degree-6 Taylor polynomial (truncation < 2e-17
//    absolute).  Accurate to a few 1e-16 absolute; callers use it where an
//    absolute error of that size is harmless (arguments of exp, or arguments
//    far from 1).
//  * rcp: the hardware reciprocal estimate (PTX rcp.approx.ftz.f64, about
//    23 correct bits) refined by two Newton-Raphson steps on f(y) = 1/y - x,
//    y <- y + y (1 - x y), each of which squares the relative error.
//  * div: a * rcp(b), then one correction of the quotient by its residual,
//    q + (a - b q) rcp(b) (P. Markstein, "Computation of elementary
//    functions on the IBM RISC System/6000 processor", IBM J. Res. Dev.
//    34(1), 1990).
//
// Arguments outside the fast ranges (non-positive, subnormal, huge, NaN,
// Inf) take the CUDA library function, so special values behave as before.
// The tables live in shared memory: a kernel declares `__shared__ MathTables`
// and calls math_tables_load() before use.  math_tables_fill() computes them
// on the host in extended precision.
#pragma once

#include <math.h>
#include <stdint.h>

namespace pbsm {

struct MathTables {
    double exp2j[256];  // 2^(j/256)
    double logc[256];   // c_j = 1 / (1 + (j + 0.5)/256), rounded to double
    double logl[256];   // -log(c_j)
};

// Filled once by the host (math_tables_fill) into device memory, staged into
// shared memory by each block that uses the functions below.
__device__ __forceinline__ void math_tables_load(MathTables& t, const MathTables* __restrict__ src) {
    const double* s = reinterpret_cast<const double*>(src);
    double* d = reinterpret_cast<double*>(&t);
    for (int k = threadIdx.x; k < 3 * 256; k += blockDim.x) d[k] = s[k];
    __syncthreads();
}

// exp(x): fast path for |x| < 700, else the library exp (NaN, Inf, overflow).
__device__ __forceinline__ double exp_t(double x, const MathTables& t) {
    const unsigned long long ax = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
    if (ax >= 0x4085E00000000000ull) return exp(x);  // |x| >= 700 or NaN
    const double kInvL = 369.3299304675746;           // 256 / ln 2
    const double kShift = 6755399441055744.0;         // 1.5 * 2^52
    const double kL1 = 2.7076061740622863e-03;        // ln2/256, high part
    const double kL2 = 9.0587766165871080e-20;        // ln2/256 - kL1
    const double tt = fma(x, kInvL, kShift);
    const int k = __double2loint(tt);  // round(x * 256/ln2)
    const double kd = tt - kShift;
    double r = fma(kd, -kL1, x);
    r = fma(kd, -kL2, r);
    const double r2 = r * r;
    double q = fma(r, 1.0 / 24.0, 1.0 / 6.0);
    q = fma(r, q, 0.5);
    const double p = fma(r2, q, r);  // e^r - 1
    const double tj = t.exp2j[k & 255];
    const double y = fma(tj, p, tj);
    // y in [1, 2.01): add n = k >> 8 to its exponent field
    const long long bits = __double_as_longlong(y) + ((long long)(k >> 8) << 52);
    return __longlong_as_double(bits);
}

// log(x): fast path for positive normal finite x, else the library log.
__device__ __forceinline__ double log_t(double x, const MathTables& t) {
    const long long b = __double_as_longlong(x);
    if (b < 0x0010000000000000ll || b >= 0x7ff0000000000000ll) return log(x);
    const int e = (int)(b >> 52) - 1023;
    const int j = (int)((b >> 44) & 255);
    const double m = __longlong_as_double((b & 0x000fffffffffffffll) | 0x3ff0000000000000ll);
    const double r = fma(m, t.logc[j], -1.0);
    // log1p(r) = r - r^2/2 + r^3/3 - r^4/4 + r^5/5 - r^6/6
    double q = fma(r, -1.0 / 6.0, 1.0 / 5.0);
    q = fma(r, q, -0.25);
    q = fma(r, q, 1.0 / 3.0);
    q = fma(r, q, -0.5);
    const double r2 = r * r;
    // e as a double without a conversion instruction: bits of 2^52 + 2^51 + e
    const double ed = __longlong_as_double(0x4338000000000000ll + e) - 6755399441055744.0;
    const double kLn2Hi = 6.9314718055994529e-01;
    const double kLn2Lo = 2.3190468138462996e-17;
    const double hi = fma(ed, kLn2Hi, t.logl[j]);
    const double lo = fma(ed, kLn2Lo, fma(r2, q, r));
    return hi + lo;
}

// 1/x for finite non-zero normal x (|x| in [2^-1000, 2^1000]), else 1.0/x:
// the hardware estimate and two Newton-Raphson steps y <- y + y (1 - x y).
__device__ __forceinline__ double rcp_t(double x) {
    const unsigned long long ax = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
    if (ax < 0x0170000000000000ull || ax >= 0x7e70000000000000ull) return 1.0 / x;
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    return y;
}

// a / b: q = a rcp(b) corrected once by its residual (Markstein 1990), within 1 ulp.
__device__ __forceinline__ double div_t(double a, double b) {
    const double y = rcp_t(b);
    const double q = a * y;
    return fma(fma(-b, q, a), y, q);
}

// (float) x, round to nearest even, on the integer pipe (an FP64->FP32
// conversion instruction issues on the FP64 pipe).  Normal results only;
// zero, subnormal, overflow, Inf and NaN take the conversion instruction.
__device__ __forceinline__ float f32_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32);
    const int e = (int)((hi >> 20) & 0x7ff) - 1023 + 127;
    if (e <= 0 || e >= 254) return (float)x;
    const unsigned long long m = b & 0x000fffffffffffffull;
    unsigned r = ((unsigned)e << 23) | (unsigned)(m >> 29);
    const unsigned long long rem = m & 0x1fffffffull;  // the 29 dropped bits
    r += (rem > 0x10000000ull || (rem == 0x10000000ull && (r & 1u))) ? 1u : 0u;
    return __uint_as_float(r | (hi & 0x80000000u));
}

// x^y = exp(y log x) for x > 0
__device__ __forceinline__ double pow_t(double x, double y, const MathTables& t) {
    return exp_t(y * log_t(x, t), t);
}

// Host: the three tables, each entry rounded once from extended precision.
void math_tables_fill(MathTables& h);

}  // namespace pbsm
