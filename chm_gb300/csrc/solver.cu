// solver.cu -- Krylov solves of the two PBSM3D systems on the GPU.
//
// Suspension (replaces the Belos GMRES(30) + Ifpack2 ILUT solve of
// LinearAlgebra.cpp:228-252): right-preconditioned BiCGStab.  The matrix is
// split A = B + N, B = the tridiagonal column of each face (diagonal, below,
// above), N = the three lateral couplings.  With M = B the preconditioned
// operator is A B^{-1} = I + N B^{-1}, so one operator application is
//   z = B^{-1} u   (Thomas sweep down and up each column, fused into the
//                   vector update that produces u)
//   y = u + N z    (gather of z at the three face neighbours, fused with the
//                   dot products that follow)
// and the vertical bands are never re-read inside the iteration.  The true
// residual b - A x is recomputed from all six FP64 bands at the end.
//
// MIXED: the same BiCGStab in FP32 (FP32 lateral bands and column factors)
// solves A d = r to a modest tolerance inside FP64 iterative refinement;
// residuals, x and all norms stay FP64.
//
// Deposition (SPD: diag(area) + eps * weighted graph Laplacian):
// Jacobi-preconditioned CG in FP64.
//
// Every reduction is deterministic: fixed grid, per-block partials, the
// last block sums them in block order.  Scalars live in device memory, so
// iterations are launched without host synchronisation; the host polls the
// iteration count every few iterations.
#include <math.h>

#include <algorithm>

#include "pbsm3d_internal.cuh"

namespace pbsm {
namespace {

template <typename V>
struct Op {
    const V* lat;    // [3][R]
    const V* l;      // [R] forward multipliers
    const V* ib;     // [R] inverse pivots
    const V* up;     // [R] above band
    const int32_t* nbr;  // [3][Tp]
    int64_t Tp, R;
    int L;
};

enum { DONE_NO = 0, DONE_CONVERGED = 1, DONE_BREAKDOWN = 2, DONE_MAXIT = 3 };

// z = B^{-1} u for one column, u already in smem column g[z*bd + tid].
template <typename V>
__device__ __forceinline__ void column_solve(const Op<V>& op, int64_t i, V* g, V* zout) {
    const int bd = blockDim.x, tid = threadIdx.x;
    V prev = 0;
    for (int z = 0; z < op.L; ++z) {
        const int64_t r = (int64_t)z * op.Tp + i;
        V gz = g[z * bd + tid] - op.l[r] * prev;
        g[z * bd + tid] = gz;
        prev = gz;
    }
    V y = 0;
    for (int z = op.L - 1; z >= 0; --z) {
        const int64_t r = (int64_t)z * op.Tp + i;
        y = (g[z * bd + tid] - op.up[r] * y) * op.ib[r];
        zout[r] = y;
    }
}

// p = r + beta (p - omega v); zp = B^{-1} p
template <typename V>
__global__ void __launch_bounds__(kBlock) k_bicg_p(Op<V> op, const V* __restrict__ r, V* __restrict__ p,
                                                   const V* __restrict__ v, V* __restrict__ zp, const Scalars* sc) {
    if (sc->done) return;
    extern __shared__ unsigned char smem_raw[];
    V* g = reinterpret_cast<V*>(smem_raw);
    const V beta = (V)sc->beta, omega = (V)sc->omega;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < op.Tp; i += (int64_t)gridDim.x * blockDim.x) {
        for (int z = 0; z < op.L; ++z) {
            const int64_t k = (int64_t)z * op.Tp + i;
            const V pk = r[k] + beta * (p[k] - omega * v[k]);
            p[k] = pk;
            g[z * blockDim.x + threadIdx.x] = pk;
        }
        column_solve(op, i, g, zp);
    }
}

// s = r - alpha v; zs = B^{-1} s
template <typename V>
__global__ void __launch_bounds__(kBlock) k_bicg_s(Op<V> op, const V* __restrict__ r, const V* __restrict__ v,
                                                   V* __restrict__ s, V* __restrict__ zs, const Scalars* sc) {
    if (sc->done) return;
    extern __shared__ unsigned char smem_raw[];
    V* g = reinterpret_cast<V*>(smem_raw);
    const V alpha = (V)sc->alpha;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < op.Tp; i += (int64_t)gridDim.x * blockDim.x) {
        for (int z = 0; z < op.L; ++z) {
            const int64_t k = (int64_t)z * op.Tp + i;
            const V sk = r[k] - alpha * v[k];
            s[k] = sk;
            g[z * blockDim.x + threadIdx.x] = sk;
        }
        column_solve(op, i, g, zs);
    }
}

// y = u + N z, with dot products (a, y) [and (y, y)]
template <typename V, int NT>
__device__ __forceinline__ void lateral_apply(const Op<V>& op, const V* __restrict__ u, const V* __restrict__ zz,
                                              V* __restrict__ y, const V* __restrict__ a, V (&acc)[2]) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < op.Tp; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t n0 = op.nbr[i], n1 = op.nbr[op.Tp + i], n2 = op.nbr[2 * op.Tp + i];
        for (int z = 0; z < op.L; ++z) {
            const int64_t base = (int64_t)z * op.Tp;
            const int64_t k = base + i;
            V yk = u[k];
            if (n0 >= 0) yk += op.lat[k] * zz[base + n0];
            if (n1 >= 0) yk += op.lat[op.R + k] * zz[base + n1];
            if (n2 >= 0) yk += op.lat[2 * op.R + k] * zz[base + n2];
            y[k] = yk;
            acc[0] += a[k] * yk;
            if (NT > 1) acc[1] += yk * yk;
        }
    }
}

// v = p + N zp; rv = (rhat, v); alpha = rho / rv
template <typename V>
__global__ void __launch_bounds__(kBlock) k_bicg_v(Op<V> op, const V* __restrict__ p, const V* __restrict__ zp,
                                                   V* __restrict__ v, const V* __restrict__ rh, Scalars* sc,
                                                   double* partials) {
    if (sc->done) return;
    V acc[2] = {0, 0};
    lateral_apply<V, 1>(op, p, zp, v, rh, acc);
    double d[1] = {(double)acc[0]}, tot[1];
    if (block_partials_last<1>(d, partials, &sc->counter[0], tot) && threadIdx.x == 0) {
        const double rv = tot[0];
        sc->rv = rv;
        if (rv == 0.0 || !isfinite(rv)) {
            sc->done = DONE_BREAKDOWN;
        } else {
            sc->alpha = sc->rho / rv;
        }
    }
}

// t = s + N zs; ts = (t, s), tt = (t, t); omega = ts / tt
template <typename V>
__global__ void __launch_bounds__(kBlock) k_bicg_t(Op<V> op, const V* __restrict__ s, const V* __restrict__ zs,
                                                   V* __restrict__ t, Scalars* sc, double* partials) {
    if (sc->done) return;
    V acc[2] = {0, 0};
    lateral_apply<V, 2>(op, s, zs, t, s, acc);
    double d[2] = {(double)acc[0], (double)acc[1]}, tot[2];
    if (block_partials_last<2>(d, partials, &sc->counter[0], tot) && threadIdx.x == 0) {
        sc->ts = tot[0];
        sc->tt = tot[1];
        sc->omega = tot[1] > 0 ? tot[0] / tot[1] : 0.0;
    }
}

// x += alpha zp + omega zs; r = s - omega t; rho' = (rhat, r), (r, r)
template <typename V, typename X>
__global__ void __launch_bounds__(kBlock) k_bicg_x(int64_t Tp, int L, X* __restrict__ x, const V* __restrict__ zp,
                                                   const V* __restrict__ zs, const V* __restrict__ s,
                                                   const V* __restrict__ t, V* __restrict__ r,
                                                   const V* __restrict__ rh, Scalars* sc, double* partials) {
    if (sc->done) return;
    const X alpha = (X)sc->alpha, omega = (X)sc->omega;
    const V om = (V)sc->omega;
    V acc[2] = {0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Tp; i += (int64_t)gridDim.x * blockDim.x) {
        for (int z = 0; z < L; ++z) {
            const int64_t k = (int64_t)z * Tp + i;
            x[k] = x[k] + alpha * (X)zp[k] + omega * (X)zs[k];
            const V rk = s[k] - om * t[k];
            r[k] = rk;
            acc[0] += rh[k] * rk;
            acc[1] += rk * rk;
        }
    }
    double d[2] = {(double)acc[0], (double)acc[1]}, tot[2];
    if (block_partials_last<2>(d, partials, &sc->counter[0], tot) && threadIdx.x == 0) {
        const double rho_new = tot[0];
        sc->rnorm2 = tot[1];
        sc->iter += 1;
        if (tot[1] <= sc->target2) {
            sc->done = DONE_CONVERGED;
        } else if (sc->omega == 0.0 || rho_new == 0.0 || !isfinite(rho_new) || !isfinite(tot[1])) {
            sc->done = DONE_BREAKDOWN;
        } else if (sc->iter >= sc->maxit) {
            sc->done = DONE_MAXIT;
        } else {
            sc->beta = (rho_new / sc->rho) * (sc->alpha / sc->omega);
        }
        sc->rho = rho_new;
    }
}

// r = b - A x with all six FP64 bands; optionally r32 = (float) r.
// Also (r, r) and (b, b).  Resets the BiCGStab state: rhat = r, p = v = 0.
template <typename V>
__global__ void __launch_bounds__(kBlock) k_residual(Params P, const double* __restrict__ band,
                                                     const int32_t* __restrict__ nbr, const double* __restrict__ x,
                                                     const double* __restrict__ b, double* __restrict__ r,
                                                     V* __restrict__ rv, V* __restrict__ rhv, V* __restrict__ pv,
                                                     V* __restrict__ vv, Scalars* sc, double* partials, double tol,
                                                     int maxit) {
    const int64_t Tp = P.Tp, R = P.R;
    double acc[3] = {0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Tp; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t nb[3] = {nbr[i], nbr[Tp + i], nbr[2 * Tp + i]};
        for (int z = 0; z < P.L; ++z) {
            const int64_t base = (int64_t)z * Tp;
            const int64_t k = base + i;
            double ax = band[k] * x[k];
#pragma unroll
            for (int j = 0; j < 3; ++j)
                if (nb[j] >= 0) ax += band[(j + 1) * R + k] * x[base + nb[j]];
            if (z > 0) ax += band[4 * R + k] * x[k - Tp];
            if (z < P.L - 1) ax += band[5 * R + k] * x[k + Tp];
            const double rk = b[k] - ax;
            r[k] = rk;
            if (rv) {
                rv[k] = (V)rk;
                rhv[k] = (V)rk;
                pv[k] = 0;
                vv[k] = 0;
            }
            acc[0] += rk * rk;
            acc[1] += b[k] * b[k];
            acc[2] += b[k] * rk;
        }
    }
    double tot[3];
    if (block_partials_last<3>(acc, partials, &sc->counter[0], tot) && threadIdx.x == 0) {
        sc->rnorm2 = tot[0];
        sc->bnorm2 = tot[1];
        sc->red0 = tot[2];  // (b, r): lets the host scale a warm start
        sc->rho = tot[0];
        sc->alpha = 1.0;
        sc->omega = 1.0;
        sc->beta = 0.0;
        sc->target2 = tol * tol * tot[0];
        sc->iter = 0;
        sc->maxit = maxit;
        sc->done = tot[0] == 0.0 ? DONE_CONVERGED : DONE_NO;
    }
}

// Warm start x0 -> gamma x0 (gamma = 0 drops it): r = (1-gamma) b + gamma r0,
// and the Krylov state restarts from the new residual.
template <typename V>
__global__ void __launch_bounds__(kBlock) k_warm_scale(int64_t n, double gamma, double* __restrict__ x,
                                                       double* __restrict__ r, const double* __restrict__ b,
                                                       V* __restrict__ rv, V* __restrict__ rhv, Scalars* sc,
                                                       double* partials) {
    double acc[1] = {0};
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        x[k] *= gamma;
        const double rk = (1.0 - gamma) * b[k] + gamma * r[k];
        r[k] = rk;
        rv[k] = (V)rk;
        rhv[k] = (V)rk;
        acc[0] += rk * rk;
    }
    double tot[1];
    if (block_partials_last<1>(acc, partials, &sc->counter[0], tot) && threadIdx.x == 0) {
        sc->rnorm2 = tot[0];
        sc->rho = tot[0];
        sc->target2 = 0.0;  // set by the host
        sc->done = tot[0] == 0.0 ? DONE_CONVERGED : DONE_NO;
    }
}

// One block-Jacobi sweep on a guess: xo = B^{-1} (b - N xi) with B the
// column tridiagonals (FP64 Thomas factors) and N the lateral couplings.
__global__ void __launch_bounds__(kBlock) k_jacobi_sweep(Op<double> op, const double* __restrict__ b,
                                                         const double* __restrict__ xi, double* __restrict__ xo) {
    extern __shared__ unsigned char smem_raw[];
    double* g = reinterpret_cast<double*>(smem_raw);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < op.Tp; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t n0 = op.nbr[i], n1 = op.nbr[op.Tp + i], n2 = op.nbr[2 * op.Tp + i];
        for (int z = 0; z < op.L; ++z) {
            const int64_t base = (int64_t)z * op.Tp;
            const int64_t k = base + i;
            double u = b[k];
            if (n0 >= 0) u -= op.lat[k] * xi[base + n0];
            if (n1 >= 0) u -= op.lat[op.R + k] * xi[base + n1];
            if (n2 >= 0) u -= op.lat[2 * op.R + k] * xi[base + n2];
            g[z * blockDim.x + threadIdx.x] = u;
        }
        column_solve(op, i, g, xo);
    }
}

// x += (double) d
__global__ void __launch_bounds__(kBlock) k_add_correction(int64_t n, double* __restrict__ x,
                                                           const float* __restrict__ d) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        x[k] += (double)d[k];
}
template <typename V>
__global__ void k_zero(int64_t n, V* __restrict__ a) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        a[k] = 0;
}

// ---------------------------------------------------------------- deposition CG
// init: r = b, z = D^{-1} b, p = z, q = A z; (r,z), (p,q), (b,b)
__global__ void __launch_bounds__(kBlock) k_cg_init(Params P, Dep D, const int32_t* __restrict__ nbr, double* r,
                                                    double* zz, double* p, double* q, Scalars* sc, double* partials,
                                                    double tol, int maxit) {
    const int64_t Tp = P.Tp;
    double acc[3] = {0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Tp; i += (int64_t)gridDim.x * blockDim.x) {
        const double bi = D.rhs[i];
        const double zi = D.dinv[i] * bi;
        double qi = D.diag[i] * zi;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int32_t nb = nbr[j * Tp + i];
            if (nb >= 0) qi += D.off[j * Tp + i] * (D.dinv[nb] * D.rhs[nb]);
        }
        r[i] = bi;
        zz[i] = zi;
        p[i] = zi;
        q[i] = qi;
        D.x[i] = 0.0;
        acc[0] += bi * zi;
        acc[1] += zi * qi;
        acc[2] += bi * bi;
    }
    double tot[3];
    if (block_partials_last<3>(acc, partials, &sc->counter[0], tot) && threadIdx.x == 0) {
        sc->rho = tot[0];
        sc->bnorm2 = tot[2];
        sc->rnorm2 = tot[2];
        sc->target2 = tol * tol * tot[2];
        sc->iter = 0;
        sc->maxit = maxit;
        if (tot[2] == 0.0) {
            sc->done = DONE_CONVERGED;
        } else if (!(tot[1] > 0.0)) {
            sc->done = DONE_BREAKDOWN;
        } else {
            sc->done = DONE_NO;
            sc->alpha = tot[0] / tot[1];
        }
    }
}

// x += alpha p; r -= alpha q; z = D^{-1} r; (r,z), (r,r)
__global__ void __launch_bounds__(kBlock) k_cg_x(Params P, Dep D, double* r, double* zz, const double* p,
                                                 const double* q, Scalars* sc, double* partials) {
    if (sc->done) return;
    const double alpha = sc->alpha;
    double acc[2] = {0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.Tp; i += (int64_t)gridDim.x * blockDim.x) {
        D.x[i] += alpha * p[i];
        const double ri = r[i] - alpha * q[i];
        r[i] = ri;
        const double zi = D.dinv[i] * ri;
        zz[i] = zi;
        acc[0] += ri * zi;
        acc[1] += ri * ri;
    }
    double tot[2];
    if (block_partials_last<2>(acc, partials, &sc->counter[0], tot) && threadIdx.x == 0) {
        sc->iter += 1;
        sc->rnorm2 = tot[1];
        sc->beta = tot[0] / sc->rho;
        sc->rho = tot[0];
        if (tot[1] <= sc->target2) sc->done = DONE_CONVERGED;
        else if (!isfinite(tot[1])) sc->done = DONE_BREAKDOWN;
        else if (sc->iter >= sc->maxit) sc->done = DONE_MAXIT;
    }
}

// p = z + beta p; q = A z + beta q; (p,q) -> alpha = rho / (p,q)
__global__ void __launch_bounds__(kBlock) k_cg_p(Params P, Dep D, const int32_t* __restrict__ nbr, const double* zz,
                                                 double* p, double* q, Scalars* sc, double* partials) {
    if (sc->done) return;
    const double beta = sc->beta;
    const int64_t Tp = P.Tp;
    double acc[1] = {0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Tp; i += (int64_t)gridDim.x * blockDim.x) {
        double az = D.diag[i] * zz[i];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int32_t nb = nbr[j * Tp + i];
            if (nb >= 0) az += D.off[j * Tp + i] * zz[nb];
        }
        const double pi = zz[i] + beta * p[i];
        const double qi = az + beta * q[i];
        p[i] = pi;
        q[i] = qi;
        acc[0] += pi * qi;
    }
    double tot[1];
    if (block_partials_last<1>(acc, partials, &sc->counter[0], tot) && threadIdx.x == 0) {
        if (!(tot[0] > 0.0)) sc->done = DONE_BREAKDOWN;
        else sc->alpha = sc->rho / tot[0];
    }
}

// r = b - A x (deposition), (r, r)
__global__ void __launch_bounds__(kBlock) k_cg_resid(Params P, Dep D, const int32_t* __restrict__ nbr, double* r,
                                                     Scalars* sc, double* partials) {
    const int64_t Tp = P.Tp;
    double acc[1] = {0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Tp; i += (int64_t)gridDim.x * blockDim.x) {
        double ax = D.diag[i] * D.x[i];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int32_t nb = nbr[j * Tp + i];
            if (nb >= 0) ax += D.off[j * Tp + i] * D.x[nb];
        }
        const double ri = D.rhs[i] - ax;
        r[i] = ri;
        acc[0] += ri * ri;
    }
    double tot[1];
    if (block_partials_last<1>(acc, partials, &sc->counter[0], tot) && threadIdx.x == 0) sc->tmp = tot[0];
}

// ---------------------------------------------------------------- persistent deposition CG
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long global_timer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr unsigned long long kBarrierLimitNs = 2000000000ull;  // 2 s
constexpr int kCgBlock = 512;  // one block per SM keeps barrier arrivals few

// Grid-wide barrier of a cooperative launch.  The wait is bounded: after
// kBarrierLimitNs a block sets gb->err and every block leaves at its next
// barrier, so a fault in the co-residency assumption ends in an error, never
// in a hang.  Returns false when the kernel must exit.
__device__ bool grid_barrier(GridBar* gb) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = ld_acquire_u32(&gb->gen);
        __threadfence();
        const unsigned arrived = atomicAdd(&gb->count, 1u);
        ok = 1;
        if (arrived == gridDim.x - 1) {
            atomicExch(&gb->count, 0u);
            __threadfence();
            atomicAdd(&gb->gen, 1u);
        } else {
            const unsigned long long t0 = global_timer_ns();
            while (ld_acquire_u32(&gb->gen) == gen) {
                if (*(volatile int*)&gb->err) {
                    ok = 0;
                    break;
                }
                if (global_timer_ns() - t0 > kBarrierLimitNs) {
                    atomicExch(&gb->err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(20);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Totals of NT per-thread values over the whole grid, identical in every
// block (each block sums all partials in block order).  buf alternates
// between two partial buffers so a fast block never overwrites partials a
// slow block is still reading.
template <int NT>
__device__ bool grid_totals(double (&v)[NT], double* partials, GridBar* gb, double (&tot)[NT]) {
    __shared__ double bc[NT];
    block_sum<NT>(v);
    if (threadIdx.x == 0)
        for (int k = 0; k < NT; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
    if (!grid_barrier(gb)) return false;
    double t[NT];
    for (int k = 0; k < NT; ++k) {
        double acc = 0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) acc += __ldcg(&partials[k * gridDim.x + b]);
        t[k] = acc;
    }
    block_sum<NT>(t);
    if (threadIdx.x == 0)
        for (int k = 0; k < NT; ++k) bc[k] = t[k];
    __syncthreads();
    for (int k = 0; k < NT; ++k) tot[k] = bc[k];
    __syncthreads();
    return true;
}

// Jacobi-preconditioned CG on the deposition system in one cooperative
// launch; at 1M faces its vectors and matrix (~100 MB) stay in L2.
__global__ void __launch_bounds__(kCgBlock) k_cg_persistent(Params P, Dep D, const int32_t* __restrict__ nbr, double* r,
                                                          double* zz, double* p, double* q, double* partials,
                                                          GridBar* gb, Scalars* sc, double tol, int maxit) {
    const int64_t Tp = P.Tp;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double* bufs[2] = {partials, partials + 4 * gridDim.x};
    int nb_buf = 0;
    // init: r = b, z = D^-1 b, p = z, q = A z
    double a3[3] = {0, 0, 0}, t3[3];
    for (int64_t i = i0; i < Tp; i += stride) {
        const double bi = D.rhs[i];
        const double zi = D.dinv[i] * bi;
        double qi = D.diag[i] * zi;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int32_t nb = nbr[j * Tp + i];
            if (nb >= 0) qi += D.off[j * Tp + i] * (D.dinv[nb] * D.rhs[nb]);
        }
        r[i] = bi;
        zz[i] = zi;
        p[i] = zi;
        q[i] = qi;
        D.x[i] = 0.0;
        a3[0] += bi * zi;
        a3[1] += zi * qi;
        a3[2] += bi * bi;
    }
    if (!grid_totals<3>(a3, bufs[nb_buf], gb, t3)) return;
    nb_buf ^= 1;
    double rho = t3[0];
    const double bb = t3[2];
    const double target2 = tol * tol * bb;
    int status = 0, it = 0;
    double rr = bb;
    if (bb == 0.0) status = 1;
    else if (!(t3[1] > 0.0)) status = 2;
    double alpha = status ? 0.0 : rho / t3[1];
    while (status == 0) {
        double a2[2] = {0, 0}, t2[2];
        for (int64_t i = i0; i < Tp; i += stride) {
            D.x[i] += alpha * p[i];
            const double ri = r[i] - alpha * q[i];
            r[i] = ri;
            const double zi = D.dinv[i] * ri;
            zz[i] = zi;
            a2[0] += ri * zi;
            a2[1] += ri * ri;
        }
        if (!grid_totals<2>(a2, bufs[nb_buf], gb, t2)) return;
        nb_buf ^= 1;
        ++it;
        rr = t2[1];
        if (rr <= target2) {
            status = 1;
            break;
        }
        if (!isfinite(rr)) {
            status = 2;
            break;
        }
        if (it >= maxit) {
            status = 3;
            break;
        }
        const double beta = t2[0] / rho;
        rho = t2[0];
        double a1[1] = {0}, t1[1];
        for (int64_t i = i0; i < Tp; i += stride) {
            double az = D.diag[i] * zz[i];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int32_t nb = nbr[j * Tp + i];
                if (nb >= 0) az += D.off[j * Tp + i] * zz[nb];
            }
            const double pi = zz[i] + beta * p[i];
            const double qi = az + beta * q[i];
            p[i] = pi;
            q[i] = qi;
            a1[0] += pi * qi;
        }
        if (!grid_totals<1>(a1, bufs[nb_buf], gb, t1)) return;
        nb_buf ^= 1;
        if (!(t1[0] > 0.0)) {
            status = 2;
            break;
        }
        alpha = rho / t1[0];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc->iter = it;
        sc->done = status;
        sc->rnorm2 = rr;
        sc->bnorm2 = bb;
    }
}

template <typename V>
Op<V> make_op(Ctx& c);
template <>
Op<double> make_op<double>(Ctx& c) {
    return Op<double>{c.A.band + c.P.R, c.A.fac_l, c.A.fac_ib, c.A.band + 5 * c.P.R, c.F.nbr, c.P.Tp, c.P.R, c.P.L};
}
template <>
Op<float> make_op<float>(Ctx& c) {
    return Op<float>{c.A.lat32, c.A.l32, c.A.ib32, c.A.up32, c.F.nbr, c.P.Tp, c.P.R, c.P.L};
}

int read_scalars(Ctx& c, cudaStream_t s, Scalars* dev) {
    PBSM_CUDA_TRY(cudaMemcpyAsync(c.sc_host, dev, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    PBSM_CUDA_TRY(cudaStreamSynchronize(s));
    return 0;
}

// Run BiCGStab iterations on the state set up by k_residual until done.
template <typename V, typename X>
int bicgstab_iterations(Ctx& c, cudaStream_t s, Scalars* sc, X* x, V* r, V* rh, V* p, V* v, V* sv, V* tv, V* zp,
                        V* zs, int& iters) {
    Op<V> op = make_op<V>(c);
    const size_t smem = (size_t)c.P.L * kBlock * sizeof(V);
    const int g = c.grid_faces;
    double* part = c.red.partials;
    const int64_t T = c.P.T, rows = T * c.P.L;
    const int64_t sv_ = sizeof(V), sx = sizeof(X);
    int chunk = 4;
    int before = 0;
    {
        int rc = read_scalars(c, s, sc);
        if (rc) return rc;
        before = c.sc_host->iter;
        if (c.sc_host->done) {
            iters = 0;
            return 0;
        }
    }
    while (true) {
        for (int k = 0; k < chunk; ++k) {
            prof_begin(c, s);
            k_bicg_p<V><<<g, kBlock, smem, s>>>(op, r, p, v, zp, sc);
            prof_end(c, s, PBSM3D_K_BICG_P, rows * 8 * sv_);
            prof_begin(c, s);
            k_bicg_v<V><<<g, kBlock, 0, s>>>(op, p, zp, v, rh, sc, part);
            prof_end(c, s, PBSM3D_K_BICG_V, rows * 7 * sv_ + T * 12);
            prof_begin(c, s);
            k_bicg_s<V><<<g, kBlock, smem, s>>>(op, r, v, sv, zs, sc);
            prof_end(c, s, PBSM3D_K_BICG_S, rows * 7 * sv_);
            prof_begin(c, s);
            k_bicg_t<V><<<g, kBlock, 0, s>>>(op, sv, zs, tv, sc, part);
            prof_end(c, s, PBSM3D_K_BICG_T, rows * 6 * sv_ + T * 12);
            prof_begin(c, s);
            k_bicg_x<V, X><<<g, kBlock, 0, s>>>(c.P.Tp, c.P.L, x, zp, zs, sv, tv, r, rh, sc, part);
            prof_end(c, s, PBSM3D_K_BICG_X, rows * (2 * sx + 6 * sv_));
        }
        int rc = read_scalars(c, s, sc);
        if (rc) return rc;
        const int ran = c.sc_host->iter - before;
        before = c.sc_host->iter;
        // launches after the converging iteration returned at once: not counted
        const int idle = chunk - ran - (c.sc_host->done == DONE_BREAKDOWN ? 1 : 0);
        if (idle > 0) prof_drop(c, 5 * idle);
        if (c.sc_host->done) break;
        chunk = std::min(16, chunk * 2);
    }
    iters = c.sc_host->iter;
    return 0;
}

}  // namespace

// Column kernels stage L values per thread in shared memory; above 48 KB the
// launch needs the opt-in limit raised.
int configure_solver_kernels(Ctx& c) {
    const int s64 = c.P.L * kBlock * 8, s32 = c.P.L * kBlock * 4;
    PBSM_CUDA_TRY(cudaFuncSetAttribute(k_jacobi_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, s64));
    PBSM_CUDA_TRY(cudaFuncSetAttribute(k_bicg_p<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, s64));
    PBSM_CUDA_TRY(cudaFuncSetAttribute(k_bicg_s<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, s64));
    PBSM_CUDA_TRY(cudaFuncSetAttribute(k_bicg_p<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, s32));
    PBSM_CUDA_TRY(cudaFuncSetAttribute(k_bicg_s<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, s32));
    return 0;
}

// xo = B^{-1} (b - N xi) on the FP64 operator (the learned warm start's smoothing)
int jacobi_sweep(Ctx& c, cudaStream_t s, const double* xi, double* xo) {
    Op<double> op = make_op<double>(c);
    prof_begin(c, s);
    k_jacobi_sweep<<<c.grid_faces, kBlock, (size_t)c.P.L * kBlock * 8, s>>>(op, c.A.rhs, xi, xo);
    prof_end(c, s, PBSM3D_K_MLP, c.P.T * c.P.L * 72 + c.P.T * 12);
    PBSM_CUDA_TRY(cudaGetLastError());
    return 0;
}

// Suspension solve: x0 = current contents of A.x.  Fills iteration stats.
int solve_suspension(Ctx& c, cudaStream_t s, pbsm3d_stats* st) {
    (void)st;
    const int g = c.grid_faces;
    double* part = c.red.partials;
    Scalars* sc0 = c.sc;      // FP64 outer / plain
    Scalars* sc1 = c.sc + 1;  // FP32 inner
    const double tol = c.cfg.susp_tol;
    int total_iters = 0, sweeps = 0;
    double bnorm2 = 0;
    const int maxit = c.cfg.susp_maxit;
    c.susp_relres = 0;
    while (true) {
        // r = b - A x, in FP64; reset the Krylov state
        if (c.P.mixed) {
            prof_begin(c, s);
            k_residual<float><<<g, kBlock, 0, s>>>(c.P, c.A.band, c.F.nbr, c.A.x, c.A.rhs, c.r, c.r32, c.rh32,
                                                   c.p32, c.v32, sc0, part, tol, maxit);
            prof_end(c, s, PBSM3D_K_RESIDUAL, c.P.T * c.P.L * 88 + c.P.T * 12);
        } else {
            prof_begin(c, s);
            k_residual<double><<<g, kBlock, 0, s>>>(c.P, c.A.band, c.F.nbr, c.A.x, c.A.rhs, c.r, c.r, c.rh, c.p,
                                                    c.v, sc0, part, tol, maxit);
            prof_end(c, s, PBSM3D_K_RESIDUAL, c.P.T * c.P.L * 96 + c.P.T * 12);
        }
        int rc = read_scalars(c, s, sc0);
        if (rc) return rc;
        if (sweeps == 0) bnorm2 = c.sc_host->bnorm2;
        if (sweeps == 0 && c.cfg.warm_start != PBSM3D_X0_ZERO && !(c.cfg.warm_flags & 1)) {
            // Scale the warm start by the gamma that minimises ||b - gamma A x0||
            // and drop it when that residual is not below ||b||: the zero
            // guess stays the fallback.  (b, A x0) = |b|^2 - (b, r0),
            // |A x0|^2 = |b|^2 - 2 (b, r0) + |r0|^2.
            const double bb = bnorm2, br = c.sc_host->red0, rr = c.sc_host->rnorm2;
            const double bax = bb - br, axax = bb - 2.0 * br + rr;
            double gamma = (axax > 0 && bax > 0) ? bax / axax : 0.0;
            const double rmin2 = axax > 0 ? bb - bax * bax / axax : bb;
            if (!(rmin2 < 0.99 * bb)) gamma = 0.0;
            c.warm_gamma = gamma;
            prof_begin(c, s);
            if (c.P.mixed)
                k_warm_scale<float><<<g, kBlock, 0, s>>>(c.P.R, gamma, c.A.x, c.r, c.A.rhs, c.r32, c.rh32, sc0, part);
            else
                k_warm_scale<double><<<g, kBlock, 0, s>>>(c.P.R, gamma, c.A.x, c.r, c.A.rhs, c.r, c.rh, sc0, part);
            prof_end(c, s, PBSM3D_K_OTHER, c.P.T * c.P.L * 40);
            rc = read_scalars(c, s, sc0);
            if (rc) return rc;
        }
        const double rn2 = c.sc_host->rnorm2;
        c.susp_relres = bnorm2 > 0 ? sqrt(rn2 / bnorm2) : 0.0;
        // ensembles: tol * min_m ||b_m|| bounds every member's residual (target_scale2 = 1 otherwise)
        const double goal2 = tol * tol * bnorm2 * c.target_scale2;
        if (rn2 <= goal2) break;
        if (total_iters >= maxit) {
            c.susp_iters = total_iters;
            c.err = "suspension solve failed to converge (relative residual " + std::to_string(c.susp_relres) + ")";
            return PBSM3D_ERR_NOT_CONVERGED;
        }
        if (!isfinite(rn2)) {
            c.err = "suspension solve produced a non-finite residual";
            return PBSM3D_ERR_NOT_CONVERGED;
        }
        int it = 0;
        if (c.P.mixed) {
            // inner: A32 d = r32, d0 = 0, to inner_tol relative -- or less when
            // the FP64 target is closer than that (no over-solving in the last sweep)
            const double need = 0.5 * sqrt(goal2 / rn2);
            const double itol = std::min(0.5, std::max(c.cfg.inner_tol, need));
            Scalars init{};
            init.rho = rn2;
            init.alpha = init.omega = 1.0;
            init.beta = 0.0;
            init.bnorm2 = rn2;
            init.target2 = itol * itol * rn2;
            init.maxit = std::max(1, maxit - total_iters);
            PBSM_CUDA_TRY(cudaMemcpyAsync(sc1, &init, sizeof(Scalars), cudaMemcpyHostToDevice, s));
            prof_begin(c, s);
            k_zero<float><<<g, kBlock, 0, s>>>(c.P.R, c.x32);
            prof_end(c, s, PBSM3D_K_OTHER, c.P.T * c.P.L * 4);
            rc = bicgstab_iterations<float, float>(c, s, sc1, c.x32, c.r32, c.rh32, c.p32, c.v32, c.s32, c.t32,
                                                   c.zp32, c.zs32, it);
            if (rc) return rc;
            prof_begin(c, s);
            k_add_correction<<<g, kBlock, 0, s>>>(c.P.R, c.A.x, c.x32);
            prof_end(c, s, PBSM3D_K_OTHER, c.P.T * c.P.L * 20);
        } else {
            // target relative to ||b|| (the state's target2 is relative to ||r||)
            Scalars* h = c.sc_host;
            h->target2 = goal2;
            h->maxit = maxit - total_iters;
            PBSM_CUDA_TRY(cudaMemcpyAsync(&sc0->target2, &h->target2, sizeof(double), cudaMemcpyHostToDevice, s));
            PBSM_CUDA_TRY(cudaMemcpyAsync(&sc0->maxit, &h->maxit, sizeof(int), cudaMemcpyHostToDevice, s));
            rc = bicgstab_iterations<double, double>(c, s, sc0, c.A.x, c.r, c.rh, c.p, c.v, c.sv, c.tv, c.zp, c.zs,
                                                     it);
            if (rc) return rc;
        }
        total_iters += it;
        sweeps++;
        if (sweeps > 64) {
            c.err = "suspension solve: refinement did not converge";
            return PBSM3D_ERR_NOT_CONVERGED;
        }
    }
    c.susp_iters = total_iters;
    c.susp_matvecs = 2 * total_iters + sweeps + 1;
    c.susp_refinements = sweeps;
    return 0;
}

int configure_cg(Ctx& c) {
    int per_sm = 0, dev = 0, sms = 0;
    PBSM_CUDA_TRY(cudaGetDevice(&dev));
    PBSM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int coop = 0;
    PBSM_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    PBSM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_persistent, kCgBlock, 0));
    const int64_t need = (c.P.Tp + kCgBlock - 1) / kCgBlock;
    // one co-resident block per SM (at most the partials workspace's 8 x grid_faces / 7 blocks)
    int64_t blocks = std::min<int64_t>(need, per_sm >= 1 ? (int64_t)sms : 0);
    blocks = std::min<int64_t>(blocks, (int64_t)c.red.nblocks);
    c.coop_blocks = coop ? (int)blocks : 0;
    return 0;
}

int solve_deposition(Ctx& c, cudaStream_t s, pbsm3d_stats* st) {
    (void)st;
    double* part = c.red.partials;
    Scalars* sc = c.sc + 2;
    const int64_t T = c.P.T;
    if (c.coop_blocks <= 0) {
        c.err = "the device does not support cooperative launches";
        return PBSM3D_ERR_CUDA;
    }
    PBSM_CUDA_TRY(cudaMemsetAsync(c.gbar, 0, sizeof(GridBar), s));
    double tol = c.cfg.dep_tol * sqrt(c.dep_target_scale2);  // ensembles: every member to dep_tol
    int maxit = c.cfg.dep_maxit;
    void* args[] = {&c.P, &c.D, &c.F.nbr, &c.dr, &c.dz_, &c.dp, &c.dq, &part, &c.gbar, &sc, &tol, &maxit};
    prof_begin(c, s);
    PBSM_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_cg_persistent, dim3(c.coop_blocks), dim3(kCgBlock),
                                              args, 0, s));
    int rc = read_scalars(c, s, sc);
    if (rc) return rc;
    const int done = c.sc_host->done;
    c.dep_iters = c.sc_host->iter;
    prof_end(c, s, PBSM3D_K_CG, T * 96 + (int64_t)c.dep_iters * T * 148);
    GridBar gb;
    PBSM_CUDA_TRY(cudaMemcpy(&gb, c.gbar, sizeof(GridBar), cudaMemcpyDeviceToHost));
    if (gb.err) {
        c.err = "deposition solve: grid barrier timed out";
        return PBSM3D_ERR_CUDA;
    }
    const double bn2 = c.sc_host->bnorm2;
    prof_begin(c, s);
    k_cg_resid<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.D, c.F.nbr, c.dr, sc, part);
    prof_end(c, s, PBSM3D_K_CG, T * 76);
    rc = read_scalars(c, s, sc);
    if (rc) return rc;
    c.dep_relres = bn2 > 0 ? sqrt(c.sc_host->tmp / bn2) : 0.0;
    if (done != DONE_CONVERGED && !(c.sc_host->tmp <= tol * tol * bn2)) {
        c.err = "deposition solve failed to converge (relative residual " + std::to_string(c.dep_relres) + ")";
        return PBSM3D_ERR_NOT_CONVERGED;
    }
    return 0;
}

}  // namespace pbsm
