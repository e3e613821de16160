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
// Jacobi-preconditioned CG in FP64 in one cooperative launch; MIXED runs
// the same CG in FP32 inside FP64 iterative refinement.
//
// Every reduction is deterministic: fixed grid, per-block partials, the
// last block sums them in block order.  Scalars live in device memory, so
// iterations are launched without host synchronisation; the host polls the
// iteration count every few iterations.
#include <math.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>

#include "fp64_math.cuh"
#include "pbsm3d_internal.cuh"

namespace pbsm {

// ---------------------------------------------------------------- launch-geometry autotuner
// The column kernels (k_bicg_p, k_bicg_s, k_bicg_neu) run at one of nine
// geometries: slices of W = 256, 128 or 64 faces a block, with 1, 2 or 4
// lanes per face column (blocks of W x lanes threads).  Their arithmetic
// does not depend on the geometry (bit-identical results), so the tuner
// times the candidates on the first solves' own iterations, one iteration
// each (the default timed first and last, its faster time counts), and keeps
// the fastest if it beats the default by more than 2%.  The choice is
// remembered per problem shape for the process.  The reduction kernels
// (lateral gathers with their dot products, x update) keep one fixed
// geometry: theirs decides the order of the floating-point sums.
const ColGeom kColGeom[kNumColGeoms] = {{256, 1}, {128, 1}, {64, 1}, {256, 2}, {128, 2},
                                        {64, 2},  {256, 4}, {128, 4}, {64, 4}};
// timing order: the default first and again last
constexpr int kTuneOrder[kNumColGeoms + 1] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 0};

struct TuneKey {
    int64_t Tp;
    int L, n, mixed, neumann;
    bool operator<(const TuneKey& o) const {
        return std::tie(Tp, L, n, mixed, neumann) < std::tie(o.Tp, o.L, o.n, o.mixed, o.neumann);
    }
};
static std::mutex g_tune_mu;
static std::map<TuneKey, int> g_tune;

static TuneKey tune_key(const Ctx& c) {
    return TuneKey{c.P.Tp, c.P.L, c.tiles.n, c.P.mixed, c.cfg.neumann > 0 ? 1 : 0};
}

int tuned_geometry(Ctx& c) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(c));
    return it == g_tune.end() ? -1 : it->second;
}

// One more candidate timed (ms per iteration per active face); after the
// last, the choice.
static void tune_record(Ctx& c, float ms) {
    const int g = kTuneOrder[c.tune_cand];
    if (c.tune_ms[g] <= 0.f || ms < c.tune_ms[g]) c.tune_ms[g] = ms;
    if (++c.tune_cand < kNumColGeoms + 1) return;
    int best = 0;
    for (int k = 1; k < kNumColGeoms; ++k)
        if (c.tune_ms[k] < c.tune_ms[best]) best = k;
    if (!(c.tune_ms[best] < 0.98f * c.tune_ms[0])) best = 0;
    c.geom = best;
    c.tuned = true;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[tune_key(c)] = best;
}

namespace {

template <typename V>
struct Op {
    const V* lat;    // [3][R] lateral bands (FP64; null in FP32)
    const V* l;      // [R] forward multipliers (FP64: scaled, ib_z lo_z)
    const V* ib;     // [R] inverse pivots
    const V* up;     // [R] above band (FP64: scaled, ib_z up_z)
    const int32_t* nbr;  // [3][Tp]
    int64_t Tp, R;
    int L;
    const float* uz;   // FP32: [R] u_z of each row
    const float* l01;  // FP32: [6][Tp] L0_f, L1_f of each face
    // FP64 with the polynomial preconditioner: the lateral bands scaled by
    // the row's inverse pivot, the pivots, and the buffer of the scaled
    // vector ib * u that the steps read (null otherwise)
    const V* latp = nullptr;  // [3][R]
    const V* piv = nullptr;   // [R]
    V* nu = nullptr;          // [R]
};

// Values a row, and bytes a face, of the lateral couplings (traffic counts).
template <typename V>
constexpr int64_t kLatRow = sizeof(V) == 4 ? 1 : 3;
template <typename V>
constexpr int64_t kLatFace = sizeof(V) == 4 ? 24 : 0;

// The lateral couplings of one face's rows.  FP64 reads the stored bands.
// FP32 recomputes lat_f = u_z L1_f + L0_f from the row's u_z and the face's
// six constants (loaded once per column): 4 bytes a row instead of 12.
template <typename V>
struct LatFace;
template <>
struct LatFace<double> {
    const double* lat;
    int64_t R;
    // a row's bands, each loaded where it is used
    struct Row {
        const double* p;
        int64_t R;
        __device__ __forceinline__ double operator[](int j) const { return p[j * R]; }
    };
    __device__ __forceinline__ LatFace(const Op<double>& op, int64_t) : lat(op.lat), R(op.R) {}
    __device__ __forceinline__ Row row(int64_t k) const { return Row{lat + k, R}; }
};
template <>
struct LatFace<float> {
    const float* uz;
    float a0, a1, a2, b0, b1, b2;  // L0_f, L1_f
    struct Row {
        float u, a0, a1, a2, b0, b1, b2;
        __device__ __forceinline__ float operator[](int j) const {
            return j == 0 ? fmaf(u, b0, a0) : j == 1 ? fmaf(u, b1, a1) : fmaf(u, b2, a2);
        }
    };
    __device__ __forceinline__ LatFace(const Op<float>& op, int64_t i) : uz(op.uz) {
        a0 = op.l01[i];
        a1 = op.l01[op.Tp + i];
        a2 = op.l01[2 * op.Tp + i];
        b0 = op.l01[3 * op.Tp + i];
        b1 = op.l01[4 * op.Tp + i];
        b2 = op.l01[5 * op.Tp + i];
    }
    __device__ __forceinline__ Row row(int64_t k) const { return Row{uz[k], a0, a1, a2, b0, b1, b2}; }
};

// DONE_HALF: stopped at the half step of a BiCGStab iteration; the column
// kernel s applies that member's x += alpha zp, and k_bicg_t2 then marks it
// DONE_CONVERGED (so later iterations of the batch do not apply it again).
enum { DONE_NO = 0, DONE_CONVERGED = 1, DONE_BREAKDOWN = 2, DONE_MAXIT = 3, DONE_HALF = 4 };

// z = B^{-1} u for one column, u already in smem column g[z*bd + col].
// FP32: the Thomas sweeps on (l, ib, up), 3 operations a row.  FP64, whose
// pipe bounds these kernels on this GPU: the caller stores ib * u, and the
// sweeps run on the factors scaled by the inverse pivots (B = L D U', so
// D^-1 L^-1 u = L''^-1 (D^-1 u) with L'' = D^-1 L D unit lower, sub-diagonal
// ib_z lo_z, and U' = D^-1 U unit upper, super-diagonal ib_z up_z): 2
// operations a row.
template <typename V>
__device__ __forceinline__ void column_solve(const Op<V>& op, int64_t i, V* g, V* zout, int bd, int col) {
    V prev = 0;
    for (int z = 0; z < op.L; ++z) {
        const int64_t r = (int64_t)z * op.Tp + i;
        V gz = g[z * bd + col] - op.l[r] * prev;
        g[z * bd + col] = gz;
        prev = gz;
    }
    V y = 0;
    for (int z = op.L - 1; z >= 0; --z) {
        const int64_t r = (int64_t)z * op.Tp + i;
        if constexpr (sizeof(V) == 8)
            y = g[z * bd + col] - op.up[r] * y;
        else
            y = (g[z * bd + col] - op.up[r] * y) * op.ib[r];
        zout[r] = y;
    }
}
// The column solve's input for row k: u itself (FP32) or ib * u (FP64),
// which the polynomial steps of an FP64 solve also read (op.nu).
template <typename V>
__device__ __forceinline__ V column_in(const Op<V>& op, int64_t k, V u) {
    if constexpr (sizeof(V) == 8) {
        const V g = u * op.ib[k];
        if (op.nu) op.nu[k] = g;
        return g;
    } else {
        return u;
    }
}

// ---------------------------------------------------------------- batched BiCGStab
// Every kernel walks the work tiles (grid-stride over tiles, one tile per
// block at a time); a tile belongs to one member, whose scalars it reads
// once.  Tiles of members that are done are skipped.

__device__ __forceinline__ float wsum(float v) { return warp_sum_f(v); }

// Block b owns the contiguous run [a0, a1) of the active-tile list (whole
// members, ascending tiles); within it each run of one member's tiles is a
// segment, flushed to the member's reduction once.
struct TileRange {
    int a0, a1;
};
__device__ __forceinline__ TileRange block_tiles(const Tiles& tl) {
    const int64_t n = tl.nact_dev ? *tl.nact_dev : tl.nact, g = gridDim.x, b = blockIdx.x;
    return TileRange{(int)(b * n / g), (int)((b + 1) * n / g)};
}
// Slices of the column kernels: each active tile (<= kBlock faces) is cut
// into S = kBlock / W slices of W faces; block b owns the contiguous run
// [u0, u1) of the nact * S slices.  A slice's face column is handled by LC
// lanes: thread t takes face t % W of the slice, lane t / W.
struct SliceRange {
    int u0, u1;
};
__device__ __forceinline__ SliceRange block_slices(const Tiles& tl, int S) {
    const int64_t n = (int64_t)(tl.nact_dev ? *tl.nact_dev : tl.nact) * S, g = gridDim.x, b = blockIdx.x;
    return SliceRange{(int)(b * n / g), (int)((b + 1) * n / g)};
}

// End (exclusive, in active-list positions) of the segment that starts at
// position a with tile t of member m.
__device__ __forceinline__ int segment_end(const Tiles& tl, const TileRange& br, int a, int t, int m) {
    return min(br.a1, a + (tl.mtile[m + 1] - t));
}

// A segment [ts, te) of member m adds NT per-thread values: the block sum
// (warp sums in the vector precision, FP64 across warps) becomes tile ts's
// partial (the segment's other tiles get 0); the block that completes
// member m's tile count sums the member's partials in tile order
// (deterministic) and returns true, with the totals in tot[] of thread 0.
template <int NT, typename V>
__device__ bool member_totals(V (&v)[NT], double* part, const Tiles& tl, int ts, int te, int m, MScal* ms,
                              double (&tot)[NT]) {
    __shared__ double shp[NT][32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if constexpr (sizeof(V) == 8) {
        double w[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) w[k] = v[k];
        warp_sums(w);
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < NT; ++k) shp[k][wid] = w[k];
    } else {
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            const V w = wsum(v[k]);
            if (lane == 0) shp[k][wid] = (double)w;
        }
    }
    __syncthreads();
    // one member: the finaliser reads only the segment heads (block starts),
    // so the other tiles' partials need no zeros
    const bool one = tl.n == 1;
    if (!one && te - ts > 1) {
        for (int q = ts + 1 + (int)threadIdx.x; q < te; q += blockDim.x)
#pragma unroll
            for (int k = 0; k < NT; ++k) part[(int64_t)k * tl.ntiles + q] = 0.0;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = (int)(blockDim.x >> 5);
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            double s = 0;
            for (int w = 0; w < nw; ++w) s += shp[k][w];
            part[(int64_t)k * tl.ntiles + ts] = s;
        }
        __threadfence();
        const unsigned nt = (unsigned)(tl.mtile[m + 1] - tl.mtile[m]), mine = (unsigned)(te - ts);
        last = atomicAdd(&ms[m].counter, mine) + mine == nt;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        double s = 0;
        if (one) {
            // the active list is every tile; block b's segment starts at b * nact / G
            const int64_t na = tl.nact_dev ? *tl.nact_dev : tl.nact, g = gridDim.x;
            for (int64_t b = threadIdx.x; b < g; b += blockDim.x) {
                const int64_t a0 = b * na / g;
                if (a0 < (b + 1) * na / g) s += __ldcg(&part[(int64_t)k * tl.ntiles + tl.act[a0]]);
            }
        } else {
            for (int q = tl.mtile[m] + threadIdx.x; q < tl.mtile[m + 1]; q += blockDim.x)
                s += __ldcg(&part[(int64_t)k * tl.ntiles + q]);
        }
        tot[k] = s;
    }
    block_sum<NT>(tot);
    if (threadIdx.x == 0) ms[m].counter = 0u;
    return true;
}

// Member m has stopped (status st); the last member to stop ends the solve.
__device__ __forceinline__ void member_stop(MScal* ms, int m, int st, Scalars* sc, int n) {
    ms[m].done = st;
    if (atomicAdd(&sc->counter[2], 1u) + 1u == (unsigned)n) sc->done = DONE_CONVERGED;
}

// The column kernels (p, s and the polynomial-preconditioner step) compute
// each row from that row's own inputs and each column's Thomas solve in one
// thread, so the launch geometry -- slice width W and lanes per face column
// LC -- changes which thread does the work, never the arithmetic: every
// geometry gives bit-identical results (the autotuner relies on it).  With
// LC > 1 the lanes split the column's layers for the row-wise part, and lane
// 0 then runs the Thomas solve from shared memory.
template <int LC>
struct ColLanes {
    int f, lane;
    __device__ __forceinline__ explicit ColLanes(int W) : f(threadIdx.x & (W - 1)), lane(threadIdx.x / W) {}
};
template <>
struct ColLanes<1> {
    int f, lane;
    __device__ __forceinline__ explicit ColLanes(int) : f(threadIdx.x), lane(0) {}
};
// slices of a tile: S = kBlock / W = 1 << sh
__device__ __forceinline__ int slice_shift(int W) { return W == kBlock ? 0 : W == kBlock / 2 ? 1 : 2; }

// p = r + beta (p - omega v); zp = B^{-1} p
template <typename V, int LC>
__global__ void __launch_bounds__(kBlock * LC, LC == 1 ? 0 : 4 / LC) k_bicg_p(Op<V> op, Tiles tl, int W, const V* __restrict__ r,
                                                        V* __restrict__ p, const V* __restrict__ v,
                                                        V* __restrict__ zp, const MScal* __restrict__ ms) {
    extern __shared__ unsigned char smem_raw[];
    V* g = reinterpret_cast<V*>(smem_raw);
    const ColLanes<LC> cl(W);
    const int sh = slice_shift(W);
    const SliceRange br = block_slices(tl, 1 << sh);
    for (int u = br.u0; u < br.u1; ++u) {
        const int t = tl.act[u >> sh], m = tl.member[t];
        if (ms[m].done) continue;
        const int64_t i = tl.start[t] + (int64_t)(u & ((1 << sh) - 1)) * W + cl.f;
        const bool valid = i < tl.start[t + 1];
        if (LC == 1 && !valid) continue;  // no block barrier with one lane
        const V beta = (V)ms[m].beta, omega = (V)ms[m].omega;
        if (valid)
            for (int z = cl.lane; z < op.L; z += LC) {
                const int64_t k = (int64_t)z * op.Tp + i;
                const V pk = r[k] + beta * (p[k] - omega * v[k]);
                p[k] = pk;
                g[z * W + cl.f] = column_in(op, k, pk);
            }
        if (LC > 1) __syncthreads();
        if (valid && cl.lane == 0) column_solve(op, i, g, zp, W, cl.f);
        if (LC > 1) __syncthreads();
    }
}

// s = r - alpha v; zs = B^{-1} s.  A member that stopped at this
// iteration's half step takes x += alpha zp instead (xh: the solve's x).
template <typename V, int LC>
__global__ void __launch_bounds__(kBlock * LC, LC == 1 ? 0 : 4 / LC) k_bicg_s(Op<V> op, Tiles tl, int W, const V* __restrict__ r,
                                                        const V* __restrict__ v, V* __restrict__ s,
                                                        V* __restrict__ zs, const MScal* __restrict__ ms,
                                                        V* __restrict__ xh, const V* __restrict__ zp) {
    extern __shared__ unsigned char smem_raw[];
    V* g = reinterpret_cast<V*>(smem_raw);
    const ColLanes<LC> cl(W);
    const int sh = slice_shift(W);
    const SliceRange br = block_slices(tl, 1 << sh);
    for (int u = br.u0; u < br.u1; ++u) {
        const int t = tl.act[u >> sh], m = tl.member[t];
        const int64_t i = tl.start[t] + (int64_t)(u & ((1 << sh) - 1)) * W + cl.f;
        const bool valid = i < tl.start[t + 1];
        if (const int d = ms[m].done) {
            // the whole block sees the same member: no barrier is skipped
            if (xh && d == DONE_HALF && valid) {
                // as k_bicg_x updates x: the step in the vector precision
                const V alpha = (V)ms[m].alpha;
                for (int z = cl.lane; z < op.L; z += LC) {
                    const int64_t k = (int64_t)z * op.Tp + i;
                    xh[k] = xh[k] + alpha * zp[k];
                }
            }
            continue;
        }
        if (LC == 1 && !valid) continue;  // no block barrier with one lane
        const V alpha = (V)ms[m].alpha;
        if (valid)
            for (int z = cl.lane; z < op.L; z += LC) {
                const int64_t k = (int64_t)z * op.Tp + i;
                const V sk = r[k] - alpha * v[k];
                s[k] = sk;
                g[z * W + cl.f] = column_in(op, k, sk);
            }
        if (LC > 1) __syncthreads();
        if (valid && cl.lane == 0) column_solve(op, i, g, zs, W, cl.f);
        if (LC > 1) __syncthreads();
    }
}

// One step of the polynomial preconditioner M^-1 = B^-1 sum_{j<=K} (-C)^j,
// C = N B^-1 (a truncated Neumann series; Saad, Iterative Methods for Sparse
// Linear Systems, section 12.3): w = u - N zin, zout = B^{-1} w.  Starting
// from zin = B^{-1} u, K steps give zout = M^-1 u, and A zout = w + N zout,
// so the lateral kernels that follow take w in place of u.  FP64 works on
// ib * w = ib * u - (ib N) zin from the stored ib * u and the scaled bands
// (5 FP64 operations a row instead of 6); its last step writes w = piv * (ib
// * w) for the lateral kernel.
template <typename V, bool WRITE_W, int LC>
__global__ void __launch_bounds__(kBlock * LC, (LC == 1 ? 6 : LC == 2 ? 2 : 1))
    k_bicg_neu(Op<V> op, Tiles tl, int W, const V* __restrict__ u, const V* __restrict__ zin, V* __restrict__ w,
               V* __restrict__ zout, const MScal* __restrict__ ms) {
    extern __shared__ unsigned char smem_raw[];
    V* g = reinterpret_cast<V*>(smem_raw);
    const ColLanes<LC> cl(W);
    const int sh = slice_shift(W);
    const SliceRange br = block_slices(tl, 1 << sh);
    for (int uu = br.u0; uu < br.u1; ++uu) {
        const int t = tl.act[uu >> sh], m = tl.member[t];
        if (ms[m].done) continue;
        const int64_t i = tl.start[t] + (int64_t)(uu & ((1 << sh) - 1)) * W + cl.f;
        const bool valid = i < tl.start[t + 1];
        if (LC == 1 && !valid) continue;  // no block barrier with one lane
        if (valid) {
            const int32_t n0 = op.nbr[i], n1 = op.nbr[op.Tp + i], n2 = op.nbr[2 * op.Tp + i];
            // FP32: the face's six coupling constants stay in registers over the
            // column (40 a thread with four layers in flight, no spills)
            Op<V> opn = op;
            if constexpr (sizeof(V) == 8) opn.lat = op.latp;
            const LatFace<V> lf(opn, i);
#pragma unroll 4
            for (int z = cl.lane; z < op.L; z += LC) {
                const int64_t base = (int64_t)z * op.Tp;
                const int64_t k = base + i;
                const auto la = lf.row(k);
                V wk = u[k];
                if (n0 >= 0) wk -= la[0] * zin[base + n0];
                if (n1 >= 0) wk -= la[1] * zin[base + n1];
                if (n2 >= 0) wk -= la[2] * zin[base + n2];
                if (WRITE_W) {  // only the last step's w is read (by the lateral kernel)
                    if constexpr (sizeof(V) == 8)
                        w[k] = wk * op.piv[k];
                    else
                        w[k] = wk;
                }
                g[z * W + cl.f] = wk;
            }
        }
        if (LC > 1) __syncthreads();
        if (valid && cl.lane == 0) column_solve(op, i, g, zout, W, cl.f);
        if (LC > 1) __syncthreads();
    }
}

// Lanes per face column of the lateral kernels (k_bicg_v, k_bicg_t2): the
// column's layers are split over them, so a block of kBlock * kLatLanes
// threads keeps twice the independent gathers in flight per face.  Their
// launch geometry is fixed (it decides the order of the dot products' sums).
constexpr int kLatLanes = 2;

// y = u + N z for layers lane, lane + LC, ... of the column of face i, with
// (a, y); NT = 2: and (y, y); NT = 3: and (b, y), (y, y)
template <typename V, int NT, int LC>
__device__ __forceinline__ void lateral_apply(const Op<V>& op, int64_t i, int lane, const V* __restrict__ u,
                                              const V* __restrict__ zz, V* __restrict__ y, const V* __restrict__ a,
                                              const V* __restrict__ b, V (&acc)[3]) {
    const int32_t n0 = op.nbr[i], n1 = op.nbr[op.Tp + i], n2 = op.nbr[2 * op.Tp + i];
    const LatFace<V> lf(op, i);
    // layers are independent here: unrolled so their loads overlap
    constexpr int kUnroll = LC == 1 ? 4 : 2;
#pragma unroll kUnroll
    for (int z = lane; z < op.L; z += LC) {
        const int64_t base = (int64_t)z * op.Tp;
        const int64_t k = base + i;
        const auto la = lf.row(k);
        V yk = u[k];
        if (n0 >= 0) yk += la[0] * zz[base + n0];
        if (n1 >= 0) yk += la[1] * zz[base + n1];
        if (n2 >= 0) yk += la[2] * zz[base + n2];
        y[k] = yk;
        acc[0] += a[k] * yk;
        if (NT == 2) acc[1] += yk * yk;
        if (NT == 3) {
            acc[1] += b[k] * yk;
            acc[2] += yk * yk;
        }
    }
}

// Below this ratio of the target to ||r||^2 the half-step norm, a difference
// of terms of the size of ||r||^2 (FP64 sums, relative error ~1e-14), could
// misjudge the target; the test is then left to the full step.
constexpr double kHalfTestFloor = 1e-11;
// The half-step iterate x + alpha zp lacks the iteration's minimal-residual
// step, and a stop just under the target leaves more error than the full
// steps, which usually land well below it: the half step stops only when
// ||s|| <= 0.3 of the target (||s||^2 <= 0.09 of target2).
constexpr double kHalfMargin2 = 0.09;
// A half step reduces ||r||^2 by 1e-6 at most (measured 1e-2..1e-6 with the
// polynomial preconditioner): its test (two more dot products and r read in
// k_bicg_v) runs only once ||r||^2 is within this factor of the target.
constexpr double kHalfWindow2 = 1e6;
__host__ __device__ __forceinline__ int half_window(double rr, double target2) {
    return rr <= kHalfWindow2 * target2 ? 1 : 0;
}

// v = p + N zp; rv = (rhat, v); alpha = rho / rv.  FP64, near the target,
// also sums (r, v) and (v, v): ||s||^2 = ||r||^2 - 2 alpha (r, v) + alpha^2
// (v, v) for s = r - alpha v is BiCGStab's half-step test (H. A. van der
// Vorst, SIAM J. Sci. Stat. Comput. 13, 1992, Alg. 1: stop with x + alpha zp
// when ||s|| meets the target), which skips the iteration's second
// preconditioner application when it passes.  The FP32 inner solve of the
// mixed form has no such test: its target, ~1e-8 of ||r||^2, puts nearly
// every iteration in the window, and FP64 sums (FP32 ones cannot resolve
// ||s||^2 there) made its v kernel 1.6x slower and the step 3% slower.
template <typename V>
__global__ void __launch_bounds__(kBlock * kLatLanes, kLatLanes == 1 ? 5 : 2) k_bicg_v(Op<V> op, Tiles tl, const V* __restrict__ p,
                                                      const V* __restrict__ zp, V* __restrict__ v,
                                                      const V* __restrict__ rh, const V* __restrict__ r,
                                                      MScal* ms, Scalars* sc, double* part) {
    const TileRange br = block_tiles(tl);
    for (int a = br.a0; a < br.a1;) {
        const int ts = tl.act[a], m = tl.member[ts];
        const int ae = segment_end(tl, br, a, ts, m), te = ts + (ae - a);
        if (ms[m].done) {
            a = ae;
            continue;
        }
        // the member's half-step test (set before the launch: the same in
        // every block of the member)
        const bool test = sizeof(V) == 8 && ms[m].half;
        V acc[3] = {0, 0, 0};
        for (int t = ts; t < te; ++t) {
            const int64_t i = tl.start[t] + threadIdx.x % kBlock;
            if (i >= tl.start[t + 1]) continue;
            if (test)
                lateral_apply<V, 3, kLatLanes>(op, i, threadIdx.x / kBlock, p, zp, v, rh, r, acc);
            else
                lateral_apply<V, 1, kLatLanes>(op, i, threadIdx.x / kBlock, p, zp, v, rh, nullptr, acc);
        }
        double tot[3] = {0, 0, 0};
        bool last;
        if (test) {
            last = member_totals<3>(acc, part, tl, ts, te, m, ms, tot);
        } else {
            V a1[1] = {acc[0]};
            double t1[1];
            last = member_totals<1>(a1, part, tl, ts, te, m, ms, t1);
            tot[0] = t1[0];
        }
        if (last && threadIdx.x == 0) {
            MScal& q = ms[m];
            const double rv = tot[0];
            if (rv == 0.0 || !isfinite(rv)) {
                member_stop(ms, m, DONE_BREAKDOWN, sc, tl.n);
            } else {
                const double alpha = q.rho / rv;
                q.alpha = alpha;
                if (test) {
                    // ||r||^2: rho itself on a sweep's first iteration (rhat = r)
                    const double rr = q.iter == 0 ? q.rho : q.rnorm2;
                    const double s2 = rr - 2.0 * alpha * tot[1] + alpha * alpha * tot[2];
                    if (q.target2 >= kHalfTestFloor * rr && s2 <= kHalfMargin2 * q.target2) {
                        q.rnorm2 = fmax(s2, 0.0);
                        q.iter += 1;
                        atomicMax(&sc->iter, q.iter);
                        atomicAdd(&sc->counter[3], 1u);
                        member_stop(ms, m, DONE_HALF, sc, tl.n);
                    }
                }
            }
        }
        a = ae;
    }
}

// t = u + N zs (u = s, or the preconditioner's last s - N z); ts = (t, s),
// tt = (t, t); omega = ts / tt
template <typename V>
__global__ void __launch_bounds__(kBlock * kLatLanes, kLatLanes == 1 ? 5 : 2) k_bicg_t2(Op<V> op, Tiles tl, const V* __restrict__ u,
                                                       const V* __restrict__ zs, V* __restrict__ tv,
                                                       const V* __restrict__ s, MScal* ms, double* part) {
    const TileRange br = block_tiles(tl);
    for (int a = br.a0; a < br.a1;) {
        const int ts = tl.act[a], m = tl.member[ts];
        const int ae = segment_end(tl, br, a, ts, m), te = ts + (ae - a);
        if (const int d = ms[m].done) {
            // a half-step exit's x update is in place (column kernel s, launched
            // before): the member is converged (every block that sees it
            // stores the same value)
            if (d == DONE_HALF && threadIdx.x == 0) ms[m].done = DONE_CONVERGED;
            a = ae;
            continue;
        }
        V acc[3] = {0, 0, 0};
        for (int t = ts; t < te; ++t) {
            const int64_t i = tl.start[t] + threadIdx.x % kBlock;
            if (i < tl.start[t + 1])
                lateral_apply<V, 2, kLatLanes>(op, i, threadIdx.x / kBlock, u, zs, tv, s, nullptr, acc);
        }
        V a2[2] = {acc[0], acc[1]};
        double tot[2];
        if (member_totals<2>(a2, part, tl, ts, te, m, ms, tot) && threadIdx.x == 0)
            ms[m].omega = tot[1] > 0 ? tot[0] / tot[1] : 0.0;
        a = ae;
    }
}

// x += alpha zp + omega zs; r = s - omega t; rho' = (rhat, r), (r, r)
template <typename V, typename X>
__global__ void __launch_bounds__(kBlock, 5) k_bicg_x(int64_t Tp, int L, Tiles tl, X* __restrict__ x,
                                                      const V* __restrict__ zp, const V* __restrict__ zs,
                                                      const V* __restrict__ s, const V* __restrict__ tv,
                                                      V* __restrict__ r, const V* __restrict__ rh, MScal* ms,
                                                      Scalars* sc, double* part) {
    const TileRange br = block_tiles(tl);
    for (int a = br.a0; a < br.a1;) {
        const int ts = tl.act[a], m = tl.member[ts];
        const int ae = segment_end(tl, br, a, ts, m), te = ts + (ae - a);
        if (ms[m].done) {
            a = ae;
            continue;
        }
        V acc[2] = {0, 0};
        const X alpha = (X)ms[m].alpha, omega = (X)ms[m].omega;
        const V om = (V)ms[m].omega;
        for (int t = ts; t < te; ++t) {
            const int64_t i = tl.start[t] + threadIdx.x;
            if (i >= tl.start[t + 1]) continue;
#pragma unroll 4
            for (int z = 0; z < L; ++z) {
                const int64_t k = (int64_t)z * Tp + i;
                x[k] = x[k] + alpha * (X)zp[k] + omega * (X)zs[k];
                const V rk = s[k] - om * tv[k];
                r[k] = rk;
                acc[0] += rh[k] * rk;
                acc[1] += rk * rk;
            }
        }
        double tot[2];
        if (member_totals<2>(acc, part, tl, ts, te, m, ms, tot) && threadIdx.x == 0) {
            MScal& q = ms[m];
            const double rho_new = tot[0];
            q.rnorm2 = tot[1];
            q.half = half_window(tot[1], q.target2);
            q.iter += 1;
            atomicMax(&sc->iter, q.iter);
            if (tot[1] <= q.target2)
                member_stop(ms, m, DONE_CONVERGED, sc, tl.n);
            else if (q.omega == 0.0 || rho_new == 0.0 || !isfinite(rho_new) || !isfinite(tot[1]))
                member_stop(ms, m, DONE_BREAKDOWN, sc, tl.n);
            else if (q.iter >= q.maxit)
                member_stop(ms, m, DONE_MAXIT, sc, tl.n);
            else
                q.beta = (rho_new / q.rho) * (q.alpha / q.omega);
            q.rho = rho_new;
        }
        a = ae;
    }
}

// r = b - A x with all six FP64 bands; optionally r32 = (float) r.  Per
// member (r, r), (b, b), (b, r) into ms[m].  Resets the Krylov vectors:
// rhat = r, p = v = 0.  Members marked done in ms are skipped (their x is
// final).
template <typename V>
__global__ void __launch_bounds__(kBlock * kLatLanes, kLatLanes == 1 ? 5 : 2)
    k_residual(Params P, Tiles tl, const double* __restrict__ band,
                                                     const int32_t* __restrict__ nbr, const double* __restrict__ x,
                                                     const double* __restrict__ b, double* __restrict__ r,
                                                     V* __restrict__ rv, V* __restrict__ rhv, V* __restrict__ pv,
                                                     V* __restrict__ vv, MScal* ms, double* part, int first,
                                                     const int* __restrict__ sweep, int x0_zero) {
    const int64_t Tp = P.Tp, R = P.R;
    // (b, b) and (b, r) serve the first refinement sweep only (the target's
    // norm and the warm start's scale): two FP64 FMAs a row fewer after it.
    // The sweep number is the host's (first) or, in a graph, the controller's.
    const bool full = sweep ? *sweep == 0 : first != 0;
    // the first sweep of a zero start has x = 0 (the assembly clears it):
    // r = b without reading the bands or x
    const bool zero_x = full && x0_zero;
    const TileRange br = block_tiles(tl);
    for (int a = br.a0; a < br.a1;) {
        const int ts = tl.act[a], m = tl.member[ts];
        const int ae = segment_end(tl, br, a, ts, m), te = ts + (ae - a);
        if (ms[m].done) {
            a = ae;
            continue;
        }
        double acc[3] = {0, 0, 0};
        // kLatLanes lanes a face column, splitting its layers (as the lateral kernels)
        const int lane = threadIdx.x / kBlock;
        // r_k, its copies and its share of the dot products; with_b: the
        // first sweep's (b, b) and (b, r) too (a compile-time choice, so the
        // later sweeps issue no FP64 instructions for them)
        auto emit = [&](int64_t k, double rk, auto with_b) {
            r[k] = rk;
            if (rv) {
                // FP32 copies rounded on the integer pipe (bit-identical to the cast)
                const V rc = sizeof(V) == 4 ? (V)f32_rn(rk) : (V)rk;
                rv[k] = rc;
                rhv[k] = rc;
                pv[k] = 0;
                vv[k] = 0;
            }
            acc[0] += rk * rk;
            if constexpr (decltype(with_b)::value) {
                acc[1] += b[k] * b[k];
                acc[2] += b[k] * rk;
            }
        };
        // r = b - A x over the column's rows of this lane
        auto spmv_rows = [&](int64_t i, auto with_b) {
            const int32_t nb[3] = {nbr[i], nbr[Tp + i], nbr[2 * Tp + i]};
#pragma unroll 1
            for (int z = lane; z < P.L; z += kLatLanes) {
                const int64_t base = (int64_t)z * Tp;
                const int64_t k = base + i;
                double ax = band[k] * x[k];
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    if (nb[j] >= 0) ax += band[(j + 1) * R + k] * x[base + nb[j]];
                if (z > 0) ax += band[4 * R + k] * x[k - Tp];
                if (z < P.L - 1) ax += band[5 * R + k] * x[k + Tp];
                emit(k, b[k] - ax, with_b);
            }
        };
        for (int t = ts; t < te; ++t) {
            const int64_t i = tl.start[t] + threadIdx.x % kBlock;
            if (i >= tl.start[t + 1]) continue;
            if (zero_x) {
                // r = b (first sweep): rows independent, unrolled so their loads overlap
#pragma unroll 4
                for (int z = lane; z < P.L; z += kLatLanes) {
                    const int64_t k = (int64_t)z * Tp + i;
                    emit(k, b[k], std::true_type{});
                }
            } else if (full) {
                spmv_rows(i, std::true_type{});
            } else {
                spmv_rows(i, std::false_type{});
            }
        }
        double tot[3];
        if (member_totals<3>(acc, part, tl, ts, te, m, ms, tot) && threadIdx.x == 0) {
            ms[m].rnorm2 = tot[0];
            if (full) {
                ms[m].bnorm2 = tot[1];
                ms[m].red0 = tot[2];
            }
        }
        a = ae;
    }
}

// Warm start x0 -> gamma_m x0 per member (gamma = 0 drops it):
// r = (1-gamma) b + gamma r0, rhat = r, and (r, r) per member.
template <typename V>
__global__ void __launch_bounds__(kBlock) k_warm_scale(Params P, Tiles tl, double* __restrict__ x,
                                                       double* __restrict__ r, const double* __restrict__ b,
                                                       V* __restrict__ rv, V* __restrict__ rhv, MScal* ms,
                                                       double* part) {
    const TileRange br = block_tiles(tl);
    for (int a = br.a0; a < br.a1;) {
        const int ts = tl.act[a], m = tl.member[ts];
        const int ae = segment_end(tl, br, a, ts, m), te = ts + (ae - a);
        if (ms[m].done) {
            a = ae;
            continue;
        }
        double acc[1] = {0};
        const double gamma = ms[m].gamma;
        for (int t = ts; t < te; ++t) {
            const int64_t i = tl.start[t] + threadIdx.x;
            if (i >= tl.start[t + 1]) continue;
            for (int z = 0; z < P.L; ++z) {
                const int64_t k = (int64_t)z * P.Tp + i;
                x[k] *= gamma;
                const double rk = (1.0 - gamma) * b[k] + gamma * r[k];
                r[k] = rk;
                rv[k] = (V)rk;
                rhv[k] = (V)rk;
                acc[0] += rk * rk;
            }
        }
        double tot[1];
        if (member_totals<1>(acc, part, tl, ts, te, m, ms, tot) && threadIdx.x == 0) ms[m].rnorm2 = tot[0];
        a = ae;
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
            g[z * blockDim.x + threadIdx.x] = u * op.ib[k];
        }
        column_solve(op, i, g, xo, (int)blockDim.x, (int)threadIdx.x);
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
// ||b - A x||^2 of the FP64 deposition system (final check, ledger residual)
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
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_timer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr unsigned long long kBarrierLimitNs = 2000000000ull;  // 2 s
// One 1024-thread block per SM (64 registers a thread): each thread's chain
// of dependent loads (neighbour index, then the gathered values) over its
// grid-stride rows is as short as with 2048 threads a SM would allow, and the
// all-reduces wait on one flag per SM (measured against two 512-thread blocks
// a SM: the same threads, twice the flags: 2% faster FP64, 5-8% FP32).
constexpr int kCgBlock = 1024;
constexpr int kCgBlocksPerSm = 1;
constexpr int kFlagStride = 32;  // one 128-byte line per block flag

// The bounded waits of the persistent CG: their limit, and one block that
// publishes no flag at all (-1: none; set only by the timeout test, whose
// other blocks' waits then run out and end the kernel with *err set).
struct GridWait {
    unsigned long long limit_ns;
    int withhold;
};

// First level of a block reduction: FP32 values are summed in FP32 across
// the warp (off the FP64 pipe), then widened.
template <int NT>
__device__ __forceinline__ void warp_level(const double (&v)[NT], double (&w)[NT]) {
#pragma unroll
    for (int k = 0; k < NT; ++k) w[k] = v[k];
    warp_sums(w);
}
template <int NT>
__device__ __forceinline__ void warp_level(const float (&v)[NT], double (&w)[NT]) {
#pragma unroll
    for (int k = 0; k < NT; ++k) w[k] = (double)warp_sum_f(v[k]);
}

// All-reduce of NT per-thread values over a cooperative grid, identical in
// every block, without atomics.  (1) Warp sums go to shared memory; (2) warp
// 0 adds them, and its lane 0 writes the block's partials and then releases
// flags[b] = epoch; (3) thread t < gridDim of every block waits for flags[t]
// and loads block t's partials, the warps holding them sum them, and (4)
// warp 0 adds those warp sums: the same order in every block
// (deterministic).  Lane 0 of warp 0 then runs `fin` on the totals -- the
// solver's scalar step (divisions, stopping tests), once a block instead of
// once a thread -- and its NX results (as double and as V) and status are
// broadcast.  Three block barriers a call.  FP64 operations are kept few
// (transposed warp sums, one warp for the block and grid levels, scalar work
// in one lane), since on this GPU they, not the flag latency, bound an
// all-reduce of many blocks.
// Partials alternate between two buffers by epoch parity: a block can only
// publish epoch e+2 after every block has published e+1, i.e. after every
// block has finished reading epoch e.  A reader therefore waits until
// flags[b] is AT LEAST its epoch (wraparound-safe difference): block b may
// already have left this all-reduce and published e+1 before a slow reader
// first loads its flag, and its epoch-e partials stay valid in the other
// buffer until every block has published e+1.  The wait is bounded: after
// gw.limit_ns (kBarrierLimitNs outside the timeout test) a block sets *err
// and every block leaves at its next all-reduce, so a broken co-residency
// assumption ends in an error, never a hang.  Returns false when the kernel
// must exit.
template <int NT, int NX, typename V, typename Fin>
__device__ bool grid_totals(const V (&v)[NT], double* partials, unsigned* flags, unsigned epoch, int* err,
                            const GridWait& gw, double (&out)[NX], V (&outv)[NX], int& st, Fin fin) {
    __shared__ double shw[NT][32], shg[NT][32], bx[NX];
    __shared__ V bv[NX];
    __shared__ int bad, good_all, bst;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    const int G = gridDim.x;
    double* pp = partials + (size_t)(epoch & 1u) * 4 * G;
    {
        double w[NT];
        warp_level<NT>(v, w);
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < NT; ++k) shw[k][wid] = w[k];
        if (threadIdx.x == 0) bad = 0;
    }
    __syncthreads();
    if (wid == 0) {
        double b[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) b[k] = lane < nw ? shw[k][lane] : 0.0;
        warp_sums(b);
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < NT; ++k) pp[k * G + blockIdx.x] = b[k];
            if ((int)blockIdx.x != gw.withhold) st_release_u32(&flags[blockIdx.x * kFlagStride], epoch);
        }
    }
    double t[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) t[k] = 0.0;
    for (int b = threadIdx.x; b < G; b += blockDim.x) {
        const unsigned long long t0 = global_timer_ns();
        bool ok = true;
        while ((int)(ld_relaxed_u32(&flags[b * kFlagStride]) - epoch) < 0) {
            if (*(volatile int*)err) {
                ok = false;
                break;
            }
            if (global_timer_ns() - t0 > gw.limit_ns) {
                atomicExch(err, 1);
                ok = false;
                break;
            }
        }
        if (!ok) bad = 1;
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
#pragma unroll
        for (int k = 0; k < NT; ++k) t[k] += __ldcg(&pp[k * G + b]);
    }
    if (wid * 32 < G) {
        warp_sums(t);
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < NT; ++k) shg[k][wid] = t[k];
    }
    __syncthreads();
    if (wid == 0) {
        const int ng = min(nw, (G + 31) >> 5);
        double g[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) g[k] = lane < ng ? shg[k][lane] : 0.0;
        warp_sums(g);
        if (lane == 0) {
            double o[NX];
            bst = fin(g, o);
#pragma unroll
            for (int k = 0; k < NX; ++k) {
                bx[k] = o[k];
                bv[k] = (V)o[k];
            }
            good_all = !bad;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NX; ++k) {
        out[k] = bx[k];
        outv[k] = bv[k];
    }
    st = bst;
    return good_all != 0;
}

// The deposition system in one precision.
template <typename V>
struct DepSys {
    const V* diag;      // [Tp]
    const V* off;       // [3][Tp]
    const V* dinv;      // [Tp] Jacobi preconditioner (per-member tile CG)
    const V* b;         // [Tp]
    V* x;               // [Tp] solution (starts at 0)
    V *r, *zz, *p, *q;  // [Tp] work
    V* r2;              // [Tp] second residual buffer; non-null selects the polynomial preconditioner
    V* s;               // [Tp] d^-1/2, the symmetric scaling of the persistent CG
    V* offs;            // [3][Tp] scaled couplings s_i a_ij s_j of the persistent CG
};

// The preconditioner z = M^-1 r at row i of the per-member tile CG.  Jacobi:
// z_i = r_i / d_i.  With D.r2 set, the order-1 truncated Neumann series of
// the Jacobi splitting A = D - R (Saad, Iterative Methods for Sparse Linear
// Systems, 2nd ed., sec. 12.3.1): M^-1 = D^-1 + D^-1 R D^-1, symmetric, and
// positive definite because the spectral radius of D^-1 R is below 1 for
// this strictly diagonally dominant matrix with non-positive off-diagonals;
// about half the iterations of Jacobi.  The neighbours' residuals are
// recomputed from the previous iteration's r and q (rn = r - alpha q), so z
// needs no grid-wide wait between the residual update and the dot products;
// the new residual goes to the other buffer, since neighbours still read the
// old one.
template <typename V>
__device__ __forceinline__ V dep_precond(const DepSys<V>& D, const int32_t* __restrict__ nbr, int64_t Tp, int64_t i,
                                         V rn, const V* __restrict__ rin, const V* __restrict__ q, V al) {
    if (!D.r2) return D.dinv[i] * rn;
    V acc = rn;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const int32_t nb = nbr[j * Tp + i];
        if (nb >= 0) acc -= D.off[j * Tp + i] * (D.dinv[nb] * (q ? rin[nb] - al * q[nb] : rin[nb]));
    }
    return D.dinv[i] * acc;
}

__device__ __forceinline__ double rsqrt_v(double d) { return rsqrt(d); }
__device__ __forceinline__ float rsqrt_v(float d) { return rsqrtf(d); }

// CG in one cooperative launch, Jacobi or polynomial preconditioner; at 1M
// faces its vectors and matrix (~100 MB in FP64) stay in L2.
//
// On this GPU the FP64 pipe, not memory or the grid all-reduce, bounds the
// FP64 iteration, so the iteration is arranged for few FP64 operations:
// - CG runs on the symmetrically scaled system S A S y = S b, S = D^-1/2
//   (x = S y), whose diagonal is one: the Jacobi preconditioner becomes the
//   identity and the order-1 Neumann polynomial M^-1 = D^-1 + D^-1 R D^-1
//   (A = D - R; Saad, Iterative Methods for Sparse Linear Systems, 2nd ed.,
//   sec. 12.3.1) becomes I + S R S.  In exact arithmetic the iterates are
//   those of the unscaled preconditioned CG, x_k = S y_k; the stopping test
//   uses the unscaled residual, ||r||^2 = sum d_i r^_i^2.
// - The polynomial's z = M^-1 r is carried by the recurrence z -= alpha
//   M^-1 q (from r -= alpha q), so an iteration gathers the neighbours' q
//   only, and no second residual buffer is needed.
// - Two all-reduces per iteration: (r, z) and (r, r) after the x/r/z update,
//   (p, q) after q = A z + beta q.
// 15 FP64 operations a row and iteration with the polynomial (21 unscaled).
// Measured slower at 1M faces and dropped: a form with one all-reduce per
// iteration (Chronopoulos-Gear recurrences, contiguous row runs per block
// and a point-to-point wait for the blocks owning neighbour rows), whose
// polynomial rebuilt each neighbour's new residual from three vectors; and
// an all-reduce whose partials are staged in shared memory for one warp to
// sum (its 24 KB of shared memory is L1 the gathers lose).
//
// `dyn`, when set, holds the stopping target (target2, relative to (b, b))
// and the iteration limit in device memory, written by a controller kernel
// of the step graph; otherwise tol and maxit are the launch's own.
template <typename V>
__global__ void __launch_bounds__(kCgBlock, kCgBlocksPerSm)
    k_cg_persistent(int64_t Tp, DepSys<V> D, const int32_t* __restrict__ nbr, double* partials, unsigned* flags,
                    int* err, Scalars* sc, double tol, int maxit, GridWait gw, const MScal* dyn) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool poly = D.r2 != nullptr;
    V *x = D.x, *r = D.r, *p = D.p, *q = D.q, *s = D.s, *offs = D.offs;
    V* z = poly ? D.zz : D.r;  // Jacobi: z = r in the scaled system
    unsigned epoch = 0;
    int st = 0;
    const auto total = [](const double (&g)[1], double (&o)[1]) {
        o[0] = g[0];
        return 0;
    };
    // set-up 1: s = d^-1/2, r = s b, y = 0; (b, b)
    double bb, rho, rr;
    V alpha = 0;  // in the vector precision (converted once, in one lane)
    {
        V a[1] = {0};
        for (int64_t i = i0; i < Tp; i += stride) {
            const V bi = D.b[i], si = rsqrt_v(D.diag[i]);
            s[i] = si;
            r[i] = si * bi;
            x[i] = 0;
            a[0] += bi * bi;
        }
        double o[1];
        V ov[1];
        if (!grid_totals<1, 1>(a, partials, flags, ++epoch, err, gw, o, ov, st, total)) return;
        bb = o[0];
    }
    // set-up 2 (every s is visible): the scaled couplings (0 without a
    // neighbour), z = M^-1 r, p = z; (r, z)
    {
        V a[1] = {0};
        for (int64_t i = i0; i < Tp; i += stride) {
            const V si = s[i], ri = r[i];
            V zi = ri;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int32_t nb = nbr[j * Tp + i];
                V o = 0;
                if (nb >= 0) {
                    o = si * D.off[j * Tp + i] * s[nb];
                    if (poly) zi -= o * r[nb];
                }
                offs[j * Tp + i] = o;
            }
            if (poly) z[i] = zi;
            p[i] = zi;
            a[0] += ri * zi;
        }
        double o[1];
        V ov[1];
        if (!grid_totals<1, 1>(a, partials, flags, ++epoch, err, gw, o, ov, st, total)) return;
        rho = o[0];
    }
    const double target2 = (dyn ? dyn->target2 : tol * tol) * bb;
    if (dyn) maxit = dyn->maxit;
    // set-up 3: q = A p; (p, q), alpha = (r, z) / (p, q)
    {
        V a[1] = {0};
        for (int64_t i = i0; i < Tp; i += stride) {
            const V pi = p[i];
            V qi = pi;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int32_t nb = nbr[j * Tp + i];
                if (nb >= 0) qi += offs[j * Tp + i] * p[nb];
            }
            q[i] = qi;
            a[0] += pi * qi;
        }
        double o[1];
        V ov[1];
        const auto first = [bb, rho](const double (&g)[1], double (&o)[1]) {
            o[0] = 0.0;
            if (bb == 0.0) return 1;
            if (!(g[0] > 0.0)) return 2;
            o[0] = rho / g[0];
            return 0;
        };
        if (!grid_totals<1, 1>(a, partials, flags, ++epoch, err, gw, o, ov, st, first)) return;
        alpha = ov[0];
    }
    int status = st, it = 0;
    rr = bb;
    while (status == 0) {
        // y += alpha p, r -= alpha q, z -= alpha M^-1 q; (r, z) and the
        // unscaled (r, r); then the stopping tests and beta in one lane
        {
            const V al = alpha;
            V a[2] = {0, 0};
            for (int64_t i = i0; i < Tp; i += stride) {
                x[i] += al * p[i];
                const V qi = q[i];
                const V ri = r[i] - al * qi;
                r[i] = ri;
                V zi = ri;
                if (poly) {
                    V mq = qi;
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        const int32_t nb = nbr[j * Tp + i];
                        if (nb >= 0) mq -= offs[j * Tp + i] * q[nb];
                    }
                    zi = z[i] - al * mq;
                    z[i] = zi;
                }
                a[0] += ri * zi;
                a[1] += ri * ri * D.diag[i];
            }
            const int itn = it + 1;
            const auto step = [=](const double (&g)[2], double (&o)[3]) {
                o[0] = g[0];
                o[1] = g[1];
                o[2] = 0.0;
                if (g[1] <= target2) return 1;
                if (!isfinite(g[1])) return 2;
                if (itn >= maxit) return 3;
                o[2] = g[0] / rho;  // beta
                return 0;
            };
            double o[3];
            V ov[3];
            if (!grid_totals<2, 3>(a, partials, flags, ++epoch, err, gw, o, ov, st, step)) return;
            it = itn;
            rr = o[1];
            if (st) {
                status = st;
                break;
            }
            rho = o[0];
            // p = z + beta p, q = A z + beta q; (p, q), alpha = rho / (p, q)
            const V be = ov[2];
            V b1[1] = {0};
            for (int64_t i = i0; i < Tp; i += stride) {
                const V zi = z[i];
                V az = zi;
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const int32_t nb = nbr[j * Tp + i];
                    if (nb >= 0) az += offs[j * Tp + i] * z[nb];
                }
                const V pi = zi + be * p[i];
                const V qi = az + be * q[i];
                p[i] = pi;
                q[i] = qi;
                b1[0] += pi * qi;
            }
            const auto step2 = [rho](const double (&g)[1], double (&o)[1]) {
                o[0] = 0.0;
                if (!(g[0] > 0.0)) return 2;
                o[0] = rho / g[0];
                return 0;
            };
            double o2[1];
            V ov2[1];
            if (!grid_totals<1, 1>(b1, partials, flags, ++epoch, err, gw, o2, ov2, st, step2)) return;
            if (st) {
                status = st;
                break;
            }
            alpha = ov2[0];
        }
    }
    // back to the unscaled solution x = S y
    for (int64_t i = i0; i < Tp; i += stride) x[i] *= s[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc->iter = it;
        sc->done = status;
        sc->rnorm2 = rr;
        sc->bnorm2 = bb;
    }
}

// ---------------------------------------------------------------- batched deposition CG (ensembles)
// Jacobi-preconditioned CG per member inside shared tile kernels, like the
// batched BiCGStab: each member its own alpha, beta, rho and stopping test
// ||b_m - A_m x_m|| <= tol ||b_m||.  Two kernels per iteration.

// r = b, z = M^-1 b, p = z, x = 0; (r, z) -> rho, (b, b) -> bnorm2
template <typename V>
__global__ void __launch_bounds__(kBlock) k_scg_start(Tiles tl, int64_t Tp, DepSys<V> D,
                                                      const int32_t* __restrict__ nbr, MScal* ms, Scalars* sc,
                                                      double* part) {
    const TileRange br = block_tiles(tl);
    for (int a = br.a0; a < br.a1;) {
        const int ts = tl.act[a], m = tl.member[ts];
        const int ae = segment_end(tl, br, a, ts, m), te = ts + (ae - a);
        if (ms[m].done) {
            a = ae;
            continue;
        }
        V acc[2] = {0, 0};
        for (int t = ts; t < te; ++t) {
            const int64_t i = tl.start[t] + threadIdx.x;
            if (i >= tl.start[t + 1]) continue;
            const V bi = D.b[i];
            const V zi = dep_precond<V>(D, nbr, Tp, i, bi, D.b, nullptr, V(0));
            D.r[i] = bi;
            D.zz[i] = zi;
            D.p[i] = zi;
            D.x[i] = 0;
            acc[0] += bi * zi;
            acc[1] += bi * bi;
        }
        double tot[2];
        if (member_totals<2>(acc, part, tl, ts, te, m, ms, tot) && threadIdx.x == 0) {
            MScal& q = ms[m];
            q.rho = tot[0];
            q.bnorm2 = tot[1];
            q.rnorm2 = tot[1];
            q.beta = 0.0;
            q.target2 *= tot[1];  // the host set tol^2: the target is relative to ||b_m||
            if (tot[1] == 0.0) member_stop(ms, m, DONE_CONVERGED, sc, tl.n);
            else if (!(tot[0] > 0.0) || !isfinite(tot[0])) member_stop(ms, m, DONE_BREAKDOWN, sc, tl.n);
        }
        a = ae;
    }
}

// q = A z + beta q, p = z + beta p; alpha = rho / (p, q)
template <typename V>
__global__ void __launch_bounds__(kBlock, 6) k_scg_q(Tiles tl, int64_t Tp, DepSys<V> D, const int32_t* __restrict__ nbr,
                                                  MScal* ms, Scalars* sc, double* part) {
    const TileRange br = block_tiles(tl);
    for (int a = br.a0; a < br.a1;) {
        const int ts = tl.act[a], m = tl.member[ts];
        const int ae = segment_end(tl, br, a, ts, m), te = ts + (ae - a);
        if (ms[m].done) {
            a = ae;
            continue;
        }
        const V be = (V)ms[m].beta;
        V acc[1] = {0};
        for (int t = ts; t < te; ++t) {
            const int64_t i = tl.start[t] + threadIdx.x;
            if (i >= tl.start[t + 1]) continue;
            V az = D.diag[i] * D.zz[i];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int32_t nb = nbr[j * Tp + i];
                if (nb >= 0) az += D.off[j * Tp + i] * D.zz[nb];
            }
            const V pi = D.zz[i] + be * D.p[i];
            const V qi = az + be * D.q[i];
            D.p[i] = pi;
            D.q[i] = qi;
            acc[0] += pi * qi;
        }
        double tot[1];
        if (member_totals<1>(acc, part, tl, ts, te, m, ms, tot) && threadIdx.x == 0) {
            if (!(tot[0] > 0.0) || !isfinite(tot[0]))
                member_stop(ms, m, DONE_BREAKDOWN, sc, tl.n);
            else
                ms[m].alpha = ms[m].rho / tot[0];
        }
        a = ae;
    }
}

// x += alpha p, r -= alpha q, z = M^-1 r; (r, z), (r, r); beta, stopping test.
// With the polynomial preconditioner the residual alternates between D.r and
// D.r2 by the member's iteration parity (k_scg_start wrote D.r).
template <typename V>
__global__ void __launch_bounds__(kBlock) k_scg_x(Tiles tl, int64_t Tp, DepSys<V> D, const int32_t* __restrict__ nbr,
                                                  MScal* ms, Scalars* sc, double* part) {
    const TileRange br = block_tiles(tl);
    for (int a = br.a0; a < br.a1;) {
        const int ts = tl.act[a], m = tl.member[ts];
        const int ae = segment_end(tl, br, a, ts, m), te = ts + (ae - a);
        if (ms[m].done) {
            a = ae;
            continue;
        }
        const V al = (V)ms[m].alpha;
        const bool odd = D.r2 && (ms[m].iter & 1);
        const V* rin = odd ? D.r2 : D.r;
        V* rout = D.r2 ? (odd ? D.r : D.r2) : D.r;
        V acc[2] = {0, 0};
        for (int t = ts; t < te; ++t) {
            const int64_t i = tl.start[t] + threadIdx.x;
            if (i >= tl.start[t + 1]) continue;
            D.x[i] += al * D.p[i];
            const V ri = rin[i] - al * D.q[i];
            rout[i] = ri;
            const V zi = dep_precond<V>(D, nbr, Tp, i, ri, rin, D.q, al);
            D.zz[i] = zi;
            acc[0] += ri * zi;
            acc[1] += ri * ri;
        }
        double tot[2];
        if (member_totals<2>(acc, part, tl, ts, te, m, ms, tot) && threadIdx.x == 0) {
            MScal& q = ms[m];
            q.rnorm2 = tot[1];
            q.iter += 1;
            atomicMax(&sc->iter, q.iter);
            if (tot[1] <= q.target2)
                member_stop(ms, m, DONE_CONVERGED, sc, tl.n);
            else if (!isfinite(tot[1]))
                member_stop(ms, m, DONE_BREAKDOWN, sc, tl.n);
            else if (q.iter >= q.maxit)
                member_stop(ms, m, DONE_MAXIT, sc, tl.n);
            else
                q.beta = tot[0] / q.rho;
            q.rho = tot[0];
        }
        a = ae;
    }
}

// r = b - A x (FP64) per member: (r, r), (b, b) into ms; r32 = (float) r
__global__ void __launch_bounds__(kBlock) k_sdep_resid(Tiles tl, Params P, Dep D, const int32_t* __restrict__ nbr,
                                                       float* __restrict__ r32, double* __restrict__ r64, MScal* ms,
                                                       double* part) {
    const int64_t Tp = P.Tp;
    const TileRange br = block_tiles(tl);
    for (int a = br.a0; a < br.a1;) {
        const int ts = tl.act[a], m = tl.member[ts];
        const int ae = segment_end(tl, br, a, ts, m), te = ts + (ae - a);
        if (ms[m].done) {
            a = ae;
            continue;
        }
        double acc[2] = {0, 0};
        for (int t = ts; t < te; ++t) {
            const int64_t i = tl.start[t] + threadIdx.x;
            if (i >= tl.start[t + 1]) continue;
            double ax = D.diag[i] * D.x[i];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int32_t nb = nbr[j * Tp + i];
                if (nb >= 0) ax += D.off[j * Tp + i] * D.x[nb];
            }
            const double bi = D.rhs[i];
            const double ri = bi - ax;
            if (r32) r32[i] = (float)ri;
            if (r64) r64[i] = ri;
            acc[0] += ri * ri;
            acc[1] += bi * bi;
        }
        double tot[2];
        if (member_totals<2>(acc, part, tl, ts, te, m, ms, tot) && threadIdx.x == 0) {
            ms[m].rnorm2 = tot[0];
            ms[m].bnorm2 = tot[1];
        }
        a = ae;
    }
}

// FP32 copies of the deposition matrix for the inner solves (MIXED).
__global__ void __launch_bounds__(kBlock) k_dep_to_f32(Params P, Dep D, float* diag, float* off, float* dinv) {
    const int64_t Tp = P.Tp;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Tp; i += (int64_t)gridDim.x * blockDim.x) {
        diag[i] = (float)D.diag[i];
        dinv[i] = (float)D.dinv[i];
        for (int j = 0; j < 3; ++j) off[j * Tp + i] = (float)D.off[j * Tp + i];
    }
}

// x += d (FP64 accumulation of an FP32 correction)
__global__ void __launch_bounds__(kBlock) k_dep_add(Params P, Dep D, const float* __restrict__ d) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.Tp; i += (int64_t)gridDim.x * blockDim.x)
        D.x[i] += (double)d[i];
}

// r = b - A x in FP64, r32 = (float) r; (r, r) -> rnorm2, (b, b) -> bnorm2
__global__ void __launch_bounds__(kBlock) k_dep_resid32(Params P, Dep D, const int32_t* __restrict__ nbr,
                                                        float* __restrict__ r32, Scalars* sc, double* partials) {
    const int64_t Tp = P.Tp;
    double acc[2] = {0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Tp; i += (int64_t)gridDim.x * blockDim.x) {
        double ax = D.diag[i] * D.x[i];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int32_t nb = nbr[j * Tp + i];
            if (nb >= 0) ax += D.off[j * Tp + i] * D.x[nb];
        }
        const double bi = D.rhs[i];
        const double ri = bi - ax;
        r32[i] = (float)ri;
        acc[0] += ri * ri;
        acc[1] += bi * bi;
    }
    double tot[2];
    if (block_partials_last<2>(acc, partials, &sc->counter[0], tot) && threadIdx.x == 0) {
        sc->rnorm2 = tot[0];
        sc->bnorm2 = tot[1];
    }
}

template <typename V>
Op<V> make_op(Ctx& c);
template <>
Op<double> make_op<double>(Ctx& c) {
    Op<double> op{c.A.band + c.P.R, c.A.fac_l, c.A.fac_ib, c.A.fac_u, c.F.nbr, c.P.Tp, c.P.R, c.P.L,
                  nullptr,          nullptr};
    op.latp = c.A.latp;
    op.piv = c.A.fac_piv;
    op.nu = c.A.latp ? c.nu64 : nullptr;
    return op;
}
template <>
Op<float> make_op<float>(Ctx& c) {
    return Op<float>{nullptr, c.A.l32, c.A.ib32, c.A.up32, c.F.nbr, c.P.Tp, c.P.R, c.P.L, c.A.uz32, c.A.l01};
}

int read_scalars(Ctx& c, cudaStream_t s, Scalars* dev) {
    PBSM_CUDA_TRY(cudaMemcpyAsync(c.sc_host, dev, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    PBSM_CUDA_TRY(cudaStreamSynchronize(s));
    return 0;
}

// Run BiCGStab iterations on the state set up by k_residual until done.
// Copy the n per-member states to the pinned host mirror.
int read_members(Ctx& c, cudaStream_t s, const MScal* dev) {
    PBSM_CUDA_TRY(
        cudaMemcpyAsync(c.ms_host, dev, sizeof(MScal) * (size_t)c.tiles.n, cudaMemcpyDeviceToHost, s));
    PBSM_CUDA_TRY(cudaStreamSynchronize(s));
    return 0;
}

// Faces of the members whose state is not done (host mirror).
int64_t active_faces(const Ctx& c) {
    int64_t f = 0;
    for (int m = 0; m < c.tiles.n; ++m)
        if (!c.ms_host[m].done) f += c.member_offsets[m + 1] - c.member_offsets[m];
    return f;
}

// Active-tile list: every tile of the members with active[m] != 0.
int set_active(Ctx& c, cudaStream_t s, const std::vector<char>& active) {
    c.act_host.clear();
    // the member tile ranges are regular: kBlock faces per tile within a member
    int t = 0;
    for (int m = 0; m < c.tiles.n; ++m) {
        const int64_t f = c.member_offsets[m + 1] - c.member_offsets[m];
        const int nt = (int)((f + kBlock - 1) / kBlock);
        if (active[m])
            for (int k = 0; k < nt; ++k) c.act_host.push_back(t + k);
        t += nt;
    }
    c.tiles.nact = (int)c.act_host.size();
    if (c.tiles.nact)
        PBSM_CUDA_TRY(cudaMemcpyAsync(c.act_buf, c.act_host.data(), sizeof(int32_t) * c.act_host.size(),
                                      cudaMemcpyHostToDevice, s));
    return 0;
}

// Faces of the members not yet converged (conv[m] == 0).
int64_t active_faces_of(const Ctx& c, const std::vector<char>& conv) {
    int64_t f = 0;
    for (int m = 0; m < c.tiles.n; ++m)
        if (!conv[m]) f += c.member_offsets[m + 1] - c.member_offsets[m];
    return f;
}

// Run BiCGStab iterations on the per-member states in ms (set up by the
// host) until every member is done.  sc holds the batch totals: done, the
// largest member iteration count and the count of stopped members.
// K steps of the polynomial preconditioner on u, whose B^-1 u the column
// kernel wrote to z0 (chosen so that the last step writes zfinal); returns
// the vector the lateral kernel adds N zfinal to (u, or the last u - N z).
// Launch of a column kernel at geometry gi: grid = one wave of its own
// residency (c.grid_geom), capped by the slices to do (all tiles' in graph
// mode, where the active count lives on the device).
template <typename V>
static int col_grid(const Ctx& c, const Tiles& tl, int gi, bool neu) {
    const int S = kBlock / kColGeom[gi].W;
    const int units = (tl.nact_dev ? tl.ntiles : tl.nact) * S;
    return std::max(1, std::min(c.grid_geom[neu ? 1 : 0][sizeof(V) == 4][gi], units));
}

template <typename V>
void launch_col_p(Ctx& c, cudaStream_t s, const Op<V>& op, const Tiles& tl, int gi, const V* r, V* p, const V* v,
                  V* zp, const MScal* ms) {
    const ColGeom G = kColGeom[gi];
    const int grid = col_grid<V>(c, tl, gi, false);
    const size_t smem = (size_t)c.P.L * G.W * sizeof(V);
    if (G.LC == 1) k_bicg_p<V, 1><<<grid, G.W, smem, s>>>(op, tl, G.W, r, p, v, zp, ms);
    else if (G.LC == 2) k_bicg_p<V, 2><<<grid, 2 * G.W, smem, s>>>(op, tl, G.W, r, p, v, zp, ms);
    else k_bicg_p<V, 4><<<grid, 4 * G.W, smem, s>>>(op, tl, G.W, r, p, v, zp, ms);
}

// xh: the solve's x (members stopped at the half step update it)
template <typename V>
void launch_col_s(Ctx& c, cudaStream_t s, const Op<V>& op, const Tiles& tl, int gi, const V* r, const V* v, V* sv,
                  V* zs, const MScal* ms, V* xh, const V* zp) {
    const ColGeom G = kColGeom[gi];
    const int grid = col_grid<V>(c, tl, gi, false);
    const size_t smem = (size_t)c.P.L * G.W * sizeof(V);
    if (G.LC == 1) k_bicg_s<V, 1><<<grid, G.W, smem, s>>>(op, tl, G.W, r, v, sv, zs, ms, xh, zp);
    else if (G.LC == 2) k_bicg_s<V, 2><<<grid, 2 * G.W, smem, s>>>(op, tl, G.W, r, v, sv, zs, ms, xh, zp);
    else k_bicg_s<V, 4><<<grid, 4 * G.W, smem, s>>>(op, tl, G.W, r, v, sv, zs, ms, xh, zp);
}


template <typename V, bool WRITE_W>
static void launch_neu_step(Ctx& c, cudaStream_t s, const Op<V>& op, const Tiles& tl, int gi, const V* u,
                            const V* zin, V* w, V* zout, const MScal* ms) {
    const ColGeom G = kColGeom[gi];
    const int grid = col_grid<V>(c, tl, gi, true);
    const size_t smem = (size_t)c.P.L * G.W * sizeof(V);
    if (G.LC == 1) k_bicg_neu<V, WRITE_W, 1><<<grid, G.W, smem, s>>>(op, tl, G.W, u, zin, w, zout, ms);
    else if (G.LC == 2) k_bicg_neu<V, WRITE_W, 2><<<grid, 2 * G.W, smem, s>>>(op, tl, G.W, u, zin, w, zout, ms);
    else k_bicg_neu<V, WRITE_W, 4><<<grid, 4 * G.W, smem, s>>>(op, tl, G.W, u, zin, w, zout, ms);
}

template <typename V>
const V* launch_neumann(Ctx& c, cudaStream_t s, const Op<V>& op, const Tiles& tl, int gi, const V* u, V* zfinal,
                        V* w, V* ztmp, const MScal* ms, int64_t rows, bool prof) {
    const int K = c.cfg.neumann;
    V* a = (K & 1) ? ztmp : zfinal;
    V* b = (K & 1) ? zfinal : ztmp;
    const V* un = op.nu ? op.nu : u;  // FP64: the steps read ib * u
    for (int j = 0; j < K; ++j) {
        const bool last = j == K - 1;
        if (prof) prof_begin(c, s);
        if (last)
            launch_neu_step<V, true>(c, s, op, tl, gi, un, a, w, b, ms);
        else
            launch_neu_step<V, false>(c, s, op, tl, gi, un, a, w, b, ms);
        // per row u, z in, z out, the lateral couplings (3 bands, or u_z in
        // FP32), the column factors (3 in FP32, 2 scaled ones in FP64), w on
        // the last step (FP64: and the pivot); per face the ids (and the FP32
        // couplings' 6 constants)
        const int64_t vals = sizeof(V) == 8 ? (last ? 7 : 5) : (last ? 7 : 6);
        if (prof)
            prof_end(c, s, PBSM3D_K_NEUMANN,
                     rows * (vals + kLatRow<V>) * sizeof(V) + rows / c.P.L * (12 + kLatFace<V>));
        std::swap(a, b);
    }
    return K > 0 ? w : u;
}

template <typename V>
V* neumann_first(Ctx& c, V* zfinal, V* ztmp) { return (c.cfg.neumann & 1) ? ztmp : zfinal; }

template <typename V, typename X>
int bicgstab_iterations(Ctx& c, cudaStream_t s, MScal* ms, Scalars* sc, X* x, V* r, V* rh, V* p, V* v, V* sv,
                        V* tv, V* zp, V* zs, V* nw, V* nz, int& iters) {
    Op<V> op = make_op<V>(c);
    double* part = c.tile_part;
    const int64_t sv_ = sizeof(V), sx = sizeof(X);
    std::vector<char> active(c.tiles.n);
    for (int m = 0; m < c.tiles.n; ++m) active[m] = c.ms_host[m].done ? 0 : 1;
    {
        int rc = set_active(c, s, active);
        if (rc) return rc;
    }
    Tiles tl = c.tiles;
    int gr = std::max(1, std::min(c.grid_red[sizeof(V) == 4], tl.nact));
    int gl = std::max(1, std::min(c.grid_lat[sizeof(V) == 4], tl.nact));
    // iterations are launched in chunks between polls of the device's
    // stopping flag; launches after it stops return at once but still cost
    // a launch each (5 + 2K a polynomial-preconditioned iteration).  The
    // first chunk is the previous solve's count; later ones grow by a
    // quarter of the iterations done, so an overshoot stays small.
    const int hint = sizeof(V) == 4 ? 1 : 0;
    int chunk = std::max(1, std::min(16, c.bicg_hint[hint]));
    int done_iters = 0;
    const int per_it = 5 + (c.cfg.neumann > 0 ? 2 * c.cfg.neumann : 0);  // profiled launches an iteration
    const int first_half = 2 + (c.cfg.neumann > 0 ? c.cfg.neumann : 0);  // p, the preconditioner, v
    unsigned half_seen = 0;
    int before = 0;
    {
        int rc = read_scalars(c, s, sc);
        if (rc) return rc;
        before = c.sc_host->iter;
        half_seen = c.sc_host->counter[3];
        if (c.sc_host->done) {
            iters = 0;
            return 0;
        }
    }
    int64_t act = active_faces(c);
    cudaEvent_t te[2] = {nullptr, nullptr};
    while (true) {
        const int64_t rows = act * c.P.L;
        const bool timing = !c.tuned;
        // the column kernels' geometry: the candidate under test (one
        // iteration a chunk while tuning), else the chosen one
        const int gi = timing ? kTuneOrder[c.tune_cand] : c.geom;
        if (timing) {
            chunk = 1;
            if (!te[0]) {
                PBSM_CUDA_TRY(cudaEventCreate(&te[0]));
                PBSM_CUDA_TRY(cudaEventCreate(&te[1]));
            }
            PBSM_CUDA_TRY(cudaEventRecord(te[0], s));
        }
        for (int k = 0; k < chunk; ++k) {
            prof_begin(c, s);
            launch_col_p<V>(c, s, op, tl, gi, r, p, v, neumann_first(c, zp, nz), ms);
            prof_end(c, s, PBSM3D_K_BICG_P, rows * (8 + (op.nu ? 1 : 0)) * sv_);
            const V* up = launch_neumann<V>(c, s, op, tl, gi, p, zp, nw, nz, ms, rows, true);
            prof_begin(c, s);
            k_bicg_v<V><<<gl, kBlock * kLatLanes, 0, s>>>(op, tl, up, zp, v, rh, r, ms, sc, part);
            // (the FP64 half-step test's read of r, in the iterations near
            // the target only, is not counted)
            prof_end(c, s, PBSM3D_K_BICG_V, rows * (4 + kLatRow<V>) * sv_ + act * (12 + kLatFace<V>));
            prof_begin(c, s);
            launch_col_s<V>(c, s, op, tl, gi, r, v, sv, neumann_first(c, zs, nz), ms, x, zp);
            prof_end(c, s, PBSM3D_K_BICG_S, rows * (7 + (op.nu ? 1 : 0)) * sv_);
            const V* us = launch_neumann<V>(c, s, op, tl, gi, sv, zs, nw, nz, ms, rows, true);
            prof_begin(c, s);
            k_bicg_t2<V><<<gl, kBlock * kLatLanes, 0, s>>>(op, tl, us, zs, tv, sv, ms, part);
            // u, s, t and the gathered zs a row (u is s itself without the
            // polynomial preconditioner, the last step's w with it)
            prof_end(c, s, PBSM3D_K_BICG_T,
                     rows * ((c.cfg.neumann > 0 ? 4 : 3) + kLatRow<V>) * sv_ + act * (12 + kLatFace<V>));
            prof_begin(c, s);
            k_bicg_x<V, X><<<gr, kBlock, 0, s>>>(c.P.Tp, c.P.L, tl, x, zp, zs, sv, tv, r, rh, ms, sc, part);
            prof_end(c, s, PBSM3D_K_BICG_X, rows * (2 * sx + 6 * sv_));
        }
        if (timing) PBSM_CUDA_TRY(cudaEventRecord(te[1], s));
        int rc = read_scalars(c, s, sc);
        if (rc) return rc;
        const int ran = c.sc_host->iter - before;
        before = c.sc_host->iter;
        const bool half_exit = c.sc_host->counter[3] > half_seen;
        if (timing && ran == chunk && !half_exit) {
            // a full chunk: its time per iteration and per active face (in
            // an ensemble later chunks carry fewer members) decides; one
            // that ended at a half step did less work and is not counted
            float ms = 0;
            PBSM_CUDA_TRY(cudaEventElapsedTime(&ms, te[0], te[1]));
            tune_record(c, ms / chunk / (float)std::max<int64_t>(1, act));
        }
        // launches after the last member stopped returned at once: not
        // counted (their bytes would inflate the classes' rates)
        done_iters += ran;
        const int idle = chunk - ran;
        if (idle > 0) prof_drop(c, per_it * idle);
        // one member that stopped at a half step: the rest of that iteration
        // (s, the second preconditioner application, t, x) did no work either
        if (tl.n == 1 && half_exit) prof_drop(c, per_it - first_half);
        half_seen = c.sc_host->counter[3];
        if (c.sc_host->done) break;
        if (tl.n > 1) {
            // members that stopped leave the active-tile list
            if ((rc = read_members(c, s, ms))) return rc;
            bool changed = false;
            for (int m = 0; m < tl.n; ++m)
                if (active[m] && c.ms_host[m].done) {
                    active[m] = 0;
                    changed = true;
                }
            if (changed) {
                if ((rc = set_active(c, s, active))) return rc;
                tl = c.tiles;
                gr = std::max(1, std::min(c.grid_red[sizeof(V) == 4], tl.nact));
                gl = std::max(1, std::min(c.grid_lat[sizeof(V) == 4], tl.nact));
            }
            act = active_faces(c);
        }
        chunk = c.tuned ? std::max(1, std::min(16, done_iters / 4)) : 1;
    }
    for (auto e : te)
        if (e) cudaEventDestroy(e);
    iters = c.sc_host->iter;
    c.bicg_hint[hint] = std::max(1, done_iters);
    return 0;
}

}  // namespace

// Column kernels stage L values per thread in shared memory; above 48 KB the
// launch needs the opt-in limit raised.
int configure_solver_kernels(Ctx& c) {
    const int s64 = c.P.L * kBlock * 8, s32 = c.P.L * kBlock * 4;
    PBSM_CUDA_TRY(cudaFuncSetAttribute(k_jacobi_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, s64));
    int dev = 0, sms = 0;
    PBSM_CUDA_TRY(cudaGetDevice(&dev));
    PBSM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // one full wave of co-resident blocks per kernel (grid-stride loops do the rest)
    auto wave_of = [&](const void* f, int block, int smem, int& out) -> int {
        int per = 0;
        PBSM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, block, smem));
        out = std::max(1, sms * std::max(per, 1));
        return 0;
    };
    int rc;
    // the column kernels at every geometry: shared-memory opt-in and one wave
    auto col_kernels = [&](auto vtag, int prec, int smax) -> int {
        using V = decltype(vtag);
        const void* kp[3] = {(const void*)k_bicg_p<V, 1>, (const void*)k_bicg_p<V, 2>, (const void*)k_bicg_p<V, 4>};
        const void* ks[3] = {(const void*)k_bicg_s<V, 1>, (const void*)k_bicg_s<V, 2>, (const void*)k_bicg_s<V, 4>};
        const void* kn0[3] = {(const void*)k_bicg_neu<V, false, 1>, (const void*)k_bicg_neu<V, false, 2>,
                              (const void*)k_bicg_neu<V, false, 4>};
        const void* kn1[3] = {(const void*)k_bicg_neu<V, true, 1>, (const void*)k_bicg_neu<V, true, 2>,
                              (const void*)k_bicg_neu<V, true, 4>};
        for (int l = 0; l < 3; ++l)
            for (const void* f : {kp[l], ks[l], kn0[l], kn1[l]})
                PBSM_CUDA_TRY(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
        for (int gi = 0; gi < kNumColGeoms; ++gi) {
            const ColGeom G = kColGeom[gi];
            const int l = G.LC == 1 ? 0 : G.LC == 2 ? 1 : 2;
            const int smem = c.P.L * G.W * (int)sizeof(V);
            int r1;
            if ((r1 = wave_of(kp[l], G.W * G.LC, smem, c.grid_geom[0][prec][gi]))) return r1;
            if ((r1 = wave_of(kn0[l], G.W * G.LC, smem, c.grid_geom[1][prec][gi]))) return r1;
        }
        return 0;
    };
    if ((rc = col_kernels(double{}, 0, s64))) return rc;
    if ((rc = col_kernels(float{}, 1, s32))) return rc;
    auto wave = [&](const void* f, int smem, int& out) -> int {
        int r1 = wave_of(f, kBlock, smem, out);
        out = std::min(out, c.grid_faces);
        return r1;
    };
    if ((rc = wave((const void*)k_bicg_x<double, double>, 0, c.grid_red[0]))) return rc;
    if ((rc = wave((const void*)k_bicg_x<float, float>, 0, c.grid_red[1]))) return rc;
    if ((rc = wave_of((const void*)k_residual<float>, kBlock * kLatLanes, 0, c.grid_res))) return rc;
    c.grid_res = std::min(c.grid_res, c.grid_faces);
    for (int k = 0; k < 2; ++k) {
        const void* f = k ? (const void*)k_bicg_v<float> : (const void*)k_bicg_v<double>;
        if ((rc = wave_of(f, kBlock * kLatLanes, 0, c.grid_lat[k]))) return rc;
        c.grid_lat[k] = std::min(c.grid_lat[k], c.grid_faces);
    }
    {
        // the tile CG: one wave of its two per-iteration kernels
        int gx[2], gq[2];
        if ((rc = wave((const void*)k_scg_x<double>, 0, gx[0]))) return rc;
        if ((rc = wave((const void*)k_scg_x<float>, 0, gx[1]))) return rc;
        if ((rc = wave((const void*)k_scg_q<double>, 0, gq[0]))) return rc;
        if ((rc = wave((const void*)k_scg_q<float>, 0, gq[1]))) return rc;
        for (int k = 0; k < 2; ++k) c.grid_cg[k] = std::min(gx[k], gq[k]);
    }
    c.geom = 0;
    c.tuned = !c.cfg.autotune;
    if (!c.tuned) {
        // a choice made for this shape by an earlier context of the process
        const int gi = tuned_geometry(c);
        if (gi >= 0) {
            c.geom = gi;
            c.tuned = true;
        }
    }
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
// Every ensemble member is its own BiCGStab (its own scalars and stopping
// test on ||b_m - A_m x_m|| <= tol ||b_m||) inside the shared kernels; a
// single mesh is the one-member case.
int solve_suspension(Ctx& c, cudaStream_t s, pbsm3d_stats* st) {
    (void)st;
    const int n = c.tiles.n;
    double* part = c.tile_part;
    Scalars* sc0 = c.sc;      // FP64 plain: batch totals
    Scalars* sc1 = c.sc + 1;  // FP32 inner: batch totals
    const double tol = c.cfg.susp_tol;
    int total_iters = 0, sweeps = 0;
    const int maxit = c.cfg.susp_maxit;
    c.susp_relres = 0;
    c.member_bb.assign(n, 0.0);
    std::vector<char> conv(n, 0);
    std::vector<MScal> init(n);
    double gamma_sum = 0;
    // residual states: every member active at the first sweep
    for (int m = 0; m < n; ++m) init[m] = MScal{};
    PBSM_CUDA_TRY(cudaMemcpyAsync(c.msR, init.data(), sizeof(MScal) * n, cudaMemcpyHostToDevice, s));
    while (true) {
        // r = b - A x in FP64 per member (converged members are skipped); reset the Krylov vectors
        const int64_t act = active_faces_of(c, conv);
        {
            std::vector<char> a(n);
            for (int m = 0; m < n; ++m) a[m] = conv[m] ? 0 : 1;
            int rc0 = set_active(c, s, a);
            if (rc0) return rc0;
        }
        const Tiles tl = c.tiles;
        const int gr = std::max(1, std::min(c.grid_red[0], tl.nact));
        const int gq = std::max(1, std::min(c.grid_res, tl.nact));
        prof_begin(c, s);
        const int x0_zero = c.cfg.warm_start == PBSM3D_X0_ZERO ? 1 : 0;
        if (c.P.mixed)
            k_residual<float><<<gq, kBlock * kLatLanes, 0, s>>>(c.P, tl, c.A.band, c.F.nbr, c.A.x, c.A.rhs, c.r, c.r32, c.rh32,
                                                    c.p32, c.v32, c.msR, part, sweeps == 0, nullptr, x0_zero);
        else
            k_residual<double><<<gq, kBlock * kLatLanes, 0, s>>>(c.P, tl, c.A.band, c.F.nbr, c.A.x, c.A.rhs, c.r, c.r, c.rh,
                                                     c.p, c.v, c.msR, part, sweeps == 0, nullptr, x0_zero);
        // b, r and the Krylov vectors' resets; the bands, x and the ids
        // unless r = b (the first sweep of a zero start)
        if (sweeps == 0 && x0_zero)
            prof_end(c, s, PBSM3D_K_RESIDUAL, act * c.P.L * (c.P.mixed ? 32 : 40));
        else
            prof_end(c, s, PBSM3D_K_RESIDUAL, act * c.P.L * (c.P.mixed ? 88 : 96) + act * 12);
        int rc = read_members(c, s, c.msR);
        if (rc) return rc;
        if (sweeps == 0) {
            for (int m = 0; m < n; ++m) c.member_bb[m] = c.ms_host[m].bnorm2;
            if (c.cfg.warm_start != PBSM3D_X0_ZERO && !(c.cfg.warm_flags & 1)) {
                // Scale each member's warm start by the gamma that minimises
                // ||b - gamma A x0|| and drop it when that residual is not
                // below ||b||: the zero guess stays the fallback.
                // (b, A x0) = |b|^2 - (b, r0), |A x0|^2 = |b|^2 - 2 (b, r0) + |r0|^2.
                for (int m = 0; m < n; ++m) {
                    const double bb = c.ms_host[m].bnorm2, br = c.ms_host[m].red0, rr = c.ms_host[m].rnorm2;
                    const double bax = bb - br, axax = bb - 2.0 * br + rr;
                    double gamma = (axax > 0 && bax > 0) ? bax / axax : 0.0;
                    const double rmin2 = axax > 0 ? bb - bax * bax / axax : bb;
                    if (!(rmin2 < 0.99 * bb)) gamma = 0.0;
                    init[m] = MScal{};
                    init[m].gamma = gamma;
                    gamma_sum += gamma;
                }
                c.warm_gamma = gamma_sum / n;
                PBSM_CUDA_TRY(cudaMemcpyAsync(c.msR, init.data(), sizeof(MScal) * n, cudaMemcpyHostToDevice, s));
                prof_begin(c, s);
                if (c.P.mixed)
                    k_warm_scale<float><<<gr, kBlock, 0, s>>>(c.P, tl, c.A.x, c.r, c.A.rhs, c.r32, c.rh32, c.msR,
                                                              part);
                else
                    k_warm_scale<double><<<gr, kBlock, 0, s>>>(c.P, tl, c.A.x, c.r, c.A.rhs, c.r, c.rh, c.msR,
                                                               part);
                prof_end(c, s, PBSM3D_K_OTHER, c.P.T * c.P.L * 40);
                if ((rc = read_members(c, s, c.msR))) return rc;
                for (int m = 0; m < n; ++m) c.ms_host[m].bnorm2 = c.member_bb[m];
            }
        }
        // per-member convergence on the true FP64 residual (members skipped
        // by the residual pass keep the value they converged with)
        bool all = true, finite = true;
        double worst = 0;
        for (int m = 0; m < n; ++m) {
            const double rr = c.ms_host[m].rnorm2, bb = c.member_bb[m];
            if (!isfinite(rr)) finite = false;
            if (bb > 0) worst = std::max(worst, rr / bb);
            if (conv[m]) continue;
            if (rr <= tol * tol * bb)
                conv[m] = 1;
            else
                all = false;
        }
        c.susp_relres = sqrt(worst);
        if (!finite) {
            c.err = "suspension solve produced a non-finite residual";
            return PBSM3D_ERR_NOT_CONVERGED;
        }
        if (all) break;
        if (total_iters >= maxit) {
            c.susp_iters = total_iters;
            c.err = "suspension solve failed to converge (relative residual " + std::to_string(c.susp_relres) + ")";
            return PBSM3D_ERR_NOT_CONVERGED;
        }
        // Krylov states: converged members are done from the start
        int ndone = 0;
        for (int m = 0; m < n; ++m) {
            const double rr = c.ms_host[m].rnorm2, bb = c.member_bb[m];
            MScal q{};
            q.rho = rr;
            q.alpha = q.omega = 1.0;
            q.beta = 0.0;
            q.maxit = std::max(1, maxit - total_iters);
            if (c.P.mixed) {
                // inner: A32 d = r32, d0 = 0, to inner_tol relative -- or less when
                // the FP64 target is closer than that (no over-solving in the last sweep)
                const double goal2 = tol * tol * bb;
                const double need = rr > 0 ? 0.5 * sqrt(goal2 / rr) : 1.0;
                const double itol = std::min(0.5, std::max(c.cfg.inner_tol, need));
                q.target2 = itol * itol * rr;
            } else {
                q.target2 = tol * tol * bb;  // relative to ||b_m||
            }
            q.half = half_window(rr, q.target2);
            q.done = conv[m] || rr == 0.0 ? DONE_CONVERGED : DONE_NO;
            ndone += q.done ? 1 : 0;
            init[m] = q;
        }
        // members whose x is final skip later residual passes
        std::vector<MScal> rs(n);
        for (int m = 0; m < n; ++m) {
            rs[m] = MScal{};
            rs[m].done = conv[m] ? 1 : 0;
            rs[m].rnorm2 = c.ms_host[m].rnorm2;
        }
        MScal* ms = c.P.mixed ? c.ms1 : c.ms0;
        Scalars* sc = c.P.mixed ? sc1 : sc0;
        Scalars tot{};
        tot.done = ndone == n ? DONE_CONVERGED : DONE_NO;
        tot.counter[2] = (unsigned)ndone;
        PBSM_CUDA_TRY(cudaMemcpyAsync(ms, init.data(), sizeof(MScal) * n, cudaMemcpyHostToDevice, s));
        PBSM_CUDA_TRY(cudaMemcpyAsync(sc, &tot, sizeof(Scalars), cudaMemcpyHostToDevice, s));
        for (int m = 0; m < n; ++m) c.ms_host[m] = init[m];
        int it = 0;
        if (c.P.mixed) {
            prof_begin(c, s);
            k_zero<float><<<c.grid_faces, kBlock, 0, s>>>(c.P.R, c.x32);
            prof_end(c, s, PBSM3D_K_OTHER, c.P.T * c.P.L * 4);
            rc = bicgstab_iterations<float, float>(c, s, ms, sc, c.x32, c.r32, c.rh32, c.p32, c.v32, c.s32, c.t32,
                                                   c.zp32, c.zs32, c.nw32, c.nz32, it);
            if (rc) return rc;
            prof_begin(c, s);
            k_add_correction<<<c.grid_faces, kBlock, 0, s>>>(c.P.R, c.A.x, c.x32);
            prof_end(c, s, PBSM3D_K_OTHER, c.P.T * c.P.L * 20);
        } else {
            rc = bicgstab_iterations<double, double>(c, s, ms, sc, c.A.x, c.r, c.rh, c.p, c.v, c.sv, c.tv, c.zp,
                                                     c.zs, c.nw, c.nz, it);
            if (rc) return rc;
        }
        PBSM_CUDA_TRY(cudaMemcpyAsync(c.msR, rs.data(), sizeof(MScal) * n, cudaMemcpyHostToDevice, s));
        total_iters += it;
        sweeps++;
        if (sweeps > 64) {
            c.err = "suspension solve: refinement did not converge";
            return PBSM3D_ERR_NOT_CONVERGED;
        }
    }
    c.susp_iters = total_iters;
    c.susp_matvecs = (2 + 2 * c.cfg.neumann) * total_iters + sweeps + 1;
    c.susp_refinements = sweeps;
    return 0;
}

int configure_cg(Ctx& c) {
    int dev = 0, sms = 0, coop = 0;
    PBSM_CUDA_TRY(cudaGetDevice(&dev));
    PBSM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PBSM_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    const int64_t need = (c.P.Tp + kCgBlock - 1) / kCgBlock;
    // up to kCgBlocksPerSm co-resident blocks per SM, within the partials
    // workspace and the flag lines
    auto blocks_for = [&](const void* f, int& out) -> int {
        int per_sm = 0;
        PBSM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, kCgBlock, 0));
        int64_t b = std::min<int64_t>(need, (int64_t)std::min(per_sm, kCgBlocksPerSm) * sms);
        b = std::min<int64_t>(b, (int64_t)c.red.nblocks);
        b = std::min<int64_t>(b, (int64_t)kMaxCgBlocks);
        out = coop ? (int)b : 0;
        return 0;
    };
    int rc;
    if ((rc = blocks_for((const void*)k_cg_persistent<double>, c.coop_blocks))) return rc;
    if ((rc = blocks_for((const void*)k_cg_persistent<float>, c.coop_blocks32))) return rc;
    return 0;
}

// The deposition CG's system and work vectors, FP64 and (MIXED) FP32; the
// second residual buffer exists with dep_neumann only.
static DepSys<double> dep_sys64(Ctx& c) {
    return DepSys<double>{c.D.diag, c.D.off, c.D.dinv, c.D.rhs, c.D.x,           c.dr,
                          c.dz_,    c.dp,    c.dq,     c.dr2,  c.dscale, c.dscale + c.P.Tp};
}

static DepSys<float> dep_sys32(Ctx& c) {
    const int64_t Tp = c.P.Tp;
    float* f = c.dep32;
    return DepSys<float>{f,          f + Tp,     f + 4 * Tp, f + 5 * Tp,  f + 6 * Tp,
                         f + 7 * Tp, f + 8 * Tp, f + 9 * Tp, f + 10 * Tp, c.cfg.dep_neumann ? f + 11 * Tp : nullptr,
                         f + 12 * Tp, f + 13 * Tp};
}

// Algorithmic bytes of the persistent CG per face: each array touched once
// per phase, the neighbour gathers as reads of the same vector.  Set-up:
// 23 values + 24 B of neighbour ids; an iteration with the polynomial
// preconditioner: 20 values + 24 B of ids, with Jacobi 15 values + 12 B.
static int64_t cg_setup_bytes(int vb) { return 23 * vb + 24; }
static int64_t cg_iter_bytes(int vb, bool poly) { return poly ? 20 * vb + 24 : 15 * vb + 12; }

// One cooperative CG launch on system D; returns the status and iterations in sc.
template <typename V>
static int launch_cg(Ctx& c, cudaStream_t s, DepSys<V> D, int blocks, Scalars* sc, double tol, int maxit) {
    if (blocks <= 0) {
        c.err = "the device does not support cooperative launches";
        return PBSM3D_ERR_CUDA;
    }
    PBSM_CUDA_TRY(cudaMemsetAsync(c.cg_flags, 0, sizeof(unsigned) * kFlagStride * (size_t)blocks, s));
    PBSM_CUDA_TRY(cudaMemsetAsync(&c.gbar->err, 0, sizeof(int), s));
    int64_t Tp = c.P.Tp;
    double* part = c.red.partials;
    int* err = &c.gbar->err;
    GridWait gw{kBarrierLimitNs, -1};
    if (c.test_limit_ns) {  // armed by the timeout test, for this launch only
        gw.limit_ns = c.test_limit_ns;
        gw.withhold = std::min(std::max(c.test_withhold, 0), blocks - 1);
        c.test_limit_ns = 0;
        c.test_withhold = -1;
    }
    const MScal* dyn = nullptr;
    void* args[] = {&Tp, &D, &c.F.nbr, &part, &c.cg_flags, &err, &sc, &tol, &maxit, &gw, &dyn};
    PBSM_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_cg_persistent<V>, dim3(blocks), dim3(kCgBlock), args,
                                              0, s));
    int rc = read_scalars(c, s, sc);
    if (rc) return rc;
    int e = 0;
    PBSM_CUDA_TRY(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        c.err = "deposition solve: grid all-reduce timed out (a block's wait ran out)";
        return PBSM3D_ERR_CUDA;
    }
    return 0;
}

// MIXED: FP64 iterative refinement around FP32 CG solves of A d = r;
// x, the residual b - A x and its norm stay FP64.
static int solve_deposition_mixed(Ctx& c, cudaStream_t s, double tol) {
    double* part = c.red.partials;
    Scalars* sc = c.sc + 2;
    const int64_t T = c.P.T, Tp = c.P.Tp;
    float* f = c.dep32;
    float *diag32 = f, *off32 = f + Tp, *dinv32 = f + 4 * Tp, *r32 = f + 5 * Tp;
    DepSys<float> D32 = dep_sys32(c);
    prof_begin(c, s);
    k_dep_to_f32<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.D, diag32, off32, dinv32);
    PBSM_CUDA_TRY(cudaMemsetAsync(c.D.x, 0, Tp * sizeof(double), s));
    k_dep_resid32<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.D, c.F.nbr, r32, sc, part);
    prof_end(c, s, PBSM3D_K_CG, T * (56 + 20 + 8 + 64));
    c.launches += 1;
    int rc = read_scalars(c, s, sc);
    if (rc) return rc;
    const double bb = c.sc_host->bnorm2;
    double rr = c.sc_host->rnorm2;
    c.dep_iters = 0;
    c.dep_refinements = 0;
    for (int pass = 0; pass < 8 && !(rr <= tol * tol * bb); ++pass) {
        // inner target relative to ||r||: what the outer target still needs,
        // no tighter than FP32 reliably reaches
        const double itol = std::max(1e-5, 0.3 * tol * sqrt(bb / rr));
        prof_begin(c, s);
        if ((rc = launch_cg<float>(c, s, D32, c.coop_blocks32, sc, itol, std::min(c.cfg.dep_maxit, 500)))) return rc;
        const int inner = c.sc_host->iter;
        prof_end(c, s, PBSM3D_K_CG, T * (cg_setup_bytes(4) + (int64_t)inner * cg_iter_bytes(4, c.cfg.dep_neumann)));
        c.dep_iters += inner;
        c.dep_refinements += 1;
        prof_begin(c, s);
        k_dep_add<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.D, D32.x);
        k_dep_resid32<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.D, c.F.nbr, r32, sc, part);
        prof_end(c, s, PBSM3D_K_CG, T * (20 + 56 + 20 + 8));
        c.launches += 1;
        rc = read_scalars(c, s, sc);
        if (rc) return rc;
        rr = c.sc_host->rnorm2;
        if (!isfinite(rr)) break;
    }
    c.dep_relres = bb > 0 ? sqrt(rr / bb) : 0.0;
    if (!(rr <= tol * tol * bb)) {
        c.err = "deposition solve failed to converge (relative residual " + std::to_string(c.dep_relres) + ")";
        return PBSM3D_ERR_NOT_CONVERGED;
    }
    // the final residual vector in FP64 for the mass ledger
    prof_begin(c, s);
    k_cg_resid<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.D, c.F.nbr, c.dr, sc, part);
    prof_end(c, s, PBSM3D_K_CG, T * 76);
    return 0;
}

// Per-member CG iterations on states set up by the host (target2 = tol^2
// relative to ||b_m||, maxit, done for members not solved); returns the
// largest member iteration count.
template <typename V>
static int scg_iterations(Ctx& c, cudaStream_t s, DepSys<V> D, MScal* ms, Scalars* sc, int& iters) {
    double* part = c.tile_part;
    const int n = c.tiles.n;
    const int64_t sv_ = sizeof(V);
    std::vector<char> active(n);
    int ndone = 0;
    for (int m = 0; m < n; ++m) {
        active[m] = c.ms_host[m].done ? 0 : 1;
        ndone += c.ms_host[m].done ? 1 : 0;
    }
    Scalars tot{};
    tot.done = ndone == n ? DONE_CONVERGED : DONE_NO;
    tot.counter[2] = (unsigned)ndone;
    PBSM_CUDA_TRY(cudaMemcpyAsync(sc, &tot, sizeof(Scalars), cudaMemcpyHostToDevice, s));
    PBSM_CUDA_TRY(cudaMemcpyAsync(ms, c.ms_host, sizeof(MScal) * n, cudaMemcpyHostToDevice, s));
    int rc = set_active(c, s, active);
    if (rc) return rc;
    Tiles tl = c.tiles;
    int g = std::max(1, std::min(c.grid_cg[sizeof(V) == 4], tl.nact));
    int64_t act = active_faces(c);
    prof_begin(c, s);
    k_scg_start<V><<<g, kBlock, 0, s>>>(tl, c.P.Tp, D, c.F.nbr, ms, sc, part);
    k_scg_q<V><<<g, kBlock, 0, s>>>(tl, c.P.Tp, D, c.F.nbr, ms, sc, part);
    prof_end(c, s, PBSM3D_K_CG, act * sv_ * 17 + act * 12);
    c.launches += 1;
    int chunk = 8, before = 0;
    while (true) {
        for (int k = 0; k < chunk; ++k) {
            prof_begin(c, s);
            k_scg_x<V><<<g, kBlock, 0, s>>>(tl, c.P.Tp, D, c.F.nbr, ms, sc, part);
            k_scg_q<V><<<g, kBlock, 0, s>>>(tl, c.P.Tp, D, c.F.nbr, ms, sc, part);
            prof_end(c, s, PBSM3D_K_CG, act * sv_ * 18 + act * 12);
            c.launches += 1;
        }
        if ((rc = read_scalars(c, s, sc))) return rc;
        const int ran = c.sc_host->iter - before;
        before = c.sc_host->iter;
        const int idle = chunk - ran;
        if (idle > 0) prof_drop(c, idle);
        if (c.sc_host->done) break;
        if ((rc = read_members(c, s, ms))) return rc;
        bool changed = false;
        for (int m = 0; m < n; ++m)
            if (active[m] && c.ms_host[m].done) {
                active[m] = 0;
                changed = true;
            }
        if (changed) {
            if ((rc = set_active(c, s, active))) return rc;
            tl = c.tiles;
            g = std::max(1, std::min(c.grid_cg[sizeof(V) == 4], tl.nact));
            act = active_faces(c);
        }
        chunk = std::min(32, chunk * 2);
    }
    iters = c.sc_host->iter;
    return 0;
}

// Ensembles: every member its own CG (FP64; MIXED: FP32 inner solves in
// per-member FP64 refinement), each to ||b_m - A_m x_m|| <= tol ||b_m||.
static int solve_deposition_members(Ctx& c, cudaStream_t s, double tol) {
    const int n = c.tiles.n;
    const int64_t Tp = c.P.Tp, T = c.P.T;
    double* part = c.tile_part;
    Scalars* sc = c.sc + 2;
    std::vector<char> conv(n, 0), all_on(n, 1);
    std::vector<double> bb(n, 0.0), rr(n, 0.0);
    c.dep_iters = 0;
    c.dep_refinements = 0;
    auto residual = [&](float* r32) -> int {
        std::vector<char> a(n);
        for (int m = 0; m < n; ++m) a[m] = conv[m] ? 0 : 1;
        int rc = set_active(c, s, a);
        if (rc) return rc;
        const Tiles tl = c.tiles;
        std::vector<MScal> z(n);
        for (int m = 0; m < n; ++m) z[m].done = conv[m] ? 1 : 0;
        PBSM_CUDA_TRY(cudaMemcpyAsync(c.msR, z.data(), sizeof(MScal) * n, cudaMemcpyHostToDevice, s));
        const int g = std::max(1, std::min(c.grid_red[0], tl.nact));
        prof_begin(c, s);
        k_sdep_resid<<<g, kBlock, 0, s>>>(tl, c.P, c.D, c.F.nbr, r32, c.dr, c.msR, part);
        prof_end(c, s, PBSM3D_K_CG, active_faces_of(c, conv) * (76 + (r32 ? 4 : 0)));
        if ((rc = read_members(c, s, c.msR))) return rc;
        for (int m = 0; m < n; ++m)
            if (!conv[m]) {
                rr[m] = c.ms_host[m].rnorm2;
                bb[m] = c.ms_host[m].bnorm2;
            }
        return 0;
    };
    auto finish = [&]() -> int {
        double worst = 0;
        bool ok = true;
        for (int m = 0; m < n; ++m) {
            if (bb[m] > 0) worst = std::max(worst, rr[m] / bb[m]);
            if (!(rr[m] <= tol * tol * bb[m])) ok = false;
        }
        c.dep_relres = sqrt(worst);
        if (!ok) {
            c.err = "deposition solve failed to converge (relative residual " + std::to_string(c.dep_relres) + ")";
            return PBSM3D_ERR_NOT_CONVERGED;
        }
        return 0;
    };
    int rc;
    if (!c.P.mixed) {
        DepSys<double> D = dep_sys64(c);
        for (int m = 0; m < n; ++m) {
            c.ms_host[m] = MScal{};
            c.ms_host[m].target2 = tol * tol;
            c.ms_host[m].maxit = c.cfg.dep_maxit;
        }
        int it = 0;
        if ((rc = scg_iterations<double>(c, s, D, c.ms0, sc, it))) return rc;
        c.dep_iters = it;
        c.dep_refinements = 1;
        // the true residual (also the mass ledger's residual vector)
        if ((rc = residual(nullptr))) return rc;
        return finish();
    }
    float* f = c.dep32;
    float *diag32 = f, *off32 = f + Tp, *dinv32 = f + 4 * Tp, *r32 = f + 5 * Tp;
    DepSys<float> D32 = dep_sys32(c);
    prof_begin(c, s);
    k_dep_to_f32<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.D, diag32, off32, dinv32);
    prof_end(c, s, PBSM3D_K_CG, T * (56 + 20));
    PBSM_CUDA_TRY(cudaMemsetAsync(c.D.x, 0, Tp * sizeof(double), s));
    for (int pass = 0;; ++pass) {
        if ((rc = residual(r32))) return rc;
        bool all = true;
        for (int m = 0; m < n; ++m) {
            if (!conv[m] && rr[m] <= tol * tol * bb[m]) conv[m] = 1;
            if (!conv[m]) all = false;
        }
        if (all || pass == 8) break;
        for (int m = 0; m < n; ++m) {
            c.ms_host[m] = MScal{};
            if (conv[m]) {
                c.ms_host[m].done = DONE_CONVERGED;
                continue;
            }
            // inner target relative to ||r_m||: what the outer target still
            // needs, no tighter than FP32 reliably reaches
            const double itol = std::max(1e-5, 0.3 * tol * sqrt(bb[m] / rr[m]));
            c.ms_host[m].target2 = itol * itol;
            c.ms_host[m].maxit = std::min(c.cfg.dep_maxit, 500);
        }
        PBSM_CUDA_TRY(cudaMemsetAsync(D32.x, 0, Tp * sizeof(float), s));
        int it = 0;
        if ((rc = scg_iterations<float>(c, s, D32, c.ms1, sc, it))) return rc;
        c.dep_iters += it;
        c.dep_refinements += 1;
        prof_begin(c, s);
        k_dep_add<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.D, D32.x);
        prof_end(c, s, PBSM3D_K_CG, T * 20);
    }
    // converged members kept the residual vector of their last pass
    return finish();
}

int solve_deposition(Ctx& c, cudaStream_t s, pbsm3d_stats* st) {
    (void)st;
    if (c.tiles.n > 1) return solve_deposition_members(c, s, c.cfg.dep_tol);
    const double tol = c.cfg.dep_tol;
    if (c.P.mixed) return solve_deposition_mixed(c, s, tol);
    c.dep_refinements = 1;
    double* part = c.red.partials;
    Scalars* sc = c.sc + 2;
    const int64_t T = c.P.T;
    DepSys<double> D = dep_sys64(c);
    prof_begin(c, s);
    int rc = launch_cg<double>(c, s, D, c.coop_blocks, sc, tol, c.cfg.dep_maxit);
    if (rc) return rc;
    const int done = c.sc_host->done;
    c.dep_iters = c.sc_host->iter;
    prof_end(c, s, PBSM3D_K_CG, T * (cg_setup_bytes(8) + (int64_t)c.dep_iters * cg_iter_bytes(8, c.cfg.dep_neumann)));
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

// ---------------------------------------------------------------- graph mode
// The device part of a step as one CUDA-graph launch.  The decisions the
// host makes between launches in the default path (the "present" tests, the
// per-member convergence and inner targets of the refinement sweeps, the
// warm-start scale, the active-tile list, the end of each Krylov loop) are
// made by one-block controller kernels, which steer conditional IF/WHILE
// nodes with cudaGraphSetConditional.  Every loop has a device-side cap:
// Krylov loops stop at their iteration limits, the refinement loops after
// 64 (suspension) or 8 (deposition) sweeps, and a guard counter over all
// loop bodies ends every loop and records an error past kGuardMax.  The
// deposition solve of one mesh is the host path's cooperative CG kernel (its
// own loop, bounded by its iteration limit and its waits); an ensemble's is
// the per-member tile CG.

namespace {

constexpr int kGuardMax = 200000;

constexpr int kGraphStamps = 6;

struct StepCtl {
    int ok, err;  // err: PBSM3D_ERR_* of the failure, 0 while ok
    int susp_present, dep_present;
    int sweep, susp_iters, dep_iters, dep_sweeps;
    int guard, n_active;
    int kernels;  // kernels the graph executed this step (tallied by the controllers)
    double susp_relres, dep_relres, susp_rhs_max, dep_rhs_max, gamma_sum;
    // with profiling on: %globaltimer at the phase boundaries (start, after
    // the assembly, the suspension solve, the post and deposition assembly,
    // the deposition solve, the update); 0 where a phase did not run
    unsigned long long stamp[kGraphStamps];
    int conv[kMaxMembers], dconv[kMaxMembers];
    double bb[kMaxMembers], dbb[kMaxMembers];
};

// A phase boundary of the step graph, stamped from the device clock by a
// one-thread kernel (kernel nodes are allowed inside conditional bodies,
// event-record nodes are not).  Slot 0 also clears the others.
__global__ void k_stamp(StepCtl* ctl, int slot) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (slot == 0)
        for (int k = 1; k < kGraphStamps; ++k) ctl->stamp[k] = 0;
    ctl->stamp[slot] = t;
}

// The conditional handles of the step graph.  A form without a warm start
// or without the mixed deposition refinement has no node for those handles;
// `valid` marks the ones that exist, and only those are ever set.
enum HandleId { H_OK1, H_SUSP, H_OUTER, H_WARM, H_INNER, H_ILOOP, H_OK2, H_DEP, H_DOUTER, H_DINNER, H_DLOOP, H_OK3,
                H_COUNT };
struct Handles {
    cudaGraphConditionalHandle h[H_COUNT];
    unsigned valid;
};

__device__ __forceinline__ void hset(const Handles& h, int id, unsigned v) {
    if (h.valid & (1u << id)) cudaGraphSetConditional(h.h[id], v);
}

__device__ __forceinline__ void stop_all(const Handles& h) {
    for (int id : {H_OUTER, H_INNER, H_ILOOP, H_WARM, H_DOUTER, H_DINNER, H_DLOOP}) hset(h, id, 0u);
}

// One block: the active-tile list of the members with active[m] != 0 (in
// shared memory, filled by the caller), in member order.
__device__ void ctl_build_act(const Tiles& tl, int32_t* act, int* nact, const int* active) {
    __shared__ int first[kMaxMembers + 1];
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int m = 0; m < tl.n; ++m) {
            first[m] = acc;
            if (active[m]) acc += tl.mtile[m + 1] - tl.mtile[m];
        }
        first[tl.n] = acc;
        *nact = acc;
    }
    __syncthreads();
    const int total = first[tl.n];
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
        // the last member whose first position is <= q; it holds position q
        // (a member without tiles in the list shares its start with the next)
        int lo = 0, hi = tl.n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (first[mid] <= q) lo = mid;
            else hi = mid - 1;
        }
        act[q] = tl.mtile[lo] + (q - first[lo]);
    }
    __syncthreads();
}

// After the suspension assembly: NaN check, per-member "present" tests.
__global__ void k_ctl_begin(StepCtl* ctl, const Scalars* sc0, Members Mb, int n, int asm_kernels, Handles h) {
    if (threadIdx.x != 0) return;
    const bool nan = sc0->nan_flag != 0.0;
    bool any = false;
    if (n == 1) {
        any = sc0->rhs_max > 1e-12;  // PBSM3D.cpp:1424-1427
    } else {
        for (int m = 0; m < n; ++m) {
            const double v = __longlong_as_double((long long)Mb.rhs_max[m]);
            Mb.susp_present[m] = v > 1e-12;
            any = any || Mb.susp_present[m];
        }
    }
    ctl->ok = !nan;
    ctl->err = nan ? PBSM3D_ERR_NAN_INPUT : 0;
    ctl->susp_present = any;
    ctl->dep_present = 0;
    ctl->susp_rhs_max = sc0->rhs_max;
    ctl->sweep = ctl->susp_iters = ctl->dep_iters = ctl->dep_sweeps = ctl->guard = 0;
    ctl->kernels = asm_kernels + 1 + (n > 1 ? 1 : 0);  // the assembly passes, this, the member mask
    ctl->susp_relres = ctl->dep_relres = ctl->gamma_sum = 0.0;
    hset(h, H_OK1, nan ? 0u : 1u);
    hset(h, H_SUSP, (!nan && any) ? 1u : 0u);
    hset(h, H_OK3, nan ? 0u : 1u);
}

// Start of the suspension solve: every member active, residual states clear.
__global__ void k_ctl_solve_init(StepCtl* ctl, MScal* msR, Tiles tl, int32_t* act, int* nact, int warm, int start_kernels,
                                 Handles h) {
    __shared__ int active[kMaxMembers];
    for (int m = threadIdx.x; m < tl.n; m += blockDim.x) {
        msR[m] = MScal{};
        active[m] = 1;
        ctl->conv[m] = 0;
    }
    ctl_build_act(tl, act, nact, active);
    if (threadIdx.x == 0) {
        ctl->kernels += 1 + start_kernels;
        hset(h, H_OUTER, 1u);
        hset(h, H_WARM, warm ? 1u : 0u);
    }
}

// Sweep 0 with a warm start: the residual-optimal scale per member
// (gamma = 0 keeps the zero guess), as the host path computes it.
__global__ void k_ctl_gamma(StepCtl* ctl, MScal* msR, int n) {
    if (threadIdx.x != 0) return;
    double gs = 0.0;
    for (int m = 0; m < n; ++m) {
        const double bb = msR[m].bnorm2, br = msR[m].red0, rr = msR[m].rnorm2;
        const double bax = bb - br, axax = bb - 2.0 * br + rr;
        double gamma = (axax > 0 && bax > 0) ? bax / axax : 0.0;
        const double rmin2 = axax > 0 ? bb - bax * bax / axax : bb;
        if (!(rmin2 < 0.99 * bb)) gamma = 0.0;
        msR[m].gamma = gamma;
        ctl->bb[m] = bb;  // ||b_m||^2 before the scaling pass overwrites nothing else
        gs += gamma;
    }
    ctl->gamma_sum = gs;
    ctl->kernels += 2;  // this and the scaling pass
}

// After a residual pass: per-member convergence on the true FP64 residual,
// then either the end of the solve or the next inner solve's states.
__global__ void k_ctl_outer(StepCtl* ctl, MScal* msR, MScal* ms, Scalars* sc, Tiles tl, int32_t* act, int* nact,
                            double tol, double inner_tol, int maxit, int mixed, Handles h) {
    __shared__ int active[kMaxMembers];
    __shared__ int s_all, s_finite, s_go;
    const int n = tl.n;
    if (threadIdx.x == 0) {
        s_all = 1;
        s_finite = 1;
    }
    __syncthreads();
    for (int m = threadIdx.x; m < n; m += blockDim.x) {
        if (ctl->sweep == 0) ctl->bb[m] = msR[m].bnorm2;
        const double rr = msR[m].rnorm2, bb = ctl->bb[m];
        if (!isfinite(rr)) atomicExch(&s_finite, 0);
        if (!ctl->conv[m] && rr <= tol * tol * bb) ctl->conv[m] = 1;
        if (!ctl->conv[m]) atomicExch(&s_all, 0);
        active[m] = !ctl->conv[m];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double worst = 0.0;
        for (int m = 0; m < n; ++m)
            if (ctl->bb[m] > 0) worst = fmax(worst, msR[m].rnorm2 / ctl->bb[m]);
        ctl->susp_relres = sqrt(worst);
        ctl->kernels += 2;  // the residual pass and this
        hset(h, H_WARM, 0u);
        int go = 0;
        if (!s_finite || ++ctl->guard > kGuardMax) {
            ctl->ok = 0;
            ctl->err = PBSM3D_ERR_NOT_CONVERGED;
        } else if (!s_all) {
            if (ctl->susp_iters >= maxit || ctl->sweep > 64) {
                ctl->ok = 0;
                ctl->err = PBSM3D_ERR_NOT_CONVERGED;
            } else {
                go = 1;
            }
        }
        s_go = go;
        if (!go) {
            hset(h, H_OUTER, 0u);
            hset(h, H_INNER, 0u);
            hset(h, H_ILOOP, 0u);
            if (!ctl->ok) {
                stop_all(h);
                hset(h, H_OK3, 0u);
            }
        }
    }
    __syncthreads();
    if (!s_go) return;
    __shared__ int s_ndone;
    if (threadIdx.x == 0) s_ndone = 0;
    __syncthreads();
    for (int m = threadIdx.x; m < n; m += blockDim.x) {
        const double rr = msR[m].rnorm2, bb = ctl->bb[m];
        MScal q{};
        q.rho = rr;
        q.alpha = q.omega = 1.0;
        q.beta = 0.0;
        q.maxit = max(1, maxit - ctl->susp_iters);
        if (mixed) {
            const double goal2 = tol * tol * bb;
            const double need = rr > 0 ? 0.5 * sqrt(goal2 / rr) : 1.0;
            const double itol = fmin(0.5, fmax(inner_tol, need));
            q.target2 = itol * itol * rr;
        } else {
            q.target2 = tol * tol * bb;
        }
        q.half = half_window(rr, q.target2);
        q.done = (ctl->conv[m] || rr == 0.0) ? 1 : 0;
        if (q.done) {
            atomicAdd(&s_ndone, 1);
            active[m] = 0;
        }
        ms[m] = q;
        msR[m].done = ctl->conv[m];
        msR[m].counter = 0u;
    }
    ctl_build_act(tl, act, nact, active);
    if (threadIdx.x == 0) {
        sc->done = s_ndone == n ? 1 : 0;
        sc->counter[2] = (unsigned)s_ndone;
        sc->counter[3] = 0u;
        sc->iter = 0;
        ctl->n_active = n - s_ndone;
        hset(h, H_OUTER, 1u);
        hset(h, H_INNER, 1u);
        hset(h, H_ILOOP, s_ndone == n ? 0u : 1u);
    }
}

// After each batched Krylov iteration: stop the loop when every member is
// done; members that stopped leave the active-tile list.
__global__ void k_ctl_inner(StepCtl* ctl, const MScal* ms, const Scalars* sc, Tiles tl, int32_t* act, int* nact,
                            int loop, int body_kernels, Handles h) {
    __shared__ int active[kMaxMembers];
    __shared__ int s_rebuild;
    if (threadIdx.x == 0) {
        s_rebuild = 0;
        ctl->kernels += body_kernels;
        if (sc->done || ++ctl->guard > kGuardMax) {
            hset(h, loop, 0u);
            if (ctl->guard > kGuardMax) {
                ctl->ok = 0;
                ctl->err = PBSM3D_ERR_NOT_CONVERGED;
                stop_all(h);
                hset(h, H_OK3, 0u);
            }
        } else if (tl.n > 1 && ctl->n_active != tl.n - (int)sc->counter[2]) {
            s_rebuild = 1;
            ctl->n_active = tl.n - (int)sc->counter[2];
        }
    }
    __syncthreads();
    if (!s_rebuild) return;
    for (int m = threadIdx.x; m < tl.n; m += blockDim.x) active[m] = ms[m].done ? 0 : 1;
    ctl_build_act(tl, act, nact, active);
}

// End of a refinement sweep of the suspension solve: count the iterations;
// the next residual pass covers the members not yet converged.
__global__ void k_ctl_sweep_end(StepCtl* ctl, const Scalars* sc, Tiles tl, int32_t* act, int* nact, int extra) {
    __shared__ int active[kMaxMembers];
    for (int m = threadIdx.x; m < tl.n; m += blockDim.x) active[m] = !ctl->conv[m];
    ctl_build_act(tl, act, nact, active);
    if (threadIdx.x == 0) {
        ctl->susp_iters += sc->iter;
        ctl->sweep += 1;
        ctl->kernels += 1 + extra;
    }
}

// After the deposition assembly: NaN check and the "present" tests.
__global__ void k_ctl_dep_begin(StepCtl* ctl, const Scalars* sc0, Members Mb, int n, int tail_kernels, Handles h) {
    if (threadIdx.x != 0) return;
    ctl->kernels += 3 + (n > 1 ? 1 : 0) + tail_kernels;  // post, deposition rows, this, mask; update
    const bool nan = sc0->nan_flag != 0.0;
    bool any = false;
    if (n == 1) {
        any = ctl->susp_present && sc0->rhs_max > 1e-12;  // PBSM3D.cpp:1661-1664
    } else {
        for (int m = 0; m < n; ++m) {
            const double v = __longlong_as_double((long long)Mb.dep_max[m]);
            Mb.dep_present[m] = v > 1e-12 && Mb.susp_present[m];
            any = any || Mb.dep_present[m];
        }
    }
    ctl->dep_rhs_max = sc0->rhs_max;
    if (nan) {
        ctl->ok = 0;
        ctl->err = PBSM3D_ERR_NAN_INPUT;
    }
    ctl->dep_present = any && !nan;
    hset(h, H_DEP, (!nan && any) ? 1u : 0u);
    hset(h, H_OK3, ctl->ok ? 1u : 0u);
}

// After the suspension solve: a failed solve ends the step, as the host path
// returns before the column post touches any state.
__global__ void k_ctl_mid(StepCtl* ctl, Handles h) {
    if (threadIdx.x != 0) return;
    ctl->kernels += 1;
    hset(h, H_OK2, ctl->ok ? 1u : 0u);
}

// Start of the step graph's second part: part 1's outcome in the control
// block opens this part's conditional nodes (the deposition solve when the
// step is ok and a deposition system is present, the update when ok).
__global__ void k_ctl_part2(StepCtl* ctl, Handles h) {
    if (threadIdx.x != 0) return;
    ctl->kernels += 1;
    const bool ok = ctl->ok != 0;
    hset(h, H_OK2, ok ? 1u : 0u);
    hset(h, H_DEP, ok && ctl->dep_present ? 1u : 0u);
    hset(h, H_OK3, ok ? 1u : 0u);
}

// Deposition CG states (plain: target tol relative to ||b_m||; mixed inner:
// itol relative to ||r_m||), all members active unless converged.
__global__ void k_ctl_dcg_init(StepCtl* ctl, MScal* ms, Scalars* sc, Tiles tl, int32_t* act, int* nact, double tol,
                               int maxit, Handles h) {
    __shared__ int active[kMaxMembers];
    for (int m = threadIdx.x; m < tl.n; m += blockDim.x) {
        MScal q{};
        q.target2 = tol * tol;
        q.maxit = maxit;
        ms[m] = q;
        active[m] = 1;
    }
    ctl_build_act(tl, act, nact, active);
    if (threadIdx.x == 0) {
        sc->done = 0;
        sc->counter[2] = 0u;
        sc->iter = 0;
        ctl->n_active = tl.n;
        ctl->kernels += 3;  // this, the CG start and its first q
        hset(h, H_DLOOP, 1u);
    }
}

// The per-member CG's residual pass: every member (plain) or the members
// not yet converged (mixed) get a fresh residual sum.
__global__ void k_ctl_dres_init(StepCtl* ctl, MScal* msR, Tiles tl, int32_t* act, int* nact, int only_open) {
    __shared__ int active[kMaxMembers];
    for (int m = threadIdx.x; m < tl.n; m += blockDim.x) {
        const int open = only_open ? !ctl->dconv[m] : 1;
        MScal q{};
        q.done = open ? 0 : 1;
        q.rnorm2 = msR[m].rnorm2;
        msR[m] = q;
        active[m] = open;
    }
    ctl_build_act(tl, act, nact, active);
    if (threadIdx.x == 0) ctl->kernels += 2;  // this and the residual pass
}

// End of the plain deposition solve: every member's true residual.
// cg_err: the cooperative CG's error word (null for the tile CG); set when
// one of its bounded grid waits ran out.
__global__ void k_ctl_dep_end(StepCtl* ctl, const MScal* msR, const Scalars* sc, int n, double tol,
                              const int* cg_err, Handles h) {
    if (threadIdx.x != 0) return;
    double worst = 0.0;
    bool ok = true;
    for (int m = 0; m < n; ++m) {
        const double rr = msR[m].rnorm2, bb = msR[m].bnorm2;
        if (bb > 0) worst = fmax(worst, rr / bb);
        if (!(rr <= tol * tol * bb)) ok = false;
    }
    ctl->dep_relres = sqrt(worst);
    ctl->dep_iters = sc->iter;
    ctl->dep_sweeps = 1;
    ctl->kernels += cg_err ? 2 : 1;  // this (and the cooperative CG)
    const bool timed_out = cg_err && *(volatile const int*)cg_err;
    if (!ok || timed_out) {
        ctl->ok = 0;
        ctl->err = timed_out ? PBSM3D_ERR_CUDA : PBSM3D_ERR_NOT_CONVERGED;
        hset(h, H_OK3, 0u);
    }
}

// Mixed deposition: start of the refinement (x = 0, nothing converged).
__global__ void k_ctl_dmix_init(StepCtl* ctl, MScal* msR, Tiles tl, int32_t* act, int* nact, Handles h) {
    __shared__ int active[kMaxMembers];
    for (int m = threadIdx.x; m < tl.n; m += blockDim.x) {
        ctl->dconv[m] = 0;
        msR[m] = MScal{};
        active[m] = 1;
    }
    ctl_build_act(tl, act, nact, active);
    if (threadIdx.x == 0) {
        ctl->dep_sweeps = 0;
        ctl->dep_iters = 0;
        ctl->kernels += 2;  // the FP32 copy and this
        hset(h, H_DOUTER, 1u);
    }
}

// Mixed deposition, after a residual pass: convergence per member, then the
// next FP32 inner solve's states or the end of the refinement.
// `solve_kernels`: the kernels of one inner solve before its first loop
// pass (zero, CG start, first q), or 1 for the cooperative CG.
__global__ void k_ctl_dmix_outer(StepCtl* ctl, MScal* msR, MScal* ms, Scalars* sc, Tiles tl, int32_t* act,
                                 int* nact, double tol, int maxit, int solve_kernels, Handles h) {
    __shared__ int active[kMaxMembers];
    __shared__ int s_all, s_go;
    const int n = tl.n;
    if (threadIdx.x == 0) s_all = 1;
    __syncthreads();
    for (int m = threadIdx.x; m < n; m += blockDim.x) {
        if (ctl->dep_sweeps == 0) ctl->dbb[m] = msR[m].bnorm2;
        const double rr = msR[m].rnorm2, bb = ctl->dbb[m];
        if (!ctl->dconv[m] && rr <= tol * tol * bb) ctl->dconv[m] = 1;
        if (!ctl->dconv[m]) atomicExch(&s_all, 0);
        active[m] = !ctl->dconv[m];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double worst = 0.0;
        for (int m = 0; m < n; ++m)
            if (ctl->dbb[m] > 0) worst = fmax(worst, msR[m].rnorm2 / ctl->dbb[m]);
        ctl->dep_relres = sqrt(worst);
        ctl->kernels += 2;  // the residual pass and this
        int go = !s_all;
        if (go && (ctl->dep_sweeps >= 8 || ++ctl->guard > kGuardMax)) {
            go = 0;
            ctl->ok = 0;
            ctl->err = PBSM3D_ERR_NOT_CONVERGED;
            stop_all(h);
            hset(h, H_OK3, 0u);
        }
        s_go = go;
        if (!go) {
            hset(h, H_DOUTER, 0u);
            hset(h, H_DINNER, 0u);
            hset(h, H_DLOOP, 0u);
        }
    }
    __syncthreads();
    if (!s_go) return;
    for (int m = threadIdx.x; m < n; m += blockDim.x) {
        MScal q{};
        if (ctl->dconv[m]) {
            q.done = 1;
        } else {
            const double rr = msR[m].rnorm2, bb = ctl->dbb[m];
            const double itol = fmax(1e-5, 0.3 * tol * sqrt(bb / rr));
            q.target2 = itol * itol;
            q.maxit = maxit;
        }
        ms[m] = q;
    }
    ctl_build_act(tl, act, nact, active);
    if (threadIdx.x == 0) {
        int nd = 0;
        for (int m = 0; m < n; ++m) nd += ctl->dconv[m] ? 1 : 0;
        sc->done = 0;
        sc->counter[2] = (unsigned)nd;
        sc->iter = 0;
        ctl->n_active = n - nd;
        ctl->kernels += solve_kernels;
        hset(h, H_DOUTER, 1u);
        hset(h, H_DINNER, 1u);
        hset(h, H_DLOOP, 1u);
    }
}

// Mixed deposition: end of an inner solve (cg_err as in k_ctl_dep_end: a
// timed-out cooperative CG ends the refinement with an error).
__global__ void k_ctl_dmix_sweep_end(StepCtl* ctl, const Scalars* sc, MScal* msR, Tiles tl, int32_t* act, int* nact,
                                     const int* cg_err, Handles h) {
    __shared__ int active[kMaxMembers];
    for (int m = threadIdx.x; m < tl.n; m += blockDim.x) {
        active[m] = !ctl->dconv[m];
        msR[m].done = ctl->dconv[m];
        msR[m].counter = 0u;
    }
    ctl_build_act(tl, act, nact, active);
    if (threadIdx.x == 0) {
        ctl->dep_iters += sc->iter;
        ctl->dep_sweeps += 1;
        ctl->kernels += 2;  // the correction and this
        if (cg_err && *(volatile const int*)cg_err) {
            ctl->ok = 0;
            ctl->err = PBSM3D_ERR_CUDA;
            stop_all(h);
            hset(h, H_OK3, 0u);
        }
    }
}

}  // namespace

struct StepGraph {
    cudaGraph_t graph = nullptr;  // part 1: assembly through the post
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph2 = nullptr;  // part 2: deposition solve and update
    cudaGraphExec_t exec2 = nullptr;
    double dt = -1.0;
    bool own_snow = false;
    StepCtl* ctl = nullptr;      // device
    StepCtl* ctl_host = nullptr;  // pinned
    int* nact = nullptr;         // device
    cudaStream_t cap[8] = {};
    bool profiled = false;       // captured with the phase stamps
};

namespace {

// Conditional node at the current capture point of stream s; its body graph
// is captured on stream t until the returned guard ends it.
struct CondBody {
    cudaStream_t t = nullptr;
    bool open = false;
    int begin(cudaStream_t s, cudaStream_t t_, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type) {
        t = t_;
        cudaStreamCaptureStatus st;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        cudaGraph_t g;
        if (cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess) return 1;
        cudaGraphNodeParams p = {};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = type;
        p.conditional.size = 1;
        cudaGraphNode_t node;
        if (cudaGraphAddNode(&node, g, deps, nullptr, nd, &p) != cudaSuccess) return 1;
        if (cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
            return 1;
        if (cudaStreamBeginCaptureToGraph(t, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeRelaxed) != cudaSuccess)
            return 1;
        open = true;
        return 0;
    }
    int end() {
        if (!open) return 0;
        open = false;
        cudaGraph_t g;
        return cudaStreamEndCapture(t, &g) != cudaSuccess;
    }
};

// The batched BiCGStab iteration (the five kernels of bicgstab_iterations).
template <typename V, typename X>
void capture_bicg_iteration(Ctx& c, cudaStream_t s, const Tiles& tl, MScal* ms, Scalars* sc, X* x, V* r, V* rh,
                            V* p, V* v, V* sv, V* tv, V* zp, V* zs, V* nw, V* nz) {
    Op<V> op = make_op<V>(c);
    const int gr = std::max(1, std::min(c.grid_red[sizeof(V) == 4], tl.ntiles));
    const int gl = std::max(1, std::min(c.grid_lat[sizeof(V) == 4], tl.ntiles));
    double* part = c.tile_part;
    launch_col_p<V>(c, s, op, tl, c.geom, r, p, v, neumann_first(c, zp, nz), ms);
    const V* up = launch_neumann<V>(c, s, op, tl, c.geom, p, zp, nw, nz, ms, 0, false);
    k_bicg_v<V><<<gl, kBlock * kLatLanes, 0, s>>>(op, tl, up, zp, v, rh, r, ms, sc, part);
    launch_col_s<V>(c, s, op, tl, c.geom, r, v, sv, neumann_first(c, zs, nz), ms, x, zp);
    const V* us = launch_neumann<V>(c, s, op, tl, c.geom, sv, zs, nw, nz, ms, 0, false);
    k_bicg_t2<V><<<gl, kBlock * kLatLanes, 0, s>>>(op, tl, us, zs, tv, sv, ms, part);
    k_bicg_x<V, X><<<gr, kBlock, 0, s>>>(c.P.Tp, c.P.L, tl, x, zp, zs, sv, tv, r, rh, ms, sc, part);
}

// The suspension solve (inside IF susp).
template <typename V>
int capture_suspension(Ctx& c, StepGraph& G, const Handles& h, int depth, const Tiles& tl) {
    cudaStream_t s = G.cap[depth];
    const int n = tl.n;
    const int gr = std::max(1, std::min(c.grid_red[0], tl.ntiles));
    const int gq = std::max(1, std::min(c.grid_res, tl.ntiles));
    double* part = c.tile_part;
    const bool mixed = c.P.mixed;
    const int warm = c.cfg.warm_start != PBSM3D_X0_ZERO && !(c.cfg.warm_flags & 1);
    const int x0_zero = c.cfg.warm_start == PBSM3D_X0_ZERO ? 1 : 0;
    MScal* ms = mixed ? c.ms1 : c.ms0;
    Scalars* sc = mixed ? c.sc + 1 : c.sc;
    const int start_kernels = (c.cfg.warm_start == PBSM3D_X0_LEARNED ? ((c.cfg.warm_flags & 2) ? 1 : 2) : 0) +
                              ((n > 1 && c.cfg.warm_start != PBSM3D_X0_ZERO) ? 1 : 0);
    k_ctl_solve_init<<<1, kBlock, 0, s>>>(G.ctl, c.msR, tl, c.act_buf, G.nact, warm, start_kernels, h);
    CondBody outer;
    if (outer.begin(s, G.cap[depth + 1], h.h[H_OUTER], cudaGraphCondTypeWhile)) return 1;
    {
        cudaStream_t t = G.cap[depth + 1];
        if (mixed)
            k_residual<float><<<gq, kBlock * kLatLanes, 0, t>>>(c.P, tl, c.A.band, c.F.nbr, c.A.x, c.A.rhs, c.r, c.r32, c.rh32,
                                                    c.p32, c.v32, c.msR, part, 1, &G.ctl->sweep, x0_zero);
        else
            k_residual<double><<<gq, kBlock * kLatLanes, 0, t>>>(c.P, tl, c.A.band, c.F.nbr, c.A.x, c.A.rhs, c.r, c.r, c.rh, c.p,
                                                     c.v, c.msR, part, 1, &G.ctl->sweep, x0_zero);
        if (warm) {
            CondBody wb;
            if (wb.begin(t, G.cap[depth + 2], h.h[H_WARM], cudaGraphCondTypeIf)) return 1;
            cudaStream_t u = G.cap[depth + 2];
            k_ctl_gamma<<<1, 32, 0, u>>>(G.ctl, c.msR, n);
            if (mixed)
                k_warm_scale<float><<<gr, kBlock, 0, u>>>(c.P, tl, c.A.x, c.r, c.A.rhs, c.r32, c.rh32, c.msR, part);
            else
                k_warm_scale<double><<<gr, kBlock, 0, u>>>(c.P, tl, c.A.x, c.r, c.A.rhs, c.r, c.rh, c.msR, part);
            if (wb.end()) return 1;
        }
        k_ctl_outer<<<1, kBlock, 0, t>>>(G.ctl, c.msR, ms, sc, tl, c.act_buf, G.nact, c.cfg.susp_tol,
                                         c.cfg.inner_tol, c.cfg.susp_maxit, mixed ? 1 : 0, h);
        CondBody inner;
        if (inner.begin(t, G.cap[depth + 2], h.h[H_INNER], cudaGraphCondTypeIf)) return 1;
        {
            cudaStream_t u = G.cap[depth + 2];
            if (mixed) k_zero<float><<<c.grid_faces, kBlock, 0, u>>>(c.P.R, c.x32);
            CondBody loop;
            if (loop.begin(u, G.cap[depth + 3], h.h[H_ILOOP], cudaGraphCondTypeWhile)) return 1;
            cudaStream_t w = G.cap[depth + 3];
            if (mixed)
                capture_bicg_iteration<float, float>(c, w, tl, ms, sc, c.x32, c.r32, c.rh32, c.p32, c.v32, c.s32,
                                                     c.t32, c.zp32, c.zs32, c.nw32, c.nz32);
            else
                capture_bicg_iteration<double, double>(c, w, tl, ms, sc, c.A.x, c.r, c.rh, c.p, c.v, c.sv, c.tv,
                                                       c.zp, c.zs, c.nw, c.nz);
            k_ctl_inner<<<1, kBlock, 0, w>>>(G.ctl, ms, sc, tl, c.act_buf, G.nact, H_ILOOP,
                                             6 + 2 * c.cfg.neumann, h);
            if (loop.end()) return 1;
            if (mixed) k_add_correction<<<c.grid_faces, kBlock, 0, u>>>(c.P.R, c.A.x, c.x32);
            k_ctl_sweep_end<<<1, kBlock, 0, u>>>(G.ctl, sc, tl, c.act_buf, G.nact, mixed ? 2 : 0);
        }
        if (inner.end()) return 1;
    }
    return outer.end();
}

// One per-member CG on system D (states set by a controller before).
template <typename V>
int capture_scg(Ctx& c, StepGraph& G, const Handles& h, int depth, const Tiles& tl, DepSys<V> D, MScal* ms,
                Scalars* sc) {
    cudaStream_t s = G.cap[depth];
    const int g = std::max(1, std::min(c.grid_cg[sizeof(V) == 4], tl.ntiles));
    double* part = c.tile_part;
    k_scg_start<V><<<g, kBlock, 0, s>>>(tl, c.P.Tp, D, c.F.nbr, ms, sc, part);
    k_scg_q<V><<<g, kBlock, 0, s>>>(tl, c.P.Tp, D, c.F.nbr, ms, sc, part);
    CondBody loop;
    if (loop.begin(s, G.cap[depth + 1], h.h[H_DLOOP], cudaGraphCondTypeWhile)) return 1;
    cudaStream_t t = G.cap[depth + 1];
    // two CG iterations per pass of the loop body, one controller: a member
    // that stops in the first is skipped by the second (its scalars say done)
    for (int k = 0; k < 2; ++k) {
        k_scg_x<V><<<g, kBlock, 0, t>>>(tl, c.P.Tp, D, c.F.nbr, ms, sc, part);
        k_scg_q<V><<<g, kBlock, 0, t>>>(tl, c.P.Tp, D, c.F.nbr, ms, sc, part);
    }
    k_ctl_inner<<<1, kBlock, 0, t>>>(G.ctl, ms, sc, tl, c.act_buf, G.nact, H_DLOOP, 5, h);
    return loop.end();
}

// The single-mesh CG as one cooperative kernel node (the host path's
// kernel; cooperative launches are allowed in conditional bodies): the
// flags and the error word are cleared by memset nodes before it.
template <typename V>
int capture_pcg(Ctx& c, cudaStream_t s, DepSys<V> D, int blocks, Scalars* sc, double tol, int maxit,
                const MScal* dyn) {
    if (cudaMemsetAsync(c.cg_flags, 0, sizeof(unsigned) * kFlagStride * (size_t)blocks, s) != cudaSuccess) return 1;
    if (cudaMemsetAsync(&c.gbar->err, 0, sizeof(int), s) != cudaSuccess) return 1;
    int64_t Tp = c.P.Tp;
    double* part = c.red.partials;
    int* err = &c.gbar->err;
    GridWait gw{kBarrierLimitNs, -1};
    void* args[] = {&Tp, &D, &c.F.nbr, &part, &c.cg_flags, &err, &sc, &tol, &maxit, &gw, &dyn};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cudaLaunchConfig_t lc{};
    lc.gridDim = dim3(blocks);
    lc.blockDim = dim3(kCgBlock);
    lc.dynamicSmemBytes = 0;
    lc.stream = s;
    lc.attrs = at;
    lc.numAttrs = 1;
    return cudaLaunchKernelExC(&lc, (const void*)k_cg_persistent<V>, args) != cudaSuccess;
}

// Whether the graph's deposition solve is the cooperative CG: one mesh,
// and the device runs cooperative launches.
static bool graph_pcg(const Ctx& c) {
    return c.tiles.n == 1 && (c.P.mixed ? c.coop_blocks32 : c.coop_blocks) > 0;
}

// The deposition solve (inside IF dep).
int capture_deposition(Ctx& c, StepGraph& G, const Handles& h, int depth, const Tiles& tl) {
    cudaStream_t s = G.cap[depth];
    const int64_t Tp = c.P.Tp;
    const double tol = c.cfg.dep_tol;
    Scalars* sc = c.sc + 2;
    const int gr = std::max(1, std::min(c.grid_red[0], tl.ntiles));
    double* part = c.tile_part;
    const bool pcg = graph_pcg(c);
    int* cg_err = pcg ? &c.gbar->err : nullptr;
    if (!c.P.mixed) {
        DepSys<double> D = dep_sys64(c);
        if (pcg) {
            if (capture_pcg<double>(c, s, D, c.coop_blocks, sc, tol, c.cfg.dep_maxit, nullptr)) return 1;
        } else {
            k_ctl_dcg_init<<<1, kBlock, 0, s>>>(G.ctl, c.ms0, sc, tl, c.act_buf, G.nact, tol, c.cfg.dep_maxit, h);
            if (capture_scg<double>(c, G, h, depth, tl, D, c.ms0, sc)) return 1;
        }
        k_ctl_dres_init<<<1, kBlock, 0, s>>>(G.ctl, c.msR, tl, c.act_buf, G.nact, 0);
        k_sdep_resid<<<gr, kBlock, 0, s>>>(tl, c.P, c.D, c.F.nbr, nullptr, c.dr, c.msR, part);
        k_ctl_dep_end<<<1, 32, 0, s>>>(G.ctl, c.msR, sc, tl.n, tol, cg_err, h);
        return 0;
    }
    float* f = c.dep32;
    float *diag32 = f, *off32 = f + Tp, *dinv32 = f + 4 * Tp, *r32 = f + 5 * Tp;
    DepSys<float> D32 = dep_sys32(c);
    k_dep_to_f32<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.D, diag32, off32, dinv32);
    if (cudaMemsetAsync(c.D.x, 0, Tp * sizeof(double), s) != cudaSuccess) return 1;
    k_ctl_dmix_init<<<1, kBlock, 0, s>>>(G.ctl, c.msR, tl, c.act_buf, G.nact, h);
    CondBody outer;
    if (outer.begin(s, G.cap[depth + 1], h.h[H_DOUTER], cudaGraphCondTypeWhile)) return 1;
    {
        cudaStream_t t = G.cap[depth + 1];
        k_sdep_resid<<<gr, kBlock, 0, t>>>(tl, c.P, c.D, c.F.nbr, r32, c.dr, c.msR, part);
        k_ctl_dmix_outer<<<1, kBlock, 0, t>>>(G.ctl, c.msR, c.ms1, sc, tl, c.act_buf, G.nact, tol,
                                              std::min(c.cfg.dep_maxit, 500), pcg ? 1 : 3, h);
        CondBody inner;
        if (inner.begin(t, G.cap[depth + 2], h.h[H_DINNER], cudaGraphCondTypeIf)) return 1;
        {
            cudaStream_t u = G.cap[depth + 2];
            if (pcg) {
                // the kernel starts from x = 0 itself; target and limit from ms1
                if (capture_pcg<float>(c, u, D32, c.coop_blocks32, sc, 0.0, 0, c.ms1)) return 1;
            } else {
                k_zero<float><<<c.grid_faces, kBlock, 0, u>>>(Tp, D32.x);
                if (capture_scg<float>(c, G, h, depth + 2, tl, D32, c.ms1, sc)) return 1;
            }
            k_dep_add<<<c.grid_faces, kBlock, 0, u>>>(c.P, c.D, D32.x);
            k_ctl_dmix_sweep_end<<<1, kBlock, 0, u>>>(G.ctl, sc, c.msR, tl, c.act_buf, G.nact, cg_err, h);
        }
        if (inner.end()) return 1;
    }
    return outer.end();
}

// The step graph is two graphs launched back to back: part 1 runs the
// assembly, the suspension solve and the column post (with the deposition
// rows); part 2 the deposition solve and the update.  Between the two
// launches the host can queue copies of the outputs that are final after
// the post on a second stream, which then overlap part 2.  Each part owns
// its conditional handles; a controller at the start of part 2 opens its
// nodes from part 1's outcome in the control block.
constexpr unsigned kPart1Handles = (1u << H_OK1) | (1u << H_SUSP) | (1u << H_OUTER) | (1u << H_WARM) |
                                   (1u << H_INNER) | (1u << H_ILOOP) | (1u << H_OK2);
constexpr unsigned kPart2Handles = (1u << H_OK2) | (1u << H_DEP) | (1u << H_DOUTER) | (1u << H_DINNER) |
                                   (1u << H_DLOOP) | (1u << H_OK3);

int build_step_graph(Ctx& c, StepGraph& G, bool own_snow) {
    cudaGraph_t g1 = nullptr, g2 = nullptr;
    auto fail = [&](const char* what, cudaError_t e) {
        if (g1) cudaGraphDestroy(g1);
        if (g2) cudaGraphDestroy(g2);
        c.err = std::string(what) + cudaGetErrorString(e);
        return PBSM3D_ERR_CUDA;
    };
    cudaError_t e = cudaGraphCreate(&g1, 0);
    if (e == cudaSuccess) e = cudaGraphCreate(&g2, 0);
    if (e != cudaSuccess) return fail("creating the step graph failed: ", e);
    const bool warm = c.cfg.warm_start != PBSM3D_X0_ZERO && !(c.cfg.warm_flags & 1);
    unsigned valid = (1u << H_COUNT) - 1u;
    if (!warm) valid &= ~(1u << H_WARM);
    if (!c.P.mixed) valid &= ~((1u << H_DOUTER) | (1u << H_DINNER));
    if (graph_pcg(c)) valid &= ~(1u << H_DLOOP);  // no tile-CG loop
    Handles h1{}, h2{};
    h1.valid = valid & kPart1Handles;
    h2.valid = valid & kPart2Handles;
    for (int id = 0; id < H_COUNT && e == cudaSuccess; ++id) {
        if (h1.valid & (1u << id)) e = cudaGraphConditionalHandleCreate(&h1.h[id], g1, 0, cudaGraphCondAssignDefault);
        if (e == cudaSuccess && (h2.valid & (1u << id)))
            e = cudaGraphConditionalHandleCreate(&h2.h[id], g2, 0, cudaGraphCondAssignDefault);
    }
    if (e != cudaSuccess) return fail("creating the step graph's conditional handles failed: ", e);
    const bool prof = c.prof;
    c.prof = false;  // per-launch events are a host-path feature
    Tiles tl = c.tiles;
    tl.nact_dev = G.nact;
    tl.nact = 0;
    cudaStream_t s = G.cap[0];
    int bad = 0;
    // phase stamps when the context profiles (the host path's per-launch
    // events have no graph equivalent)
    auto stamp = [&](cudaStream_t st, int slot) {
        if (prof) k_stamp<<<1, 1, 0, st>>>(G.ctl, slot);
    };
    c.graph_dep_flag = &G.ctl->dep_present;
    // ---- part 1: assembly, suspension solve, post and deposition rows
    e = cudaStreamBeginCaptureToGraph(s, g1, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
        stamp(s, 0);
        cudaMemcpyAsync(c.x_prev, c.A.x, c.P.R * 8, cudaMemcpyDeviceToDevice, s);
        if (c.Mb.n > 1) {
            cudaMemsetAsync(c.Mb.rhs_max, 0, c.Mb.n * 8, s);
            cudaMemsetAsync(c.Mb.dep_max, 0, c.Mb.n * 8, s);
        }
        launch_assemble_suspension(c, s);
        k_ctl_begin<<<1, 32, 0, s>>>(G.ctl, c.sc, c.Mb, c.Mb.n, c.asm_kernels, h1);
        if (c.Mb.n > 1) launch_member_mask_norm(c, s, 0);
        stamp(s, 1);
        CondBody ok1;
        bad |= ok1.begin(s, G.cap[1], h1.h[H_OK1], cudaGraphCondTypeIf);
        if (!bad) {
            cudaStream_t t = G.cap[1];
            CondBody susp;
            bad |= susp.begin(t, G.cap[2], h1.h[H_SUSP], cudaGraphCondTypeIf);
            if (!bad) {
                cudaStream_t u = G.cap[2];
                if (c.cfg.warm_start == PBSM3D_X0_PREVIOUS)
                    cudaMemcpyAsync(c.A.x, c.x_prev, c.P.R * 8, cudaMemcpyDeviceToDevice, u);
                if (c.cfg.warm_start == PBSM3D_X0_LEARNED) {
                    if (c.cfg.warm_flags & 2) {
                        bad |= launch_mlp_infer(c, u, c.A.x);
                    } else {
                        bad |= launch_mlp_infer(c, u, c.r);
                        bad |= jacobi_sweep(c, u, c.r, c.A.x);
                    }
                }
                if (c.Mb.n > 1 && c.cfg.warm_start != PBSM3D_X0_ZERO) launch_member_zero(c, u, c.A.x);
                if (!bad) bad |= c.P.mixed ? capture_suspension<float>(c, G, h1, 2, tl)
                                           : capture_suspension<double>(c, G, h1, 2, tl);
                bad |= susp.end();
            }
            stamp(t, 2);
            k_ctl_mid<<<1, 32, 0, t>>>(G.ctl, h1);
            CondBody ok2;
            bad |= ok2.begin(t, G.cap[2], h1.h[H_OK2], cudaGraphCondTypeIf);
            if (!bad) {
                cudaStream_t u = G.cap[2];
                launch_post_and_assemble_deposition(c, u);
                // decides the deposition's presence in the control block
                // (its handles belong to part 2)
                k_ctl_dep_begin<<<1, 32, 0, u>>>(G.ctl, c.sc, c.Mb, c.Mb.n, own_snow ? 2 : 1, h1);
                if (c.Mb.n > 1) launch_member_mask_norm(c, u, 1);
                stamp(u, 3);
                bad |= ok2.end();
            }
            bad |= ok1.end();
        }
        cudaGraph_t out;
        const cudaError_t ee = cudaStreamEndCapture(s, &out);
        if (ee != cudaSuccess) e = ee;
    }
    // ---- part 2: deposition solve and update
    if (e == cudaSuccess && !bad) {
        e = cudaStreamBeginCaptureToGraph(s, g2, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            k_ctl_part2<<<1, 32, 0, s>>>(G.ctl, h2);
            CondBody ok2;
            bad |= ok2.begin(s, G.cap[1], h2.h[H_OK2], cudaGraphCondTypeIf);
            if (!bad) {
                cudaStream_t t = G.cap[1];
                CondBody dep;
                bad |= dep.begin(t, G.cap[2], h2.h[H_DEP], cudaGraphCondTypeIf);
                if (!bad) {
                    bad |= capture_deposition(c, G, h2, 2, tl);
                    bad |= dep.end();
                }
                stamp(t, 4);
                CondBody ok3;
                bad |= ok3.begin(t, G.cap[2], h2.h[H_OK3], cudaGraphCondTypeIf);
                if (!bad) {
                    launch_update(c, G.cap[2]);
                    if (own_snow) launch_consume_drift(c, G.cap[2]);
                    stamp(G.cap[2], 5);
                    bad |= ok3.end();
                }
                bad |= ok2.end();
            }
            cudaGraph_t out;
            const cudaError_t ee = cudaStreamEndCapture(s, &out);
            if (ee != cudaSuccess) e = ee;
        }
    }
    c.graph_dep_flag = nullptr;
    c.prof = prof;
    if (bad || e != cudaSuccess)
        return fail("building the step graph failed: ", e != cudaSuccess ? e : cudaGetLastError());
    cudaGraphExec_t x1 = nullptr, x2 = nullptr;
    e = cudaGraphInstantiate(&x1, g1, 0);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&x2, g2, 0);
    if (e != cudaSuccess) {
        if (x1) cudaGraphExecDestroy(x1);
        return fail("instantiating the step graph failed: ", e);
    }
    G.graph = g1;
    G.exec = x1;
    G.graph2 = g2;
    G.exec2 = x2;
    G.own_snow = own_snow;
    G.profiled = prof;
    G.dt = c.P.dt;
    return 0;
}

}  // namespace

void graph_destroy(Ctx& c) {
    if (!c.graph) return;
    StepGraph& G = *c.graph;
    if (G.exec) cudaGraphExecDestroy(G.exec);
    if (G.graph) cudaGraphDestroy(G.graph);
    if (G.exec2) cudaGraphExecDestroy(G.exec2);
    if (G.graph2) cudaGraphDestroy(G.graph2);
    for (auto& st : G.cap)
        if (st) cudaStreamDestroy(st);
    if (G.ctl_host) cudaFreeHost(G.ctl_host);
    delete c.graph;
    c.graph = nullptr;
}

int graph_step(Ctx& c, cudaStream_t s, bool own_snow, const std::function<int()>& between) {
    if (!c.graph) {
        c.graph = new StepGraph();
        StepGraph& G = *c.graph;
        for (auto& st : G.cap) PBSM_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        bool ok = true;
        G.ctl = dalloc<StepCtl>(c, 1, ok);
        G.nact = dalloc<int>(c, 1, ok);
        if (!ok || cudaMallocHost(&G.ctl_host, sizeof(StepCtl)) != cudaSuccess) {
            c.err = "out of memory for the step graph";
            return PBSM3D_ERR_OUT_OF_MEMORY;
        }
    }
    StepGraph& G = *c.graph;
    if (!G.exec || G.dt != c.P.dt || G.own_snow != own_snow || G.profiled != c.prof) {
        if (G.exec) {
            cudaGraphExecDestroy(G.exec);
            cudaGraphDestroy(G.graph);
            cudaGraphExecDestroy(G.exec2);
            cudaGraphDestroy(G.graph2);
            G.exec = G.exec2 = nullptr;
            G.graph = G.graph2 = nullptr;
        }
        // the capture streams must follow s's earlier work
        PBSM_CUDA_TRY(cudaStreamSynchronize(s));
        int rc = build_step_graph(c, G, own_snow);
        if (rc) return rc;
        c.bytes = 0;
    }
    PBSM_CUDA_TRY(cudaGraphLaunch(G.exec, s));
    if (between) {
        const int rc = between();
        if (rc) {
            cudaStreamSynchronize(s);
            return rc;
        }
    }
    PBSM_CUDA_TRY(cudaGraphLaunch(G.exec2, s));
    PBSM_CUDA_TRY(cudaMemcpyAsync(G.ctl_host, G.ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost, s));
    return 0;
}

int graph_finish(Ctx& c) {
    const StepCtl& k = *c.graph->ctl_host;
    const StepGraph& G = *c.graph;
    c.suspension_present = k.susp_present;
    c.deposition_present = k.dep_present;
    c.susp_iters = k.susp_iters;
    c.susp_refinements = k.sweep;
    c.susp_matvecs = (2 + 2 * c.cfg.neumann) * k.susp_iters + k.sweep + 1;
    c.susp_relres = k.susp_relres;
    c.dep_iters = k.dep_iters;
    c.dep_refinements = k.dep_sweeps;
    c.dep_relres = k.dep_relres;
    c.warm_gamma = c.tiles.n ? k.gamma_sum / c.tiles.n : 0.0;
    c.launches = k.kernels;  // kernels the one graph launch executed
    c.graph_rhs_max[0] = k.susp_rhs_max;
    c.graph_rhs_max[1] = k.dep_rhs_max;
    // phase times from the stamps (a phase that did not run counts 0; the
    // next stamp that did run closes the span)
    for (int p = 0; p < kGraphStamps - 1; ++p) c.graph_phase_ms[p] = 0.0;
    c.graph_phases = G.profiled && k.stamp[0] != 0;
    if (c.graph_phases) {
        unsigned long long prev = k.stamp[0];
        for (int p = 1; p < kGraphStamps; ++p)
            if (k.stamp[p] >= prev && k.stamp[p] != 0) {
                c.graph_phase_ms[p - 1] = (double)(k.stamp[p] - prev) * 1e-6;
                prev = k.stamp[p];
            }
    }
    if (k.err) {
        c.err = k.err == PBSM3D_ERR_NAN_INPUT ? "NaN in an assembled system (check the forcing)"
                : k.err == PBSM3D_ERR_CUDA    ? "deposition solve: grid all-reduce timed out (a block's wait ran out)"
                                              : "a Krylov solve failed to converge";
        return k.err;
    }
    return 0;
}

}  // namespace pbsm
