// wind.cu -- the modules that produce PBSM3D's wind inputs, on the device:
// scale_wind_vert (U_2m_above_srf, scale_wind_vert.cpp:53-227) and fetchr
// (fetch, fetchr.cpp:55-117).  Per-face work, one thread per face.
//
//  * scale_wind_vert: the log / exponential wind profile through the canopy
//    and over the snow (Atmosphere.cpp:32-46), then the thin plate spline of
//    the three neighbours' values at the face centre (TPSpline.cpp:55-157):
//    an (n+1)x(n+1) system per face (n <= 3 neighbours) with the basis
//    -(log q + c + E1(q)), solved with full pivoting in registers.
//  * fetchr: fetch_steps nearest-face queries per face along the upwind
//    bearing.  The reference queries a kd-tree of face centres; here a
//    uniform grid per ensemble member (about one face per cell) is searched
//    in rings around the query's cell until no unvisited cell can hold a
//    nearer centre.  Distances are computed with explicitly rounded
//    operations, and the lowest face index wins a tie, as in the oracle's
//    brute-force search.
//  * uniform_wind (interp_met/uniform_wind.cpp:58-127): each face
//    interpolates its stations' wind components (thin plate spline, inverse
//    distance or nearest, interpolation/*.cpp) from the station lists that
//    pbsm3d_set_stations builds the way CHM's core does.
#include <math.h>

#include "pbsm3d_internal.cuh"

namespace pbsm {
namespace {

constexpr double kZUR = 50.0;     // Atmosphere.h:31 (Z_U_R)
constexpr double kZ0Snow = 0.01;  // Snow.h:31 (Z0_SNOW)

__device__ __forceinline__ bool is_nan_chm(double v) { return fabs(v - -9999.0) < 1e-5 || isnan(v); }
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }

// Atmosphere.cpp:32-38 (z0 = Z0_SNOW) and :41-46
__device__ __forceinline__ double log_scale_wind(double u, double Z_in, double Z_out, double sd) {
    return u * log((Z_out - (sd + kZ0Snow)) / kZ0Snow) / log((Z_in - (sd + kZ0Snow)) / kZ0Snow);
}
__device__ __forceinline__ double exp_scale_wind(double u, double Z_in, double Z_out, double alpha) {
    return u * exp(alpha * (Z_out / Z_in - 1));
}

// Exponential integral E1(x), x > 0: the power series for x <= 1, the
// continued fraction (modified Lentz) above (Press et al., Numerical
// Recipes, section 6.3).  Bounded loops.
__device__ double expint_e1(double x) {
    const double euler = 0.57721566490153286061;
    if (x <= 1.0) {
        double sum = 0, term = 1;
        for (int k = 1; k < 200; ++k) {
            term *= -x / k;
            const double d = -term / k;
            sum += d;
            if (fabs(d) < fabs(sum) * 1e-17) break;
        }
        return -euler - log(x) + sum;
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
        if (fabs(del - 1.0) < 1e-17) break;
    }
    return h * exp(-x);
}

// The thin-plate-spline basis of TPSpline.cpp:110-113 (weight 0.01, c = 0.577215)
__device__ __forceinline__ double tps_basis(double dx, double dy) {
    double d = sqrt(dx * dx + dy * dy);
    d = (d * 0.01 / 2.0) * (d * 0.01 / 2.0);
    return -(log(d) + 0.577215 + expint_e1(d));
}

// thin_plate_spline::operator() for n <= 3 samples at the query (qx, qy)
__device__ double tps_interp(const double* sx, const double* sy, const double* sz, int n, double qx, double qy) {
    const int m = n + 1;
    double A[4][4], b[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        b[i] = 0.0;
#pragma unroll
        for (int j = 0; j < 4; ++j) A[i][j] = 0.0;
    }
    for (int i = 0; i < n; ++i)
        for (int j = i; j < n; ++j) {
            const double xd = sx[i] - sx[j], yd = sy[i] - sy[j];
            if (xd == 0. && yd == 0.) continue;  // a duplicate point is left out (:83-85)
            const double Rd = j == i ? 0.0 : tps_basis(xd, yd);
            A[i][j + 1] = Rd;
            A[j][i + 1] = Rd;
        }
    for (int i = 0; i < m; ++i) {
        A[i][0] = 1;
        A[m - 1][i] = 1;
    }
    A[m - 1][0] = 0;
    for (int i = 0; i < n; ++i) b[i] = sz[i];
    b[m - 1] = 0.0;
    // Gaussian elimination with full pivoting (Eigen::FullPivLU in the reference)
    int colp[4] = {0, 1, 2, 3};
    for (int k = 0; k < m; ++k) {
        int pr = k, pc = k;
        double best = -1;
        for (int i = k; i < m; ++i)
            for (int j = k; j < m; ++j)
                if (fabs(A[i][j]) > best) {
                    best = fabs(A[i][j]);
                    pr = i;
                    pc = j;
                }
        if (best == 0) break;
        for (int j = 0; j < m; ++j) {
            const double t = A[k][j];
            A[k][j] = A[pr][j];
            A[pr][j] = t;
        }
        {
            const double t = b[k];
            b[k] = b[pr];
            b[pr] = t;
        }
        for (int i = 0; i < m; ++i) {
            const double t = A[i][k];
            A[i][k] = A[i][pc];
            A[i][pc] = t;
        }
        {
            const int t = colp[k];
            colp[k] = colp[pc];
            colp[pc] = t;
        }
        for (int i = k + 1; i < m; ++i) {
            const double f = A[i][k] / A[k][k];
            for (int j = k; j < m; ++j) A[i][j] -= f * A[k][j];
            b[i] -= f * b[k];
        }
    }
    double y[4] = {0, 0, 0, 0}, x[4] = {0, 0, 0, 0};
    for (int k = m - 1; k >= 0; --k) {
        double v = b[k];
        for (int j = k + 1; j < m; ++j) v -= A[k][j] * y[j];
        y[k] = A[k][k] != 0 ? v / A[k][k] : 0.0;
    }
    for (int k = 0; k < m; ++k) x[colp[k]] = y[k];
    double z0 = x[0];
    for (int i = 1; i < m; ++i) z0 += x[i] * tps_basis(sx[i - 1] - qx, sy[i - 1] - qy);
    return z0;
}

// scale_wind_vert::point_scale (scale_wind_vert.cpp:53-145)
__global__ void k_wind_point(int64_t T, Wind w, int ignore_canopy, const double* __restrict__ U_R,
                             const double* __restrict__ sd_in, double* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < T; i += (int64_t)gridDim.x * blockDim.x) {
        const double U = U_R[i];
        const double Z_R = kZUR;
        const double Z_CanTop = ignore_canopy ? 0.0 : w.canopy[i];
        const double Z_CanBot = Z_CanTop / 2.0;
        double sd = sd_in ? sd_in[i] : 0.0;
        if (is_nan_chm(sd)) sd = 0.0;
        const double Z_2m = sd + 2.0;
        if (Z_2m >= Z_R) {
            out[i] = U;
            continue;
        }
        double u;
        if (!ignore_canopy && (Z_CanTop > 0.0) && (Z_2m < Z_CanTop)) {
            const double alpha = w.lai[i];
            if (sd < Z_CanTop) {
                const double U_CanTop = log_scale_wind(U, Z_R, Z_CanTop, sd);
                const double U_CanBot = exp_scale_wind(U_CanTop, Z_CanTop, Z_CanBot, alpha);
                if (Z_2m < Z_CanBot)
                    u = log_scale_wind(U_CanBot, Z_CanBot, Z_2m, sd);
                else
                    u = exp_scale_wind(U_CanTop, Z_CanTop, Z_2m, alpha);
            } else {
                u = log_scale_wind(U, Z_R, Z_2m, sd);
            }
        } else {
            u = log_scale_wind(U, Z_R, Z_2m, sd);
        }
        out[i] = smax(0.1, u);
    }
}

// scale_wind_vert::run, the neighbour smoothing (:181-227)
__global__ void k_wind_smooth(int64_t T, int64_t Tp, Wind w, const int32_t* __restrict__ nbr,
                              const double* __restrict__ pt, double* __restrict__ u2m) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < T; i += (int64_t)gridDim.x * blockDim.x) {
        double sx[3], sy[3], sz[3];
        int n = 0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int32_t nb = nbr[j * Tp + i];
            if (nb < 0) continue;
            sx[n] = w.cx[nb];
            sy[n] = w.cy[nb];
            sz[n] = pt[nb];
            ++n;
        }
        u2m[i] = n > 0 ? smax(0.1, tps_interp(sx, sy, sz, n, w.cx[i], w.cy[i])) : smax(0.1, pt[i]);
    }
}

// squared distance with explicitly rounded operations (the oracle's order)
__device__ __forceinline__ double dist2(double ax, double ay, double qx, double qy) {
    const double dx = __dsub_rn(ax, qx), dy = __dsub_rn(ay, qy);
    return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
}

// Nearest face centre to (qx, qy) in member grid g.  Rings r = 0, 1, ... of
// cells around the query's (clamped) cell; after ring r the unvisited cells
// lie beyond the block [ci-r, ci+r] x [cj-r, cj+r], so their centres are at
// least the distance to the nearest block side that has cells beyond it.
// Bounded by the grid size.
__device__ int32_t nearest_face(const GridM& g, const int32_t* __restrict__ cs, const int32_t* __restrict__ cf,
                                const double* __restrict__ cx, const double* __restrict__ cy, double qx, double qy) {
    int ci = (int)floor((qx - g.x0) / g.h), cj = (int)floor((qy - g.y0) / g.h);
    ci = min(max(ci, 0), g.nx - 1);
    cj = min(max(cj, 0), g.ny - 1);
    double best = INFINITY;
    int32_t bf = -1;
    const int rmax = max(g.nx, g.ny);
    for (int r = 0; r <= rmax; ++r) {
        for (int dj = -r; dj <= r; ++dj) {
            const int j = cj + dj;
            if (j < 0 || j >= g.ny) continue;
            const bool edge_row = dj == -r || dj == r;
            for (int di = -r; di <= r; di += (edge_row || r == 0) ? 1 : 2 * r) {
                const int ii = ci + di;
                if (ii < 0 || ii >= g.nx) continue;
                const int cell = g.cell0 + j * g.nx + ii;
                for (int k = cs[cell]; k < cs[cell + 1]; ++k) {
                    const int32_t f = cf[k];
                    const double d2 = dist2(cx[f], cy[f], qx, qy);
                    if (d2 < best || (d2 == best && f < bf)) {
                        best = d2;
                        bf = f;
                    }
                }
            }
        }
        double lb = INFINITY;
        if (ci - r - 1 >= 0) lb = fmin(lb, fmax(0.0, qx - (g.x0 + (ci - r) * g.h)));
        if (ci + r + 1 < g.nx) lb = fmin(lb, fmax(0.0, g.x0 + (ci + r + 1) * g.h - qx));
        if (cj - r - 1 >= 0) lb = fmin(lb, fmax(0.0, qy - (g.y0 + (cj - r) * g.h)));
        if (cj + r + 1 < g.ny) lb = fmin(lb, fmax(0.0, g.y0 + (cj + r + 1) * g.h - qy));
        if (lb == INFINITY) break;        // every cell visited
        if (best < lb * lb) break;        // nothing unvisited can be as near
    }
    return bf;
}

// fetchr::run (fetchr.cpp:55-117)
__global__ void k_fetchr(int64_t T, Wind w, const int32_t* __restrict__ face_member, int steps, double max_distance,
                         double I, int incl_veg, const double* __restrict__ dir, double* __restrict__ fetch) {
    const double size_of_step = max_distance / steps;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < T; i += (int64_t)gridDim.x * blockDim.x) {
        double out = max_distance;
        if (incl_veg && w.canopy[i] > 1) {
            fetch[i] = 0;
            continue;
        }
        const GridM g = w.grid[face_member[i]];
        double sb, cb;
        sincos(dir[i] * (M_PI / 180.0), &sb, &cb);
        const double cx = w.cx[i], cy = w.cy[i], cz = w.cz[i];
        for (int j = 1; j <= steps; ++j) {
            const double distance = j * size_of_step;
            const double qx = __dadd_rn(cx, __dmul_rn(distance, sb)), qy = __dadd_rn(cy, __dmul_rn(distance, cb));
            const int32_t f = nearest_face(g, w.cell_start, w.cell_face, w.cx, w.cy, qx, qy);
            if (f < 0) break;
            const double Z_CanTop = incl_veg ? w.canopy[f] : 0.0;
            const double Z_test = w.cz[f] + Z_CanTop;
            const double Z_core = cz + distance * I;
            const double z0_1 = 0.12 * Z_CanTop, z0_2 = 0.001, n = 1.0 / 0.8, h = 5;
            const double x_sss = pow(((33.33333333 * h - 25. * z0_2) / (log(z0_1 / z0_2) * z0_2)), n) * z0_2;
            if (Z_test >= Z_core || (incl_veg && distance < x_sss)) {
                out = distance;
                break;
            }
        }
        fetch[i] = out;
    }
}

// The thin plate spline of n <= 16 samples carrying two fields at once (the
// system does not depend on the field), full pivoting; local-memory arrays.
__device__ void tps_interp2(const double* sx, const double* sy, const double* z0v, const double* z1v, int n,
                            double qx, double qy, double& o0, double& o1) {
    const int m = n + 1;
    double A[17][17], b[2][17];
    int colp[17];
    for (int i = 0; i < m; ++i) {
        colp[i] = i;
        b[0][i] = b[1][i] = 0.0;
        for (int j = 0; j < m; ++j) A[i][j] = 0.0;
    }
    for (int i = 0; i < n; ++i)
        for (int j = i; j < n; ++j) {
            const double xd = sx[i] - sx[j], yd = sy[i] - sy[j];
            if (xd == 0. && yd == 0.) continue;
            const double Rd = j == i ? 0.0 : tps_basis(xd, yd);
            A[i][j + 1] = Rd;
            A[j][i + 1] = Rd;
        }
    for (int i = 0; i < m; ++i) {
        A[i][0] = 1;
        A[m - 1][i] = 1;
    }
    A[m - 1][0] = 0;
    for (int i = 0; i < n; ++i) {
        b[0][i] = z0v[i];
        b[1][i] = z1v[i];
    }
    for (int k = 0; k < m; ++k) {
        int pr = k, pc = k;
        double best = -1;
        for (int i = k; i < m; ++i)
            for (int j = k; j < m; ++j)
                if (fabs(A[i][j]) > best) {
                    best = fabs(A[i][j]);
                    pr = i;
                    pc = j;
                }
        if (best == 0) break;
        for (int j = 0; j < m; ++j) {
            const double t = A[k][j];
            A[k][j] = A[pr][j];
            A[pr][j] = t;
        }
        for (int f = 0; f < 2; ++f) {
            const double t = b[f][k];
            b[f][k] = b[f][pr];
            b[f][pr] = t;
        }
        for (int i = 0; i < m; ++i) {
            const double t = A[i][k];
            A[i][k] = A[i][pc];
            A[i][pc] = t;
        }
        {
            const int t = colp[k];
            colp[k] = colp[pc];
            colp[pc] = t;
        }
        for (int i = k + 1; i < m; ++i) {
            const double g = A[i][k] / A[k][k];
            for (int j = k; j < m; ++j) A[i][j] -= g * A[k][j];
            b[0][i] -= g * b[0][k];
            b[1][i] -= g * b[1][k];
        }
    }
    double out[2];
    for (int f = 0; f < 2; ++f) {
        double y[17], x[17];
        for (int k = m - 1; k >= 0; --k) {
            double v = b[f][k];
            for (int j = k + 1; j < m; ++j) v -= A[k][j] * y[j];
            y[k] = A[k][k] != 0 ? v / A[k][k] : 0.0;
        }
        for (int k = 0; k < m; ++k) x[colp[k]] = y[k];
        double z = x[0];
        for (int i = 1; i < m; ++i) z += x[i] * tps_basis(sx[i - 1] - qx, sy[i - 1] - qy);
        out[f] = z;
    }
    o0 = out[0];
    o1 = out[1];
}

// inv_dist::operator() (interpolation/inv_dist.cpp:36-78): weights 1/d^2; a
// sample at the query resets the sums to it and later samples still add.
__device__ double idw_interp(const double* sx, const double* sy, const double* sz, int n, double qx, double qy) {
    double numerator = 0.0, denominator = 0.0;
    for (int i = 0; i < n; ++i) {
        const double xdiff = sx[i] - qx, ydiff = sy[i] - qy;
        const double di = pow(sqrt(pow(xdiff, 2.0) + pow(ydiff, 2.0)), 2.0);
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

// uniform_wind::run (interp_met/uniform_wind.cpp:58-127)
__global__ void k_uniform_wind(int64_t T, Wind w, Stations st, double* __restrict__ U_R,
                               double* __restrict__ vw_dir) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < T; i += (int64_t)gridDim.x * blockDim.x) {
        double px[16], py[16], pu[16], pv[16];
        int m = 0;
        for (int k = st.start[i]; k < st.start[i + 1] && m < 16; ++k) {
            const int s = st.idx[k];
            const double su = st.u[s], sd = st.dir[s];
            if (is_nan_chm(su) || is_nan_chm(sd)) continue;
            const double W = smax(su, 0.1);
            const double theta = sd * M_PI / 180.;
            double sn, cs;
            sincos(theta, &sn, &cs);
            px[m] = st.x[s];
            py[m] = st.y[s];
            pu[m] = -W * sn;
            pv[m] = -W * cs;
            ++m;
        }
        if (m == 0) {
            atomicExch(st.bad, 1);
            continue;
        }
        const double qx = w.cx[i], qy = w.cy[i];
        double zu, zv;
        if (st.interp == PBSM3D_INTERP_SPLINE) {
            tps_interp2(px, py, pu, pv, m, qx, qy, zu, zv);
        } else if (st.interp == PBSM3D_INTERP_IDW) {
            zu = idw_interp(px, py, pu, m, qx, qy);
            zv = idw_interp(px, py, pv, m, qx, qy);
        } else {
            zu = pu[0];
            zv = pv[0];
        }
        double theta = 3.0 * M_PI * 0.5 - atan2(zv, zu);
        if (theta > 2 * M_PI) theta = theta - 2 * M_PI;
        U_R[i] = smax(sqrt(zu * zu + zv * zv), 0.1);
        vw_dir[i] = theta * 180.0 / M_PI;
    }
}

}  // namespace

void launch_uniform_wind(Ctx& c, cudaStream_t s, double* U_R, double* vw_dir) {
    k_uniform_wind<<<c.grid_faces, kBlock, 0, s>>>(c.P.T, c.wnd, c.st, U_R, vw_dir);
}

void launch_scale_wind_vert(Ctx& c, cudaStream_t s, const double* U_R, const double* sd, double* u2m) {
    k_wind_point<<<c.grid_faces, kBlock, 0, s>>>(c.P.T, c.wnd, c.cfg.wind_ignore_canopy, U_R, sd, c.wnd.tmp);
    k_wind_smooth<<<c.grid_faces, kBlock, 0, s>>>(c.P.T, c.P.Tp, c.wnd, c.F.nbr, c.wnd.tmp, u2m);
}

void launch_fetchr(Ctx& c, cudaStream_t s, const double* dir, double* fetch) {
    k_fetchr<<<c.grid_faces, kBlock, 0, s>>>(c.P.T, c.wnd, c.Mb.face_member, c.cfg.fetch_steps,
                                            c.cfg.fetch_max_distance, c.cfg.fetch_I, c.cfg.fetch_incl_veg, dir,
                                            fetch);
}

}  // namespace pbsm
