// physics.cu -- per-face physics and system assembly of the PBSM3D step.
//
// The assembly is bound by the FP64 pipe (GB300 issues FP64 at a small
// fraction of its FP32 rate, and a warp instruction costs the same however
// many of its lanes are active), so it is written to spend as few FP64 warp
// instructions per row as the accuracy bar allows:
//  * three passes keep warps convergent: per-face saltation (pass 1), the
//    height-dependent particle terms of the rows of saltating faces, one
//    row per lane (pass 2), and the row assembly (pass 3), which reads those
//    terms from pass 2 or, for faces without a saltation layer, from a
//    per-layer table; saltating faces are spatially random, so a single
//    per-face pass would run both paths in nearly every warp;
//  * exp / log / 1/x are the table-driven routines of fp64_math.cuh, x^y for
//    x > 0 is exp(y log x), and log(u_z) is assembled from per-face and
//    per-layer logarithms so that u_z^1.36 is one exp per row;
//  * NaN/Inf detection, the |rhs| maximum and sign tests run on the integer
//    pipe (bit patterns);
//  * multiply-adds contract to FMA, except in the saltation concentration
//    whose bracket 1 - tau - u*_th^2/u*^2 cancels near the threshold and is
//    evaluated with explicitly rounded operations in the reference's order.
// The assembled entries agree with a C++ evaluation of
// src/modules/PBSM3D.cpp to ~1e-15 relative.
#include <math.h>

#include "pbsm3d_internal.cuh"
#include "roots.cuh"

namespace pbsm {
namespace {

constexpr double kKappa = 0.4;    // PhysConst.h:31
constexpr double kRhoIce = 917;   // PhysConst.h:39
constexpr double kZUR = 50.0;     // Atmosphere.h:31

// Bit-pattern tests that keep comparisons off the FP64 pipe.
__device__ __forceinline__ bool nonfinite(double x) {
    return ((unsigned)(__double_as_longlong(x) >> 32) & 0x7ff00000u) == 0x7ff00000u;
}
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
// x > 0 for a non-NaN x (false for +0 and -0)
__device__ __forceinline__ bool gt0(double x) { return __double_as_longlong(x) > 0; }

// module_base.hpp:471-479: -9999 or NaN
__device__ __forceinline__ bool is_nan_chm(double v) { return fabs(v - -9999.0) < 1e-5 || isnan(v); }
// std::max(a, b) == (a < b) ? b : a (NaN in b yields a)
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }

// Atmosphere.cpp:32-38
__device__ __forceinline__ double log_scale_wind(double u, double Z_in, double Z_out, double sd, double z0) {
    return u * log((Z_out - (sd + z0)) / z0) / log((Z_in - (sd + z0)) / z0);
}

// Atmosphere.cpp:62-80 (T in K against Tfreeze = 0: the water branch for any T > 0 K)
__device__ __forceinline__ double saturated_vapour_pressure(double T, const MathTables& mt) {
    const double TA = T - 273.15;
    if (T >= 0.) return 611.21 * exp_t((17.502 * TA) * rcp_t(240.97 + TA), mt);
    return 611.15 * exp_t((22.452 * TA) * rcp_t(272.55 + TA), mt);
}

// coordinates.cpp:112-131
__device__ __forceinline__ void bearing_to_cartesian(double bearing, double& x, double& y) {
    double h = 450. - bearing;
    if (h > 360.) h = h - 360.;
    const double theta = h * M_PI / 180.;
    sincos(theta, &y, &x);
}

// MeteoIO standard atmosphere (PBSM3D.cpp:785): p(z) / (R_dry T)
__device__ __forceinline__ double std_dry_air_density(double altitude, double temperature, const MathTables& mt) {
    const double p0 = 101325., lapse = 0.0065, T0 = 288.15, Rd = 287.058, g = 9.80665, R0 = 6356766.0;
    const double expo = g / (lapse * Rd);
    const double p = p0 * pow_t(1. - ((lapse * R0 * altitude) / (T0 * (R0 + altitude))), expo, mt);
    return p / (287.058 * temperature);
}

// armadillo's 3-vector dot with a zero z on one side: (a0*b0 + a2*b2) + a1*b1
__device__ __forceinline__ double dot2(double ax, double ay, double bx, double by) {
    double v1 = 0, v2 = 0;
    v1 += ax * bx;
    v2 += ay * by;
    return v1 + v2;
}

// Height-dependent terms of one suspension layer centred at cz
// (PBSM3D.cpp:1003-1028, 1113-1120, 1157): mean particle radius and mass,
// radius of the mean-mass particle, settling velocity, the log(cz) factor of
// the undersaturation, the radiation term and the mixing length; and the
// wind-profile logarithm log((cz - z0)/z0) with its 1.36th power.
// hz_minus_d0 is the reference's Z_out - (snow depth + z0) of
// log_scale_wind (Atmosphere.cpp:32-38).
__device__ __forceinline__ void cz_coeffs(double cz, double hz_minus_d0, double z0, double settling_scale,
                                          const Params& P, const MathTables& t, CzCoef& o) {
    const double lcz = log_t(cz, t);
    const double rm = 4.6e-5 * exp_t(-0.258 * lcz, t);             // 4.6e-5 cz^-0.258
    const double ia = rcp_t(4.08 + 12.6 * cz);                       // 1 / mm_alpha
    const double mm = 4. / 3. * M_PI * kRhoIce * rm * rm * rm * (1.0 + 3.0 * ia + 2. * (ia * ia));
    const double inv_mm = rcp_t(mm);
    const double lq = 0.3333333 * log_t((3.0 * mm) * (1.0 / (4 * M_PI * kRhoIce)), t);
    const double r_z = exp_t(lq, t);                                 // (3 mm / 4 pi rho)^0.3333333
    double omega = P.settling_velocity;
    if (!P.do_fixed_settling) omega = 1.1e7 * exp_t(1.8 * lq, t);   // 1.1e7 r_z^1.8
    o.omega = omega * settling_scale;
    // the radiation term, or with iterative_subl, whose rate has no radiation
    // term, the mean radius itself; over the particle mass
    o.qr_m = (P.iterative_subl ? rm : 0.9 * M_PI * rm * rm * 120.0) * inv_mm;
    const double sigfac = 1.019 + 0.027 * lcz;
    const double kz = kKappa * (cz + z0);
    o.l = kz * 40.0 * rcp_t(kz + 40.0);
    o.rz2nu = 2.0 * r_z * (1.0 / 1.88e-5);                          // Re = rz2nu * Vr
    o.rsig_m = r_z * sigfac * inv_mm;
    o.lwarg = log_t(hz_minus_d0 * rcp_t(z0), t);
    // u_z^1.36 = (uref / logden)^1.36 lwarg^1.36: the face's factor times
    // this one, so the row needs no exp (lwarg <= 0 gives NaN, as log does)
    o.ew = exp_t(1.36 * log_t(o.lwarg, t), t);
    o.cz = cz;
}

// z0_ustar_coupling (PBSM3D.cpp:691-712): u* over snow with partly buried
// vegetation, the root of Li and Pomeroy (2000) eqn 5
//     g(u) = u2 kappa / log(2 / (c u^2 + lambda/2)) - u,  c = 0.6131702345e-2,
// which falls with u, from guess 1 (roots.cuh).  false: no bracket.
__device__ bool coupled_ustar(double u2, double lambda, const MathTables& mt, double& ustar) {
    const double c = 0.6131702345e-2, A = u2 * kKappa, h = .5 * lambda;
    auto g = [&](double u) { return div_t(A, log_t(div_t(2.0, c * u * u + h), mt)) - u; };
    auto dg = [&](double u) {
        const double q = c * u * u + h;
        const double ell = log_t(div_t(2.0, q), mt);
        return div_t(A * (2.0 * c * u), q * ell * ell) - 1.0;
    };
    return bracket_solve(g, dg, 1.0, false, ustar);
}

// iterative_subl (PBSM3D.cpp:1062-1096): the ice-bulb temperature Ti (C),
// root of f(Ti) = T + D L (rho/1000 - .611 mw e(Ti) / (R (Ti+273.15) 1000)) / lambda_t - Ti,
// e(Ti) = exp(17.3 Ti / (237.3 + Ti)), by the reference's
// newton_raphson_iterate(f, T, -50, 0, 6 digits): Newton steps from T, the
// result being the iterate after the first step no larger than |Ti| 2^-5.  A
// step that would reach a bound goes half the way to it; the bound on the
// side a step left from moves to the point it left.  At most 100 steps.
__device__ double ice_bulb_temperature(double T, double t, double ea, double D, double lambda_t, double L,
                                       const MathTables& mt) {
    const double mw = 0.01801528 * 1000.0, R = 8.31441 / 1000.0;
    const double rho = div_t(mw * ea, R * t);
    const double k = div_t(D * L, lambda_t);
    const double sat0 = .611 * mw * (1.0 / (R * 1000.0));
    double lo = -50, hi = 0;
    double x = T;
    for (int it = 0; it < 100; ++it) {
        const double iw = rcp_t(237.3 + x), ik = rcp_t(x + 273.15);
        const double sat = sat0 * exp_t(17.3 * x * iw, mt) * ik;  // saturation vapour density (kg/m^3)
        const double f = T + k * (rho * 1e-3 - sat) - x;
        if (f == 0) break;
        // d sat/dTi = sat (17.3 * 237.3 / (237.3 + Ti)^2 - 1 / (Ti + 273.15))
        const double df = -k * sat * (17.3 * 237.3 * iw * iw - ik) - 1.0;
        const double from = x;
        double step = div_t(f, df);
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
        if (!(fabs(x * (1.0 / 32.0)) < fabs(step))) break;
    }
    return x;
}

// The same terms for every layer of a face with no saltation layer (hs = 0).
__global__ void k_cz_table(Params P, Members Mb, CzCoef* tab) {
    __shared__ MathTables mt;
    math_tables_load(mt, P.mt);
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= Mb.n * P.L) return;
    const int m = q / P.L, z = q % P.L;
    const double cz = z * P.dz + P.dz / 2.;
    const double z0 = Mb.prm[m].z0;
    CzCoef o;
    cz_coeffs(cz, cz - z0, z0, Mb.prm[m].settling_scale, P, mt, o);
    tab[q] = o;
}

// Pass 1 of the suspension assembly, one thread per face: saltation
// (PBSM3D.cpp:436-925) and the per-face constants of the layer loop
// (:927-1233).  Faces that carry a saltation layer (hs > 0: their layer
// heights differ from the per-layer table) are appended to a list, so that
// pass 2 computes their height-dependent terms with every lane busy.
__global__ void __launch_bounds__(kBlock) k_salt_faces(Params P, Faces G, Forcing F, FaceState S, Susp A, Members Mb) {
    __shared__ MathTables mt;
    math_tables_load(mt, P.mt);
    const int64_t Tp = P.Tp;
    const int lane = threadIdx.x & 31;
    // Tp is a multiple of the block size: every lane of a warp runs the same iterations
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Tp; i += (int64_t)gridDim.x * blockDim.x) {
        bool slow = false;
        if (i < P.T) {
            const Member mp = Mb.prm[Mb.face_member[i]];
            const double uref = F.UR[i];
            double snow_depth = F.sd[i];
            snow_depth = is_nan_chm(snow_depth) ? 0 : snow_depth;
            const double u2 = F.U2[i];
            double height_diff = smax(0.0, G.canopy[i] - snow_depth);
            if (!P.enable_veg) height_diff = 0;
            double ustar = 1.3;
            double lambda = 0;
            bool saltation = false;
            const double T_c = F.t[i];
            // u*_th decides saltation (ustar >= u*_th) and enters the cancelling
            // c_salt bracket: evaluated without contraction, in the reference's order
            double uth =
                __dadd_rn(__dadd_rn(0.35, __dmul_rn(1.0 / 150.0, T_c)), __dmul_rn(__dmul_rn(1.0 / 8200.0, T_c), T_c));
            uth = __dmul_rn(uth, mp.uth_scale);
            const double stalkN = G.stalkN[i], stalkD = G.stalkD[i];
            // PBSM3D.cpp:480-645: the subgrid holding capacity and contributing fraction
            const double min_sd_trans_avg = P.subgrid ? S.sub[SG_HOLD * Tp + i] : P.min_sd_trans;
            if (height_diff <= P.cutoff && snow_depth >= min_sd_trans_avg && !G.water[i]) {
                if (P.use_R94_lambda)
                    lambda = 0.5 * G.lai[i] * height_diff;
                else
                    lambda = stalkN * stalkD * height_diff;
                if (P.z0_ustar_coupling) {
                    double u;
                    if (coupled_ustar(u2, lambda, mt, u)) ustar = u;  // no bracket: u* stays 1.3 (:710-713)
                } else {
                    ustar = u2 * kKappa / P.log_2_0002;
                }
                if (ustar >= uth) saltation = true;
            }
            // z0 is the member's snow roughness (:740-754), or with the
            // coupling, Li and Pomeroy 2000 eqn 4 on saltating faces (:736),
            // at least the snow roughness (:753)
            double z0 = mp.z0;
            if (P.z0_ustar_coupling && saltation)
                z0 = smax(mp.z0, 0.6131702345e-2 * ustar * ustar + .5 * lambda);
            if (!saltation) ustar = smax(0.01, kKappa * uref / mp.log_zur_z0);
            ustar = smax(0.01, ustar);
            // the saltation terms (hs, c_salt, Qsalt, the over-erosion check)
            // of the saltating faces run in pass 1b over their compacted list,
            // so that warps do not carry them for the ~70% of faces without
            // saltation; the other faces are final here
            slow = saltation;  // hs > 0
            const double t = F.t[i] + 273.15;
            double vx, vy;
            bearing_to_cartesian(F.dir[i], vx, vy);
            const double ux = -vx, uy = -vy;
            double mx[3], my[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                mx[j] = G.mx[j * Tp + i];
                my[j] = G.my[j * Tp + i];
            }
            double* fv = A.face_v;
            fv[FV_UX * Tp + i] = ux;
            fv[FV_UY * Tp + i] = uy;
            if (saltation) {
                fv[FV_LAMBDA * Tp + i] = lambda;
            } else {
                fv[FV_HS * Tp + i] = 0.0;
                fv[FV_CSALT * Tp + i] = 0.0;
                S.Qsalt[i] = 0.0;
                S.saltation[i] = false;
            }

            // per-face constants of the layer loop.  Division by a per-face or
            // constant value becomes a product with its reciprocal and the
            // sublimation rate is regrouped so that no division is left per
            // row (each change moves a result by a few ulps).
            const double rh = F.rh[i] / 100.;
            const double es = saturated_vapour_pressure(t, mt);
            const double D = 2.06e-5 * pow_t(t * (1.0 / 273.15), 1.75, mt);
            const double lambda_t = 0.000063 * t + 0.00673;
            const double Ls = 2.838e6, M = 18.01, Rg = 8313;
            const double rho = (M * es) * rcp_t(Rg * t);
            // dm/dt = Sh rho D (2 pi Nu R r sigma t^2 lt - L M Qr + Qr R t) /
            //         (D L Sh (L M - R t) rho + lt t^2 Nu R),  Sh = Nu,
            //       = q * ((c1 (rh-1)) Nu (r sigfac) - Qr (L M - R t))
            const double Rgt = Rg * t;
            const double c1r = 6.283185308 * Rg * (t * t * lambda_t) * (rh - 1.0);
            double q_sub = (rho * D) * rcp_t(D * Ls * (Ls * M - Rgt) * rho + lambda_t * t * t * Rg);
            if (P.iterative_subl) {
                // dm/dt = 2 pi rm lambda_t / L Nu (Ts - (t + 273.15)) (:1099, t already
                // in K): q_sub carries everything but rm Nu
                const double Ti = ice_bulb_temperature(T_c, t, rh * es / 1000., D, lambda_t, Ls, mt);
                q_sub = 2.0 * M_PI * lambda_t * (1.0 / Ls) * ((Ti + 273.15) - (t + 273.15));
            }
            const double LR = Ls * M - Rgt;
            const double sdz0 = snow_depth + z0;
            const double logden = log_t((kZUR - sdz0) * rcp_t(z0), mt);
            const double inv_logden = rcp_t(logden);
            // u_z^1.36 = (uref / logden)^1.36 lwarg^1.36: this face's factor,
            // with the constants of the particle-velocity term 3 cos(pi/4) 0.005 u_z^1.36
            const double ef = uref > 0.0 ? (0.015 * P.cos_pi_4) * exp_t(1.36 * (log_t(uref, mt) - log_t(logden, mt)), mt)
                                         : 0.0;
            // the two sublimation terms' per-face factors
            const double qc = P.iterative_subl ? q_sub : q_sub * c1r, ql = P.iterative_subl ? 0.0 : q_sub * LR;
            double v1 = 0, v2 = 0;
            v1 += ux * ux;
            v2 += uy * uy;
            const double inv_nrm = rcp_t(sqrt(v1 + v2));
            fv[FV_USTAR * Tp + i] = ustar;
            fv[FV_UTH * Tp + i] = uth;
            fv[FV_QC * Tp + i] = qc;
            fv[FV_QL * Tp + i] = ql;
            fv[FV_EF * Tp + i] = ef;
            fv[FV_INVLOGDEN * Tp + i] = inv_logden;
            if (P.z0_ustar_coupling) fv[FV_Z0 * Tp + i] = z0;
            // lateral faces: udotm_f = u_z * k_f with k_f = (u_hat . m_f) / |u_hat|
#pragma unroll
            for (int f = 0; f < 3; ++f) fv[(FV_K0 + f) * Tp + i] = inv_nrm * dot2(ux, uy, mx[f], my[f]);
        }
        // append the faces with a saltation layer (one atomic per warp)
        const unsigned ball = __ballot_sync(0xffffffffu, slow);
        if (ball) {
            int base = 0;
            if (lane == 0) base = atomicAdd(A.n_slow, __popc(ball));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (slow) A.slow_list[base + __popc(ball & ((1u << lane) - 1u))] = (int32_t)i;
        }
    }
}

// Pass 1b, one thread per face on the list of saltating faces (hs > 0): the
// saltation layer's height, the saltation concentration and flux with the
// fetch, probability and subgrid factors, and the over-erosion check
// (PBSM3D.cpp:763-925), in the reference's order and rounding.
__global__ void __launch_bounds__(kBlock) k_salt_terms(Params P, Faces G, Forcing F, FaceState S, Susp A, Members Mb) {
    __shared__ MathTables mt;
    math_tables_load(mt, P.mt);
    const int64_t Tp = P.Tp;
    const int n = *A.n_slow;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int64_t i = A.slow_list[k];
        const Member mp = Mb.prm[Mb.face_member[i]];
        double* fv = A.face_v;
        const double ustar = fv[FV_USTAR * Tp + i], uth = fv[FV_UTH * Tp + i], lambda = fv[FV_LAMBDA * Tp + i];
        double fetch = 1000;
        if (P.use_exp_fetch || P.use_tanh_fetch) fetch = F.fetch[i];
        const double uref = F.UR[i];
        double snow_depth = F.sd[i];
        snow_depth = is_nan_chm(snow_depth) ? 0 : snow_depth;
        double swe = F.swe[i];
        swe = is_nan_chm(swe) ? 0 : swe;
        const double T_c = F.t[i];
        const double t = T_c + 273.15;
        bool saltation = true;
        const double hs = 0.08436 * pow_t(ustar, 1.27, mt);
        const double ux = fv[FV_UX * Tp + i], uy = fv[FV_UY * Tp + i];
        const double rho_f = std_dry_air_density(G.zc[i], t, mt);
        const double Beta = 202.0, mB = 0.16;
        const double mbl = __dmul_rn(__dmul_rn(mB, Beta), lambda);
        const double tau_n_ratio = __ddiv_rn(mbl, __dadd_rn(1.0, mbl));
        // the bracket cancels near the threshold: no contraction here
        const double bracket =
            __dsub_rn(__dsub_rn(1.0, tau_n_ratio), __ddiv_rn(__dmul_rn(uth, uth), __dmul_rn(ustar, ustar)));
        double c_salt = __dmul_rn(__ddiv_rn(rho_f, __dmul_rn(3.29, ustar)), bracket);
        if (c_salt < 0 || isnan(c_salt)) {
            c_salt = 0;
            saltation = false;
        }
        if (P.use_exp_fetch && fetch < 500) {
            const double fetch_ref = 500, mu = 3.0;
            c_salt *= 1.0 - exp(-mu * fetch / fetch_ref);
        } else if (P.use_tanh_fetch && fetch <= 300.) {
            c_salt *= P.Lc_tanh;  // 0.5*tanh(0.01333*fetch_ref - 2)+0.5 with fetch_ref = 300
        }
        if (P.use_PomLi) {  // PBSM3D.cpp:848-865
            double height_diff = smax(0.0, G.canopy[i] - snow_depth);
            if (!P.enable_veg) height_diff = 0;
            const double z10 = 10. + snow_depth;
            const double u10 = z10 < kZUR ? log_scale_wind(uref, kZUR, z10, snow_depth, mp.z0) : uref;
            const double Ah = F.psh[i];
            const double u_mean = 11.2 + 0.365 * T_c + 0.00706 * T_c * T_c + 0.9 * log(Ah);
            const double delta = 0.145 * T_c + 0.00196 * T_c * T_c + 4.3;
            const double z0v = (G.stalkN[i] * G.stalkD[i] * height_diff) / 2.0;
            const double us = u10 / sqrt((1 + 340.0 * z0v));
            const double Pu10 = 1.0 / (1.0 + exp((sqrt(M_PI) * (u_mean - us)) / delta));
            S.bsp[i] = Pu10;
            c_salt *= Pu10;
        }
        if (P.subgrid) c_salt *= S.sub[SG_FRAC * Tp + i];  // :867-870
        const double uhs = 2.8 * uth;
        double Qsalt = c_salt * uhs * hs;
        double mass = 0;
        for (int j = 0; j < 3; ++j) {
            const double udm = __dadd_rn(__dmul_rn(ux, G.mx[j * Tp + i]), __dmul_rn(uy, G.my[j * Tp + i]));
            mass = __dadd_rn(mass, __dmul_rn(__dmul_rn(-G.E[j * Tp + i], Qsalt), udm));
        }
        mass = __dmul_rn(__ddiv_rn(mass, G.area[i]), P.dt);
        if (mass < 0 && fabs(mass) > swe) {
            c_salt = 0;
            Qsalt = c_salt * uhs * hs;
        }
        S.Qsalt[i] = Qsalt;
        S.saltation[i] = saltation;
        fv[FV_HS * Tp + i] = hs;
        fv[FV_CSALT * Tp + i] = c_salt;
    }
}

// Pass 2, one thread per row of a face on the list: the height-dependent
// terms of its layer (cz = z dz + hs + dz/2), stored by row as pass 3
// reads them.  Every lane of a warp does the same work.
__global__ void __launch_bounds__(kBlock) k_salt_rows(Params P, Forcing F, Susp A, Members Mb) {
    __shared__ MathTables mt;
    math_tables_load(mt, P.mt);
    const int64_t n = *A.n_slow;
    const int64_t tasks = n * P.L, Tp = P.Tp, R = P.R;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tasks; q += (int64_t)gridDim.x * blockDim.x) {
        const int z = (int)(q / n);
        const int64_t i = A.slow_list[q - (int64_t)z * n];
        const Member mp = Mb.prm[Mb.face_member[i]];
        double snow_depth = F.sd[i];
        snow_depth = is_nan_chm(snow_depth) ? 0 : snow_depth;
        const double hs = A.face_v[FV_HS * Tp + i];
        const double z0 = P.z0_ustar_coupling ? A.face_v[FV_Z0 * Tp + i] : mp.z0;
        const double cz = z * P.dz + hs + P.dz / 2.;
        CzCoef o;
        cz_coeffs(cz, cz + snow_depth - (snow_depth + z0), z0, mp.settling_scale, P, mt, o);
        const int64_t r = (int64_t)z * Tp + i;
        double* w = A.slow_rows + r;
        w[0 * R] = o.omega;
        w[1 * R] = o.qr_m;
        w[2 * R] = o.l;
        w[3 * R] = o.rz2nu;
        w[4 * R] = o.rsig_m;
        w[5 * R] = o.lwarg;
        w[6 * R] = o.ew;
    }
}

// Pass 3, one thread per face: the suspension rows (PBSM3D.cpp:1236-1404)
// from the layer terms (table or pass 2) and the face constants (pass 1),
// and the Thomas factorisation of the column.
__global__ void __launch_bounds__(kBlock, 2) k_assemble_suspension(Params P, Faces G, Forcing F, FaceState S, Susp A,
                                                               Members Mb, double* partials, Scalars* sc) {
    __shared__ MathTables mt;
    math_tables_load(mt, P.mt);
    unsigned long long vmax_bits = 0;
    bool bad = false;
    // per-member max |rhs| of this block (ensembles), folded into Mb.rhs_max at the end
    __shared__ unsigned long long mb_max[kMaxMembers];
    if (Mb.n > 1) {
        for (int m = threadIdx.x; m < Mb.n; m += blockDim.x) mb_max[m] = 0ull;
        __syncthreads();
    }
    const int64_t Tp = P.Tp, R = P.R;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Tp; i += (int64_t)gridDim.x * blockDim.x) {
        if (i >= P.T) {  // padding face: identity rows
            for (int z = 0; z < P.L; ++z) {
                const int64_t r = (int64_t)z * Tp + i;
                A.band[r] = 1.0;
                for (int k = 1; k < 6; ++k) A.band[k * R + r] = 0.0;
                A.rhs[r] = 0.0;
                A.x[r] = 0.0;
                A.u_z[r] = 0.0;
                A.csubl[r] = 0.0;
                A.fac_l[r] = 0.0;
                A.fac_ib[r] = 1.0;
                A.fac_u[r] = 0.0;
                if (A.latp) {
                    A.fac_piv[r] = 1.0;
                    for (int k = 0; k < 3; ++k) A.latp[k * R + r] = 0.0;
                }
                if (P.mixed) {
                    A.uz32[r] = 0.f;
                    if (z == 0)
                        for (int k = 0; k < 6; ++k) A.l01[k * Tp + i] = 0.f;
                    A.l32[r] = 0.f;
                    A.ib32[r] = 1.f;
                    A.up32[r] = 0.f;
                }
            }
            continue;
        }
        const int mem = Mb.face_member[i];
        const CzCoef* tab = A.cztab + (int64_t)mem * P.L;
        const double* fv = A.face_v;
        const double hs = fv[FV_HS * Tp + i];
        const double ustar = fv[FV_USTAR * Tp + i];
        const double uth = fv[FV_UTH * Tp + i];
        const double c_salt = fv[FV_CSALT * Tp + i];
        const double qc = fv[FV_QC * Tp + i];
        const double ql = fv[FV_QL * Tp + i];
        const double ef = fv[FV_EF * Tp + i];
        const double inv_logden = fv[FV_INVLOGDEN * Tp + i];
        const double kxr = 0.015 * P.cos_pi_4;  // 3 cos(pi/4) 0.005
        const bool saltation = S.saltation[i];
        const double uref = F.UR[i];
        double snow_depth = F.sd[i];
        snow_depth = is_nan_chm(snow_depth) ? 0 : snow_depth;
        double height_diff = smax(0.0, G.canopy[i] - snow_depth);
        if (!P.enable_veg) height_diff = 0;
        const double area = G.area[i];
        const double V5 = area * P.dz / 5.0;
        const double areaK = area * P.inv_dz;
        double Ak[3], al[3];
        bool out_f[3];
        int32_t nb[3];
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const double kf = fv[(FV_K0 + f) * Tp + i];
            const double Af = G.E[f * Tp + i] * P.dz;
            nb[f] = G.nbr[f * Tp + i];
            Ak[f] = Af * kf;
            out_f[f] = gt0(kf);
            al[f] = P.do_lateral_diff ? Af * 0.00001 : 0.0;
        }
        // Lateral faces, PBSM3D.cpp:1248-1284: with the face's out/in and
        // neighbour flags fixed, each face adds to the row
        //   dg  += V5cs + ca_f alpha_f + cA_f (u_z A_f k_f)
        //   lat_f = L0_f + u_z L1_f
        // (out+nbr: ca -1, cA -1, lat alpha; out, no nbr: ca -0.01, cA -1;
        //  in+nbr: ca -1, cA 0, lat alpha - Au; in, no nbr: ca -0.01, cA -0.99),
        // so the three faces fold into per-face constants and a row costs
        // four FMAs instead of lane-divergent branches.
        double dg_a = 0.0, dg_u = 0.0, L0[3], L1[3];
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const bool has = nb[f] >= 0;
            dg_a += (has ? -1.0 : -0.01) * al[f];
            dg_u += (out_f[f] ? -1.0 : (has ? 0.0 : -0.99)) * Ak[f];
            L0[f] = has ? al[f] : 0.0;
            L1[f] = (has && !out_f[f]) ? -Ak[f] : 0.0;
        }
        if (P.mixed)
#pragma unroll
            for (int f = 0; f < 3; ++f) {
                A.l01[f * Tp + i] = f32_rn(L0[f]);
                A.l01[(3 + f) * Tp + i] = f32_rn(L1[f]);
            }
        const double ust_dc = P.snow_diffusion_const * ustar;
        // Per-face versions of the per-row branch tests (no FP64 compare per
        // row): the canopy test cz < height_diff can only hold when
        // height_diff > 0, and hz < 50 m holds for every layer when the top of
        // the suspension column is below 50 m.
        const bool fast = hs == 0.0;
        const bool in_canopy_possible = height_diff > 0.0;
        const bool all_below_zur = snow_depth + hs + 5.0 + P.dz < kZUR;
        const long long b001 = __double_as_longlong(0.01);
        const bool uref_pos = uref > 0.0;
        double prev_up = 0.0, prev_ib = 1.0;
        float prev_up32 = 0.f, prev_ib32 = 1.f;
        unsigned long long face_max = 0;
        for (int z = 0; z < P.L; ++z) {
            const int64_t r = (int64_t)z * Tp + i;
            // layer terms: the member's table row, or this row of pass 2
            const double* lp = fast ? &tab[z].omega : A.slow_rows + r;
            const int64_t ls = fast ? 1 : R;
            const double omega = lp[0], qr_m = lp[ls], lmix = lp[2 * ls], rz2nu = lp[3 * ls];
            const double rsig_m = lp[4 * ls], lwarg = lp[5 * ls], ew = lp[6 * ls];
            // the layer centre is only needed by the canopy and 50 m tests,
            // which the per-face flags usually settle
            const bool need_cz = in_canopy_possible || !all_below_zur;
            const double cz = need_cz ? z * P.dz + hs + P.dz / 2. : 0.0;
            // u_z and xr = 3 cos(pi/4) 0.005 u_z^1.36: in the open below 50 m
            // with a positive wind, the face's factor times the layer's (no
            // exp per row); else u_z^1.36 directly (a branch, not a select)
            double u_z, xr = 0.0;
            bool direct = true;
            if (in_canopy_possible && saltation && cz < height_diff) {
                u_z = 2.8 * uth;
            } else if (in_canopy_possible && cz < height_diff) {
                u_z = 0.01;
            } else if (all_below_zur || cz + snow_depth < kZUR) {
                // log_scale_wind(uref, 50, hz, snow_depth, z0), clamped at 0.01 m/s
                const double u_raw = uref * lwarg * inv_logden;
                const long long ub = __double_as_longlong(u_raw);
                const bool above = ub > b001 && ub <= 0x7ff0000000000000ll;  // 0.01 < u_raw, not NaN
                u_z = above ? u_raw : 0.01;
                if (above && uref_pos) {
                    xr = ef * ew;
                    direct = false;
                }
            } else {
                u_z = fmax(0.01, uref);
            }
            if (direct) xr = kxr * pow_t(u_z, 1.36, mt);
            const double Vr = omega + xr;
            const double Nu = 1.79 + 0.606 * sqrt(rz2nu * Vr);
            // dm/dt / mm (PBSM3D.cpp:1113-1120 regrouped: the face factors qc, ql
            // times the layer factors over the mass)
            double csubl = P.iterative_subl ? qc * Nu * qr_m : fma(qc * Nu, rsig_m, -ql * qr_m);
            const double w = omega;
            double K34;
            if (P.rouault)
                K34 = (1.0 / (1.0 + (1.0 * w * w) / (1.56 * ustar * ustar))) * ustar * lmix;
            else
                K34 = ust_dc * lmix;
            if (!P.do_sublimation) csubl = 0.0;
            A.u_z[r] = u_z;
            A.csubl[r] = csubl;
            const double V5cs = V5 * csubl;
            // Vertical faces (PBSM3D.cpp:1286-1404): udotm = -w on the top
            // face, +w on the bottom one; alpha = area K / dz on both, except
            // the bottom of layer 0, which couples to the saltation layer.
            const double aw = area * w;    // area * |udotm| of a vertical face
            const double aK = areaK * K34;  // alpha[3] = alpha[4]
            const bool top_out = gt0(-w), bot_out = gt0(w);
            double lat[3], lo = 0.0, up = 0.0, b = 0.0;
#pragma unroll
            for (int f = 0; f < 3; ++f) lat[f] = fma(u_z, L1[f], L0[f]);
            // lateral faces plus the top face (every layer has one)
            double dg = fma(u_z, dg_u, fma(4.0, V5cs, dg_a)) - aK;
            if (top_out) dg += aw;
            if (z == 0) {
                const double alpha4 = area * K34 / (hs / 2.0 + P.dz / 2.0);  // once per face
                dg += V5cs - aw - alpha4;
                b = -alpha4 * c_salt;
                if (P.L > 1) up = top_out ? aK : aw + aK;
            } else {
                // bottom face; the top boundary of the last layer has no coupling
                dg += V5cs - aK;
                if (bot_out) dg -= aw;
                lo = bot_out ? aK : aK - aw;
                if (z < P.L - 1) up = top_out ? aK : aw + aK;
            }
            A.band[r] = dg;
            A.band[1 * R + r] = lat[0];
            A.band[2 * R + r] = lat[1];
            A.band[3 * R + r] = lat[2];
            A.band[4 * R + r] = lo;
            A.band[5 * R + r] = up;
            A.rhs[r] = b;
            A.x[r] = 0.0;
            // Thomas factorisation of the column: beta_z = d_z - l_z * up_{z-1}
            float l32 = 0.f, ib32 = 1.f;
            const float up32 = P.mixed ? f32_rn(up) : 0.f;
            if (P.fac64) {
                const double lz = (z == 0) ? 0.0 : lo * prev_ib;
                const double beta = (z == 0) ? dg : dg - lz * prev_up;
                const double ib = rcp_t(beta);
                // the factors scaled by the inverse pivot (the FP64 column
                // solve's form), and for the FP64 polynomial steps the pivot
                // and the lateral bands times ib
                A.fac_l[r] = ib * lo;
                A.fac_ib[r] = ib;
                A.fac_u[r] = ib * up;
                if (A.latp) {
                    A.fac_piv[r] = beta;
#pragma unroll
                    for (int f = 0; f < 3; ++f) A.latp[f * R + r] = ib * lat[f];
                }
                if (P.mixed) {
                    l32 = f32_rn(lz);
                    ib32 = f32_rn(ib);
                }
                prev_ib = ib;
                if (nonfinite(ib)) bad = true;
            } else {
                // MIXED, no FP64 factors needed: the FP32 preconditioner's own
                // factorisation of the FP32-rounded column, on the FP32 pipe.
                // It only preconditions; the refinement's FP64 residual decides.
                const float dg32 = f32_rn(dg);
                l32 = (z == 0) ? 0.f : f32_rn(lo) * prev_ib32;
                ib32 = __frcp_rn((z == 0) ? dg32 : __fmaf_rn(-l32, prev_up32, dg32));
                prev_ib32 = ib32;
            }
            if (P.mixed) {
                A.uz32[r] = f32_rn(u_z);
                A.l32[r] = l32;
                A.ib32[r] = ib32;
                A.up32[r] = up32;
            }
            prev_up = up;
            prev_up32 = up32;
            vmax_bits = max(vmax_bits, abs_bits(b));
            face_max = max(face_max, abs_bits(b));
            if (nonfinite(dg) | nonfinite(b) | nonfinite(lat[0]) | nonfinite(lat[1]) | nonfinite(lat[2]) |
                nonfinite(lo) | nonfinite(up))
                bad = true;
        }
        if (Mb.n > 1) atomicMax(&mb_max[mem], face_max);
    }
    if (Mb.n > 1) {
        __syncthreads();
        for (int m = threadIdx.x; m < Mb.n; m += blockDim.x)
            if (mb_max[m]) atomicMax(&Mb.rhs_max[m], mb_max[m]);
    }
    // ||rhs||_inf (as the bit pattern of a non-negative double, whose integer
    // order is its numeric order) and the NaN/Inf flag: last block finalises
    const double vmax = __longlong_as_double((long long)vmax_bits), vnan = bad ? 1.0 : 0.0;
    double mv[2] = {vmax, vnan}, tot[2];
    if (block_partials_last_max<2>(mv, partials, &sc->counter[0], tot) && threadIdx.x == 0) {
        sc->rhs_max = tot[0];
        sc->nan_flag = tot[1];
    }
}

// PBSM3D.cpp:1467-1503 (column post) fused with :1516-1658 (deposition rows).
// Qsusp/Qsalt of the neighbours are needed, so the post runs first in its own
// kernel; the deposition kernel then gathers.
__global__ void __launch_bounds__(kBlock) k_post(Params P, Susp A, FaceState S) {
    const int64_t Tp = P.Tp;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.T; i += (int64_t)gridDim.x * blockDim.x) {
        double Qsusp = 0, Qsubl = 0;
        for (int z = 0; z < P.L; ++z) {
            const int64_t r = (int64_t)z * Tp + i;
            double c = A.x[r];
            c = c < 0 || is_nan_chm(c) ? 0 : c;
            Qsusp += c * A.u_z[r] * P.dz;
            Qsubl += A.csubl[r] * c * P.dz;
        }
        S.Qsusp[i] = Qsusp;
        S.Qsubl[i] = Qsubl;
        const double qm = Qsubl * P.dt;
        S.Qsubl_mass[i] = qm;
        S.sum_subl[i] += qm;
    }
}

__global__ void __launch_bounds__(kBlock) k_assemble_deposition(Params P, Faces G, Forcing F, FaceState S, Dep D,
                                                               Members Mb, const double* __restrict__ face_v,
                                                               double* partials, Scalars* sc) {
    const int64_t Tp = P.Tp;
    double vmax = 0, vnan = 0;
    __shared__ unsigned long long mb_max[kMaxMembers];
    if (Mb.n > 1) {
        for (int m = threadIdx.x; m < Mb.n; m += blockDim.x) mb_max[m] = 0ull;
        __syncthreads();
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Tp; i += (int64_t)gridDim.x * blockDim.x) {
        if (i >= P.T) {
            D.diag[i] = 1.0;
            D.dinv[i] = 1.0;
            for (int j = 0; j < 3; ++j) D.off[j * Tp + i] = 0.0;
            D.rhs[i] = 0.0;
            D.x[i] = 0.0;
            continue;
        }
        // the unit wind vector of pass 1
        const double ux = face_v[FV_UX * Tp + i], uy = face_v[FV_UY * Tp + i];
        double dg = G.area[i];  // replace, PBSM3D.cpp:1546
        double b = 0.0;
        const double Qs_self = S.Qsusp[i], Qa_self = S.Qsalt[i];
        for (int j = 0; j < 3; ++j) {
            const double udm = dot2(ux, uy, G.mx[j * Tp + i], G.my[j * Tp + i]);
            const double Ej = G.E[j * Tp + i];
            const int32_t nb = G.nbr[j * Tp + i];
            double Qtj, Qsj;
            if (udm > 0) {
                Qtj = Qs_self;
                Qsj = Qa_self;
            } else if (nb >= 0) {
                Qtj = S.Qsusp[nb];
                Qsj = S.Qsalt[nb];
                if (is_nan_chm(Qsj)) Qsj = 0;
            } else {
                Qtj = Qs_self;
                Qsj = Qa_self;
            }
            double off = 0.0;
            if (nb >= 0) {
                const double w = G.depw[j * Tp + i];  // eps E_j / dx_j
                dg += w;
                off += -w;
            }
            D.off[j * Tp + i] = off;
            b += -Ej * (Qtj + Qsj) * udm;
        }
        D.diag[i] = dg;
        D.dinv[i] = 1.0 / dg;
        D.rhs[i] = b;
        D.x[i] = 0.0;
        vmax = fmax(vmax, fabs(b));
        if (Mb.n > 1) atomicMax(&mb_max[Mb.face_member[i]], abs_bits(b));
        if (isnan(dg) || isnan(b)) vnan = 1.0;
    }
    if (Mb.n > 1) {
        __syncthreads();
        for (int m = threadIdx.x; m < Mb.n; m += blockDim.x)
            if (mb_max[m]) atomicMax(&Mb.dep_max[m], mb_max[m]);
    }
    double mv[2] = {vmax, vnan}, tot[2];
    if (block_partials_last_max<2>(mv, partials, &sc->counter[0], tot) && threadIdx.x == 0) {
        sc->rhs_max = tot[0];
        sc->nan_flag = tot[1];
    }
}

// PBSM3D.cpp:1710-1740 plus the FP64 mass ledger (deterministic partial sums).
// rres holds b - A q from the solver's final residual.
__global__ void __launch_bounds__(kBlock) k_update(Params P, Faces G, Forcing F, FaceState S, Dep D, const double* rres,
                                                   int deposition_present, const int* dep_flag, Members Mb,
                                                   double* partials, Scalars* sc, double* ledger) {
    if (dep_flag) deposition_present = *dep_flag;  // graph mode: decided on the device
    double v[4] = {0, 0, 0, 0};  // divergence, deposited, clipped, residual
    double snow = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.T; i += (int64_t)gridDim.x * blockDim.x) {
        double swe = F.swe[i];
        swe = is_nan_chm(swe) ? 0 : swe;
        const double area = G.area[i];
        snow += area * swe;
        if (!deposition_present) continue;
        if (Mb.n > 1 && !Mb.dep_present[Mb.face_member[i]]) continue;  // this member had no deposition
        const double q = D.x[i];
        const double qdep = is_nan_chm(q) ? 0 : q;
        double mass = qdep * P.dt;
        if (mass < 0 && fabs(mass) > swe) {
            S.more[i] = 1;
            mass = -swe;
        }
        if (mass < 0 && !S.saltation[i]) mass = 0;
        S.drift_mass[i] = mass;
        S.sum_drift[i] += mass;
        v[0] += P.dt * D.rhs[i];
        v[1] += P.dt * area * q;
        v[2] += area * (mass - q * P.dt);
        v[3] += P.dt * rres[i];
    }
    double w[5] = {v[0], v[1], v[2], v[3], snow}, tot[5];
    if (block_partials_last<5>(w, partials, &sc->counter[1], tot) && threadIdx.x == 0)
        for (int k = 0; k < 5; ++k) ledger[k] = tot[k];
}

// The drift consumer of CHM's snow models on the device (snobal.cpp:363-387
// and its _adj_snow): erosion removes depth at the pack's bulk density,
// deposition adds it at drift_density; a pack whose depth or mass reaches 0
// is removed.
__global__ void __launch_bounds__(kBlock) k_consume_drift(Params P, FaceState S, Forcing F, double drift_density) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.T; i += (int64_t)gridDim.x * blockDim.x) {
        double mass = S.drift_mass[i];
        mass = is_nan_chm(mass) ? 0.0 : mass;
        double swe = F.swe[i], depth = F.sd[i];
        swe = is_nan_chm(swe) ? 0.0 : swe;
        depth = is_nan_chm(depth) ? 0.0 : depth;
        const double rho = (mass < 0.0 && depth > 0.0) ? swe / depth : drift_density;
        depth += mass / rho;
        swe += mass;
        if (depth <= 0.0 || swe <= 0.0) {
            depth = 0.0;
            swe = 0.0;
        }
        F.swe[i] = swe;
        F.sd[i] = depth;
    }
}

// Ensembles: zero the right-hand sides of members without suspension (or
// deposition) so their solution is exactly 0, as the reference's skipped
// solve leaves it; and ||rhs_m||^2 per member.
__global__ void k_member_mask_norm(Params P, Members Mb, double* rhs, int layers, const int* present, double* bb) {
    __shared__ double sbb[kMaxMembers];
    for (int m = threadIdx.x; m < Mb.n; m += blockDim.x) sbb[m] = 0.0;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.T; i += (int64_t)gridDim.x * blockDim.x) {
        const int m = Mb.face_member[i];
        double acc = 0.0;
        for (int z = 0; z < layers; ++z) {
            const int64_t r = (int64_t)z * P.Tp + i;
            if (!present[m]) rhs[r] = 0.0;
            acc += rhs[r] * rhs[r];
        }
        atomicAdd(&sbb[m], acc);
    }
    __syncthreads();
    for (int m = threadIdx.x; m < Mb.n; m += blockDim.x)
        if (sbb[m] != 0.0) atomicAdd(&bb[m], sbb[m]);
}

// Ensembles: a warm start of a member without suspension is reset to 0 (its
// right-hand side is 0, so the joint Krylov solve then keeps it exactly 0).
__global__ void k_member_zero(Params P, Members Mb, double* x, const int* present) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.T; i += (int64_t)gridDim.x * blockDim.x) {
        if (present[Mb.face_member[i]]) continue;
        for (int z = 0; z < P.L; ++z) x[(int64_t)z * P.Tp + i] = 0.0;
    }
}

// Centroid distances to neighbours (distance_UTM, coordinates.cpp:100-106).
// The deposition rows' static couplings eps E_j / dx_j (PBSM3D.cpp:1560-1580,
// dx the centroid distance, distance_UTM), once per mesh instead of per step.
__global__ void k_init_static(Params P, Faces G, const double* cx, const double* cy) {
    const int64_t Tp = P.Tp;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Tp; i += (int64_t)gridDim.x * blockDim.x) {
        for (int j = 0; j < 3; ++j) {
            const int32_t nb = G.nbr[j * Tp + i];
            double w = 0.0;
            if (nb >= 0 && i < P.T) {
                const double ddx = cx[i] - cx[nb];
                const double ddy = cy[i] - cy[nb];
                const double d = sqrt(ddx * ddx + ddy * ddy);
                w = P.eps * G.E[j * Tp + i] / d;
            }
            G.depw[j * Tp + i] = w;
        }
    }
}

}  // namespace

void launch_member_mask_norm(Ctx& c, cudaStream_t s, int which) {
    cudaMemsetAsync(c.Mb.bb, 0, sizeof(double) * c.Mb.n, s);
    prof_begin(c, s);
    if (which == 0)
        k_member_mask_norm<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.Mb, c.A.rhs, c.P.L, c.Mb.susp_present, c.Mb.bb);
    else
        k_member_mask_norm<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.Mb, c.D.rhs, 1, c.Mb.dep_present, c.Mb.bb);
    prof_end(c, s, PBSM3D_K_OTHER, c.P.T * (which == 0 ? c.P.L : 1) * 16);
}

void launch_member_zero(Ctx& c, cudaStream_t s, double* x) {
    prof_begin(c, s);
    k_member_zero<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.Mb, x, c.Mb.susp_present);
    prof_end(c, s, PBSM3D_K_OTHER, c.P.T * 4);
}

void launch_assemble_suspension(Ctx& c, cudaStream_t s) {
    const int64_t T = c.P.T, rows = T * c.P.L;
    // the three passes count as one assembly; the algorithmic bytes are those
    // of the whole step: per face 8 forcing + 133 B geometry in, Qsalt + flag
    // out (+6 floats of coupling constants MIXED); per row 10 doubles out, 3
    // more with the FP64 column factors, 4 more with the FP64 polynomial
    // preconditioner's scaled bands and pivot, 4 floats MIXED
    prof_begin(c, s);
    cudaMemsetAsync(c.A.n_slow, 0, sizeof(int), s);
    // the wind inputs on the device (scale_wind_vert, fetchr), when asked for
    if (c.cfg.derive_wind) launch_scale_wind_vert(c, s, c.Fo.UR, c.Fo.sd, c.Fo.U2);
    if (c.cfg.derive_fetch) launch_fetchr(c, s, c.Fo.dir, c.Fo.fetch);
    if (c.P.subgrid) launch_subgrid(c, s);
    k_salt_faces<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.F, c.Fo, c.S, c.A, c.Mb);
    k_salt_terms<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.F, c.Fo, c.S, c.A, c.Mb);
    k_salt_rows<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.Fo, c.A, c.Mb);
    k_assemble_suspension<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.F, c.Fo, c.S, c.A, c.Mb, c.red.partials, c.sc);
    prof_end(c, s, PBSM3D_K_ASSEMBLE,
             T * (64 + 133 + 9 + (c.P.mixed ? 24 : 0)) +
                 rows * (80 + (c.P.fac64 ? 24 : 0) + (c.A.latp ? 32 : 0) + (c.P.mixed ? 16 : 0)));
    c.launches += c.asm_kernels;
}

void launch_post_and_assemble_deposition(Ctx& c, cudaStream_t s) {
    const int64_t T = c.P.T, rows = T * c.P.L;
    prof_begin(c, s);
    k_post<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.A, c.S);
    prof_end(c, s, PBSM3D_K_POST, rows * 24 + T * 40);
    prof_begin(c, s);
    k_assemble_deposition<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.F, c.Fo, c.S, c.D, c.Mb, c.A.face_v, c.red.partials,
                                                          c.sc);
    prof_end(c, s, PBSM3D_K_DEP_ASSEMBLE, T * 196);
}

void launch_consume_drift(Ctx& c, cudaStream_t s) {
    prof_begin(c, s);
    k_consume_drift<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.S, c.Fo, c.drift_density);
    prof_end(c, s, PBSM3D_K_UPDATE, c.P.T * 40);
}

void launch_update(Ctx& c, cudaStream_t s) {
    prof_begin(c, s);
    k_update<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.F, c.Fo, c.S, c.D, c.dr, c.deposition_present ? 1 : 0,
                                             c.graph_dep_flag, c.Mb, c.red.partials, c.sc, c.ledger);
    prof_end(c, s, PBSM3D_K_UPDATE, c.P.T * 81);
}

// cx, cy: the centroid x/y staged in the CG work vectors by pbsm3d_create
void launch_init_static(Ctx& c, cudaStream_t s) {
    k_cz_table<<<(c.Mb.n * c.P.L + 63) / 64, 64, 0, s>>>(c.P, c.Mb, c.A.cztab);
    k_init_static<<<c.grid_faces, kBlock, 0, s>>>(c.P, c.F, c.dr, c.dz_);
}

void math_tables_fill(MathTables& h) {
    for (int j = 0; j < 256; ++j) {
        h.exp2j[j] = (double)exp2l((long double)j / 256.0L);
        const double c = 1.0 / (1.0 + (j + 0.5) / 256.0);
        h.logc[j] = c;
        h.logl[j] = (double)(-logl((long double)c));
    }
}

}  // namespace pbsm
