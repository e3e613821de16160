/*
 * pbsm3d_oracle.h -- CPU oracle of the PBSM3D blowing-snow step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for
 * libpbsm3d_cuda: only the test suite, the smoke check and the CPU-baseline
 * leg of the benchmark load it.  The product path never links or calls it.
 *
 * It restates, loop by loop, CHM's src/modules/PBSM3D.cpp (init :221-398,
 * run :400-1748, checkpoint :1753-1773) and the solver settings of
 * src/math/LinearAlgebra.cpp:31-252 (GMRES(30), ILUT drop 1e-4 fill 3,
 * tol 1e-8, x0 = 0).  Trilinos (Belos/Ifpack2 15.0.0) and MeteoIO are not
 * available; their published algorithms are restated here (see the
 * function comments).  Parity status: the helpers log_scale_wind and
 * saturatedVapourPressure are pinned against the reference's own
 * src/physics/Atmosphere.cpp compiled from source; mesh adjacency and
 * geometry are pinned against the reference's mesh fixtures; the PBSM3D
 * step itself has no reference test or golden vector, so its parity is
 * unpinned beyond this restatement.
 */
#ifndef PBSM3D_ORACLE_H
#define PBSM3D_ORACLE_H

#include "../include/pbsm3d.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

/* Solver settings of the oracle.  Defaults = the reference's
 * (LinearAlgebra.cpp:164-187): restart 30, maxit 1000, tol 1e-8,
 * ILUT drop 1e-4, level-of-fill 3, one block (one MPI rank). nblocks > 1
 * factors ILUT independently per contiguous block of faces (what Ifpack2
 * does per MPI rank) and runs the blocks on OpenMP threads. */
typedef struct oracle_solver_cfg {
    int32_t restart;
    int32_t maxit;
    double tol;
    double ilut_drop;
    double ilut_fill;
    int32_t nblocks;
    int32_t dep_maxit;
    double dep_tol;
} oracle_solver_cfg;

int oracle_create(const pbsm3d_mesh_desc* mesh, const pbsm3d_config* cfg, oracle_ctx** out);
void oracle_destroy(oracle_ctx* ctx);
void oracle_solver_defaults(oracle_solver_cfg* s);
int oracle_set_solver(oracle_ctx* ctx, const oracle_solver_cfg* s);
/* OpenMP threads of the process's later parallel regions (the CPU timing at
 * a stated core count); returns the count in effect before the call. */
int oracle_set_threads(int n);
const char* oracle_last_error(const oracle_ctx* ctx);

/* Whole step (PBSM3D::run). */
int oracle_step(oracle_ctx* ctx, const pbsm3d_forcing* f, double dt, const pbsm3d_outputs* out,
                pbsm3d_stats* stats);

/* The same step in stages, so a test can substitute an exact solution. */
int oracle_stage_assemble_suspension(oracle_ctx* ctx, const pbsm3d_forcing* f, double dt);
int oracle_stage_solve_suspension(oracle_ctx* ctx);
int oracle_stage_set_suspension_solution(oracle_ctx* ctx, const double* x);
int oracle_stage_post_and_assemble_deposition(oracle_ctx* ctx);
int oracle_stage_solve_deposition(oracle_ctx* ctx);
int oracle_stage_set_deposition_solution(oracle_ctx* ctx, const double* q);
int oracle_stage_update(oracle_ctx* ctx, const pbsm3d_outputs* out, pbsm3d_stats* stats);

/* CSR of the last assembled system (which: 0 suspension, 1 deposition), graph
 * order per row (self, lateral 0..2 present, below, above).  rowptr [rows+1]. */
int64_t oracle_rows(const oracle_ctx* ctx, int32_t which);
int64_t oracle_nnz(const oracle_ctx* ctx, int32_t which);
int oracle_get_system(const oracle_ctx* ctx, int32_t which, int64_t* rowptr, int32_t* cols, double* vals,
                      double* rhs, double* x);
/* Per-face intermediate fields of the last step: saltation flag, hs, z0,
 * ustar, c_salt, u*_th; per-row u_z and csubl ([nLayer*n]). NULL = skip. */
int oracle_get_face_fields(const oracle_ctx* ctx, double* saltation, double* hs, double* z0, double* ustar,
                           double* c_salt, double* ustar_th, double* u_z, double* csubl);
int oracle_get_state(const oracle_ctx* ctx, double* sum_drift, double* sum_subl, double* drift_mass,
                     double* more_than_avail);
int oracle_set_state(oracle_ctx* ctx, const double* sum_drift, const double* sum_subl, const double* drift_mass,
                     const double* more_than_avail);

/* Helpers restated from the reference, exported for unit tests. */
double oracle_log_scale_wind(double u, double z_in, double z_out, double snowdepthavg, double z0);
double oracle_saturated_vapour_pressure(double T);
void oracle_bearing_to_cartesian(double bearing, double* xy);
double oracle_std_dry_air_density(double altitude, double temperature);
/* Li and Pomeroy (2000) eqn 5 friction velocity (z0_ustar_coupling); returns
 * 0 when no bracket is found, 1 otherwise. */
int oracle_coupled_ustar(double u2, double lambda, double* ustar);
/* ice-bulb temperature (C) of iterative_subl: T in C, t in K, ea in kPa */
double oracle_ice_bulb_temperature(double T, double t, double ea, double D, double lambda_t, double L);
/* regularised incomplete gamma P(a, x), Q(a, x) and the gamma density (shape a, scale b) */
void oracle_incomplete_gamma(double a, double x, double* P, double* Q);
double oracle_gamma_pdf(double x, double a, double b);
/* subgrid topography of one face (use_subgrid_topo / _V2 per cfg): tpi[5] =
 * TPI_mean, TPI_std, TPI_neg_frac, TPI_neg_mean, TPI_neg_std; out[5] =
 * hold_topo, frac_contrib, frac_contrib_nosnw, tpi_lim, test_int (-9999 when
 * the normalisation integral is not evaluated) */
void oracle_subgrid_face(const pbsm3d_config* cfg, double snow_depth, const double* tpi, double* out);
/* the wind-input modules: scale_wind_vert (U_2m_above_srf from U_R) and fetchr
 * (fetch from vw_dir) over the context's mesh; snowdepthavg may be NULL */
int oracle_scale_wind_vert(const oracle_ctx* c, int ignore_canopy, const double* U_R, const double* snowdepthavg,
                           double* u2m);
int oracle_fetchr(const oracle_ctx* c, int steps, double max_distance, double I, int incl_veg, const double* vw_dir,
                  double* fetch);
/* uniform_wind from stations (interp 0 spline, 1 IDW, 2 nearest) and the face's
 * station list (n_nearest > 0, or radius); -1 when a face has no valid station */
int oracle_uniform_wind(const oracle_ctx* c, int64_t ns, const double* sx, const double* sy, int n_nearest,
                        double radius, int interp, const double* st_U, const double* st_dir, double* U_R,
                        double* vw_dir);
double oracle_expint_e1(double x);
double oracle_tps(const double* sx, const double* sy, const double* sz, int n, double qx, double qy);
/* Face geometry of a triangle mesh (triangulation.hpp:1443-1498,1577-1589,1830-1856).
 * xyz [3*nv], tri [3*nt] vertex ids; outputs [3*nt], [6*nt], [nt], [3*nt]. */
void oracle_face_geometry(int64_t nv, const double* xyz, int64_t nt, const int32_t* tri, double* edge_length,
                          double* edge_normal, double* area, double* center);
/* Face adjacency: neigh[3*i+j] = face across the edge opposite vertex j, -1 if none. */
int oracle_face_neighbors(int64_t nv, int64_t nt, const int32_t* tri, int32_t* neigh);

/* Fixed-size dense MLP reference in FP64 (learned warm start), for gradient
 * checks of the GPU training kernels.  Layers: 14->128->128->128->1, ReLU.
 * Weights row-major [out][in].  Computes the loss 0.5*mean((y-t)^2) over
 * n rows and its gradients. */
double oracle_mlp_loss_grad(int64_t n, const float* x, const float* target, const float* w0, const float* b0,
                            const float* w1, const float* b1, const float* w2, const float* b2, const float* w3,
                            const float* b3, double* gw0, double* gb0, double* gw1, double* gb1, double* gw2,
                            double* gb2, double* gw3, double* gb3, double* y_out);

#ifdef __cplusplus
}
#endif
#endif
