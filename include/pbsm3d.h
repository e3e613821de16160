/*
 * pbsm3d.h -- C ABI of libpbsm3d_cuda, the GB300 (sm_103a) implementation of
 * CHM's PBSM3D blowing-snow timestep.
 *
 * One context owns one mesh resident in HBM.  A step runs, entirely on the
 * GPU: saltation, suspension coefficients, the sliced-ELL assembly of the
 * 3-D suspension advection-diffusion system, its Krylov solve, the column
 * post-processing (Qsusp, Qsubl), the assembly and solve of the 2-D drift
 * flux-divergence (deposition) system and the erosion/deposition update.
 *
 * Reference interfaces replaced (Chrismarsh/CHM):
 *   pbsm3d_create   <- PBSM3D::PBSM3D(config_file)   src/modules/PBSM3D.cpp:103-219
 *                      PBSM3D::init(mesh&)           src/modules/PBSM3D.cpp:221-398
 *                      NearestNeighborProblem ctor   src/math/LinearAlgebra.cpp:31-197
 *   pbsm3d_step     <- PBSM3D::run(mesh&)            src/modules/PBSM3D.cpp:400-1748
 *   pbsm3d_get_state/pbsm3d_set_state
 *                   <- PBSM3D::checkpoint / load_checkpoint
 *                                                    src/modules/PBSM3D.cpp:1753-1773
 *   error codes     <- CHM_THROW_EXCEPTION(module_error, ...)
 *                                                    src/modules/PBSM3D.cpp:1447,1704
 * and, around the step: the upstream wind modules (pbsm3d_scale_wind_vert,
 * pbsm3d_fetchr, pbsm3d_uniform_wind), the snow models' consumption of
 * drift_mass (pbsm3d_set_snow), CHM's JSON mesh reader (pbsm3d_mesh_read),
 * and batched parameter ensembles (pbsm3d_ensemble_create).
 *
 * Conventions
 *   - Plain C structs, POD arrays, no exceptions across the ABI.
 *   - Per-face arrays are indexed by the face's position in the mesh
 *     (CHM cell_local_id == cell_global_id for a single-process mesh,
 *     src/mesh/triangulation.cpp:300-302).  [3*n] arrays are row-major
 *     (face, j).  neighbor[3*i+j] is the face across the edge opposite
 *     vertex j (CGAL convention), -1 when there is none.
 *   - Layered arrays ([nLayer*n]) are layer-major: index z*n + i, the
 *     ordering of the reference's extruded map (LinearAlgebra.cpp:46-55).
 *   - Return 0 on success, a negative PBSM3D_ERR_* on failure; the message
 *     is available from pbsm3d_last_error().
 *   - A context is not thread-safe; use one context per host thread.
 */
#ifndef PBSM3D_H
#define PBSM3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBSM3D_ABI_VERSION 3

enum pbsm3d_status {
    PBSM3D_OK = 0,
    PBSM3D_ERR_INVALID_ARG = -1,
    PBSM3D_ERR_BAD_MESH = -2,
    PBSM3D_ERR_NAN_INPUT = -3,
    PBSM3D_ERR_NOT_CONVERGED = -4,
    PBSM3D_ERR_CUDA = -5,
    PBSM3D_ERR_UNSUPPORTED = -6,
    PBSM3D_ERR_OUT_OF_MEMORY = -7
};

/* Krylov method of the suspension solve. */
enum pbsm3d_solver {
    PBSM3D_SOLVER_BICGSTAB = 0, /* right-preconditioned BiCGStab (default) */
    PBSM3D_SOLVER_GMRES = 1     /* right-preconditioned restarted GMRES(m) */
};

/* Arithmetic of the suspension solve. */
enum pbsm3d_precision {
    PBSM3D_FP64 = 0,  /* FP64 matrix, preconditioner and Krylov vectors */
    PBSM3D_MIXED = 1  /* FP32 SpMV + preconditioner inside FP64 iterative refinement */
};

/* Initial guess of the suspension solve. */
enum pbsm3d_warm_start {
    PBSM3D_X0_ZERO = 0,     /* x0 = 0 every step, as the reference (LinearAlgebra.cpp:199-206) */
    PBSM3D_X0_PREVIOUS = 1, /* previous step's concentration field */
    PBSM3D_X0_LEARNED = 2   /* per-row MLP prediction (pbsm3d_set_mlp) */
};

/*
 * Module configuration.  Every key of the reference is here with the
 * reference default (PBSM3D.cpp:123-145, 223-258); pbsm3d_config_defaults()
 * fills them.  Fields after "debug_output" are this library's additions and
 * default to the reference behaviour.
 */
typedef struct pbsm3d_config {
    int32_t abi_version;            /* PBSM3D_ABI_VERSION */
    int32_t nLayer;                 /* "nLayer" 10 */
    int32_t do_fixed_settling;      /* "do_fixed_settling" false */
    int32_t do_sublimation;         /* "do_sublimation" true */
    int32_t do_lateral_diff;        /* "do_lateral_diff" true */
    int32_t rouault_diffusion_coef; /* "rouault_diffusion_coef" false */
    int32_t enable_veg;             /* "enable_veg" true */
    int32_t iterative_subl;         /* "iterative_subl" false */
    int32_t use_exp_fetch;          /* "use_exp_fetch" false */
    int32_t use_tanh_fetch;         /* "use_tanh_fetch" true */
    int32_t use_PomLi_probability;  /* "use_PomLi_probability" false */
    int32_t z0_ustar_coupling;      /* "z0_ustar_coupling" false */
    int32_t use_subgrid_topo;       /* "use_subgrid_topo" false */
    int32_t use_subgrid_topo_V2;    /* "use_subgrid_topo_V2" false */
    int32_t use_R94_lambda;         /* "use_R94_lambda" true */
    int32_t debug_output;           /* "debug_output" false (diagnostics: pbsm3d_get_debug) */
    double settling_velocity;       /* "settling_velocity" 0.5 m/s, must be >= 0 */
    double smooth_coeff;            /* "smooth_coeff" 820 (Laplacian smoothing eps) */
    double min_sd_trans;            /* "min_sd_trans" 0.1 m */
    double cutoff;                  /* "cutoff" 0.3 m */
    double snow_diffusion_const;    /* "snow_diffusion_const" 0.3 */

    /* Parameter perturbations of an ensemble member (identity defaults). */
    double ustar_th_scale;  /* multiplies the threshold friction velocity, 1.0 */
    double z0_snow;         /* aerodynamic roughness of snow, 0.01 m (Snow::Z0_SNOW) */
    double settling_scale;  /* multiplies the settling velocity, 1.0 */

    /* Solver settings. */
    int32_t solver;         /* enum pbsm3d_solver, BICGSTAB */
    int32_t precision;      /* enum pbsm3d_precision, FP64 */
    int32_t warm_start;     /* enum pbsm3d_warm_start, ZERO */
    int32_t gmres_restart;  /* GMRES(m) restart length, 30 (LinearAlgebra.cpp:166) */
    int32_t susp_maxit;     /* 1000 (LinearAlgebra.cpp:167) */
    int32_t dep_maxit;      /* 1000 */
    double susp_tol;        /* relative residual ||b-Ax||/||b||, 1e-8 (LinearAlgebra.cpp:168) */
    double dep_tol;         /* deposition relative residual, 1e-10 */
    double inner_tol;       /* MIXED: FP32 inner relative reduction per refinement sweep, 1e-4 */
    int32_t warm_flags;     /* warm starts: bit 0 = no residual-optimal rescaling of x0,
                               bit 1 = no block-Jacobi sweep after the learned guess; 0 */
    int32_t graph;          /* 1: run each step as one CUDA-graph launch with device-side control
                               (conditional nodes; no host round trip inside the step); 0 */
    int32_t autotune;       /* 1: the first suspension solves time the column kernels (the vector
                               updates fused with the column Thomas solves, and the polynomial-
                               preconditioner steps) at nine launch geometries -- slices of 256, 128
                               or 64 faces a block, 1, 2 or 4 threads a face column -- one iteration
                               each, and keep the fastest (shared by later contexts of the same
                               shape).  Every geometry gives bit-identical results; 1 */
    int32_t neumann;        /* order K (0..9) of the polynomial preconditioner of the suspension
                               Krylov solve: M^-1 = B^-1 sum_{j<=K} (-N B^-1)^j, B the column
                               (tridiagonal) blocks, N the lateral couplings; 0 = B^-1 alone.
                               Odd K make A M^-1 = I - (N B^-1)^(K+1), whose spectrum stays on one
                               side of 1, and converge best */
    /* The wind inputs on the device (the upstream modules of PBSM3D in a CHM
     * configuration), see pbsm3d_scale_wind_vert / pbsm3d_fetchr below. */
    int32_t derive_wind;         /* 1: every step computes U_2m_above_srf from U_R and the snow depth
                                    (scale_wind_vert) and ignores the forcing's; 0 */
    int32_t wind_ignore_canopy;  /* scale_wind_vert "ignore_canopy", false */
    int32_t derive_fetch;        /* 1: every step computes fetch from vw_dir (fetchr); 0 */
    int32_t fetch_steps;         /* fetchr "steps", 10 */
    int32_t fetch_incl_veg;      /* fetchr "incl_veg", true */
    int32_t dep_neumann;         /* 1: the deposition CG preconditioned by the order-1 truncated Neumann
                                    series of its Jacobi splitting, M^-1 = D^-1 + D^-1 R D^-1
                                    (A = D - R; SPD for the diagonally dominant deposition matrix),
                                    about half the iterations of Jacobi; 0 = D^-1 alone */
    int32_t reserved[2];
    double fetch_max_distance;   /* fetchr "max_distance", 1000 m */
    double fetch_I;              /* fetchr "I", 0.06 */
} pbsm3d_config;

/*
 * Mesh description: per-face geometry as CHM's triangulation computes it.
 *   edge_length[3*i+j]  face->edge_length(j)          triangulation.hpp:1493-1498
 *   edge_normal[6*i+2j+{0,1}] face->edge_unit_normal(j) triangulation.hpp:1443-1463
 *   area[i]             face->get_area()              triangulation.hpp:1830-1856
 *   center[3*i+{0,1,2}] face->center() (centroid x, y, z)  triangulation.hpp:1577-1589
 * Optional arrays may be NULL.  has_vegetation NULL with canopy_height
 * non-NULL means every face has vegetation; canopy_height NULL means none.
 * All pointers are host pointers, read during pbsm3d_create only.
 */
typedef struct pbsm3d_mesh_desc {
    int64_t n_faces;
    const int32_t* neighbor;       /* [3*n] */
    const double* edge_length;     /* [3*n] */
    const double* edge_normal;     /* [6*n] */
    const double* area;            /* [n] */
    const double* center;          /* [3*n] */
    const uint8_t* has_vegetation; /* [n] or NULL */
    const double* canopy_height;   /* [n] "CanopyHeight" or NULL */
    const double* lai;             /* [n] "LAI" or NULL */
    const double* stalk_number;    /* [n] "stalk_number" or NULL (default 1) */
    const double* stalk_diameter;  /* [n] "stalk_diameter" or NULL (default 0.8) */
    const uint8_t* is_water;       /* [n] landcover is_water flag or NULL */
    /* Subgrid topographic-position-index statistics, the mesh parameters
     * read by use_subgrid_topo_V2 (TPI_mean, TPI_std; PBSM3D.cpp:494-498) and
     * use_subgrid_topo (TPI_neg_frac, TPI_neg_mean, TPI_neg_std; :607-613).
     * NULL, NaN or -9999 on a face: the parameter is undefined there and the
     * branch keeps its defaults for that face. */
    const double* tpi_mean;        /* [n] "TPI_mean" or NULL */
    const double* tpi_std;         /* [n] "TPI_std" or NULL */
    const double* tpi_neg_frac;    /* [n] "TPI_neg_frac" or NULL */
    const double* tpi_neg_mean;    /* [n] "TPI_neg_mean" or NULL */
    const double* tpi_neg_std;     /* [n] "TPI_neg_std" or NULL */
} pbsm3d_mesh_desc;

/*
 * Per-step forcing, SoA, n_faces doubles each (the depends list of
 * PBSM3D.cpp:105-138).  CHM's "nan" value -9999 is accepted where the
 * reference accepts it (swe, snowdepthavg).  fetch may be NULL when neither
 * fetch formulation is enabled; p_snow_hours is read only by
 * use_PomLi_probability.  on_device: 0 = host pointers (copied in by the
 * step), 1 = device pointers already resident in HBM.
 */
typedef struct pbsm3d_forcing {
    const double* U_R;
    const double* U_2m_above_srf;
    const double* vw_dir;
    const double* swe;
    const double* t;
    const double* rh;
    const double* snowdepthavg;
    const double* fetch;
    const double* p_snow_hours;
    int32_t on_device;
} pbsm3d_forcing;

/*
 * Per-step outputs (the provides list of PBSM3D.cpp:112-188), n_faces
 * doubles each, NULL = not wanted.  drift_mass, sum_drift, sum_subl,
 * pbsm_more_than_avail and blowingsnow_probability are module state held in
 * the context and copied out every step: like the reference, drift_mass keeps
 * its previous value in a step without deposition (PBSM3D.cpp:1742-1745) and
 * starts at -9999.  c, when non-NULL, receives the nLayer*n_faces suspension
 * concentrations (kg m^-3), layer-major.
 */
typedef struct pbsm3d_outputs {
    double* Qsalt;
    double* Qsusp;
    double* Qsubl;
    double* Qsubl_mass;
    double* sum_subl;
    double* drift_mass;
    double* sum_drift;
    double* pbsm_more_than_avail;
    double* blowingsnow_probability;
    double* c;
    /* provided with use_subgrid_topo / use_subgrid_topo_V2 (PBSM3D.cpp:204-218):
     * frac_contrib and hold_topo with either, frac_contrib_nosnw with
     * use_subgrid_topo, tpi_lim and test_int with use_subgrid_topo_V2.
     * test_int keeps its previous value (from -9999) on faces where the
     * normalisation integral is not evaluated. */
    double* frac_contrib;
    double* frac_contrib_nosnw;
    double* hold_topo;
    double* tpi_lim;
    double* test_int;
    int32_t on_device;
} pbsm3d_outputs;

/* Step diagnostics.  Times are CUDA-event milliseconds on the context's stream. */
typedef struct pbsm3d_stats {
    int32_t suspension_present;  /* ||b_susp||_inf > 1e-12 (PBSM3D.cpp:1424-1427) */
    int32_t deposition_present;  /* suspension_present && ||b_dep||_inf > 1e-12 */
    int32_t susp_iters;          /* BiCGStab iterations; one that stops at its half step counts as one */
    int32_t susp_matvecs;        /* operator applications, all precisions (every iteration counted whole) */
    int32_t susp_refinements;    /* MIXED: FP64 refinement sweeps */
    int32_t dep_iters;
    double susp_rel_residual;    /* final ||b-Ax||/||b|| in FP64 */
    double dep_rel_residual;
    double susp_rhs_max;
    double dep_rhs_max;
    double ms_coefficients;      /* saltation + layer coefficients + assembly + factorisation */
    double ms_susp_solve;
    double ms_post;              /* Qsusp/Qsubl column reduction */
    double ms_dep_assembly;
    double ms_dep_solve;
    double ms_update;
    double ms_total;             /* whole step on the device, incl. copies when on_device=0 */
    /* Mass ledger of the deposition update, kg, summed in FP64 over faces. */
    double ledger_divergence;    /* dt * sum_i b_dep[i]  (net drift flux into the faces) */
    double ledger_deposited;     /* dt * sum_i area[i] * q[i]  (solution) */
    double ledger_clipped;       /* sum_i area[i] * (drift_mass[i] - q[i]*dt)  (caps, no-erosion rule) */
    double ledger_snow_mass;     /* sum_i area[i] * swe[i] before the step */
    double ledger_residual;      /* dt * sum_i (b - A q)[i] */
    int64_t bytes_moved;         /* algorithmic HBM bytes of the step (model of the kernels) */
    int32_t gpu_launches;        /* kernels launched by the step */
    int32_t profiled;            /* 1 when the kern_* fields below were measured */
    /* Per kernel class (enum pbsm3d_kernel): CUDA-event time of the launches
     * that did work, their count and their algorithmic HBM bytes.  Filled only
     * when profiling is on (pbsm3d_set_profiling). */
    double kern_ms[16];
    int64_t kern_bytes[16];
    int32_t kern_launches[16];
    int32_t dep_refinements;     /* MIXED: FP64 refinement sweeps of the deposition solve (1 otherwise) */
    int32_t n_slow_faces;        /* faces with a saltation layer (per-row particle terms) */
} pbsm3d_stats;

/* Kernel classes reported in pbsm3d_stats.kern_*. */
enum pbsm3d_kernel {
    PBSM3D_K_ASSEMBLE = 0,   /* saltation + layer coefficients + ELL rows + column factors */
    PBSM3D_K_BICG_P = 1,     /* p update fused with the column (Thomas) preconditioner */
    PBSM3D_K_BICG_V = 2,     /* v = p + N B^-1 p (lateral gather) + dot */
    PBSM3D_K_BICG_S = 3,     /* s update fused with the column preconditioner */
    PBSM3D_K_BICG_T = 4,     /* t = s + N B^-1 s + two dots */
    PBSM3D_K_BICG_X = 5,     /* x, r update + two dots */
    PBSM3D_K_RESIDUAL = 6,   /* FP64 true residual b - A x */
    PBSM3D_K_POST = 7,       /* Qsusp / Qsubl column reduction */
    PBSM3D_K_DEP_ASSEMBLE = 8,
    PBSM3D_K_CG = 9,         /* deposition CG iterations (both kernels) */
    PBSM3D_K_UPDATE = 10,    /* erosion/deposition update + mass ledger */
    PBSM3D_K_OTHER = 11,
    PBSM3D_K_MLP = 12,       /* learned warm start: features + fused 3-layer tensor-core MLP */
    PBSM3D_K_NEUMANN = 13,   /* polynomial preconditioner steps: lateral gather + column solve */
    PBSM3D_K_COUNT = 14
};

typedef struct pbsm3d_ctx pbsm3d_ctx;

/* Parameters of one ensemble member (the perturbed constants of config 4). */
typedef struct pbsm3d_member {
    double ustar_th_scale;  /* multiplies the threshold friction velocity */
    double z0_snow;         /* aerodynamic roughness of snow (m) */
    double settling_scale;  /* multiplies the settling velocity */
} pbsm3d_member;

/* Fill *cfg with the reference defaults. */
void pbsm3d_config_defaults(pbsm3d_config* cfg);

/* Validate the config (the checks of PBSM3D.cpp:132-135, 237-240), pack the
 * mesh into device SoA, build the sliced-ELL pattern of both systems.
 * Replaces PBSM3D::PBSM3D + PBSM3D::init + the two NearestNeighborProblem ctors. */
int pbsm3d_create(const pbsm3d_mesh_desc* mesh, const pbsm3d_config* cfg, pbsm3d_ctx** out);

/* A batched ensemble: n_members independent meshes of any sizes, each with
 * its own parameters, in one context.  Every step advances all members with
 * the same kernels: one joint system over the disjoint union of the meshes,
 * each member with the reference's own "suspension/deposition present"
 * tests and its own relative tolerance.  Forcing and output arrays of
 * pbsm3d_step are the members' arrays concatenated in member order
 * (pbsm3d_member_offsets gives the face ranges).  cfg.ustar_th_scale,
 * z0_snow and settling_scale are ignored (members[] replaces them).
 * No counterpart in the reference. */
int pbsm3d_ensemble_create(int32_t n_members, const pbsm3d_mesh_desc* meshes, const pbsm3d_member* members,
                           const pbsm3d_config* cfg, pbsm3d_ctx** out);
/* offsets[0..n_members] face ranges of the members; returns n_members. */
int pbsm3d_member_offsets(const pbsm3d_ctx* ctx, int64_t* offsets);

/* One timestep of dt seconds (global_param->dt(), integer seconds in CHM).
 * Replaces PBSM3D::run.  stats may be NULL.  Host output buffers in
 * page-locked memory let the outputs that are final after the column post
 * (Qsalt, Qsusp, Qsubl, Qsubl_mass, sum_subl, blowingsnow_probability, c)
 * reach the host while the deposition solve runs; with pageable buffers
 * every output is copied after the step.  After an error return the output
 * buffers' contents are unspecified; a step that fails before the column
 * post (NaN input, suspension solve) leaves the module state unchanged. */
int pbsm3d_step(pbsm3d_ctx* ctx, const pbsm3d_forcing* forcing, double dt,
                const pbsm3d_outputs* out, pbsm3d_stats* stats);

/* Module state for checkpoint/restart (host arrays of n_faces doubles, NULL = skip).
 * The reference checkpoints sum_drift only ("PBSM3D:sum_drift", PBSM3D.cpp:1753-1773). */
int pbsm3d_get_state(pbsm3d_ctx* ctx, double* sum_drift, double* sum_subl,
                     double* drift_mass, double* pbsm_more_than_avail);
int pbsm3d_set_state(pbsm3d_ctx* ctx, const double* sum_drift, const double* sum_subl,
                     const double* drift_mass, const double* pbsm_more_than_avail);

/* Device-resident snow state: the drift consumer of CHM's snow models on the
 * GPU, so multi-step runs keep swe and snow depth in HBM.  After
 * pbsm3d_set_snow, a step whose forcing leaves swe and snowdepthavg NULL
 * reads them from the context, and every step ends by applying its
 * drift_mass to them as snobal does (snobal.cpp:363-387, _adj_snow):
 *   mass = drift_mass (0 when NaN or -9999);
 *   depth change = mass / rho, rho = the snowpack's bulk density swe/depth
 *   for erosion (mass < 0), drift_density for deposition;
 *   swe += mass, depth += depth change; the pack is removed (both 0) when
 *   either reaches 0.
 * swe (kg m^-2) and depth (m) are n_faces doubles (device pointers when
 * on_device); drift_density > 0 (CHM default 300 kg m^-3).
 * pbsm3d_get_snow copies the current state out.  No counterpart in the
 * reference module itself: this is the caller side of its drift_mass output. */
int pbsm3d_set_snow(pbsm3d_ctx* ctx, const double* swe, const double* depth, double drift_density, int on_device);
int pbsm3d_get_snow(pbsm3d_ctx* ctx, double* swe, double* depth, int on_device);

/*
 * The modules that produce PBSM3D's wind inputs, on the context's mesh (all
 * members of an ensemble), with the settings in its config:
 *   pbsm3d_scale_wind_vert <- scale_wind_vert::run(mesh&)   scale_wind_vert.cpp:53-227
 *     U_2m_above_srf from U_R through the canopy/snow log-exp profile
 *     (Atmosphere.cpp:32-46), then the thin plate spline of the three
 *     neighbours' values at the face centre (TPSpline.cpp:55-157), >= 0.1.
 *     snowdepthavg may be NULL (the reference's optional variable; 0).
 *   pbsm3d_fetchr          <- fetchr::run                    fetchr.cpp:55-117
 *     fetch (m) from vw_dir: the upwind search in fetch_steps steps of
 *     fetch_max_distance/fetch_steps, each taking the face whose centre is
 *     nearest the search point (a kd-tree query in the reference,
 *     triangulation.cpp:170-178; a uniform grid per member here, lowest index
 *     on a tie), nearest within the face's own member mesh.
 * on_device as for the forcing.  With derive_wind / derive_fetch the step
 * runs them itself, before the assembly.
 */
int pbsm3d_scale_wind_vert(pbsm3d_ctx* ctx, const double* U_R, const double* snowdepthavg, double* U_2m_above_srf,
                           int on_device);
int pbsm3d_fetchr(pbsm3d_ctx* ctx, const double* vw_dir, double* fetch, int on_device);

/*
 * Met stations and the station-driven wind provider uniform_wind
 * (interp_met/uniform_wind.cpp:28-127).  pbsm3d_set_stations takes the
 * stations' x, y (host arrays, the mesh's projection) and builds each face's
 * station list as CHM's core does (core.cpp:168-205, metdata.cpp:591-622):
 * the n_nearest nearest (station_N_nearest; nearest first, the lower index on
 * a tie) or, with n_nearest = 0 and radius > 0, every station within radius
 * (station_search_radius; ascending index).  n_nearest = 0 and radius = 0 take
 * the core's defaults: 1 for NEAREST, 5 otherwise.  SPLINE and IDW need at
 * least 2 stations per list, NEAREST exactly 1 (the reference throws
 * otherwise); at most 16 per face.  pbsm3d_uniform_wind interpolates one
 * time step of the stations' U_R and vw_dir (n_stations each; a station with
 * -9999/NaN in either is skipped) to every face: U_R (>= 0.1 m/s) and vw_dir
 * (degrees).  PBSM3D_ERR_NAN_INPUT when a face is left without a station.
 */
enum pbsm3d_interp { PBSM3D_INTERP_SPLINE = 0, PBSM3D_INTERP_IDW = 1, PBSM3D_INTERP_NEAREST = 2 };
int pbsm3d_set_stations(pbsm3d_ctx* ctx, int64_t n_stations, const double* x, const double* y, int32_t n_nearest,
                        double radius, int32_t interp);
int pbsm3d_uniform_wind(pbsm3d_ctx* ctx, const double* station_U_R, const double* station_vw_dir, double* U_R,
                        double* vw_dir, int on_device);

/*
 * CHM's JSON mesh files (triangulation.cpp:206-356): a .mesh file
 * {"mesh": {"vertex", "elem", "neigh", "nvertex", "nelem", "is_geographic", ...}}
 * and an optional .param file of per-face parameters.  The geometry is
 * computed as CHM's face class does; the neighbour lists are taken as given.
 * Parameters read: area, TPI_mean, TPI_std, TPI_neg_frac, TPI_neg_mean,
 * TPI_neg_std, CanopyHeight, LAI (the last two stand in for CHM's landcover
 * table).  Geographic meshes return PBSM3D_ERR_UNSUPPORTED; malformed files
 * PBSM3D_ERR_BAD_MESH with the reason in pbsm3d_mesh_last_error().
 * pbsm3d_mesh_describe fills a description whose arrays point into the mesh
 * (valid until pbsm3d_mesh_free).  CHM's HDF5 mesh and parameter files
 * (triangulation.cpp:724-1035, 1237-1383: /mesh/vertex, /mesh/elem,
 * /mesh/neighbor, root attributes "/mesh/...", /parameters/<name>) are read
 * too, either path of the pair, chosen by the file's signature, with no HDF5
 * library (the subset of the format those files use).  One file of a
 * multi-process partition (is_partition, or cell_global_id out of file
 * order) is refused: the step runs on the whole mesh.
 */
/*
 * Diagnostics of the last step by the names debug_output gives them in the
 * reference (PBSM3D.cpp:141-186): per face "hs", "ustar", "u*_th", "csalt",
 * "z0", "is_drifting"; per layer z (0-based) "c<z>", "csubl<z>", "u_z<z>",
 * "cz<z>".  n_faces doubles.  Unknown names: PBSM3D_ERR_INVALID_ARG.  The
 * reference's other debug variables (K, rm, mm, dm/dt, uvw, ...) are not kept.
 */
int pbsm3d_get_debug(pbsm3d_ctx* ctx, const char* name, double* out, int on_device);

typedef struct pbsm3d_mesh pbsm3d_mesh;
int pbsm3d_mesh_read(const char* mesh_path, const char* param_path, pbsm3d_mesh** out);
int pbsm3d_mesh_describe(const pbsm3d_mesh* mesh, pbsm3d_mesh_desc* desc);
int pbsm3d_mesh_arrays(const pbsm3d_mesh* mesh, int64_t* n_vertices, const double** vertex, const int32_t** elem);
void pbsm3d_mesh_free(pbsm3d_mesh* mesh);
const char* pbsm3d_mesh_last_error(void);

/* Sliced-ELL export of the last assembled systems in the reference row order
 * (row = z*n_faces + face) and the reference graph's slot order: self, lateral
 * neighbours in face order 0..2 (present ones only), below, above
 * (LinearAlgebra.cpp:67-116).  cols/vals are [rows*6], unused slots col=-1.
 * rhs and x (solution) are [rows].  Any pointer may be NULL. */
int pbsm3d_export_suspension(pbsm3d_ctx* ctx, int32_t* cols, double* vals, double* rhs, double* x);
int pbsm3d_export_deposition(pbsm3d_ctx* ctx, int32_t* cols, double* vals, double* rhs, double* x);

/*
 * Learned warm start (x0 of the suspension solve when cfg.warm_start ==
 * PBSM3D_X0_LEARNED): a per-row MLP 14 -> 128 -> 128 -> 128 -> 1 (ReLU),
 * BF16 weights and activations, FP32 accumulation on the tensor cores.
 * Parameters are one packed FP32 vector of pbsm3d_mlp_num_params() values:
 *   W0[128][14] b0[128] W1[128][128] b1[128] W2[128][128] b2[128] w3[128] b3
 * (W row-major [out][in]).  feat_mean/feat_scale standardise the 14 inputs:
 * x = (f - mean) * scale.  No counterpart in the reference.
 */
int pbsm3d_mlp_num_params(void);
int pbsm3d_set_mlp(pbsm3d_ctx* ctx, const float* params, const float* feat_mean, const float* feat_scale);

/* Training data of the last step: the 14 raw features of every row
 * (reference row order, [nLayer*n_faces][14]) computed from the step's
 * system and the previous step's solution c_prev, and the target
 * 100*(c - c_prev), the change of the step's solution.  Host arrays, or device arrays when on_device != 0;
 * either may be NULL. */
int pbsm3d_mlp_features(pbsm3d_ctx* ctx, float* features, float* targets, int32_t on_device);
/* The loaded MLP's prediction of the last step's concentrations,
 * c_prev + network/100 (before the block-Jacobi sweep the warm start applies),
 * [nLayer*n_faces] host doubles, reference order. */
int pbsm3d_mlp_predict(pbsm3d_ctx* ctx, double* c_out);

/* GPU trainer of the MLP (Adam, loss 0.5 mean((y - t)^2)); batch rows a
 * multiple of 128 (and of 1024 above 1024). */
typedef struct pbsm3d_mlp_trainer pbsm3d_mlp_trainer;
int pbsm3d_mlp_trainer_create(int32_t batch, const float* params, const float* feat_mean, const float* feat_scale,
                              pbsm3d_mlp_trainer** out);
/* `steps` minibatches drawn (seeded) from device arrays features [rows][14], targets [rows]. */
int pbsm3d_mlp_train(pbsm3d_mlp_trainer* tr, const float* features, const float* targets, int64_t rows,
                     int32_t steps, float lr, uint64_t seed, float* loss_per_step);
/* One forward/backward over exactly `batch` host rows: gradients (packed), loss, outputs. */
int pbsm3d_mlp_grad(pbsm3d_mlp_trainer* tr, const float* features, const float* targets, float* grads, float* loss,
                    float* outputs);
int pbsm3d_mlp_get_params(pbsm3d_mlp_trainer* tr, float* params);
void pbsm3d_mlp_trainer_destroy(pbsm3d_mlp_trainer* tr);
/* The tensor-core GEMM the MLP is built from: C[M][N] (FP32) = A[M][K] B[N][K]^T,
 * A and B BF16 (raw 16-bit patterns), host arrays; M a multiple of 128,
 * N in {16, 128}, K = 16 or a multiple of 64. */
int pbsm3d_mlp_gemm_bf16(const uint16_t* A, const uint16_t* B, float* C, int32_t M, int32_t N, int32_t K);

/* Per-launch CUDA-event timing of every kernel (off by default).  When on,
 * the step records an event pair around each launch on the context's stream
 * and fills pbsm3d_stats.kern_*. */
int pbsm3d_set_profiling(pbsm3d_ctx* ctx, int32_t on);

/*
 * Launch geometry of the suspension solve's column kernels.  No counterpart
 * in the reference (its Krylov solve is Belos/Tpetra's, LinearAlgebra.cpp:
 * 228-252).  set: fix the geometry (width 256, 128 or 64 faces a block;
 * lanes 1, 2 or 4 threads a face column), which also ends autotuning; the
 * results do not depend on it, bit for bit.  get: the geometry in force and
 * whether it is final (tuned = 1) or still being tuned.
 */
int pbsm3d_set_column_geometry(pbsm3d_ctx* ctx, int32_t width, int32_t lanes);
int pbsm3d_get_column_geometry(const pbsm3d_ctx* ctx, int32_t* width, int32_t* lanes, int32_t* tuned);

/*
 * Test of the device-side wait limits.  No counterpart in the reference,
 * whose failure path is a solver exception (PBSM3D.cpp:1690-1705).  Every
 * wait of the persistent deposition CG (one cooperative launch whose blocks
 * synchronise through flags in global memory) is bounded; this arms, for the
 * next such launch of this context only, a block (withhold_block, clamped to
 * the grid) that publishes none of its flags, and a wait limit of limit_ms
 * (at most 2000; the default limit is 2 s).  The other blocks' waits run
 * out, every block leaves, and that step returns PBSM3D_ERR_CUDA ("grid
 * all-reduce timed out") with the context usable for the next step.
 * Single-mesh, host-driven contexts only (PBSM3D_ERR_INVALID_ARG otherwise;
 * a graph-mode context's wait limit is fixed when its graph is captured).
 */
int pbsm3d_arm_wait_timeout_test(pbsm3d_ctx* ctx, int32_t withhold_block, double limit_ms);

/* Device-side timing of a region on the context's stream (measurement
 * plumbing): pbsm3d_timer_mark records CUDA event `slot` (0..15) on the
 * stream; pbsm3d_timer_elapsed waits for both and returns the milliseconds
 * between them. */
int pbsm3d_timer_mark(pbsm3d_ctx* ctx, int32_t slot);
int pbsm3d_timer_elapsed(pbsm3d_ctx* ctx, int32_t a, int32_t b, double* ms);

/*
 * Deposition solve without device allocation.  No counterpart in the
 * reference: it exists for hosts that own all device memory and do not let
 * a library call cudaMalloc (a model that reserves the GPU at start-up and
 * forbids allocation inside its time loop, or a framework whose memory pool
 * is the only allocator on the device).  Solves the SPD deposition system
 *   diag[i] x[i] + sum_j off[j*n+i] x[neighbor[j*n+i]] = rhs[i]
 * (the layout pbsm3d_step assembles: SoA, j = 0..2, neighbour -1 = none) by
 * Jacobi-preconditioned CG to ||rhs - A x|| <= tol ||rhs||, x0 = 0.  All
 * arrays are device pointers of the current device, owned by the caller.
 * Work space is a fixed static device array sized for at most 1,048,576
 * faces (32 MiB, held by every device that loads the library until exit);
 * larger n_faces returns PBSM3D_ERR_INVALID_ARG.  The first call on a device
 * looks up that array's address (make it before any stream capture), and
 * the first call after a cudaDeviceReset looks it up again where the driver
 * reports context ids (CUDA 12+ drivers); with an older driver, do not reset
 * the device after the first call.  Calls that overlap on one device race on
 * the shared array.  Runs on the legacy default stream and returns when done,
 * after at most maxit iterations: a launch failure returns PBSM3D_ERR_CUDA,
 * a solve that reaches maxit above tol PBSM3D_ERR_NOT_CONVERGED (with *iters
 * and *rel_residual set).  Messages: pbsm3d_last_error(NULL).
 */
int pbsm3d_deposition_solve_noalloc(int64_t n_faces, const int32_t* neighbor, const double* diag,
                                    const double* off, const double* rhs, double* x, double tol, int32_t maxit,
                                    int32_t* iters, double* rel_residual);

/*
 * Validation of the library's table-driven FP64 routines.  No counterpart in
 * the reference: the assembly evaluates exp, log, x^y, 1/x and a/b with its
 * own routines (Tang's table-driven exp and log, a Newton-Raphson-refined
 * reciprocal) and rounds FP64 to FP32 on the integer pipe; this evaluates
 * one of them, or the CUDA function it stands in for, elementwise over n
 * device values: out[i] = f(a[i]) or f(a[i], b[i]) (b only for DIV and POW).
 * Synchronous, on the legacy default stream.
 */
enum {
    PBSM3D_MATH_EXP = 0,
    PBSM3D_MATH_LOG = 1,
    PBSM3D_MATH_RCP = 2,
    PBSM3D_MATH_DIV = 3,
    PBSM3D_MATH_POW = 4,
    PBSM3D_MATH_F32 = 5,       /* (double)(float) rounding on the integer pipe */
    PBSM3D_MATH_CUDA_EXP = 6,  /* CUDA's exp, log, 1.0/x, a/b, pow, (float) */
    PBSM3D_MATH_CUDA_LOG = 7,
    PBSM3D_MATH_CUDA_RCP = 8,
    PBSM3D_MATH_CUDA_DIV = 9,
    PBSM3D_MATH_CUDA_POW = 10,
    PBSM3D_MATH_CUDA_F32 = 11
};
int pbsm3d_math_eval(int32_t fn, int64_t n, const double* a, const double* b, double* out);

/* The GPU's FP64 fused multiply-add rate (thread operations a second),
 * measured on the current device by a kernel of independent FMA chains that
 * touches no memory (about 10 ms).  Measurement plumbing for the FP64
 * roofline of the FP64 kernels, whose bound on this GPU is the FP64 pipe; no
 * reference counterpart. */
int pbsm3d_fp64_rate(double* fma_per_s);

/* Message of the last failure on this context (or of the last failed create
 * when ctx is NULL). */
const char* pbsm3d_last_error(const pbsm3d_ctx* ctx);

void pbsm3d_destroy(pbsm3d_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* PBSM3D_H */
