// pbsm3d_internal.cuh -- device data layout and kernel entry points of
// libpbsm3d_cuda (sm_103a).
//
// HBM layout (all SoA, 256-byte aligned allocations):
//   faces      i in [0, Tp), Tp = n_faces rounded up to a multiple of 256;
//              faces >= n_faces are padding with identity rows.
//   rows       r = z*Tp + i (layer-major, the reference's extruded ordering
//              row = z*n_global + gid, LinearAlgebra.cpp:46-55, with a
//              padded stride).  R = nLayer*Tp.
//   suspension matrix: sliced ELL, one slice per layer, 6 slots per row
//              stored slot-major: band[k*R + r], k = 0 diag, 1..3 lateral
//              face 0..2, 4 below (z-1), 5 above (z+1).  Column indices are
//              implicit: lateral = z*Tp + nbr[j*Tp + i], vertical = r -/+ Tp.
//   column preconditioner: Thomas factors of each face's tridiagonal column
//              fac_l[r] (forward multiplier), fac_ib[r] (1/pivot); the upper
//              band is band 5.
//   deposition matrix: dep_diag[Tp], dep_off[j*Tp + i] (j = 0..2).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <string>
#include <vector>

#include "../../include/pbsm3d.h"
#include "fp64_math.cuh"

namespace pbsm {

constexpr int kBlock = 256;
constexpr int kMaxLayers = 64;
constexpr int kMaxTerms = 4;
constexpr int kMaxMembers = 256;
constexpr int kMaxCgBlocks = 1024;  // blocks of a cooperative CG launch
// launch geometries of the column kernels: W faces a block, LC lanes a face column
struct ColGeom {
    int W, LC;
};
constexpr int kNumColGeoms = 9;
extern const ColGeom kColGeom[kNumColGeoms];

// Configuration scalars every kernel sees (passed by value).
struct Params {
    int64_t T, Tp, R;
    int L;
    double dz, inv_dz, dt;
    int use_exp_fetch, use_tanh_fetch, use_PomLi, use_R94_lambda, enable_veg;
    int do_fixed_settling, do_sublimation, do_lateral_diff, rouault;
    double settling_velocity, eps, min_sd_trans, cutoff, snow_diffusion_const;
    // constants computed once on the host with the C library, the way the
    // reference computes them (compile-time or libm): cos(pi/4), the tanh
    // fetch factor, log(2/0.0002).  The per-member constants (threshold
    // scale, z0, settling scale, log(50/z0)) are in Member.
    double cos_pi_4, Lc_tanh, log_2_0002;
    int mixed;
    int fac64;  // FP64 Thomas factors needed (FP64 solves, or the learned start's sweep)
    int z0_ustar_coupling, iterative_subl;  // the reference's non-default branches
    int subgrid;  // bit 0: use_subgrid_topo, bit 1: use_subgrid_topo_V2
    const MathTables* mt;  // exp/log tables (device)
};

// Per-face static geometry (device pointers).
struct Faces {
    int32_t* nbr;     // [3][Tp]
    double* E;        // [3][Tp]
    double* mx;       // [3][Tp]
    double* my;       // [3][Tp]
    double* area;     // [Tp]
    double* zc;       // [Tp] centroid elevation
    double* depw;     // [3][Tp] deposition coupling eps E_j / |c_i - c_nb| across edge j (0 without a neighbour)
    double* canopy;   // [Tp]
    double* lai;
    double* stalkN;
    double* stalkD;
    uint8_t* water;   // [Tp]
};

// Per-step forcing resident in HBM.
struct Forcing {
    double *UR, *U2, *dir, *swe, *t, *rh, *sd, *fetch, *psh;
};

// Per-face work/state.
struct FaceState {
    uint8_t* saltation;
    double *Qsalt, *Qsusp, *Qsubl, *Qsubl_mass, *sum_subl, *drift_mass, *sum_drift, *more, *bsp;
    double* sub;  // [SG_COUNT][Tp] subgrid results, NULL unless a subgrid branch is on
};

// Subgrid topography results per face, rows of FaceState::sub: the holding
// capacity that gates saltation (min_sd_trans_avg, output "hold_topo"), the
// contributing fraction that scales c_salt, and the other outputs.
enum SubgridValue { SG_HOLD, SG_FRAC, SG_NOSNW, SG_TPILIM, SG_TESTINT, SG_COUNT };

// Per-member uniform grid of face centres for the nearest-face queries of fetchr.
struct GridM {
    double x0, y0, h;
    int nx, ny, cell0;  // this member's cells are [cell0, cell0 + nx * ny) of the concatenated list
    int pad;
};

// The wind-input modules (scale_wind_vert, fetchr) on the device.
struct Wind {
    double *cx = nullptr, *cy = nullptr, *cz = nullptr;  // [Tp] face centres
    double* canopy = nullptr;  // [Tp] canopy height, 0 on faces without vegetation
    double* lai = nullptr;     // [Tp]
    GridM* grid = nullptr;     // [n_members]
    int32_t* cell_start = nullptr;  // [ncells + 1]
    int32_t* cell_face = nullptr;   // [T] faces by cell
    double* tmp = nullptr;     // [Tp] scale_wind_vert's per-face pass
    double *in0 = nullptr, *in1 = nullptr, *out = nullptr;  // [Tp] staging of the stand-alone calls
};

// Met stations of the station-driven modules (uniform_wind) and each face's
// station list, [start[i], start[i+1]) of idx.
struct Stations {
    int64_t n = 0;
    int interp = 0;                 // PBSM3D_INTERP_*
    double *x = nullptr, *y = nullptr;
    int32_t *start = nullptr, *idx = nullptr;
    double *u = nullptr, *dir = nullptr;  // [n] this call's station values
    double *out_u = nullptr, *out_dir = nullptr;  // [Tp] staging
    int* bad = nullptr;             // set when a face has no valid station
};

// Static inputs of the subgrid branches (device).
struct Subgrid {
    double* tpi;        // [5][Tp] TPI_mean, TPI_std, TPI_neg_frac, TPI_neg_mean, TPI_neg_std (NaN = undefined)
    double* I0;         // [Tp] normalisation integral of the filling function (use_subgrid_topo_V2)
};

// Height-dependent coefficients of one layer (see cz_coeffs in physics.cu).
// The first kRowTerms fields are also the per-row layout of Susp::slow_rows.
// The particle mass mm divides the sublimation rate, so it is folded into the
// two terms the rate combines (one multiply a row fewer).
struct CzCoef {
    double omega;   // settling velocity
    double qr_m;    // Qr / mm: the radiation term (iterative_subl: the mean radius) over the mass
    double l;       // mixing length
    double rz2nu;   // 2 r_z / nu: Re = rz2nu * Vr
    double rsig_m;  // r_z sigfac / mm
    double lwarg;   // log((cz - z0) / z0), the wind-profile numerator
    double ew;      // lwarg^1.36: the layer's factor of u_z^1.36
    double cz;      // layer centre height above the snow surface
};
constexpr int kRowTerms = 7;  // doubles per row of Susp::slow_rows

// Per-face values the saltation pass hands to the row assembly, [FV_COUNT][Tp].
enum FaceValue {
    // FV_QC, FV_QL: the face's factors of the two sublimation terms; FV_EF:
    // its factor of the particle-velocity term 3 cos(pi/4) 0.005 u_z^1.36
    // FV_LAMBDA: the roughness element density of a saltating face (pass 1
    // to its saltation terms, pass 1b)
    // FV_UX, FV_UY: the unit wind vector -bearing_to_cartesian(dir) (pass 1
    // to pass 1b and the deposition rows)
    FV_HS, FV_USTAR, FV_UTH, FV_CSALT, FV_QC, FV_QL, FV_EF, FV_INVLOGDEN, FV_K0, FV_K1, FV_K2, FV_Z0, FV_LAMBDA,
    FV_UX, FV_UY,
    FV_COUNT
};

// Parameters of one ensemble member (a plain context is one member).
struct Member {
    double uth_scale, z0, settling_scale, log_zur_z0;
};

// Per-member bookkeeping on the device.
struct Members {
    int n;
    const int32_t* face_member;     // [Tp] member of each face (padding: 0)
    const Member* prm;              // [n]
    unsigned long long* rhs_max;    // [n] bit patterns of max |rhs| (suspension)
    unsigned long long* dep_max;    // [n] bit patterns of max |rhs| (deposition)
    double* bb;                     // [n] ||rhs_m||^2 (suspension), then deposition
    int* susp_present;              // [n]
    int* dep_present;               // [n]
};

// Suspension system.
struct Susp {
    CzCoef* cztab;    // [n_members][L] for faces with hs == 0
    double* face_v;   // [FV_COUNT][Tp] saltation pass results
    int32_t* slow_list;  // [Tp] faces with a saltation layer (hs > 0)
    int* n_slow;      // device count of slow_list
    double* slow_rows;   // [kRowTerms][R] layer terms of those faces' rows
    double* band;     // [6][R]
    double* rhs;      // [R]
    double* x;        // [R]
    double* u_z;      // [R]
    double* csubl;    // [R]
    // FP64 Thomas factors of the column tridiagonals: the inverse pivots ib,
    // and the off-diagonals scaled by them (ib_z lo_z, ib_z up_z)
    double* fac_l;    // [R]
    double* fac_ib;   // [R]
    double* fac_u;    // [R]
    // FP64 with the polynomial preconditioner: the pivots and the lateral
    // bands scaled by ib (null otherwise)
    double* fac_piv = nullptr;  // [R]
    double* latp = nullptr;     // [3][R]
    // MIXED: the FP32 operator.  Its lateral bands are not stored: a row's
    // lat_f = u_z L1_f + L0_f comes from its u_z and its face's constants
    float* uz32;      // [R] u_z
    float* l01;       // [6][Tp] L0_0..2, L1_0..2 of each face
    float* l32;       // [R]
    float* ib32;      // [R]
    float* up32;      // [R]
};

// Deposition system.
struct Dep {
    double* diag;     // [Tp]
    double* off;      // [3][Tp]
    double* dinv;     // [Tp]
    double* rhs;      // [Tp]
    double* x;        // [Tp]
};

// Device scalars of one Krylov solve (one cache line each group).
struct Scalars {
    double rho, alpha, omega, beta;
    double bnorm2, rnorm2, target2, tmp;
    double rv, ts, tt, pq;
    double rhs_max, nan_flag, red0, red1;
    int iter, done, maxit, status;
    unsigned counter[8];
};

// Krylov state of one ensemble member in a batched solve: each member runs
// its own BiCGStab recurrences (its own alpha, omega, beta, rho) inside the
// shared kernels, and stops on its own residual.  One 128-byte line each.
struct MScal {
    double rho, alpha, omega, beta;
    double rnorm2, bnorm2, target2, red0;  // red0 = (b, r) of the residual pass
    double gamma, pad0;                    // warm-start scale (set by the host)
    int iter, done, maxit;
    unsigned counter;                      // tiles reported to the current reduction
    int half;                              // FP64: the next iteration tests its half step
    int pad1[3];
};

// Work tiles of the batched Krylov kernels: runs of at most kBlock faces
// that never span two members, so a tile's block sum belongs to one member.
struct Tiles {
    const int32_t* start;   // [ntiles + 1] first face of each tile
    const int32_t* member;  // [ntiles]
    const int32_t* mtile;   // [n + 1] first tile of each member
    const int32_t* act;     // [nact] tiles of the members still iterating, ascending
    int ntiles, n, nact;
    const int* nact_dev;    // graph mode: nact lives in device memory (set by the controllers)
};

// Grid-wide barrier state of a persistent (cooperative) kernel.
struct GridBar {
    unsigned count, gen;
    int err, pad;
};

// Reduction workspace: per-block partials.
struct ReduceWs {
    double* partials;  // [kMaxTerms][nblocks]
    int nblocks;
};

struct Ctx;

// physics.cu
void launch_assemble_suspension(Ctx& c, cudaStream_t s);
void launch_post_and_assemble_deposition(Ctx& c, cudaStream_t s);
void launch_update(Ctx& c, cudaStream_t s);
void launch_init_static(Ctx& c, cudaStream_t s);
void launch_member_mask_norm(Ctx& c, cudaStream_t s, int which);
void launch_member_zero(Ctx& c, cudaStream_t s, double* x);
void launch_consume_drift(Ctx& c, cudaStream_t s);

// subgrid.cu
void launch_subgrid(Ctx& c, cudaStream_t s);
int subgrid_init(Ctx& c, cudaStream_t s);

// wind.cu
void launch_scale_wind_vert(Ctx& c, cudaStream_t s, const double* U_R, const double* sd, double* u2m);
void launch_fetchr(Ctx& c, cudaStream_t s, const double* dir, double* fetch);
void launch_uniform_wind(Ctx& c, cudaStream_t s, double* U_R, double* vw_dir);

// solver.cu
int solve_suspension(Ctx& c, cudaStream_t s, pbsm3d_stats* st);
// graph mode: the device part of a step as one CUDA-graph launch (built on
// first use); fills the iteration/residual fields of c like the host path
// One step as the two launches of the step graph; `between` (may be empty)
// runs on the host after part 1 is queued and before part 2 is.  The step's
// control block comes back with the queued work: after the caller's
// synchronisation of s, graph_finish reads it (iterations, residuals, the
// step's error).
int graph_step(Ctx& c, cudaStream_t s, bool own_snow, const std::function<int()>& between);
int graph_finish(Ctx& c);
void graph_destroy(Ctx& c);
int solve_deposition(Ctx& c, cudaStream_t s, pbsm3d_stats* st);
int configure_solver_kernels(Ctx& c);
int tuned_geometry(Ctx& c);          // autotuner: the choice cached for this shape (-1 = none)
int configure_cg(Ctx& c);
int jacobi_sweep(Ctx& c, cudaStream_t s, const double* xi, double* xo);
// mlp.cu
int launch_mlp_infer(Ctx& c, cudaStream_t s, double* x0);
int mlp_features(Ctx& c, float* feat_dev, float* target_dev);
int mlp_load(Ctx& c, const float* params, const float* fmean, const float* fscale);
// capi.cu: the message pbsm3d_last_error(NULL) returns
void set_global_error(const std::string& msg);

struct Ctx {
    pbsm3d_config cfg;
    Params P;
    Faces F;
    Forcing Fo;
    FaceState S;
    Subgrid sg;
    Wind wnd;
    Stations st;
    int asm_kernels = 3;  // kernels of one suspension assembly (+1 subgrid, +2 derived wind, +1 derived fetch)
    Susp A;
    Dep D;
    Members Mb;
    std::vector<int64_t> member_offsets;  // host, [n+1] face ranges
    std::vector<double> member_z0;        // host, [n] snow roughness of each member
    double target_scale2 = 1.0;           // min_m ||b_m||^2 / ||b||^2 over present members
    double dep_target_scale2 = 1.0;
    // Krylov work vectors (FP64), [R] each
    double *r, *rh, *p, *v, *sv, *tv, *zp, *zs;
    // FP32 work vectors for MIXED, [R] each
    float *r32, *rh32, *p32, *v32, *s32, *t32, *zp32, *zs32, *x32;
    // polynomial preconditioner (neumann > 0): the last u - N z and the other z, [R] each
    double *nw = nullptr, *nz = nullptr;
    double* nu64 = nullptr;  // FP64 with neumann > 0: ib * u, read by the polynomial steps [R]
    float *nw32 = nullptr, *nz32 = nullptr;
    // deposition CG vectors [Tp]
    double *dr, *dz_, *dp, *dq;
    double* dr2 = nullptr;     // second residual buffer of the polynomial deposition tile CG (FP64)
    double* dscale = nullptr;  // [4][Tp] the persistent CG's d^-1/2 and scaled couplings (FP64)
    // reductions
    Scalars* sc;       // device
    Scalars* sc_host;  // pinned mirror
    int* n_slow_host = nullptr;  // pinned: faces with a saltation layer in the last assembly
    int n_slow = 0;
    // graph mode (cfg.graph): the step as one CUDA graph, see solver.cu
    const int* graph_dep_flag = nullptr;  // set only while the graph is captured
    struct StepGraph* graph = nullptr;
    double graph_rhs_max[2] = {0, 0};  // graph mode: ||rhs||_inf of the two systems
    // graph mode with profiling: the step's phase times from device stamps
    // (assembly, suspension solve, post + deposition assembly, deposition
    // solve, update)
    bool graph_phases = false;
    double graph_phase_ms[5] = {0, 0, 0, 0, 0};
    // device-resident snow state (pbsm3d_set_snow): swe and depth live in Fo.swe / Fo.sd
    bool snow_state = false;
    double drift_density = 300.0;
    ReduceWs red;
    int grid_rows, grid_faces;
    // batched Krylov: tiles, per-member states (residual sums, FP64 plain /
    // outer, FP32 inner), their pinned host mirror and the tile partials
    Tiles tiles;
    int32_t* act_buf = nullptr;      // device [ntiles]: the active-tile list
    std::vector<int32_t> act_host;
    MScal *msR = nullptr, *ms0 = nullptr, *ms1 = nullptr;
    MScal* ms_host = nullptr;
    double* tile_part = nullptr;  // [4][ntiles]
    std::vector<double> member_bb;  // ||b_m||^2 of the current suspension solve
    int grid_red[2] = {1, 1};  // BiCGStab gather + reduction kernels
    int grid_lat[2] = {1, 1};  // the lateral kernels (v, t), kLatLanes lanes a face
    int grid_res = 1;          // the FP64 residual kernel, kLatLanes lanes a face
    int grid_cg[2] = {1, 1};   // the tile CG's kernels (k_scg_x, k_scg_q): one wave
    // column kernels (p, s, polynomial step): one wave of blocks at each
    // geometry, [p/s or polynomial step][FP64, FP32][geometry]; the geometry
    // in force; the autotuner's state (cfg.autotune): next candidate, best
    // time per iteration and per face of each, tuned = a choice is in force
    int grid_geom[2][2][kNumColGeoms] = {};
    int geom = 0;
    int tune_cand = 0;
    int bicg_hint[2] = {4, 4};  // iterations of the last host-driven BiCGStab call (FP64, FP32): the first chunk
    float tune_ms[kNumColGeoms] = {};
    bool tuned = false;
    // ledger partial sums
    double* ledger;    // device [8]
    GridBar* gbar;     // device
    // previous step's solution (warm starts, training features) [R]
    double* x_prev;
    // learned warm start: BF16 weights (W0 padded to 16 inputs), FP32 rest
    void* mlp_w;       // bf16: W0[128*16] W1[128*128] W2[128*128]
    float* mlp_f;      // b0 b1 b2 w3 [4*128], b3, fmean[14], fscale[14]
    bool mlp_loaded = false;
    float mlp_b3 = 0.0f;
    int coop_blocks;   // co-resident blocks of the persistent CG kernel
    int coop_blocks32 = 0;  // ... of its FP32 instance (MIXED)
    unsigned* cg_flags;     // [kMaxCgBlocks][32] all-reduce flags of the persistent CG
    // the timeout test (pbsm3d_arm_wait_timeout_test): for the next
    // persistent CG launch only, a block that publishes no flag and the wait
    // limit in ns (0: none armed)
    int test_withhold = -1;
    unsigned long long test_limit_ns = 0;
    // MIXED deposition: FP32 matrix (diag, off[3], dinv), right-hand side and
    // the five CG vectors, [11][Tp]
    float* dep32 = nullptr;
    cudaStream_t stream;
    cudaStream_t copy_stream = nullptr;  // host copies of outputs final before the deposition solve
    cudaEvent_t copy_ev[2] = {nullptr, nullptr};
    cudaEvent_t ev[16];
    cudaEvent_t user_ev[16];
    std::vector<void*> allocations;
    std::string err;
    int launches;
    int64_t bytes;
    // per-launch profiling (pbsm3d_set_profiling)
    bool prof = false;
    std::vector<cudaEvent_t> pev;
    std::vector<int> pcat;
    std::vector<int64_t> pbytes;
    int pused = 0;
    double kern_ms[16];
    int64_t kern_bytes[16];
    int kern_launches[16];
    bool suspension_present, deposition_present;
    int susp_iters, susp_matvecs, susp_refinements, dep_iters, dep_refinements = 1;
    double susp_relres, dep_relres;
    double warm_gamma = 0.0;  // scale applied to the last warm start (0 = dropped)
};

// Device allocation owned by the context (freed with it); ok turns false on failure.
template <typename T>
T* dalloc(Ctx& c, size_t n, bool& ok) {
    void* p = nullptr;
    if (n == 0) n = 1;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
        ok = false;
        return nullptr;
    }
    c.allocations.push_back(p);
    return static_cast<T*>(p);
}

// Record the start of a kernel launch of class cat with the given algorithmic
// bytes (profiling only).  Every launch also adds its bytes to c.bytes.
void prof_begin(Ctx& c, cudaStream_t s);
void prof_end(Ctx& c, cudaStream_t s, int cat, int64_t bytes);
// Forget the last n recorded launches (no-op launches after convergence).
void prof_drop(Ctx& c, int n);

#define PBSM_CUDA_TRY(expr)                                                           \
    do {                                                                              \
        cudaError_t e_ = (expr);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            c.err = std::string(#expr) + ": " + cudaGetErrorString(e_);               \
            return PBSM3D_ERR_CUDA;                                                   \
        }                                                                             \
    } while (0)

// ---------------------------------------------------------------- device helpers
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// Warp sums of NT FP64 values, every lane ending with the totals (the same
// order in every call: deterministic).  The FP64 pipe of this GPU issues a
// small fraction of the FP32 rate, so the values share the first butterfly
// steps: with two, each half-warp adds one of them and the four remaining
// steps carry one value a lane (5 FP64 adds a lane instead of 10); with
// three, the quarter-warps take v0, v1, v2 and a zero after two shared steps
// (6 instead of 15).
__device__ __forceinline__ void warp_sums(double (&v)[1]) { v[0] = warp_sum(v[0]); }
__device__ __forceinline__ void warp_sums(double (&v)[2]) {
    const bool lo = (threadIdx.x & 31) < 16;
    double keep = lo ? v[0] : v[1];
    keep += __shfl_xor_sync(0xffffffffu, lo ? v[1] : v[0], 16);
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) keep += __shfl_xor_sync(0xffffffffu, keep, o);
    v[0] = __shfl_sync(0xffffffffu, keep, 0);
    v[1] = __shfl_sync(0xffffffffu, keep, 16);
}
__device__ __forceinline__ void warp_sums(double (&v)[3]) {
    const int lane = threadIdx.x & 31;
    const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0;
    // lanes < 16 carry (v0, v1), lanes >= 16 carry (v2, 0)
    double a = h16 ? v[2] : v[0], b = h16 ? 0.0 : v[1];
    a += __shfl_xor_sync(0xffffffffu, h16 ? v[0] : v[2], 16);
    b += __shfl_xor_sync(0xffffffffu, h16 ? v[1] : 0.0, 16);
    // lanes with bit 3 clear keep a, the others b
    double c = h8 ? b : a;
    c += __shfl_xor_sync(0xffffffffu, h8 ? a : b, 8);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    v[0] = __shfl_sync(0xffffffffu, c, 0);
    v[1] = __shfl_sync(0xffffffffu, c, 8);
    v[2] = __shfl_sync(0xffffffffu, c, 16);
}
template <int NT>
__device__ __forceinline__ void warp_sums(double (&v)[NT]) {
#pragma unroll
    for (int k = 0; k < NT; ++k) v[k] = warp_sum(v[k]);
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Deterministic block reduction of NT values (sum), result valid in thread 0.
template <int NT>
__device__ __forceinline__ void block_sum(double (&v)[NT]) {
    __shared__ double sh[NT][32];  // up to 1024 threads
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    {
        double w[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) w[k] = v[k];
        warp_sums(w);
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < NT; ++k) sh[k][wid] = w[k];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NT; ++k) v[k] = lane < (int)(blockDim.x >> 5) ? sh[k][lane] : 0.0;
        warp_sums(v);
    }
    __syncthreads();
}

// Write this block's NT partials; the last block to arrive sums all partials
// in a fixed order (deterministic) and returns true in every thread of that
// block with the totals in tot[] (valid in thread 0 only).
template <int NT>
__device__ __forceinline__ bool block_partials_last(double (&v)[NT], double* partials, unsigned* counter,
                                                    double (&tot)[NT]) {
    block_sum<NT>(v);
    __shared__ bool is_last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NT; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
        __threadfence();
        unsigned prev = atomicAdd(counter, 1u);
        is_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        double s = 0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += __ldcg(&partials[k * gridDim.x + b]);
        tot[k] = s;
    }
    block_sum<NT>(tot);
    if (threadIdx.x == 0) *counter = 0u;
    return true;
}

// Maxima of non-negative values (no order to fix): as block_partials_last,
// the last block reducing all partials with every thread.
template <int NT>
__device__ __forceinline__ bool block_partials_last_max(double (&v)[NT], double* partials, unsigned* counter,
                                                        double (&tot)[NT]) {
    __shared__ double shm[NT][32];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    auto block_max = [&](double (&x)[NT]) {
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            const double w = warp_max(x[k]);
            if (lane == 0) shm[k][wid] = w;
        }
        __syncthreads();
        if (wid == 0) {
#pragma unroll
            for (int k = 0; k < NT; ++k) x[k] = warp_max(lane < nw ? shm[k][lane] : 0.0);
        }
        __syncthreads();
    };
    block_max(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NT; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
        __threadfence();
        is_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        double m = 0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) m = fmax(m, __ldcg(&partials[k * gridDim.x + b]));
        tot[k] = m;
    }
    block_max(tot);
    if (threadIdx.x == 0) *counter = 0u;
    return true;
}

// Same for FP32 per-thread values: the warp-level sums stay in FP32 (off the
// FP64 pipe); each warp's sum is widened to FP64 for the block and grid sums.
__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <int NT>
__device__ __forceinline__ bool block_partials_last(float (&vf)[NT], double* partials, unsigned* counter,
                                                    double (&tot)[NT]) {
    __shared__ double shf[NT][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        const float w = warp_sum_f(vf[k]);
        if (lane == 0) shf[k][wid] = (double)w;
    }
    __syncthreads();
    __shared__ bool is_last;
    if (threadIdx.x == 0) {
        const int nw = (int)(blockDim.x >> 5);
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            double s = 0;
            for (int w = 0; w < nw; ++w) s += shf[k][w];
            partials[k * gridDim.x + blockIdx.x] = s;
        }
        __threadfence();
        const unsigned prev = atomicAdd(counter, 1u);
        is_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        double s = 0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += __ldcg(&partials[k * gridDim.x + b]);
        tot[k] = s;
    }
    block_sum<NT>(tot);
    if (threadIdx.x == 0) *counter = 0u;
    return true;
}

}  // namespace pbsm
