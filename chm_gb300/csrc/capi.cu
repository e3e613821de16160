// capi.cu -- the extern "C" boundary of libpbsm3d_cuda (declared in
// include/pbsm3d.h): context creation (PBSM3D::PBSM3D + init + the two
// NearestNeighborProblem constructors), the step (PBSM3D::run) and the
// checkpoint state; the ensemble constructor, the device snow state, the
// stand-alone wind modules and the diagnostics.  The step never falls back
// to the CPU: a missing or failing GPU is an error returned to the caller.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <new>
#include <string>
#include <vector>

#include "pbsm3d_internal.cuh"

using namespace pbsm;

struct pbsm3d_ctx {
    Ctx c;
};

static thread_local std::string g_create_error;

namespace pbsm {

void set_global_error(const std::string& msg) { g_create_error = msg; }

void prof_begin(Ctx& c, cudaStream_t s) {
    c.launches++;
    if (!c.prof) return;
    if ((size_t)(2 * c.pused + 2) > c.pev.size()) {
        size_t old = c.pev.size();
        c.pev.resize(std::max<size_t>(256, old * 2));
        for (size_t k = old; k < c.pev.size(); ++k) cudaEventCreate(&c.pev[k]);
    }
    cudaEventRecord(c.pev[2 * c.pused], s);
}

void prof_end(Ctx& c, cudaStream_t s, int cat, int64_t bytes) {
    c.bytes += bytes;
    if (c.prof) cudaEventRecord(c.pev[2 * c.pused + 1], s);
    if ((int)c.pcat.size() <= c.pused) {
        c.pcat.resize(c.pused + 64);
        c.pbytes.resize(c.pused + 64);
    }
    c.pcat[c.pused] = cat;
    c.pbytes[c.pused] = bytes;
    c.pused++;
}

// The last n launches returned at once (the solve had converged): their
// bytes and event records are removed.
void prof_drop(Ctx& c, int n) {
    for (int k = 0; k < n && c.pused > 0; ++k) {
        c.pused--;
        c.bytes -= c.pbytes[c.pused];
    }
}

}  // namespace pbsm

namespace {

void free_all(Ctx& c) {
    graph_destroy(c);
    for (void* p : c.allocations) cudaFree(p);
    c.allocations.clear();
    for (auto& e : c.pev) cudaEventDestroy(e);
    c.pev.clear();
    for (auto& e : c.ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : c.user_ev)
        if (e) cudaEventDestroy(e);
    if (c.sc_host) cudaFreeHost(c.sc_host);
    c.sc_host = nullptr;
    if (c.n_slow_host) cudaFreeHost(c.n_slow_host);
    c.n_slow_host = nullptr;
    if (c.ms_host) cudaFreeHost(c.ms_host);
    c.ms_host = nullptr;
    if (c.stream) cudaStreamDestroy(c.stream);
    c.stream = nullptr;
    if (c.copy_stream) cudaStreamDestroy(c.copy_stream);
    c.copy_stream = nullptr;
    for (auto& e : c.copy_ev)
        if (e) cudaEventDestroy(e);
}

// SoA [3][Tp] from row-major [n][3]
template <typename T>
void to_soa3(const T* src, int64_t n, int64_t Tp, std::vector<T>& dst, T pad) {
    dst.assign(3 * Tp, pad);
    for (int64_t i = 0; i < n; ++i)
        for (int j = 0; j < 3; ++j) dst[j * Tp + i] = src[3 * i + j];
}

int upload(Ctx& c, void* dst, const void* src, size_t bytes) {
    PBSM_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c.stream));
    return 0;
}

}  // namespace

extern "C" {

void pbsm3d_config_defaults(pbsm3d_config* cfg) {
    memset(cfg, 0, sizeof(*cfg));
    cfg->abi_version = PBSM3D_ABI_VERSION;
    cfg->nLayer = 10;
    cfg->do_fixed_settling = 0;
    cfg->do_sublimation = 1;
    cfg->do_lateral_diff = 1;
    cfg->rouault_diffusion_coef = 0;
    cfg->enable_veg = 1;
    cfg->iterative_subl = 0;
    cfg->use_exp_fetch = 0;
    cfg->use_tanh_fetch = 1;
    cfg->use_PomLi_probability = 0;
    cfg->z0_ustar_coupling = 0;
    cfg->use_subgrid_topo = 0;
    cfg->use_subgrid_topo_V2 = 0;
    cfg->use_R94_lambda = 1;
    cfg->debug_output = 0;
    cfg->settling_velocity = 0.5;
    cfg->smooth_coeff = 820;
    cfg->min_sd_trans = 0.1;
    cfg->cutoff = 0.3;
    cfg->snow_diffusion_const = 0.3;
    cfg->ustar_th_scale = 1.0;
    cfg->z0_snow = 0.01;
    cfg->settling_scale = 1.0;
    cfg->solver = PBSM3D_SOLVER_BICGSTAB;
    cfg->precision = PBSM3D_FP64;
    cfg->warm_start = PBSM3D_X0_ZERO;
    cfg->gmres_restart = 30;
    cfg->susp_maxit = 1000;
    cfg->dep_maxit = 1000;
    cfg->susp_tol = 1e-8;
    cfg->fetch_steps = 10;  // fetchr.cpp:34-45
    cfg->fetch_incl_veg = 1;
    cfg->fetch_max_distance = 1000.0;
    cfg->fetch_I = 0.06;
    cfg->dep_tol = 1e-10;
    cfg->inner_tol = 1e-4;
    cfg->autotune = 1;
}

const char* pbsm3d_last_error(const pbsm3d_ctx* ctx) {
    return ctx ? ctx->c.err.c_str() : g_create_error.c_str();
}

static int create_core(const pbsm3d_mesh_desc* mesh, const pbsm3d_config* cfg_in,
                       const std::vector<int64_t>& offsets, const std::vector<Member>& members, pbsm3d_ctx** out) {
    if (!out) return PBSM3D_ERR_INVALID_ARG;
    *out = nullptr;
    if (!mesh || !cfg_in) {
        g_create_error = "null mesh or config";
        return PBSM3D_ERR_INVALID_ARG;
    }
    const pbsm3d_config& cfg = *cfg_in;
    if (cfg.abi_version != PBSM3D_ABI_VERSION) {
        g_create_error = "config abi_version mismatch (use pbsm3d_config_defaults)";
        return PBSM3D_ERR_INVALID_ARG;
    }
    for (const Member& m : members)
        if (!(m.z0 > 0) || !std::isfinite(m.z0) || !(m.uth_scale > 0) || !std::isfinite(m.uth_scale) ||
            !(m.settling_scale >= 0) || !std::isfinite(m.settling_scale)) {
            g_create_error = "z0_snow and ustar_th_scale must be positive, settling_scale non-negative";
            return PBSM3D_ERR_INVALID_ARG;
        }
    if (mesh->n_faces <= 0 || mesh->n_faces > (int64_t)INT32_MAX / 2 || !mesh->neighbor || !mesh->edge_length ||
        !mesh->edge_normal || !mesh->area || !mesh->center) {
        g_create_error = "invalid mesh description";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (cfg.use_exp_fetch && cfg.use_tanh_fetch) {  // PBSM3D.cpp:132-135
        g_create_error = "PBSM3d: Cannot specify both exp_fetch and tanh_fetch";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (!(cfg.settling_velocity >= 0)) {  // PBSM3D.cpp:237-240
        g_create_error = "PBSM3D settling velocity must be positive";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (cfg.nLayer < 1 || cfg.nLayer > kMaxLayers) {
        g_create_error = "nLayer must be in [1, 64]";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (cfg.fetch_steps < 1 || cfg.fetch_steps > 100000 || !(cfg.fetch_max_distance > 0) ||
        !std::isfinite(cfg.fetch_max_distance) || !std::isfinite(cfg.fetch_I)) {
        g_create_error = "fetch_steps must be in [1, 100000], fetch_max_distance positive, fetch_I finite";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (cfg.neumann < 0 || cfg.neumann > 9) {
        g_create_error = "neumann must be in [0, 9]";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (cfg.dep_neumann != 0 && cfg.dep_neumann != 1) {
        g_create_error = "dep_neumann must be 0 or 1";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (cfg.solver != PBSM3D_SOLVER_BICGSTAB) {
        g_create_error = "only the BiCGStab suspension solver is implemented";
        return PBSM3D_ERR_UNSUPPORTED;
    }
    if (cfg.warm_start < PBSM3D_X0_ZERO || cfg.warm_start > PBSM3D_X0_LEARNED) {
        g_create_error = "unknown warm_start";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (!(cfg.susp_tol > 0) || !(cfg.dep_tol > 0) || cfg.susp_maxit < 1 || cfg.dep_maxit < 1 ||
        (cfg.precision == PBSM3D_MIXED && !(cfg.inner_tol > 0 && cfg.inner_tol < 1))) {
        g_create_error = "invalid solver tolerance or iteration limit";
        return PBSM3D_ERR_INVALID_ARG;
    }
    const int64_t T = mesh->n_faces;
    for (int64_t k = 0; k < 3 * T; ++k) {
        const int32_t nb = mesh->neighbor[k];
        if (nb < -1 || nb >= T || nb == k / 3) {
            g_create_error = "neighbour index out of range at face " + std::to_string(k / 3);
            return PBSM3D_ERR_BAD_MESH;
        }
    }
    for (int64_t i = 0; i < T; ++i)
        if (!(mesh->area[i] > 0) || !isfinite(mesh->area[i])) {
            g_create_error = "face " + std::to_string(i) + " has a non-positive or non-finite area";
            return PBSM3D_ERR_BAD_MESH;
        }
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
        g_create_error = "no CUDA device";
        return PBSM3D_ERR_CUDA;
    }

    auto* h = new (std::nothrow) pbsm3d_ctx();
    if (!h) return PBSM3D_ERR_OUT_OF_MEMORY;
    Ctx& c = h->c;
    c.cfg = cfg;
    const int L = cfg.nLayer;
    const int64_t Tp = (T + 255) / 256 * 256;
    const int64_t R = Tp * L;
    Params& P = c.P;
    P.T = T;
    P.Tp = Tp;
    P.R = R;
    P.L = L;
    P.dz = 5.0 / (double)L;  // susp_depth / nLayer, PBSM3D.cpp:225-226
    P.inv_dz = 1.0 / P.dz;
    P.dt = 0;
    P.use_exp_fetch = cfg.use_exp_fetch;
    P.use_tanh_fetch = cfg.use_tanh_fetch;
    P.use_PomLi = cfg.use_PomLi_probability;
    P.use_R94_lambda = cfg.use_R94_lambda;
    bool all_veg = mesh->canopy_height != nullptr;
    if (all_veg && mesh->has_vegetation)
        for (int64_t i = 0; i < T; ++i) all_veg = all_veg && mesh->has_vegetation[i];
    P.enable_veg = cfg.enable_veg && all_veg;  // PBSM3D.cpp:283-325
    P.do_fixed_settling = cfg.do_fixed_settling;
    P.do_sublimation = cfg.do_sublimation;
    P.do_lateral_diff = cfg.do_lateral_diff;
    P.rouault = cfg.rouault_diffusion_coef;
    P.settling_velocity = cfg.settling_velocity;
    P.eps = cfg.smooth_coeff;
    P.min_sd_trans = cfg.min_sd_trans;
    P.cutoff = cfg.cutoff;
    P.snow_diffusion_const = cfg.snow_diffusion_const;
    P.cos_pi_4 = cos(M_PI / 4.0);
    {
        const double fetch_ref = 300;
        P.Lc_tanh = 0.5 * tanh(0.1333333333e-1 * fetch_ref - 2.0) + 0.5;
    }
    P.log_2_0002 = log(2.0 / 0.0002);
    P.mixed = cfg.precision == PBSM3D_MIXED;
    P.fac64 = !P.mixed || cfg.warm_start == PBSM3D_X0_LEARNED;
    P.z0_ustar_coupling = cfg.z0_ustar_coupling != 0;
    P.iterative_subl = cfg.iterative_subl != 0;
    P.subgrid = (cfg.use_subgrid_topo ? 1 : 0) | (cfg.use_subgrid_topo_V2 ? 2 : 0);
    c.asm_kernels = 4 + (P.subgrid ? 1 : 0) + (cfg.derive_wind ? 2 : 0) + (cfg.derive_fetch ? 1 : 0);
    c.member_offsets = offsets;
    c.member_z0.resize(members.size());
    for (size_t m = 0; m < members.size(); ++m) c.member_z0[m] = members[m].z0;
    const int nm = (int)members.size();

    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
    c.grid_faces = (int)std::max<int64_t>(1, std::min<int64_t>((Tp + kBlock - 1) / kBlock, (int64_t)sms * 8));
    c.grid_rows = c.grid_faces;
    c.red.nblocks = c.grid_faces;

    if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) {
        g_create_error = "cudaStreamCreate failed";
        delete h;
        return PBSM3D_ERR_CUDA;
    }
    for (auto& e : c.ev) cudaEventCreate(&e);
    for (auto& e : c.user_ev) cudaEventCreate(&e);
    // outputs that are final before the deposition solve go to the host on a
    // second stream while the solve runs
    if (cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c.copy_ev[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c.copy_ev[1], cudaEventDisableTiming) != cudaSuccess) {
        g_create_error = "cudaStreamCreate failed";
        free_all(c);
        delete h;
        return PBSM3D_ERR_CUDA;
    }
    if (cudaMallocHost(&c.sc_host, sizeof(Scalars)) != cudaSuccess ||
        cudaMallocHost(&c.n_slow_host, sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&c.ms_host, sizeof(MScal) * members.size()) != cudaSuccess) {
        g_create_error = "cudaMallocHost failed";
        free_all(c);
        delete h;
        return PBSM3D_ERR_OUT_OF_MEMORY;
    }

    bool ok = true;
    Faces& F = c.F;
    F.nbr = dalloc<int32_t>(c, 3 * Tp, ok);
    F.E = dalloc<double>(c, 3 * Tp, ok);
    F.mx = dalloc<double>(c, 3 * Tp, ok);
    F.my = dalloc<double>(c, 3 * Tp, ok);
    F.area = dalloc<double>(c, Tp, ok);
    F.zc = dalloc<double>(c, Tp, ok);
    F.depw = dalloc<double>(c, 3 * Tp, ok);
    F.canopy = dalloc<double>(c, Tp, ok);
    F.lai = dalloc<double>(c, Tp, ok);
    F.stalkN = dalloc<double>(c, Tp, ok);
    F.stalkD = dalloc<double>(c, Tp, ok);
    F.water = dalloc<uint8_t>(c, Tp, ok);
    Forcing& Fo = c.Fo;
    double* fbuf = dalloc<double>(c, 9 * Tp, ok);
    if (ok) {
        Fo.UR = fbuf;
        Fo.U2 = fbuf + Tp;
        Fo.dir = fbuf + 2 * Tp;
        Fo.swe = fbuf + 3 * Tp;
        Fo.t = fbuf + 4 * Tp;
        Fo.rh = fbuf + 5 * Tp;
        Fo.sd = fbuf + 6 * Tp;
        Fo.fetch = fbuf + 7 * Tp;
        Fo.psh = fbuf + 8 * Tp;
    }
    FaceState& S = c.S;
    S.saltation = dalloc<uint8_t>(c, Tp, ok);
    double* sbuf = dalloc<double>(c, 9 * Tp, ok);
    if (ok) {
        S.Qsalt = sbuf;
        S.Qsusp = sbuf + Tp;
        S.Qsubl = sbuf + 2 * Tp;
        S.Qsubl_mass = sbuf + 3 * Tp;
        S.sum_subl = sbuf + 4 * Tp;
        S.drift_mass = sbuf + 5 * Tp;
        S.sum_drift = sbuf + 6 * Tp;
        S.more = sbuf + 7 * Tp;
        S.bsp = sbuf + 8 * Tp;
    }
    c.wnd = Wind{};
    c.wnd.cx = dalloc<double>(c, Tp, ok);
    c.wnd.cy = dalloc<double>(c, Tp, ok);
    c.wnd.cz = F.zc;
    c.wnd.canopy = dalloc<double>(c, Tp, ok);
    c.wnd.lai = dalloc<double>(c, Tp, ok);
    c.wnd.tmp = dalloc<double>(c, Tp, ok);
    c.wnd.grid = dalloc<GridM>(c, nm, ok);
    c.wnd.cell_face = dalloc<int32_t>(c, T, ok);
    S.sub = nullptr;
    c.sg = Subgrid{};
    if (P.subgrid) {
        S.sub = dalloc<double>(c, (size_t)SG_COUNT * Tp, ok);
        c.sg.tpi = dalloc<double>(c, 5 * Tp, ok);
        c.sg.I0 = dalloc<double>(c, Tp, ok);
    }
    Susp& A = c.A;
    A.band = dalloc<double>(c, 6 * R, ok);
    A.cztab = dalloc<CzCoef>(c, (size_t)kMaxLayers * nm, ok);
    A.face_v = dalloc<double>(c, (size_t)FV_COUNT * Tp, ok);
    A.slow_list = dalloc<int32_t>(c, Tp, ok);
    A.n_slow = dalloc<int>(c, 1, ok);
    A.slow_rows = dalloc<double>(c, (size_t)kRowTerms * R, ok);
    MathTables* mt = dalloc<MathTables>(c, 1, ok);
    P.mt = mt;
    // batched-Krylov tiles: runs of at most kBlock faces within one member
    std::vector<int32_t> t_start, t_member, m_tile(nm + 1, 0);
    for (int m = 0; m < nm; ++m) {
        m_tile[m] = (int32_t)t_start.size();
        for (int64_t f = offsets[m]; f < offsets[m + 1]; f += kBlock) {
            t_start.push_back((int32_t)f);
            t_member.push_back(m);
        }
    }
    m_tile[nm] = (int32_t)t_start.size();
    const int ntiles = (int)t_start.size();
    t_start.push_back((int32_t)T);
    int32_t* tile_buf = dalloc<int32_t>(c, (size_t)2 * ntiles + 1 + nm + 1, ok);
    c.tiles.start = tile_buf;
    c.tiles.member = tile_buf + ntiles + 1;
    c.tiles.mtile = tile_buf + 2 * ntiles + 1;
    c.tiles.ntiles = ntiles;
    c.tiles.n = nm;
    c.act_buf = dalloc<int32_t>(c, ntiles, ok);
    c.tiles.act = c.act_buf;
    c.tiles.nact = 0;
    c.tile_part = dalloc<double>(c, (size_t)4 * ntiles, ok);
    c.msR = dalloc<MScal>(c, nm, ok);
    c.ms0 = dalloc<MScal>(c, nm, ok);
    c.ms1 = dalloc<MScal>(c, nm, ok);
    int32_t* face_member = dalloc<int32_t>(c, Tp, ok);
    Member* prm = dalloc<Member>(c, nm, ok);
    c.Mb.n = nm;
    c.Mb.face_member = face_member;
    c.Mb.prm = prm;
    c.Mb.rhs_max = dalloc<unsigned long long>(c, nm, ok);
    c.Mb.dep_max = dalloc<unsigned long long>(c, nm, ok);
    c.Mb.bb = dalloc<double>(c, nm, ok);
    c.Mb.susp_present = dalloc<int>(c, nm, ok);
    c.Mb.dep_present = dalloc<int>(c, nm, ok);
    A.rhs = dalloc<double>(c, R, ok);
    A.x = dalloc<double>(c, R, ok);
    c.x_prev = dalloc<double>(c, R, ok);
    A.u_z = dalloc<double>(c, R, ok);
    A.csubl = dalloc<double>(c, R, ok);
    A.fac_l = dalloc<double>(c, R, ok);
    A.fac_ib = dalloc<double>(c, R, ok);
    A.fac_u = dalloc<double>(c, R, ok);
    if (!P.mixed && cfg.neumann > 0) {
        A.fac_piv = dalloc<double>(c, R, ok);
        A.latp = dalloc<double>(c, (size_t)3 * R, ok);
        c.nu64 = dalloc<double>(c, R, ok);
    }
    c.r = dalloc<double>(c, R, ok);
    if (P.mixed) {
        A.uz32 = dalloc<float>(c, R, ok);
        A.l01 = dalloc<float>(c, (size_t)6 * Tp, ok);
        A.l32 = dalloc<float>(c, R, ok);
        A.ib32 = dalloc<float>(c, R, ok);
        A.up32 = dalloc<float>(c, R, ok);
        c.r32 = dalloc<float>(c, R, ok);
        c.rh32 = dalloc<float>(c, R, ok);
        c.p32 = dalloc<float>(c, R, ok);
        c.v32 = dalloc<float>(c, R, ok);
        c.s32 = dalloc<float>(c, R, ok);
        c.t32 = dalloc<float>(c, R, ok);
        c.zp32 = dalloc<float>(c, R, ok);
        c.zs32 = dalloc<float>(c, R, ok);
        c.x32 = dalloc<float>(c, R, ok);
        if (cfg.neumann > 0) {
            c.nw32 = dalloc<float>(c, R, ok);
            c.nz32 = dalloc<float>(c, R, ok);
        }
    } else {
        c.rh = dalloc<double>(c, R, ok);
        c.p = dalloc<double>(c, R, ok);
        c.v = dalloc<double>(c, R, ok);
        c.sv = dalloc<double>(c, R, ok);
        c.tv = dalloc<double>(c, R, ok);
        c.zp = dalloc<double>(c, R, ok);
        c.zs = dalloc<double>(c, R, ok);
        if (cfg.neumann > 0) {
            c.nw = dalloc<double>(c, R, ok);
            c.nz = dalloc<double>(c, R, ok);
        }
    }
    Dep& D = c.D;
    D.diag = dalloc<double>(c, Tp, ok);
    D.off = dalloc<double>(c, 3 * Tp, ok);
    D.dinv = dalloc<double>(c, Tp, ok);
    D.rhs = dalloc<double>(c, Tp, ok);
    D.x = dalloc<double>(c, Tp, ok);
    c.dr = dalloc<double>(c, Tp, ok);
    c.dz_ = dalloc<double>(c, Tp, ok);
    c.dp = dalloc<double>(c, Tp, ok);
    c.dq = dalloc<double>(c, Tp, ok);
    // the polynomial deposition preconditioner reads the previous residual
    // of its neighbours while the new one is written: a second buffer
    if (cfg.dep_neumann && !P.mixed) c.dr2 = dalloc<double>(c, Tp, ok);
    // the persistent CG's scaling d^-1/2 and scaled couplings
    if (!P.mixed) c.dscale = dalloc<double>(c, (size_t)4 * Tp, ok);
    if (P.mixed) c.dep32 = dalloc<float>(c, (size_t)16 * Tp, ok);
    c.cg_flags = dalloc<unsigned>(c, (size_t)kMaxCgBlocks * 32, ok);
    c.sc = dalloc<Scalars>(c, 4, ok);
    c.red.partials = dalloc<double>(c, (size_t)8 * c.red.nblocks, ok);
    c.ledger = dalloc<double>(c, 8, ok);
    c.gbar = dalloc<GridBar>(c, 1, ok);
    if (!ok) {
        g_create_error = "out of device memory for " + std::to_string(T) + " faces x " + std::to_string(L) + " layers";
        free_all(c);
        delete h;
        return PBSM3D_ERR_OUT_OF_MEMORY;
    }

    // ---- pack the mesh (PBSM3D.cpp:278-392) into SoA
    int rc = 0;
    std::vector<int32_t> nb;
    to_soa3<int32_t>(mesh->neighbor, T, Tp, nb, -1);
    std::vector<double> E, mx(3 * Tp, 0.0), my(3 * Tp, 0.0), tmp(Tp, 0.0), cx(Tp, 0.0), cy(Tp, 0.0);
    to_soa3<double>(mesh->edge_length, T, Tp, E, 0.0);
    for (int64_t i = 0; i < T; ++i)
        for (int j = 0; j < 3; ++j) {
            mx[j * Tp + i] = mesh->edge_normal[6 * i + 2 * j];
            my[j * Tp + i] = mesh->edge_normal[6 * i + 2 * j + 1];
        }
    rc |= upload(c, F.nbr, nb.data(), nb.size() * 4);
    rc |= upload(c, F.E, E.data(), E.size() * 8);
    rc |= upload(c, F.mx, mx.data(), mx.size() * 8);
    rc |= upload(c, F.my, my.data(), my.size() * 8);
    std::vector<double> area(Tp, 1.0), zc(Tp, 0.0);
    for (int64_t i = 0; i < T; ++i) {
        area[i] = mesh->area[i];
        cx[i] = mesh->center[3 * i];
        cy[i] = mesh->center[3 * i + 1];
        zc[i] = mesh->center[3 * i + 2];
    }
    rc |= upload(c, F.area, area.data(), Tp * 8);
    rc |= upload(c, F.zc, zc.data(), Tp * 8);
    rc |= upload(c, c.wnd.cx, cx.data(), Tp * 8);
    rc |= upload(c, c.wnd.cy, cy.data(), Tp * 8);
    {
        // the wind modules read the raw vegetation (scale_wind_vert.cpp:66-69,
        // fetchr.cpp:66-72): canopy height 0 where a face has none
        std::vector<double> wc(Tp, 0.0), wl(Tp, 0.0);
        if (mesh->canopy_height)
            for (int64_t i = 0; i < T; ++i)
                if (!mesh->has_vegetation || mesh->has_vegetation[i]) {
                    wc[i] = mesh->canopy_height[i];
                    wl[i] = mesh->lai ? mesh->lai[i] : 0.0;
                }
        rc |= upload(c, c.wnd.canopy, wc.data(), Tp * 8);
        rc |= upload(c, c.wnd.lai, wl.data(), Tp * 8);
        // fetchr's nearest-face grids: per member, about one face centre per cell
        std::vector<GridM> grids(nm);
        std::vector<int32_t> cell_start(1, 0), cell_face(T);
        for (int m = 0; m < nm; ++m) {
            const int64_t f0 = offsets[m], f1 = offsets[m + 1], n = f1 - f0;
            double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
            for (int64_t i = f0; i < f1; ++i) {
                x0 = std::min(x0, cx[i]);
                x1 = std::max(x1, cx[i]);
                y0 = std::min(y0, cy[i]);
                y1 = std::max(y1, cy[i]);
            }
            const double w = x1 - x0, hgt = y1 - y0;
            double h = std::sqrt(w * hgt / (double)n);
            if (!(h > 0) || !std::isfinite(h)) h = std::max(std::max(w, hgt) / std::max(1.0, std::sqrt((double)n)), 1.0);
            GridM g{};
            g.x0 = x0;
            g.y0 = y0;
            g.h = h;
            g.nx = (int)std::min<int64_t>(std::max<int64_t>(1, (int64_t)std::floor(w / h) + 1), 1 << 20);
            g.ny = (int)std::min<int64_t>(std::max<int64_t>(1, (int64_t)std::floor(hgt / h) + 1), 1 << 20);
            g.cell0 = (int)(cell_start.size() - 1);
            const int64_t nc = (int64_t)g.nx * g.ny;
            std::vector<int32_t> cnt(nc + 1, 0);
            auto cell_of = [&](int64_t i) {
                const int ci = std::min(std::max((int)std::floor((cx[i] - g.x0) / g.h), 0), g.nx - 1);
                const int cj = std::min(std::max((int)std::floor((cy[i] - g.y0) / g.h), 0), g.ny - 1);
                return (int64_t)cj * g.nx + ci;
            };
            for (int64_t i = f0; i < f1; ++i) cnt[cell_of(i) + 1]++;
            for (int64_t k = 0; k < nc; ++k) cnt[k + 1] += cnt[k];
            std::vector<int32_t> pos(cnt.begin(), cnt.end() - 1);
            const int32_t base = cell_start.back();
            for (int64_t i = f0; i < f1; ++i) cell_face[base + pos[cell_of(i)]++] = (int32_t)i;
            for (int64_t k = 1; k <= nc; ++k) cell_start.push_back(base + cnt[k]);
            grids[m] = g;
        }
        c.wnd.cell_start = dalloc<int32_t>(c, cell_start.size(), ok);
        if (!ok) rc = 1;
        rc |= upload(c, c.wnd.grid, grids.data(), nm * sizeof(GridM));
        if (ok) rc |= upload(c, c.wnd.cell_start, cell_start.data(), cell_start.size() * 4);
        rc |= upload(c, c.wnd.cell_face, cell_face.data(), T * 4);
    }
    std::vector<double> canopy(Tp, 0.0), lai(Tp, 0.0), sN(Tp, 0.0), sD(Tp, 0.0);
    if (P.enable_veg)
        for (int64_t i = 0; i < T; ++i) {
            canopy[i] = mesh->canopy_height[i];
            if (cfg.use_R94_lambda) {
                lai[i] = mesh->lai ? mesh->lai[i] : 0.0;
            } else {
                sN[i] = mesh->stalk_number ? mesh->stalk_number[i] : 1.0;
                sD[i] = mesh->stalk_diameter ? mesh->stalk_diameter[i] : 0.8;
            }
        }
    rc |= upload(c, F.canopy, canopy.data(), Tp * 8);
    rc |= upload(c, F.lai, lai.data(), Tp * 8);
    rc |= upload(c, F.stalkN, sN.data(), Tp * 8);
    rc |= upload(c, F.stalkD, sD.data(), Tp * 8);
    std::vector<uint8_t> water(Tp, 0);
    if (mesh->is_water)
        for (int64_t i = 0; i < T; ++i) water[i] = mesh->is_water[i] ? 1 : 0;
    rc |= upload(c, F.water, water.data(), Tp);
    {
        std::vector<int32_t> fm(Tp, 0);
        for (int m = 0; m < nm; ++m)
            for (int64_t i = offsets[m]; i < offsets[m + 1]; ++i) fm[i] = m;
        rc |= upload(c, face_member, fm.data(), Tp * 4);
        rc |= upload(c, prm, members.data(), nm * sizeof(Member));
        std::vector<int> ones(nm, 1);
        rc |= upload(c, c.Mb.susp_present, ones.data(), nm * 4);
        rc |= upload(c, c.Mb.dep_present, ones.data(), nm * 4);
    }
    {
        MathTables h;
        math_tables_fill(h);
        rc |= upload(c, mt, &h, sizeof(h));
        rc |= upload(c, tile_buf, t_start.data(), (ntiles + 1) * 4);
        rc |= upload(c, tile_buf + ntiles + 1, t_member.data(), ntiles * 4);
        rc |= upload(c, tile_buf + 2 * ntiles + 1, m_tile.data(), (nm + 1) * 4);
    }
    rc |= upload(c, c.dr, cx.data(), Tp * 8);
    rc |= upload(c, c.dz_, cy.data(), Tp * 8);
    // module state: CHM face variables start at -9999, sum_drift/sum_subl at 0
    std::vector<double> nanv(Tp, -9999.0), zero(Tp, 0.0);
    rc |= upload(c, S.Qsalt, nanv.data(), Tp * 8);
    rc |= upload(c, S.Qsusp, nanv.data(), Tp * 8);
    rc |= upload(c, S.Qsubl, nanv.data(), Tp * 8);
    rc |= upload(c, S.Qsubl_mass, nanv.data(), Tp * 8);
    rc |= upload(c, S.sum_subl, zero.data(), Tp * 8);
    rc |= upload(c, S.drift_mass, nanv.data(), Tp * 8);
    rc |= upload(c, S.sum_drift, zero.data(), Tp * 8);
    rc |= upload(c, S.more, nanv.data(), Tp * 8);
    rc |= upload(c, S.bsp, nanv.data(), Tp * 8);
    rc |= upload(c, Fo.fetch, std::vector<double>(Tp, 1000.0).data(), Tp * 8);
    rc |= upload(c, Fo.psh, zero.data(), Tp * 8);
    if (P.subgrid) {
        // TPI statistics, NaN where the mesh has none; outputs start at -9999
        std::vector<double> tpi(5 * Tp, NAN);
        const double* src[5] = {mesh->tpi_mean, mesh->tpi_std, mesh->tpi_neg_frac, mesh->tpi_neg_mean,
                                mesh->tpi_neg_std};
        for (int k = 0; k < 5; ++k)
            if (src[k]) std::copy(src[k], src[k] + T, tpi.begin() + k * Tp);
        rc |= upload(c, c.sg.tpi, tpi.data(), 5 * Tp * 8);
        std::vector<double> sub((size_t)SG_COUNT * Tp, -9999.0);
        rc |= upload(c, S.sub, sub.data(), sub.size() * 8);
        rc |= subgrid_init(c, c.stream);
    }
    if (cudaMemsetAsync(c.sc, 0, 4 * sizeof(Scalars), c.stream) != cudaSuccess) rc = 1;
    if (cudaMemsetAsync(A.x, 0, R * 8, c.stream) != cudaSuccess) rc = 1;
    if (cudaMemsetAsync(c.x_prev, 0, R * 8, c.stream) != cudaSuccess) rc = 1;
    if (configure_solver_kernels(c)) rc = 1;
    if (configure_cg(c)) rc = 1;
    launch_init_static(c, c.stream);
    if (cudaStreamSynchronize(c.stream) != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = 1;
    if (rc) {
        g_create_error = "device upload failed: " + c.err;
        free_all(c);
        delete h;
        return PBSM3D_ERR_CUDA;
    }
    c.launches = 0;
    c.bytes = 0;
    *out = h;
    return 0;
}

int pbsm3d_create(const pbsm3d_mesh_desc* mesh, const pbsm3d_config* cfg, pbsm3d_ctx** out) {
    if (!mesh || !cfg) {
        g_create_error = "null mesh or config";
        return PBSM3D_ERR_INVALID_ARG;
    }
    Member m{cfg->ustar_th_scale, cfg->z0_snow, cfg->settling_scale, log(50.0 / cfg->z0_snow)};
    return create_core(mesh, cfg, {0, mesh->n_faces}, {m}, out);
}

int pbsm3d_ensemble_create(int32_t n_members, const pbsm3d_mesh_desc* meshes, const pbsm3d_member* members,
                           const pbsm3d_config* cfg, pbsm3d_ctx** out) {
    if (!out || !meshes || !members || !cfg || n_members < 1 || n_members > kMaxMembers) {
        g_create_error = "ensemble: 1..256 members with meshes, member parameters and a config";
        return PBSM3D_ERR_INVALID_ARG;
    }
    // the members' meshes as one disjoint union (faces in member order,
    // neighbour ids shifted by each member's face offset)
    std::vector<int64_t> off(n_members + 1, 0);
    // vegetation is a per-domain switch in the reference (PBSM3D.cpp:283-325):
    // the members must agree on it
    bool veg = true, lai = false, sn = false, sd = false, water = false, tpi_any[5] = {false, false, false, false, false};
    for (int m = 0; m < n_members; ++m) {
        const pbsm3d_mesh_desc& d = meshes[m];
        if (d.n_faces <= 0 || !d.neighbor || !d.edge_length || !d.edge_normal || !d.area || !d.center) {
            g_create_error = "ensemble: invalid mesh of member " + std::to_string(m);
            return PBSM3D_ERR_INVALID_ARG;
        }
        off[m + 1] = off[m] + d.n_faces;
        bool mveg = d.canopy_height != nullptr;
        if (mveg && d.has_vegetation)
            for (int64_t i = 0; i < d.n_faces; ++i) mveg = mveg && d.has_vegetation[i];
        if (m > 0 && mveg != veg) {
            g_create_error = "ensemble: members must all have vegetation on every face, or none";
            return PBSM3D_ERR_INVALID_ARG;
        }
        veg = mveg;
        lai = lai || d.lai;
        sn = sn || d.stalk_number;
        sd = sd || d.stalk_diameter;
        water = water || d.is_water;
        const double* tp[5] = {d.tpi_mean, d.tpi_std, d.tpi_neg_frac, d.tpi_neg_mean, d.tpi_neg_std};
        for (int k = 0; k < 5; ++k) tpi_any[k] = tpi_any[k] || tp[k];
    }
    const int64_t T = off[n_members];
    std::vector<int32_t> nb(3 * T);
    std::vector<double> E(3 * T), M(6 * T), area(T), C(3 * T), ch, la, sN, sD;
    std::vector<uint8_t> wat;
    if (veg) ch.resize(T);
    if (veg && lai) la.assign(T, 0.0);
    if (veg && sn) sN.assign(T, 1.0);
    if (veg && sd) sD.assign(T, 0.8);
    if (water) wat.assign(T, 0);
    std::vector<double> tpi[5];
    for (int k = 0; k < 5; ++k)
        if (tpi_any[k]) tpi[k].assign(T, NAN);
    for (int m = 0; m < n_members; ++m) {
        const pbsm3d_mesh_desc& d = meshes[m];
        const int64_t o = off[m], n = d.n_faces;
        for (int64_t k = 0; k < 3 * n; ++k) {
            const int32_t v = d.neighbor[k];
            if (v < -1 || v >= n) {
                g_create_error = "ensemble: neighbour out of range in member " + std::to_string(m);
                return PBSM3D_ERR_BAD_MESH;
            }
            nb[3 * o + k] = v >= 0 ? (int32_t)(v + o) : -1;
        }
        std::copy(d.edge_length, d.edge_length + 3 * n, E.begin() + 3 * o);
        std::copy(d.edge_normal, d.edge_normal + 6 * n, M.begin() + 6 * o);
        std::copy(d.area, d.area + n, area.begin() + o);
        std::copy(d.center, d.center + 3 * n, C.begin() + 3 * o);
        if (veg) std::copy(d.canopy_height, d.canopy_height + n, ch.begin() + o);
        if (veg && lai && d.lai) std::copy(d.lai, d.lai + n, la.begin() + o);
        if (veg && sn && d.stalk_number) std::copy(d.stalk_number, d.stalk_number + n, sN.begin() + o);
        if (veg && sd && d.stalk_diameter) std::copy(d.stalk_diameter, d.stalk_diameter + n, sD.begin() + o);
        if (water && d.is_water) std::copy(d.is_water, d.is_water + n, wat.begin() + o);
        const double* tp[5] = {d.tpi_mean, d.tpi_std, d.tpi_neg_frac, d.tpi_neg_mean, d.tpi_neg_std};
        for (int k = 0; k < 5; ++k)
            if (tp[k]) std::copy(tp[k], tp[k] + n, tpi[k].begin() + o);
    }
    pbsm3d_mesh_desc u{};
    u.n_faces = T;
    u.neighbor = nb.data();
    u.edge_length = E.data();
    u.edge_normal = M.data();
    u.area = area.data();
    u.center = C.data();
    u.canopy_height = veg ? ch.data() : nullptr;
    u.lai = la.empty() ? nullptr : la.data();
    u.stalk_number = sN.empty() ? nullptr : sN.data();
    u.stalk_diameter = sD.empty() ? nullptr : sD.data();
    u.has_vegetation = nullptr;
    u.is_water = wat.empty() ? nullptr : wat.data();
    u.tpi_mean = tpi[0].empty() ? nullptr : tpi[0].data();
    u.tpi_std = tpi[1].empty() ? nullptr : tpi[1].data();
    u.tpi_neg_frac = tpi[2].empty() ? nullptr : tpi[2].data();
    u.tpi_neg_mean = tpi[3].empty() ? nullptr : tpi[3].data();
    u.tpi_neg_std = tpi[4].empty() ? nullptr : tpi[4].data();
    std::vector<Member> mp(n_members);
    for (int m = 0; m < n_members; ++m)
        mp[m] = Member{members[m].ustar_th_scale, members[m].z0_snow, members[m].settling_scale,
                       log(50.0 / members[m].z0_snow)};
    return create_core(&u, cfg, off, mp, out);
}

int pbsm3d_member_offsets(const pbsm3d_ctx* h, int64_t* offsets) {
    if (!h || !offsets) return PBSM3D_ERR_INVALID_ARG;
    std::copy(h->c.member_offsets.begin(), h->c.member_offsets.end(), offsets);
    return (int)h->c.member_offsets.size() - 1;
}

void pbsm3d_destroy(pbsm3d_ctx* h) {
    if (!h) return;
    cudaStreamSynchronize(h->c.stream);
    free_all(h->c);
    delete h;
}

int pbsm3d_set_profiling(pbsm3d_ctx* h, int32_t on) {
    if (!h) return PBSM3D_ERR_INVALID_ARG;
    h->c.prof = on != 0;
    return 0;
}

int pbsm3d_set_column_geometry(pbsm3d_ctx* h, int32_t width, int32_t lanes) {
    if (!h) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    for (int gi = 0; gi < kNumColGeoms; ++gi)
        if (kColGeom[gi].W == width && kColGeom[gi].LC == lanes) {
            if (c.graph && c.geom != gi) graph_destroy(c);  // captured with the old geometry
            c.geom = gi;
            c.tuned = true;
            return 0;
        }
    c.err = "column geometry must be width 64, 128 or 256 and lanes 1, 2 or 4";
    return PBSM3D_ERR_INVALID_ARG;
}

int pbsm3d_get_column_geometry(const pbsm3d_ctx* h, int32_t* width, int32_t* lanes, int32_t* tuned) {
    if (!h) return PBSM3D_ERR_INVALID_ARG;
    const Ctx& c = h->c;
    if (width) *width = kColGeom[c.geom].W;
    if (lanes) *lanes = kColGeom[c.geom].LC;
    if (tuned) *tuned = c.tuned ? 1 : 0;
    return 0;
}

int pbsm3d_arm_wait_timeout_test(pbsm3d_ctx* h, int32_t withhold_block, double limit_ms) {
    if (!h || withhold_block < 0 || !(limit_ms > 0.0) || limit_ms > 2000.0) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    if (c.tiles.n > 1 || c.cfg.graph) {
        c.err = "the wait-timeout test needs a single-mesh, host-driven context (persistent deposition CG)";
        return PBSM3D_ERR_INVALID_ARG;
    }
    c.test_withhold = withhold_block;
    c.test_limit_ns = (unsigned long long)(limit_ms * 1e6);
    return 0;
}

int pbsm3d_timer_mark(pbsm3d_ctx* h, int32_t slot) {
    if (!h || slot < 0 || slot >= 16) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    PBSM_CUDA_TRY(cudaEventRecord(c.user_ev[slot], c.stream));
    return 0;
}

int pbsm3d_timer_elapsed(pbsm3d_ctx* h, int32_t a, int32_t b, double* ms) {
    if (!h || !ms || a < 0 || a >= 16 || b < 0 || b >= 16) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    PBSM_CUDA_TRY(cudaEventSynchronize(c.user_ev[b]));
    float f = 0;
    PBSM_CUDA_TRY(cudaEventElapsedTime(&f, c.user_ev[a], c.user_ev[b]));
    *ms = f;
    return 0;
}

int pbsm3d_set_mlp(pbsm3d_ctx* h, const float* params, const float* feat_mean, const float* feat_scale) {
    if (!h || !params || !feat_mean || !feat_scale) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    int rc = mlp_load(c, params, feat_mean, feat_scale);
    return rc;
}

int pbsm3d_mlp_features(pbsm3d_ctx* h, float* features, float* targets, int32_t on_device) {
    if (!h) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    const int64_t rows = c.P.T * c.P.L;
    if (on_device) {
        int rc = mlp_features(c, features, targets);
        if (!rc && cudaStreamSynchronize(c.stream) != cudaSuccess) rc = PBSM3D_ERR_CUDA;
        return rc;
    }
    float *df = nullptr, *dt = nullptr;
    PBSM_CUDA_TRY(cudaMalloc(&df, rows * 14 * 4));
    if (cudaMalloc(&dt, rows * 4) != cudaSuccess) {
        cudaFree(df);
        c.err = "out of device memory";
        return PBSM3D_ERR_OUT_OF_MEMORY;
    }
    int rc = mlp_features(c, df, dt);
    if (!rc && features)
        rc = cudaMemcpyAsync(features, df, rows * 14 * 4, cudaMemcpyDeviceToHost, c.stream) ? PBSM3D_ERR_CUDA : 0;
    if (!rc && targets)
        rc = cudaMemcpyAsync(targets, dt, rows * 4, cudaMemcpyDeviceToHost, c.stream) ? PBSM3D_ERR_CUDA : 0;
    if (cudaStreamSynchronize(c.stream) != cudaSuccess) rc = PBSM3D_ERR_CUDA;
    cudaFree(df);
    cudaFree(dt);
    return rc;
}

int pbsm3d_mlp_predict(pbsm3d_ctx* h, double* c_out) {
    if (!h || !c_out) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    double* tmp = nullptr;
    PBSM_CUDA_TRY(cudaMalloc(&tmp, c.P.R * 8));
    int rc = launch_mlp_infer(c, c.stream, tmp);
    if (!rc && cudaMemcpy2DAsync(c_out, c.P.T * 8, tmp, c.P.Tp * 8, c.P.T * 8, c.P.L, cudaMemcpyDeviceToHost,
                                 c.stream) != cudaSuccess)
        rc = PBSM3D_ERR_CUDA;
    if (cudaStreamSynchronize(c.stream) != cudaSuccess) rc = PBSM3D_ERR_CUDA;
    cudaFree(tmp);
    return rc;
}

// Ensembles (which 0: suspension, 1: deposition): each member's own
// "present" test (||rhs_m||_inf > 1e-12, PBSM3D.cpp:1424-1427, 1661-1664);
// absent members get a zero right-hand side (solution exactly 0, and no
// update), and the joint Krylov target becomes tol * min_m ||rhs_m|| so every
// present member reaches its own relative tolerance.
static int member_presence(Ctx& c, cudaStream_t s, int which) {
    const int n = c.Mb.n;
    std::vector<unsigned long long> mx(n);
    std::vector<int> present(n), susp(n);
    PBSM_CUDA_TRY(cudaMemcpyAsync(mx.data(), which ? c.Mb.dep_max : c.Mb.rhs_max, n * 8, cudaMemcpyDeviceToHost, s));
    if (which) PBSM_CUDA_TRY(cudaMemcpyAsync(susp.data(), c.Mb.susp_present, n * 4, cudaMemcpyDeviceToHost, s));
    PBSM_CUDA_TRY(cudaStreamSynchronize(s));
    bool any = false;
    for (int m = 0; m < n; ++m) {
        double v;
        memcpy(&v, &mx[m], 8);
        present[m] = v > 1e-12 && (!which || susp[m]);
        any = any || present[m];
    }
    PBSM_CUDA_TRY(cudaMemcpyAsync(which ? c.Mb.dep_present : c.Mb.susp_present, present.data(), n * 4,
                                  cudaMemcpyHostToDevice, s));
    launch_member_mask_norm(c, s, which);
    std::vector<double> bb(n);
    PBSM_CUDA_TRY(cudaMemcpyAsync(bb.data(), c.Mb.bb, n * 8, cudaMemcpyDeviceToHost, s));
    PBSM_CUDA_TRY(cudaStreamSynchronize(s));
    double tot = 0, mn = -1;
    for (int m = 0; m < n; ++m)
        if (present[m]) {
            tot += bb[m];
            if (mn < 0 || bb[m] < mn) mn = bb[m];
        }
    const double scale2 = (any && tot > 0) ? mn / tot : 1.0;
    if (which) {
        c.deposition_present = any;
        c.dep_target_scale2 = scale2;
    } else {
        c.suspension_present = any;
        c.target_scale2 = scale2;
    }
    return 0;
}

static int copy_in(Ctx& c, double* dst, const double* src, int on_device) {
    PBSM_CUDA_TRY(cudaMemcpyAsync(dst, src, c.P.T * 8, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  c.stream));
    return 0;
}
static int copy_out(Ctx& c, double* dst, const double* src, int on_device, cudaStream_t s = nullptr) {
    if (!dst) return 0;
    PBSM_CUDA_TRY(cudaMemcpyAsync(dst, src, c.P.T * 8, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                  s ? s : c.stream));
    return 0;
}

// Output k of the step (pbsm3d_outputs order) is final once the suspension
// post has run: Qsalt, Qsusp, Qsubl, Qsubl_mass, sum_subl, blowing-snow
// probability (and c).  The others change in the deposition update.
static bool final_after_post(int k) { return k <= 4 || k == 8; }

// Whether the outputs that are final after the post can be copied to the
// host while the step goes on: host outputs in page-locked memory (a copy
// into pageable memory returns only when it is done, so queued early it
// would hold the host, and the rest of the step, until then).
static bool early_copies(const pbsm3d_outputs* out) {
    if (!out || out->on_device) return false;
    const void* ptrs[7] = {out->Qsalt, out->Qsusp, out->Qsubl, out->Qsubl_mass, out->sum_subl,
                           out->blowingsnow_probability, out->c};
    bool any = false;
    for (const void* p : ptrs) {
        if (!p) continue;
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (a.type != cudaMemoryTypeHost) return false;
        any = true;
    }
    return any;
}

// Queue the host copies of the outputs that are final after the post (and
// c) on the second stream, after the work queued so far on s; copy_ev[1]
// marks their end and `early` records that they are in flight.
static int copy_final_outputs(Ctx& c, cudaStream_t s, const pbsm3d_outputs* out, bool& early) {
    double* outs[9] = {out->Qsalt, out->Qsusp, out->Qsubl, out->Qsubl_mass, out->sum_subl,
                       out->drift_mass, out->sum_drift, out->pbsm_more_than_avail, out->blowingsnow_probability};
    const double* srcs[9] = {c.S.Qsalt, c.S.Qsusp, c.S.Qsubl, c.S.Qsubl_mass, c.S.sum_subl,
                             c.S.drift_mass, c.S.sum_drift, c.S.more, c.S.bsp};
    PBSM_CUDA_TRY(cudaEventRecord(c.copy_ev[0], s));
    PBSM_CUDA_TRY(cudaStreamWaitEvent(c.copy_stream, c.copy_ev[0], 0));
    early = true;
    int rc = 0;
    for (int k = 0; k < 9; ++k)
        if (final_after_post(k) && (rc = copy_out(c, outs[k], srcs[k], 0, c.copy_stream))) break;
    if (!rc && out->c)
        rc = cudaMemcpy2DAsync(out->c, c.P.T * 8, c.A.x, c.P.Tp * 8, c.P.T * 8, c.P.L, cudaMemcpyDeviceToHost,
                               c.copy_stream) == cudaSuccess ? 0 : PBSM3D_ERR_CUDA;
    if (!rc) rc = cudaEventRecord(c.copy_ev[1], c.copy_stream) == cudaSuccess ? 0 : PBSM3D_ERR_CUDA;
    if (rc) {
        cudaStreamSynchronize(c.copy_stream);
        c.err = "output copy failed";
    }
    return rc;
}

static float ev_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

int pbsm3d_step(pbsm3d_ctx* h, const pbsm3d_forcing* f, double dt, const pbsm3d_outputs* out, pbsm3d_stats* st) {
    if (!h) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    c.err.clear();
    if (!f) {
        c.err = "missing forcing";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if ((c.cfg.use_exp_fetch || c.cfg.use_tanh_fetch) && !f->fetch && !c.cfg.derive_fetch) {
        c.err = "fetch forcing is required by use_exp_fetch/use_tanh_fetch (or derive_fetch)";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (c.cfg.use_PomLi_probability && !f->p_snow_hours) {
        c.err = "p_snow_hours forcing is required by use_PomLi_probability";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (!(dt > 0) || !isfinite(dt)) {
        c.err = "dt must be positive";
        return PBSM3D_ERR_INVALID_ARG;
    }
    cudaStream_t s = c.stream;
    c.P.dt = dt;
    c.launches = 0;
    c.bytes = 0;
    c.pused = 0;
    c.susp_iters = c.susp_matvecs = c.susp_refinements = c.dep_iters = 0;
    c.susp_relres = c.dep_relres = 0;
    int rc;
    PBSM_CUDA_TRY(cudaEventRecord(c.ev[0], s));
    const int dev = f->on_device;
    // swe and snow depth come from the context's snow state when the caller
    // set one and leaves them NULL
    const bool own_snow = c.snow_state && !f->swe && !f->snowdepthavg;
    if (!own_snow && (!f->swe || !f->snowdepthavg)) {
        c.err = "forcing swe and snowdepthavg are required (or pbsm3d_set_snow)";
        return PBSM3D_ERR_INVALID_ARG;
    }
    const bool derive_wind = c.cfg.derive_wind != 0, derive_fetch = c.cfg.derive_fetch != 0;
    if (!f->U_R || (!f->U_2m_above_srf && !derive_wind) || !f->vw_dir || !f->t || !f->rh) {
        c.err = "forcing U_R, U_2m_above_srf (unless derive_wind), vw_dir, t and rh are required";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if ((rc = copy_in(c, c.Fo.UR, f->U_R, dev)) ||
        (!derive_wind && (rc = copy_in(c, c.Fo.U2, f->U_2m_above_srf, dev))) ||
        (rc = copy_in(c, c.Fo.dir, f->vw_dir, dev)) || (rc = copy_in(c, c.Fo.t, f->t, dev)) ||
        (rc = copy_in(c, c.Fo.rh, f->rh, dev)))
        return rc;
    if (!own_snow) {
        if ((rc = copy_in(c, c.Fo.swe, f->swe, dev)) || (rc = copy_in(c, c.Fo.sd, f->snowdepthavg, dev))) return rc;
        // a caller that passes its own snow state takes over from the context's
        c.snow_state = false;
    }
    if (f->fetch && !derive_fetch && (rc = copy_in(c, c.Fo.fetch, f->fetch, dev))) return rc;
    if (f->p_snow_hours && (rc = copy_in(c, c.Fo.psh, f->p_snow_hours, dev))) return rc;
    const int64_t h2d = dev ? 0
                            : c.P.T * 8 *
                                  ((own_snow ? 5 : 7) - (derive_wind ? 1 : 0) + (f->fetch && !derive_fetch ? 1 : 0) +
                                   (f->p_snow_hours ? 1 : 0));

    double susp_rhs_max = 0.0, dep_rhs_max = 0.0;
    bool early_out = false;  // some host outputs already copied on the second stream
    bool graph_run = false;  // the step graph is queued on s (its outcome comes after the sync)
    // whatever path leaves the step, no copy into the caller's buffers outlives it
    struct CopyGuard {
        Ctx& c;
        const bool& on;
        const bool& queued;
        ~CopyGuard() {
            if (on) cudaStreamSynchronize(c.copy_stream);
            if (queued) cudaStreamSynchronize(c.stream);
        }
    } copy_guard{c, early_out, graph_run};
    // graph mode; with the autotuner on, the first step runs host-driven so
    // that the geometry is tuned before the graph is built
    if (c.cfg.graph && c.tuned) {
        // the device part of the step as the step graph's two launches; host
        // outputs final after the post are copied while part 2 runs (on a
        // failed step they may hold the post's fields or the last step's)
        PBSM_CUDA_TRY(cudaEventRecord(c.ev[1], s));
        // Nothing waits for the graph here: the remaining output copies
        // follow it on s, and its outcome is read after the step's one
        // synchronisation below.
        std::function<int()> between;
        if (early_copies(out)) between = [&]() { return copy_final_outputs(c, s, out, early_out); };
        graph_run = true;
        if ((rc = graph_step(c, s, own_snow, between))) return rc;
        for (int k = 2; k <= 6; ++k) PBSM_CUDA_TRY(cudaEventRecord(c.ev[k], s));
    } else {
        // the previous step's solution (the assembly zeroes x, as the reference's
        // zeroSystem does): kept for the warm starts and the MLP features
        PBSM_CUDA_TRY(cudaMemcpyAsync(c.x_prev, c.A.x, c.P.R * 8, cudaMemcpyDeviceToDevice, s));

        PBSM_CUDA_TRY(cudaEventRecord(c.ev[1], s));
        if (c.Mb.n > 1) {
            PBSM_CUDA_TRY(cudaMemsetAsync(c.Mb.rhs_max, 0, c.Mb.n * 8, s));
            PBSM_CUDA_TRY(cudaMemsetAsync(c.Mb.dep_max, 0, c.Mb.n * 8, s));
        }
        launch_assemble_suspension(c, s);
        PBSM_CUDA_TRY(cudaGetLastError());
        PBSM_CUDA_TRY(cudaMemcpyAsync(c.sc_host, c.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
        PBSM_CUDA_TRY(cudaMemcpyAsync(c.n_slow_host, c.A.n_slow, sizeof(int), cudaMemcpyDeviceToHost, s));
        PBSM_CUDA_TRY(cudaEventRecord(c.ev[2], s));
        PBSM_CUDA_TRY(cudaStreamSynchronize(s));
        if (c.sc_host->nan_flag != 0.0) {
            c.err = "NaN in the assembled suspension system (check the forcing)";
            return PBSM3D_ERR_NAN_INPUT;
        }
        c.n_slow = *c.n_slow_host;
        susp_rhs_max = c.sc_host->rhs_max;
        c.suspension_present = susp_rhs_max > 1e-12;  // PBSM3D.cpp:1424-1427
        c.target_scale2 = 1.0;
        if (c.Mb.n > 1 && (rc = member_presence(c, s, 0))) return rc;
        if (c.suspension_present) {
            if (c.cfg.warm_start == PBSM3D_X0_PREVIOUS)
                PBSM_CUDA_TRY(cudaMemcpyAsync(c.A.x, c.x_prev, c.P.R * 8, cudaMemcpyDeviceToDevice, s));
            if (c.cfg.warm_start == PBSM3D_X0_LEARNED) {
                // network guess, then one block-Jacobi sweep: each column then
                // satisfies its own vertical balance exactly and only the lateral
                // couplings act on the network's error
                if (c.cfg.warm_flags & 2) {
                    if ((rc = launch_mlp_infer(c, s, c.A.x))) return rc;
                } else {
                    if ((rc = launch_mlp_infer(c, s, c.r))) return rc;
                    if ((rc = jacobi_sweep(c, s, c.r, c.A.x))) return rc;
                }
            }
            if (c.Mb.n > 1 && c.cfg.warm_start != PBSM3D_X0_ZERO) launch_member_zero(c, s, c.A.x);
            rc = solve_suspension(c, s, st);
            PBSM_CUDA_TRY(cudaGetLastError());
            if (rc) return rc;
        }
        PBSM_CUDA_TRY(cudaEventRecord(c.ev[3], s));
        launch_post_and_assemble_deposition(c, s);
        PBSM_CUDA_TRY(cudaGetLastError());
        PBSM_CUDA_TRY(cudaMemcpyAsync(c.sc_host, c.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
        PBSM_CUDA_TRY(cudaEventRecord(c.ev[4], s));
        PBSM_CUDA_TRY(cudaStreamSynchronize(s));
        if (c.sc_host->nan_flag != 0.0) {
            c.err = "NaN in the assembled deposition system";
            return PBSM3D_ERR_NAN_INPUT;
        }
        dep_rhs_max = c.sc_host->rhs_max;
        c.deposition_present = c.suspension_present && dep_rhs_max > 1e-12;  // PBSM3D.cpp:1661-1664
        c.dep_target_scale2 = 1.0;
        if (c.Mb.n > 1 && (rc = member_presence(c, s, 1))) return rc;
        if (c.deposition_present) {
            // host outputs already final: copied on the second stream while
            // the deposition solve runs
            if (early_copies(out) && (rc = copy_final_outputs(c, s, out, early_out))) return rc;
            rc = solve_deposition(c, s, st);
            PBSM_CUDA_TRY(cudaGetLastError());
            if (rc) {
                // no copy into the caller's buffers outlives the call
                if (early_out) cudaStreamSynchronize(c.copy_stream);
                return rc;
            }
        }
        PBSM_CUDA_TRY(cudaEventRecord(c.ev[5], s));
        launch_update(c, s);
        if (own_snow) launch_consume_drift(c, s);
        PBSM_CUDA_TRY(cudaGetLastError());
        PBSM_CUDA_TRY(cudaEventRecord(c.ev[6], s));
    }
    int64_t d2h = 0;
    if (out) {
        const int od = out->on_device;
        double* outs[9] = {out->Qsalt, out->Qsusp, out->Qsubl, out->Qsubl_mass, out->sum_subl,
                           out->drift_mass, out->sum_drift, out->pbsm_more_than_avail, out->blowingsnow_probability};
        const double* srcs[9] = {c.S.Qsalt, c.S.Qsusp, c.S.Qsubl, c.S.Qsubl_mass, c.S.sum_subl,
                                 c.S.drift_mass, c.S.sum_drift, c.S.more, c.S.bsp};
        for (int k = 0; k < 9; ++k) {
            if (!(early_out && final_after_post(k)) && (rc = copy_out(c, outs[k], srcs[k], od))) {
                if (early_out) cudaStreamSynchronize(c.copy_stream);
                return rc;
            }
            if (outs[k] && !od) d2h += c.P.T * 8;
        }
        if (c.S.sub) {
            double* souts[5] = {out->hold_topo, out->frac_contrib, out->frac_contrib_nosnw, out->tpi_lim, out->test_int};
            const int rows[5] = {SG_HOLD, SG_FRAC, SG_NOSNW, SG_TPILIM, SG_TESTINT};
            for (int k = 0; k < 5; ++k) {
                if ((rc = copy_out(c, souts[k], c.S.sub + (size_t)rows[k] * c.P.Tp, od))) return rc;
                if (souts[k] && !od) d2h += c.P.T * 8;
            }
        }
        if (out->c) {
            // layer-major with stride n_faces (the device stride is the padded Tp)
            if (!early_out)
                PBSM_CUDA_TRY(cudaMemcpy2DAsync(out->c, c.P.T * 8, c.A.x, c.P.Tp * 8, c.P.T * 8, c.P.L,
                                                od ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
            if (!od) d2h += c.P.T * c.P.L * 8;
        }
    }
    double ledger[8] = {0};
    PBSM_CUDA_TRY(cudaMemcpyAsync(ledger, c.ledger, 5 * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (early_out) PBSM_CUDA_TRY(cudaStreamWaitEvent(s, c.copy_ev[1], 0));
    PBSM_CUDA_TRY(cudaEventRecord(c.ev[7], s));
    PBSM_CUDA_TRY(cudaStreamSynchronize(s));
    if (graph_run) {
        graph_run = false;
        if ((rc = graph_finish(c))) return rc;  // the output buffers' contents are unspecified
        susp_rhs_max = c.graph_rhs_max[0];
        dep_rhs_max = c.graph_rhs_max[1];
    }
    if (st) {
        memset(st, 0, sizeof(*st));
        st->suspension_present = c.suspension_present;
        st->deposition_present = c.deposition_present;
        st->susp_iters = c.susp_iters;
        st->susp_matvecs = c.susp_matvecs;
        st->susp_refinements = c.susp_refinements;
        st->dep_iters = c.dep_iters;
        st->dep_refinements = c.dep_refinements;
        st->n_slow_faces = c.n_slow;
        st->susp_rel_residual = c.susp_relres;
        st->dep_rel_residual = c.dep_relres;
        st->susp_rhs_max = susp_rhs_max;
        st->dep_rhs_max = dep_rhs_max;
        if (c.cfg.graph && c.tuned && c.graph_phases) {
            // one graph launch: the phases from the device stamps in the graph
            st->ms_coefficients = c.graph_phase_ms[0];
            st->ms_susp_solve = c.graph_phase_ms[1];
            st->ms_post = c.graph_phase_ms[2];
            st->ms_dep_solve = c.graph_phase_ms[3];
            st->ms_update = c.graph_phase_ms[4];
        } else {
            st->ms_coefficients = ev_ms(c.ev[1], c.ev[2]);
            st->ms_susp_solve = ev_ms(c.ev[2], c.ev[3]);
            st->ms_post = ev_ms(c.ev[3], c.ev[4]);
            st->ms_dep_solve = ev_ms(c.ev[4], c.ev[5]);
            st->ms_update = ev_ms(c.ev[5], c.ev[6]);
        }
        st->ms_dep_assembly = 0;
        st->ms_total = ev_ms(c.ev[0], c.ev[7]);
        if (c.deposition_present) {
            st->ledger_divergence = ledger[0];
            st->ledger_deposited = ledger[1];
            st->ledger_clipped = ledger[2];
            st->ledger_residual = ledger[3];
        }
        st->ledger_snow_mass = ledger[4];
        st->bytes_moved = c.bytes + h2d + d2h;
        st->gpu_launches = c.launches;
        if (c.prof && !c.cfg.graph) {  // a graph replay records no per-launch events
            st->profiled = 1;
            for (int k = 0; k < c.pused; ++k) {
                const int cat = c.pcat[k];
                st->kern_ms[cat] += ev_ms(c.pev[2 * k], c.pev[2 * k + 1]);
                st->kern_bytes[cat] += c.pbytes[k];
                st->kern_launches[cat] += 1;
            }
        }
    }
    return 0;
}

int pbsm3d_get_state(pbsm3d_ctx* h, double* sum_drift, double* sum_subl, double* drift_mass, double* more) {
    if (!h) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    int rc;
    if ((rc = copy_out(c, sum_drift, c.S.sum_drift, 0)) || (rc = copy_out(c, sum_subl, c.S.sum_subl, 0)) ||
        (rc = copy_out(c, drift_mass, c.S.drift_mass, 0)) || (rc = copy_out(c, more, c.S.more, 0)))
        return rc;
    PBSM_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return 0;
}

int pbsm3d_set_state(pbsm3d_ctx* h, const double* sum_drift, const double* sum_subl, const double* drift_mass,
                     const double* more) {
    if (!h) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    int rc;
    if ((sum_drift && (rc = copy_in(c, c.S.sum_drift, sum_drift, 0))) ||
        (sum_subl && (rc = copy_in(c, c.S.sum_subl, sum_subl, 0))) ||
        (drift_mass && (rc = copy_in(c, c.S.drift_mass, drift_mass, 0))) ||
        (more && (rc = copy_in(c, c.S.more, more, 0))))
        return rc;
    PBSM_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return 0;
}

int pbsm3d_set_snow(pbsm3d_ctx* h, const double* swe, const double* depth, double drift_density, int on_device) {
    if (!h || !swe || !depth || !(drift_density > 0) || !std::isfinite(drift_density)) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    int rc;
    if ((rc = copy_in(c, c.Fo.swe, swe, on_device)) || (rc = copy_in(c, c.Fo.sd, depth, on_device))) return rc;
    PBSM_CUDA_TRY(cudaStreamSynchronize(c.stream));
    c.snow_state = true;
    c.drift_density = drift_density;
    return 0;
}

int pbsm3d_get_snow(pbsm3d_ctx* h, double* swe, double* depth, int on_device) {
    if (!h) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    int rc;
    if ((rc = copy_out(c, swe, c.Fo.swe, on_device)) || (rc = copy_out(c, depth, c.Fo.sd, on_device))) return rc;
    PBSM_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return 0;
}

// Diagnostics of the last step by the reference's debug_output names
// (PBSM3D.cpp:141-186): per face "hs", "ustar", "u*_th", "csalt", "z0",
// "is_drifting"; per layer z "c<z>", "csubl<z>", "u_z<z>", "cz<z>".
int pbsm3d_get_debug(pbsm3d_ctx* h, const char* name, double* out, int on_device) {
    if (!h || !name || !out) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    c.err.clear();
    const int64_t T = c.P.T, Tp = c.P.Tp;
    const std::string n(name);
    auto face_row = [&](int fv) { return copy_out(c, out, c.A.face_v + (size_t)fv * Tp, on_device); };
    auto layer_of = [&](const char* prefix, int& z) -> bool {
        const size_t lp = strlen(prefix);
        if (n.size() <= lp || n.compare(0, lp, prefix) != 0) return false;
        const std::string rest = n.substr(lp);
        if (rest.find_first_not_of("0123456789") != std::string::npos || rest.size() > 3) return false;
        z = std::stoi(rest);
        return z >= 0 && z < c.P.L;
    };
    // host-computed rows (copied to the device when asked for there)
    auto put_host = [&](const std::vector<double>& v) -> int {
        PBSM_CUDA_TRY(cudaMemcpy(out, v.data(), T * 8, on_device ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost));
        return 0;
    };
    int rc = 0, z = 0;
    if (n == "hs")
        rc = face_row(FV_HS);
    else if (n == "ustar")
        rc = face_row(FV_USTAR);
    else if (n == "u*_th")
        rc = face_row(FV_UTH);
    else if (n == "csalt")
        rc = face_row(FV_CSALT);
    else if (n == "z0" && c.P.z0_ustar_coupling)
        rc = face_row(FV_Z0);  // written for every face by the saltation pass with the coupling
    else if (n == "z0") {
        std::vector<double> z0v(T);
        for (int m = 0; m < (int)c.member_offsets.size() - 1; ++m)
            for (int64_t i = c.member_offsets[m]; i < c.member_offsets[m + 1]; ++i) z0v[i] = c.member_z0[m];
        rc = put_host(z0v);
    } else if (n == "is_drifting") {
        std::vector<uint8_t> salt(T);
        PBSM_CUDA_TRY(cudaStreamSynchronize(c.stream));
        PBSM_CUDA_TRY(cudaMemcpy(salt.data(), c.S.saltation, T, cudaMemcpyDeviceToHost));
        std::vector<double> v(T);
        for (int64_t i = 0; i < T; ++i) v[i] = salt[i] ? 1.0 : 0.0;
        rc = put_host(v);
    } else if (layer_of("csubl", z))
        rc = copy_out(c, out, c.A.csubl + (size_t)z * Tp, on_device);
    else if (layer_of("u_z", z))
        rc = copy_out(c, out, c.A.u_z + (size_t)z * Tp, on_device);
    else if (layer_of("cz", z)) {
        std::vector<double> hs(T), v(T);
        PBSM_CUDA_TRY(cudaStreamSynchronize(c.stream));
        PBSM_CUDA_TRY(cudaMemcpy(hs.data(), c.A.face_v + (size_t)FV_HS * Tp, T * 8, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < T; ++i) v[i] = z * c.P.dz + hs[i] + c.P.dz / 2.;  // PBSM3D.cpp:941
        rc = put_host(v);
    } else if (layer_of("c", z))
        rc = copy_out(c, out, c.A.x + (size_t)z * Tp, on_device);
    else {
        c.err = "unknown diagnostic " + n;
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (rc) return rc;
    PBSM_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return 0;
}

// staging buffers of the stand-alone wind calls, allocated on first use
static int wind_staging(Ctx& c) {
    if (c.wnd.in0) return 0;
    bool ok = true;
    c.wnd.in0 = dalloc<double>(c, c.P.Tp, ok);
    c.wnd.in1 = dalloc<double>(c, c.P.Tp, ok);
    c.wnd.out = dalloc<double>(c, c.P.Tp, ok);
    if (!ok) {
        c.err = "out of device memory for the wind staging buffers";
        return PBSM3D_ERR_OUT_OF_MEMORY;
    }
    return 0;
}

int pbsm3d_scale_wind_vert(pbsm3d_ctx* h, const double* U_R, const double* snowdepthavg, double* U_2m_above_srf,
                           int on_device) {
    if (!h || !U_R || !U_2m_above_srf) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    c.err.clear();
    int rc;
    if ((rc = wind_staging(c))) return rc;
    if ((rc = copy_in(c, c.wnd.in0, U_R, on_device))) return rc;
    if (snowdepthavg && (rc = copy_in(c, c.wnd.in1, snowdepthavg, on_device))) return rc;
    launch_scale_wind_vert(c, c.stream, c.wnd.in0, snowdepthavg ? c.wnd.in1 : nullptr, c.wnd.out);
    PBSM_CUDA_TRY(cudaGetLastError());
    if ((rc = copy_out(c, U_2m_above_srf, c.wnd.out, on_device))) return rc;
    PBSM_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return 0;
}

int pbsm3d_fetchr(pbsm3d_ctx* h, const double* vw_dir, double* fetch, int on_device) {
    if (!h || !vw_dir || !fetch) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    c.err.clear();
    int rc;
    if ((rc = wind_staging(c))) return rc;
    if ((rc = copy_in(c, c.wnd.in0, vw_dir, on_device))) return rc;
    launch_fetchr(c, c.stream, c.wnd.in0, c.wnd.out);
    PBSM_CUDA_TRY(cudaGetLastError());
    if ((rc = copy_out(c, fetch, c.wnd.out, on_device))) return rc;
    PBSM_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return 0;
}

int pbsm3d_set_stations(pbsm3d_ctx* h, int64_t ns, const double* x, const double* y, int32_t n_nearest,
                        double radius, int32_t interp) {
    if (!h || ns < 1 || !x || !y || n_nearest < 0 || !(radius >= 0) || interp < PBSM3D_INTERP_SPLINE ||
        interp > PBSM3D_INTERP_NEAREST)
        return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    c.err.clear();
    if (n_nearest > 0 && radius > 0) {
        c.err = "Cannot have both station_search_radius and station_N_nearest set.";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (n_nearest == 0 && radius == 0) n_nearest = interp == PBSM3D_INTERP_NEAREST ? 1 : 5;  // core.cpp:183-196
    if (n_nearest > 0 && n_nearest < 2 && interp != PBSM3D_INTERP_NEAREST) {
        c.err = "station_N_nearest must be >= 2 if spline or idw is used";
        return PBSM3D_ERR_INVALID_ARG;
    }
    if (n_nearest > 16) {
        c.err = "at most 16 stations per face";
        return PBSM3D_ERR_INVALID_ARG;
    }
    const int64_t T = c.P.T;
    std::vector<double> cx(T), cy(T);
    PBSM_CUDA_TRY(cudaMemcpy(cx.data(), c.wnd.cx, T * 8, cudaMemcpyDeviceToHost));
    PBSM_CUDA_TRY(cudaMemcpy(cy.data(), c.wnd.cy, T * 8, cudaMemcpyDeviceToHost));
    std::vector<int32_t> start(T + 1, 0), idx;
    idx.reserve(T * (size_t)std::max(1, n_nearest));
    std::vector<std::pair<double, int32_t>> d(ns);
    for (int64_t i = 0; i < T; ++i) {
        for (int64_t k = 0; k < ns; ++k) {
            const double dx = x[k] - cx[i], dy = y[k] - cy[i];
            d[k] = {dx * dx + dy * dy, (int32_t)k};
        }
        int n = 0;
        if (n_nearest > 0) {
            const int64_t take = std::min<int64_t>(n_nearest, ns);
            std::partial_sort(d.begin(), d.begin() + take, d.end());
            for (int64_t k = 0; k < take; ++k) idx.push_back(d[k].second);
            n = (int)take;
        } else {
            for (int64_t k = 0; k < ns; ++k)
                if (d[k].first <= radius * radius) {
                    idx.push_back((int32_t)k);
                    ++n;
                }
        }
        if (n == 0 || n > 16 || (interp == PBSM3D_INTERP_NEAREST && n != 1)) {
            c.err = "face " + std::to_string(i) + " has " + std::to_string(n) +
                    " stations (NEAREST needs exactly 1, the others 1 to 16)";
            return PBSM3D_ERR_INVALID_ARG;
        }
        start[i + 1] = (int32_t)idx.size();
    }
    // replace any earlier station set
    Stations& st = c.st;
    auto drop = [&](void* p) {
        if (!p) return;
        cudaFree(p);
        c.allocations.erase(std::remove(c.allocations.begin(), c.allocations.end(), p), c.allocations.end());
    };
    for (void* p : {(void*)st.x, (void*)st.y, (void*)st.start, (void*)st.idx, (void*)st.u, (void*)st.dir,
                    (void*)st.out_u, (void*)st.out_dir, (void*)st.bad})
        drop(p);
    st = Stations{};
    bool ok = true;
    st.n = ns;
    st.interp = interp;
    st.x = dalloc<double>(c, ns, ok);
    st.y = dalloc<double>(c, ns, ok);
    st.start = dalloc<int32_t>(c, T + 1, ok);
    st.idx = dalloc<int32_t>(c, idx.size(), ok);
    st.u = dalloc<double>(c, ns, ok);
    st.dir = dalloc<double>(c, ns, ok);
    st.out_u = dalloc<double>(c, c.P.Tp, ok);
    st.out_dir = dalloc<double>(c, c.P.Tp, ok);
    st.bad = dalloc<int>(c, 1, ok);
    if (!ok) {
        c.err = "out of device memory for the stations";
        return PBSM3D_ERR_OUT_OF_MEMORY;
    }
    PBSM_CUDA_TRY(cudaMemcpy(st.x, x, ns * 8, cudaMemcpyHostToDevice));
    PBSM_CUDA_TRY(cudaMemcpy(st.y, y, ns * 8, cudaMemcpyHostToDevice));
    PBSM_CUDA_TRY(cudaMemcpy(st.start, start.data(), (T + 1) * 4, cudaMemcpyHostToDevice));
    PBSM_CUDA_TRY(cudaMemcpy(st.idx, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice));
    return 0;
}

int pbsm3d_uniform_wind(pbsm3d_ctx* h, const double* st_U, const double* st_dir, double* U_R, double* vw_dir,
                        int on_device) {
    if (!h || !st_U || !st_dir || !U_R || !vw_dir) return PBSM3D_ERR_INVALID_ARG;
    Ctx& c = h->c;
    c.err.clear();
    Stations& st = c.st;
    if (!st.x) {
        c.err = "no stations (pbsm3d_set_stations)";
        return PBSM3D_ERR_INVALID_ARG;
    }
    const cudaMemcpyKind in = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    PBSM_CUDA_TRY(cudaMemcpyAsync(st.u, st_U, st.n * 8, in, c.stream));
    PBSM_CUDA_TRY(cudaMemcpyAsync(st.dir, st_dir, st.n * 8, in, c.stream));
    PBSM_CUDA_TRY(cudaMemsetAsync(st.bad, 0, sizeof(int), c.stream));
    launch_uniform_wind(c, c.stream, st.out_u, st.out_dir);
    PBSM_CUDA_TRY(cudaGetLastError());
    int bad = 0, rc;
    PBSM_CUDA_TRY(cudaMemcpyAsync(&bad, st.bad, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    PBSM_CUDA_TRY(cudaStreamSynchronize(c.stream));
    if (bad) {
        c.err = "uniform_wind: a face has no station with a valid U_R and vw_dir";
        return PBSM3D_ERR_NAN_INPUT;
    }
    if ((rc = copy_out(c, U_R, st.out_u, on_device)) || (rc = copy_out(c, vw_dir, st.out_dir, on_device))) return rc;
    PBSM_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return 0;
}

static int export_system(Ctx& c, int which, int32_t* cols, double* vals, double* rhs, double* x) {
    const int64_t T = c.P.T, Tp = c.P.Tp;
    const int L = which == 0 ? c.P.L : 1;
    const int64_t R = which == 0 ? c.P.R : Tp;
    std::vector<int32_t> nb(3 * Tp);
    PBSM_CUDA_TRY(cudaMemcpy(nb.data(), c.F.nbr, 3 * Tp * 4, cudaMemcpyDeviceToHost));
    std::vector<double> band, b(R), xv(R);
    if (which == 0) {
        band.resize(6 * R);
        PBSM_CUDA_TRY(cudaMemcpy(band.data(), c.A.band, 6 * R * 8, cudaMemcpyDeviceToHost));
        PBSM_CUDA_TRY(cudaMemcpy(b.data(), c.A.rhs, R * 8, cudaMemcpyDeviceToHost));
        PBSM_CUDA_TRY(cudaMemcpy(xv.data(), c.A.x, R * 8, cudaMemcpyDeviceToHost));
    } else {
        band.assign(6 * R, 0.0);
        PBSM_CUDA_TRY(cudaMemcpy(band.data(), c.D.diag, Tp * 8, cudaMemcpyDeviceToHost));
        PBSM_CUDA_TRY(cudaMemcpy(band.data() + R, c.D.off, 3 * Tp * 8, cudaMemcpyDeviceToHost));
        PBSM_CUDA_TRY(cudaMemcpy(b.data(), c.D.rhs, R * 8, cudaMemcpyDeviceToHost));
        PBSM_CUDA_TRY(cudaMemcpy(xv.data(), c.D.x, R * 8, cudaMemcpyDeviceToHost));
    }
    for (int z = 0; z < L; ++z)
        for (int64_t i = 0; i < T; ++i) {
            const int64_t rr = z * T + i;   // reference row
            const int64_t rd = z * Tp + i;  // device row
            int k = 0;
            auto put = [&](int64_t col, double v) {
                if (cols) cols[6 * rr + k] = (int32_t)col;
                if (vals) vals[6 * rr + k] = v;
                ++k;
            };
            put(rr, band[rd]);
            for (int j = 0; j < 3; ++j) {
                const int32_t n = nb[j * Tp + i];
                if (n >= 0) put(z * T + n, band[(1 + j) * R + rd]);
            }
            if (z > 0) put(rr - T, band[4 * R + rd]);
            if (z < L - 1) put(rr + T, band[5 * R + rd]);
            while (k < 6) {
                if (cols) cols[6 * rr + k] = -1;
                if (vals) vals[6 * rr + k] = 0.0;
                ++k;
            }
            if (rhs) rhs[rr] = b[rd];
            if (x) x[rr] = xv[rd];
        }
    return 0;
}

int pbsm3d_export_suspension(pbsm3d_ctx* h, int32_t* cols, double* vals, double* rhs, double* x) {
    if (!h) return PBSM3D_ERR_INVALID_ARG;
    cudaStreamSynchronize(h->c.stream);
    return export_system(h->c, 0, cols, vals, rhs, x);
}

int pbsm3d_export_deposition(pbsm3d_ctx* h, int32_t* cols, double* vals, double* rhs, double* x) {
    if (!h) return PBSM3D_ERR_INVALID_ARG;
    cudaStreamSynchronize(h->c.stream);
    return export_system(h->c, 1, cols, vals, rhs, x);
}

}  // extern "C"
