// PBSM3D_gpu.cpp -- the PBSM3D module over libpbsm3d_cuda.
//   ctor        <- PBSM3D::PBSM3D     src/modules/PBSM3D.cpp:103-219
//   init        <- PBSM3D::init       src/modules/PBSM3D.cpp:221-398
//   run         <- PBSM3D::run        src/modules/PBSM3D.cpp:400-1748
//   checkpoint  <- PBSM3D::checkpoint / load_checkpoint  :1753-1773
#include "PBSM3D_gpu.hpp"

#include <cstring>

namespace chm {

REGISTER_MODULE_CPP(PBSM3D);

static const char* kForcing[9] = {"U_R", "U_2m_above_srf", "vw_dir", "swe", "t", "rh", "snowdepthavg", "fetch",
                                  "p_snow_hours"};
static const char* kOutputs[9] = {"Qsalt",     "Qsusp",     "Qsubl",
                                  "Qsubl_mass", "sum_subl",  "drift_mass",
                                  "sum_drift", "pbsm_more_than_avail", "blowingsnow_probability"};

PBSM3D::PBSM3D(config_file c) : module_base("PBSM3D", parallel::domain, c) {
    depends("U_2m_above_srf");
    depends("vw_dir");
    depends("swe");
    depends("t");
    depends("rh");
    depends("U_R");
    provides("pbsm_more_than_avail");
    provides("global_cell_id");
    use_exp_fetch = cfg.get("use_exp_fetch", false);
    use_tanh_fetch = cfg.get("use_tanh_fetch", true);
    use_PomLi_probability = cfg.get("use_PomLi_probability", false);
    if (use_exp_fetch && use_tanh_fetch) throw module_error("PBSM3d: Cannot specify both exp_fetch and tanh_fetch");
    if (use_exp_fetch || use_tanh_fetch)
        depends("fetch");
    else
        depends("p_snow_hours");
    provides("blowingsnow_probability");
    for (const char* v : {"Qsubl", "Qsubl_mass", "sum_subl", "drift_mass", "Qsusp", "Qsalt", "sum_drift"}) provides(v);
    use_subgrid_topo = cfg.get("use_subgrid_topo", false);
    use_subgrid_topo_V2 = cfg.get("use_subgrid_topo_V2", false);
    if (use_subgrid_topo)  // PBSM3D.cpp:204-209
        for (const char* v : {"frac_contrib", "frac_contrib_nosnw", "hold_topo"}) provides(v);
    if (use_subgrid_topo_V2)  // :211-218
        for (const char* v : {"frac_contrib", "hold_topo", "test_int", "test_err", "tpi_lim"}) provides(v);
    if (cfg.get("debug_output", false)) {  // PBSM3D.cpp:141-186, the variables kept here
        for (const char* v : {"hs", "ustar", "u*_th", "csalt", "z0", "is_drifting"}) provides(v);
        for (int z = 0; z < cfg.get("nLayer", 10); ++z)
            for (const char* v : {"c", "csubl", "u_z", "cz"}) provides(v + std::to_string(z));
    }
    pbsm3d_config_defaults(&gpu_cfg);
    // this library's solver switches (not reference keys); the plain FP64
    // form without them
    pbsm3d_config& g = gpu_cfg;
    if (cfg.get("solver.mixed", false)) g.precision = PBSM3D_MIXED;
    const std::string x0 = cfg.get<std::string>("solver.warm_start", "zero");
    if (x0 == "previous")
        g.warm_start = PBSM3D_X0_PREVIOUS;
    else if (x0 != "zero")  // the learned start needs weights: the C ABI's pbsm3d_set_mlp
        throw module_error("solver.warm_start must be zero or previous, not '" + x0 + "'");
    g.graph = cfg.get("solver.graph", false) ? 1 : 0;
    g.neumann = cfg.get("solver.neumann", 0);
    if (g.neumann < 0 || g.neumann > 9) throw module_error("solver.neumann must be in [0, 9]");
    g.dep_neumann = cfg.get("solver.dep_neumann", false) ? 1 : 0;
}

PBSM3D::~PBSM3D() { pbsm3d_destroy(ctx_); }

void PBSM3D::check(int rc, const char* what) const {
    if (rc != PBSM3D_OK) throw module_error(std::string(what) + ": " + pbsm3d_last_error(ctx_));
}

void PBSM3D::init(mesh& domain) {
    pbsm3d_config& g = gpu_cfg;
    g.nLayer = cfg.get("nLayer", 10);
    g.do_fixed_settling = cfg.get("do_fixed_settling", false);
    g.settling_velocity = cfg.get("settling_velocity", 0.5);
    if (g.settling_velocity < 0) throw module_error("PBSM3D settling velocity must be positive");
    g.do_sublimation = cfg.get("do_sublimation", true);
    g.do_lateral_diff = cfg.get("do_lateral_diff", true);
    g.smooth_coeff = cfg.get("smooth_coeff", 820.0);
    g.min_sd_trans = cfg.get("min_sd_trans", 0.1);
    g.cutoff = cfg.get("cutoff", 0.3);
    g.snow_diffusion_const = cfg.get("snow_diffusion_const", 0.3);
    g.rouault_diffusion_coef = cfg.get("rouault_diffusion_coef", false);
    g.enable_veg = cfg.get("enable_veg", true);
    g.iterative_subl = cfg.get("iterative_subl", false);
    g.use_exp_fetch = use_exp_fetch;
    g.use_tanh_fetch = use_tanh_fetch;
    g.use_PomLi_probability = use_PomLi_probability;
    g.z0_ustar_coupling = cfg.get("z0_ustar_coupling", false);
    g.use_subgrid_topo = use_subgrid_topo;
    g.use_subgrid_topo_V2 = use_subgrid_topo_V2;
    g.use_R94_lambda = cfg.get("use_R94_lambda", true);
    g.debug_output = cfg.get("debug_output", false);
    mesh_store& m = *domain;
    const int64_t n = m.size_faces();
    pbsm3d_mesh_desc d{};
    d.n_faces = n;
    d.neighbor = m.neighbor.data();
    d.edge_length = m.edge_length.data();
    d.edge_normal = m.edge_unit_normal.data();
    d.area = m.area.data();
    d.center = m.center.data();
    d.canopy_height = m.canopy_height.empty() ? nullptr : m.canopy_height.data();
    d.lai = m.lai.empty() ? nullptr : m.lai.data();
    d.stalk_number = m.stalk_number.empty() ? nullptr : m.stalk_number.data();
    d.stalk_diameter = m.stalk_diameter.empty() ? nullptr : m.stalk_diameter.data();
    d.is_water = m.is_water.empty() ? nullptr : m.is_water.data();
    d.tpi_mean = m.tpi_mean.empty() ? nullptr : m.tpi_mean.data();
    d.tpi_std = m.tpi_std.empty() ? nullptr : m.tpi_std.data();
    d.tpi_neg_frac = m.tpi_neg_frac.empty() ? nullptr : m.tpi_neg_frac.data();
    d.tpi_neg_mean = m.tpi_neg_mean.empty() ? nullptr : m.tpi_neg_mean.data();
    d.tpi_neg_std = m.tpi_neg_std.empty() ? nullptr : m.tpi_neg_std.data();
    pbsm3d_destroy(ctx_);
    ctx_ = nullptr;
    check(pbsm3d_create(&d, &g, &ctx_), "PBSM3D init");
    m.var("sum_drift").assign(n, 0.0);  // PBSM3D.cpp:392
    for (auto& v : f_) v.resize(n);
}

void PBSM3D::run(mesh& domain) {
    mesh_store& m = *domain;
    const int64_t n = m.size_faces();
    // gather the depends variables of every face into SoA host buffers
    pbsm3d_forcing f{};
    const double** slots[9] = {&f.U_R, &f.U_2m_above_srf, &f.vw_dir, &f.swe, &f.t, &f.rh, &f.snowdepthavg, &f.fetch,
                               &f.p_snow_hours};
    for (int k = 0; k < 9; ++k) {
        if (k == 7 && !(use_exp_fetch || use_tanh_fetch)) continue;
        if (k == 8 && !use_PomLi_probability) continue;
        const std::string name = kForcing[k];
        if (!m.has_var(name)) {
            if (k == 6) {  // snowdepthavg is read without a depends entry; absent = CHM's -9999
                m.var(name);
            } else {
                throw module_error("PBSM3D: missing variable " + name);
            }
        }
        std::memcpy(f_[k].data(), m.var(name).data(), n * sizeof(double));
        *slots[k] = f_[k].data();
    }
    f.on_device = 0;
    // outputs go straight into the face variables (module state is in the context)
    pbsm3d_outputs o{};
    double** oslots[9] = {&o.Qsalt, &o.Qsusp, &o.Qsubl, &o.Qsubl_mass, &o.sum_subl, &o.drift_mass, &o.sum_drift,
                          &o.pbsm_more_than_avail, &o.blowingsnow_probability};
    for (int k = 0; k < 9; ++k) *oslots[k] = m.var(kOutputs[k]).data();
    if (use_subgrid_topo || use_subgrid_topo_V2) {
        o.frac_contrib = m.var("frac_contrib").data();
        o.hold_topo = m.var("hold_topo").data();
    }
    if (use_subgrid_topo) o.frac_contrib_nosnw = m.var("frac_contrib_nosnw").data();
    if (use_subgrid_topo_V2) {
        o.tpi_lim = m.var("tpi_lim").data();
        o.test_int = m.var("test_int").data();
    }
    o.on_device = 0;
    check(pbsm3d_step(ctx_, &f, (double)dt, &o, &last_stats), "PBSM3D run");
    if (gpu_cfg.debug_output) {
        // the diagnostics the library keeps, under the reference's names
        for (const char* v : {"hs", "ustar", "u*_th", "csalt", "z0", "is_drifting"})
            check(pbsm3d_get_debug(ctx_, v, m.var(v).data(), 0), "PBSM3D debug_output");
        for (int z = 0; z < gpu_cfg.nLayer; ++z)
            for (const char* v : {"c", "csubl", "u_z", "cz"}) {
                const std::string name = v + std::to_string(z);
                check(pbsm3d_get_debug(ctx_, name.c_str(), m.var(name).data(), 0), "PBSM3D debug_output");
            }
    }
}

void PBSM3D::checkpoint(mesh& domain, netcdf& chkpt) {
    const int64_t n = domain->size_faces();
    std::vector<double> sd(n);
    check(pbsm3d_get_state(ctx_, sd.data(), nullptr, nullptr, nullptr), "PBSM3D checkpoint");
    chkpt.create_variable1D("PBSM3D:sum_drift", n);
    for (int64_t i = 0; i < n; ++i) chkpt.put_var1D("PBSM3D:sum_drift", i, sd[i]);
}

void PBSM3D::load_checkpoint(mesh& domain, netcdf& chkpt) {
    const int64_t n = domain->size_faces();
    std::vector<double> sd(n);
    for (int64_t i = 0; i < n; ++i) sd[i] = chkpt.get_var1D("PBSM3D:sum_drift", i);
    check(pbsm3d_set_state(ctx_, sd.data(), nullptr, nullptr, nullptr), "PBSM3D load_checkpoint");
    domain->var("sum_drift") = sd;
}

}  // namespace chm
