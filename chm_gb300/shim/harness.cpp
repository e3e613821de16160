// harness.cpp -- drives the PBSM3D module the way CHM's core does:
// factory create -> init(mesh) -> per timestep: forcing into the face
// variables, run(mesh), outputs read back from the face variables.
//
//   pbsm3d_harness --selftest            host-side checks, no GPU
//   pbsm3d_harness <case_dir> <out_dir>  run a case written by the tests:
//       case_dir/meta.txt     "n_faces nLayer n_steps dt" then "key value" config lines
//       case_dir/<array>.bin  raw little-endian arrays (see load_case)
//       out_dir/<var>_<step>.bin for the 9 output variables
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>

#include "PBSM3D_gpu.hpp"

using namespace chm;

template <typename T>
static std::vector<T> read_bin(const std::string& path, size_t n) {
    std::vector<T> v(n);
    std::ifstream f(path, std::ios::binary);
    if (!f || !f.read(reinterpret_cast<char*>(v.data()), n * sizeof(T))) throw std::runtime_error("cannot read " + path);
    return v;
}
template <typename T>
static void write_bin(const std::string& path, const std::vector<T>& v) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(T));
}

static int selftest() {
    int fails = 0;
    auto expect = [&](bool ok, const char* what) {
        if (!ok) {
            std::cerr << "FAIL: " << what << "\n";
            ++fails;
        }
    };
    auto keys = module_factory::registered_keys();
    expect(keys.size() == 1 && keys[0] == "PBSM3D", "PBSM3D registered under its class name");
    config_file c;
    c.put("nLayer", "10");
    auto m = module_factory::create("PBSM3D", c);
    auto has = [](const std::vector<std::string>& v, const char* s) {
        for (auto& x : v)
            if (x == s) return true;
        return false;
    };
    for (const char* v : {"U_2m_above_srf", "vw_dir", "swe", "t", "rh", "U_R", "fetch"})
        expect(has(m->depends(), v), "depends");
    for (const char* v : {"Qsubl", "Qsubl_mass", "sum_subl", "drift_mass", "Qsusp", "Qsalt", "sum_drift",
                          "pbsm_more_than_avail", "blowingsnow_probability"})
        expect(has(m->provides(), v), "provides");
    expect(m->type == parallel::domain, "domain-parallel module");
    config_file bad;
    bad.put("use_exp_fetch", "true");
    bad.put("use_tanh_fetch", "true");
    bool threw = false;
    try {
        module_factory::create("PBSM3D", bad);
    } catch (module_error&) {
        threw = true;
    }
    expect(threw, "both fetch formulations rejected");
    threw = false;
    try {
        module_factory::create("NoSuchModule", c);
    } catch (module_not_found&) {
        threw = true;
    }
    expect(threw, "unknown module rejected");
    config_file ph;
    ph.put("use_tanh_fetch", "false");
    auto m2 = module_factory::create("PBSM3D", ph);
    expect(has(m2->depends(), "p_snow_hours") && !has(m2->depends(), "fetch"), "p_snow_hours dependency");
    config_file fast;
    fast.put("solver.mixed", "true");
    fast.put("solver.warm_start", "previous");
    fast.put("solver.graph", "true");
    fast.put("solver.neumann", "5");
    fast.put("solver.dep_neumann", "true");
    auto m3 = module_factory::create("PBSM3D", fast);
    const pbsm3d_config& g = dynamic_cast<PBSM3D&>(*m3).gpu_cfg;
    expect(g.precision == PBSM3D_MIXED && g.warm_start == PBSM3D_X0_PREVIOUS && g.graph == 1 && g.neumann == 5 &&
               g.dep_neumann == 1,
           "solver keys");
    const pbsm3d_config& g0 = dynamic_cast<PBSM3D&>(*m).gpu_cfg;
    expect(g0.precision == PBSM3D_FP64 && g0.warm_start == PBSM3D_X0_ZERO && g0.graph == 0 && g0.neumann == 0 &&
               g0.dep_neumann == 0,
           "plain form by default");
    for (auto kv : {std::pair<const char*, const char*>{"solver.warm_start", "learned"}, {"solver.neumann", "10"}}) {
        config_file b2;
        b2.put(kv.first, kv.second);
        threw = false;
        try {
            module_factory::create("PBSM3D", b2);
        } catch (module_error&) {
            threw = true;
        }
        expect(threw, kv.first);
    }
    std::cout << (fails ? "selftest FAILED\n" : "selftest ok\n");
    return fails ? 1 : 0;
}

int main(int argc, char** argv) {
    if (argc == 2 && std::string(argv[1]) == "--selftest") return selftest();
    if (argc != 3) {
        std::cerr << "usage: pbsm3d_harness --selftest | <case_dir> <out_dir>\n";
        return 2;
    }
    const std::string dir = argv[1], out = argv[2];
    try {
        std::ifstream meta(dir + "/meta.txt");
        int64_t n;
        int L, steps, dt;
        meta >> n >> L >> steps >> dt;
        config_file cfg;
        std::string k, v;
        while (meta >> k >> v) cfg.put(k, v);
        auto dom = std::make_shared<mesh_store>(n);
        dom->neighbor = read_bin<int32_t>(dir + "/neighbor.bin", 3 * n);
        dom->edge_length = read_bin<double>(dir + "/edge_length.bin", 3 * n);
        dom->edge_unit_normal = read_bin<double>(dir + "/edge_normal.bin", 6 * n);
        dom->area = read_bin<double>(dir + "/area.bin", n);
        dom->center = read_bin<double>(dir + "/center.bin", 3 * n);
        dom->canopy_height.assign(n, 0.0);
        dom->lai.assign(n, 0.0);
        mesh domain = dom;
        auto mod = module_factory::create("PBSM3D", cfg);
        mod->dt = dt;
        mod->init(domain);
        const char* fvars[8] = {"U_R", "U_2m_above_srf", "vw_dir", "swe", "t", "rh", "snowdepthavg", "fetch"};
        const char* ovars[9] = {"Qsalt", "Qsusp", "Qsubl", "Qsubl_mass", "sum_subl", "drift_mass", "sum_drift",
                                "pbsm_more_than_avail", "blowingsnow_probability"};
        for (int s = 0; s < steps; ++s) {
            for (const char* fv : fvars)
                domain->var(fv) = read_bin<double>(dir + "/" + fv + "_" + std::to_string(s) + ".bin", n);
            mod->run(domain);
            for (const char* ov : ovars) write_bin(out + "/" + ov + "_" + std::to_string(s) + ".bin", domain->var(ov));
            auto* p = dynamic_cast<PBSM3D*>(mod.get());
            std::cout << "step " << s << " iters " << p->last_stats.susp_iters << " residual "
                      << p->last_stats.susp_rel_residual << "\n";
        }
        netcdf chk;
        mod->checkpoint(domain, chk);
        write_bin(out + "/checkpoint_sum_drift.bin", chk.vars["PBSM3D:sum_drift"]);
    } catch (std::exception& e) {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
