// PBSM3D_gpu.hpp -- CHM's PBSM3D module (src/modules/PBSM3D.hpp:306-423) on
// GB300: same registered name, config keys, defaults, depends and provides;
// the step runs in libpbsm3d_cuda through the C ABI of include/pbsm3d.h.
#pragma once

#include "../../include/pbsm3d.h"
#include "chm_module.hpp"

namespace chm {

class PBSM3D : public module_base {
    REGISTER_MODULE_HPP(PBSM3D)
   public:
    explicit PBSM3D(config_file cfg);
    ~PBSM3D() override;
    void init(mesh& domain) override;
    void run(mesh& domain) override;
    void checkpoint(mesh& domain, netcdf& chkpt) override;
    void load_checkpoint(mesh& domain, netcdf& chkpt) override;

    pbsm3d_stats last_stats{};
    // solver settings beyond the reference keys ("solver.mixed", "solver.warm_start",
    // "solver.graph", "solver.neumann", "solver.dep_neumann")
    pbsm3d_config gpu_cfg{};

   private:
    void check(int rc, const char* what) const;
    bool use_exp_fetch, use_tanh_fetch, use_PomLi_probability, use_subgrid_topo, use_subgrid_topo_V2;
    pbsm3d_ctx* ctx_ = nullptr;
    std::vector<double> f_[9], o_[9];
};

}  // namespace chm
