// chm_module.hpp -- the slice of CHM's module plugin interface that a
// process module needs, restated so the GPU PBSM3D module can be built and
// driven outside CHM.  Names and semantics follow the reference:
//   module_base             src/modules/module_base.hpp:142-540
//   factory / registration  src/factory.hpp:34-106, module_base.hpp:533-540
//   module_error            src/exception.hpp:46
//   config_file             boost::property_tree::ptree (module_base.hpp:68),
//                           here a flat key -> string map with typed get()
//   mesh / face storage     src/mesh/triangulation.hpp (per-face variables
//                           default to -9999, variablestorage.hpp:271)
// Inside CHM the module compiles against CHM's own headers instead.
#pragma once

#include <cmath>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace chm {

struct module_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct module_not_found : module_error {
    using module_error::module_error;
};

// ptree-style typed access with defaults ("true"/"false"/numbers as strings)
class config_file {
   public:
    void put(const std::string& k, const std::string& v) { kv_[k] = v; }
    bool has(const std::string& k) const { return kv_.count(k) != 0; }
    template <typename T>
    T get(const std::string& k, T def) const {
        auto it = kv_.find(k);
        if (it == kv_.end()) return def;
        return parse<T>(k, it->second);
    }

   private:
    template <typename T>
    static T parse(const std::string& k, const std::string& v);
    std::map<std::string, std::string> kv_;
};
template <>
inline bool config_file::parse<bool>(const std::string& k, const std::string& v) {
    if (v == "true" || v == "1") return true;
    if (v == "false" || v == "0") return false;
    throw module_error("config key " + k + ": cannot parse '" + v + "' as bool");
}
template <>
inline int config_file::parse<int>(const std::string&, const std::string& v) { return (int)std::stod(v); }
template <>
inline double config_file::parse<double>(const std::string&, const std::string& v) { return std::stod(v); }
template <>
inline std::string config_file::parse<std::string>(const std::string&, const std::string& v) { return v; }

// A triangle mesh with CHM's per-face variable store.
class mesh_store {
   public:
    mesh_store(int64_t n_faces) : n_(n_faces) {}
    int64_t size_faces() const { return n_; }
    int64_t size_global_faces() const { return n_; }
    // geometry and adjacency as CHM's face API returns them
    std::vector<int32_t> neighbor;        // [3n], -1 = none
    std::vector<double> edge_length;      // [3n]
    std::vector<double> edge_unit_normal; // [6n]
    std::vector<double> area;             // [n]
    std::vector<double> center;           // [3n]
    std::vector<double> canopy_height, lai, stalk_number, stalk_diameter;  // vegetation parameters or empty
    // subgrid parameters TPI_mean, TPI_std, TPI_neg_frac, TPI_neg_mean, TPI_neg_std, or empty
    std::vector<double> tpi_mean, tpi_std, tpi_neg_frac, tpi_neg_mean, tpi_neg_std;
    std::vector<uint8_t> is_water;
    // per-face variables ((*face)["name"_s]); created on first use at -9999
    std::vector<double>& var(const std::string& name) {
        auto it = vars_.find(name);
        if (it == vars_.end()) it = vars_.emplace(name, std::vector<double>(n_, -9999.0)).first;
        return it->second;
    }
    bool has_var(const std::string& name) const { return vars_.count(name) != 0; }

   private:
    int64_t n_;
    std::unordered_map<std::string, std::vector<double>> vars_;
};
using mesh = std::shared_ptr<mesh_store>;

// checkpoint file stand-in: named 1-D double variables (CHM uses NetCDF)
struct netcdf {
    std::map<std::string, std::vector<double>> vars;
    void create_variable1D(const std::string& n, size_t len) { vars[n].assign(len, 0.0); }
    void put_var1D(const std::string& n, size_t i, double v) { vars[n].at(i) = v; }
    double get_var1D(const std::string& n, size_t i) const { return vars.at(n).at(i); }
};

enum class parallel { data, domain };

class module_base {
   public:
    module_base(std::string ID, parallel type, config_file cfg) : ID(std::move(ID)), type(type), cfg(std::move(cfg)) {}
    virtual ~module_base() = default;
    virtual void init(mesh&) {}
    virtual void run(mesh&) {}
    virtual void checkpoint(mesh&, netcdf&) {}
    virtual void load_checkpoint(mesh&, netcdf&) {}
    const std::vector<std::string>& depends() const { return depends_; }
    const std::vector<std::string>& provides() const { return provides_; }
    const std::vector<std::string>& optionals() const { return optional_; }
    std::string ID;
    parallel type;
    config_file cfg;
    int dt = 3600;  // global_param->dt(), seconds

   protected:
    void depends(const std::string& v) { depends_.push_back(v); }
    void provides(const std::string& v) { provides_.push_back(v); }
    void optional(const std::string& v) { optional_.push_back(v); }

   private:
    std::vector<std::string> depends_, provides_, optional_;
};

class module_factory {
   public:
    using ctor = std::function<module_base*(config_file)>;
    static std::shared_ptr<module_base> create(const std::string& name, config_file cfg) {
        auto it = registry().find(name);
        if (it == registry().end()) throw module_not_found("Requested module not found in registry: [" + name + "]");
        return std::shared_ptr<module_base>(it->second(std::move(cfg)));
    }
    static void register_factory_function(const std::string& name, ctor c) { registry()[name] = std::move(c); }
    static std::vector<std::string> registered_keys() {
        std::vector<std::string> k;
        for (auto& e : registry()) k.push_back(e.first);
        return k;
    }

   private:
    static std::map<std::string, ctor>& registry() {
        static std::map<std::string, ctor> r;
        return r;
    }
};

template <class T>
struct registration_helper {
    explicit registration_helper(const std::string& name) {
        module_factory::register_factory_function(name, [](config_file c) -> module_base* { return new T(c); });
    }
};

}  // namespace chm

#define REGISTER_MODULE_HPP(x) static chm::registration_helper<x> registrar_;
#define REGISTER_MODULE_CPP(x) chm::registration_helper<x> x::registrar_(#x)
