// ref_atmosphere_shim.cpp -- C entry points over the reference's own
// src/physics/Atmosphere.cpp, compiled from the reference source tree by
// oracle/build_oracle.py into oracle/_ref/libref_atmosphere.so.
// TEST INFRASTRUCTURE ONLY: used to pin the oracle's restatement of
// Atmosphere::log_scale_wind and Atmosphere::saturatedVapourPressure.
namespace Atmosphere {
double log_scale_wind(double u, double Z_in, double Z_out, double snowdepthavg, double z0);
double saturatedVapourPressure(const double& T);
}  // namespace Atmosphere

extern "C" double ref_log_scale_wind(double u, double z_in, double z_out, double sd, double z0) {
    return Atmosphere::log_scale_wind(u, z_in, z_out, sd, z0);
}
extern "C" double ref_saturated_vapour_pressure(double T) { return Atmosphere::saturatedVapourPressure(T); }
