"""Python host mirror of CHM's PBSM3D module over libpbsm3d_cuda.

Mirrors the reference's module interface (src/modules/module_base.hpp:142-540,
src/factory.hpp:34-106, src/modules/PBSM3D.cpp:103-398): a class registered
as "PBSM3D" in a factory, built from a config of string/bool/number values
with the reference's keys and defaults, exposing ``depends``/``provides``,
``init(mesh)``, ``run(...)`` (one timestep), ``checkpoint``/``load_checkpoint``.
Errors raise ``ModuleError`` like CHM_THROW_EXCEPTION(module_error, ...).
The step itself always runs in the CUDA library; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi


class ModuleError(RuntimeError):
    """CHM's module_error."""


class ModuleNotFound(ModuleError):
    """CHM's module_not_found (factory.hpp:72-74)."""


def _get(cfg: dict, key: str, default):
    """ptree-style typed get with default (CHM config values are often strings)."""
    if key not in cfg:
        return default
    v = cfg[key]
    if isinstance(default, bool):
        if isinstance(v, str):
            s = v.strip().lower()
            if s in ("true", "1", "yes"):
                return True
            if s in ("false", "0", "no"):
                return False
            raise ModuleError(f"config key {key}: cannot parse '{v}' as bool")
        return bool(v)
    if isinstance(default, int):
        return int(float(v)) if isinstance(v, str) else int(v)
    if isinstance(default, float):
        return float(v)
    return v


_REGISTRY: dict = {}


def register_module(name: str):
    def deco(cls):
        _REGISTRY[name] = cls
        return cls
    return deco


def create(name: str, cfg: dict | None = None):
    """factory<module_base, config_file>::create (factory.hpp:65-79)."""
    if name not in _REGISTRY:
        raise ModuleNotFound(f"Requested module not found in registry: [{name}]")
    return _REGISTRY[name](cfg or {})


def registered_keys():
    return sorted(_REGISTRY)


FORCING_KEYS = ("U_R", "U_2m_above_srf", "vw_dir", "swe", "t", "rh", "snowdepthavg", "fetch", "p_snow_hours")
OUTPUT_KEYS = ("Qsalt", "Qsusp", "Qsubl", "Qsubl_mass", "sum_subl", "drift_mass", "sum_drift",
               "pbsm_more_than_avail", "blowingsnow_probability")


@register_module("PBSM3D")
class PBSM3D:
    name = "PBSM3D"
    parallel = "domain"  # module_base("PBSM3D", parallel::domain, cfg), PBSM3D.cpp:103

    def __init__(self, cfg: dict):
        self.cfg = dict(cfg)
        g = lambda k, d: _get(self.cfg, k, d)  # noqa: E731
        self.depends = ["U_2m_above_srf", "vw_dir", "swe", "t", "rh", "U_R"]
        self.provides = ["pbsm_more_than_avail", "global_cell_id"]
        self.use_exp_fetch = g("use_exp_fetch", False)
        self.use_tanh_fetch = g("use_tanh_fetch", True)
        self.use_PomLi_probability = g("use_PomLi_probability", False)
        self.z0_ustar_coupling = g("z0_ustar_coupling", False)
        self.use_subgrid_topo = g("use_subgrid_topo", False)
        self.use_subgrid_topo_V2 = g("use_subgrid_topo_V2", False)
        if self.use_exp_fetch and self.use_tanh_fetch:
            raise ModuleError("PBSM3d: Cannot specify both exp_fetch and tanh_fetch")
        if self.use_exp_fetch or self.use_tanh_fetch:
            self.depends.append("fetch")
        else:
            self.depends.append("p_snow_hours")
        self.use_R94_lambda = g("use_R94_lambda", True)
        self.provides.append("blowingsnow_probability")
        self.debug_output = g("debug_output", False)
        if self.debug_output:  # PBSM3D.cpp:141-186, the diagnostics this library keeps (debug())
            self.provides += ["hs", "ustar", "u*_th", "csalt", "z0", "is_drifting"]
            self.provides += [f"{v}{z}" for z in range(int(g("nLayer", 10))) for v in ("c", "csubl", "u_z", "cz")]
        self.provides += ["Qsubl", "Qsubl_mass", "sum_subl", "drift_mass", "Qsusp", "Qsalt", "sum_drift"]
        if self.use_subgrid_topo:
            self.provides += ["frac_contrib", "frac_contrib_nosnw", "hold_topo"]
        if self.use_subgrid_topo_V2:
            self.provides += ["frac_contrib", "hold_topo", "test_int", "test_err", "tpi_lim"]
        self._lib = None
        self._ctx = None
        self._keep = []
        self.n_faces = 0
        self.last_stats = None

    # PBSM3D::init (PBSM3D.cpp:221-398)
    def init(self, mesh, **solver):
        lib = capi.load()
        cfg = self.make_config(lib, **solver)
        desc = capi.mesh_desc(mesh, self._keep)
        ctx = C.c_void_p()
        rc = lib.pbsm3d_create(C.byref(desc), C.byref(cfg), C.byref(ctx))
        if rc != 0:
            raise ModuleError(f"pbsm3d_create: {capi.STATUS_NAMES.get(rc, rc)}: "
                              f"{lib.pbsm3d_last_error(None).decode()}")
        self._lib = lib
        self._ctx = ctx
        self.n_faces = mesh.n_faces

    def make_config(self, lib, **solver) -> capi.Config:
        """The library's config struct from this module's keys (PBSM3D.cpp:221-280)
        plus solver fields of the struct given by name."""
        g = lambda k, d: _get(self.cfg, k, d)  # noqa: E731
        self.nLayer = g("nLayer", 10)
        settling = g("settling_velocity", 0.5)
        if settling < 0:
            raise ModuleError("PBSM3D settling velocity must be positive")
        cfg = capi.default_config(lib)
        cfg.nLayer = self.nLayer
        cfg.do_fixed_settling = int(g("do_fixed_settling", False))
        cfg.settling_velocity = float(settling)
        cfg.do_sublimation = int(g("do_sublimation", True))
        cfg.do_lateral_diff = int(g("do_lateral_diff", True))
        cfg.smooth_coeff = float(g("smooth_coeff", 820.0))
        cfg.min_sd_trans = float(g("min_sd_trans", 0.1))
        cfg.cutoff = float(g("cutoff", 0.3))
        cfg.snow_diffusion_const = float(g("snow_diffusion_const", 0.3))
        cfg.rouault_diffusion_coef = int(g("rouault_diffusion_coef", False))
        cfg.enable_veg = int(g("enable_veg", True))
        cfg.iterative_subl = int(g("iterative_subl", False))
        cfg.use_exp_fetch = int(self.use_exp_fetch)
        cfg.use_tanh_fetch = int(self.use_tanh_fetch)
        cfg.use_PomLi_probability = int(self.use_PomLi_probability)
        cfg.z0_ustar_coupling = int(self.z0_ustar_coupling)
        cfg.use_subgrid_topo = int(self.use_subgrid_topo)
        cfg.use_subgrid_topo_V2 = int(self.use_subgrid_topo_V2)
        cfg.use_R94_lambda = int(self.use_R94_lambda)
        cfg.debug_output = int(self.debug_output)
        for k, v in solver.items():
            if not hasattr(cfg, k):
                raise ModuleError(f"unknown solver setting {k}")
            setattr(cfg, k, v)
        self._cfg_struct = cfg
        return cfg

    def set_profiling(self, on: bool):
        self._lib.pbsm3d_set_profiling(self._ctx, int(on))

    def _error(self, rc, what):
        msg = self._lib.pbsm3d_last_error(self._ctx).decode()
        raise ModuleError(f"{what}: {capi.STATUS_NAMES.get(rc, rc)}: {msg}")

    # PBSM3D::run (PBSM3D.cpp:400-1748)
    def run(self, forcing, dt: float, want_c: bool = False, outputs: dict | None = None) -> dict:
        if self._ctx is None:
            raise ModuleError("PBSM3D.run before init")
        n = self.n_faces
        f = capi.ForcingDesc()
        keep = []
        src = forcing if isinstance(forcing, dict) else forcing.arrays()
        for k in FORCING_KEYS:
            a = src.get(k)
            if a is None:
                continue
            a = np.ascontiguousarray(a, dtype=np.float64)
            if a.shape != (n,):
                raise ModuleError(f"forcing {k} has shape {a.shape}, expected ({n},)")
            keep.append(a)
            setattr(f, k, capi.ptr(a))
        f.on_device = 0
        out = outputs if outputs is not None else {k: np.empty(n) for k in self.output_keys()}
        if want_c and "c" not in out:
            out["c"] = np.empty(self.nLayer * n)
        o = capi.Outputs()
        for k, a in out.items():
            setattr(o, k, capi.ptr(a))
        o.on_device = 0
        st = capi.Stats()
        rc = self._lib.pbsm3d_step(self._ctx, C.byref(f), float(dt), C.byref(o), C.byref(st))
        if rc != 0:
            self._error(rc, "pbsm3d_step")
        self.last_stats = st.as_dict()
        return out

    def scale_wind_vert(self, U_R, snowdepthavg=None) -> np.ndarray:
        """U_2m_above_srf from U_R on the device (scale_wind_vert.cpp:53-227),
        with the context's wind_ignore_canopy."""
        u = np.ascontiguousarray(U_R, dtype=np.float64)
        sd = None if snowdepthavg is None else np.ascontiguousarray(snowdepthavg, dtype=np.float64)
        out = np.empty(self.n_faces)
        rc = self._lib.pbsm3d_scale_wind_vert(self._ctx, capi.ptr(u), capi.ptr(sd) if sd is not None else None,
                                              capi.ptr(out), 0)
        if rc != 0:
            self._error(rc, "pbsm3d_scale_wind_vert")
        return out

    def fetchr(self, vw_dir) -> np.ndarray:
        """fetch from vw_dir on the device (fetchr.cpp:55-117), with the
        context's fetch_* settings."""
        d = np.ascontiguousarray(vw_dir, dtype=np.float64)
        out = np.empty(self.n_faces)
        rc = self._lib.pbsm3d_fetchr(self._ctx, capi.ptr(d), capi.ptr(out), 0)
        if rc != 0:
            self._error(rc, "pbsm3d_fetchr")
        return out

    def set_stations(self, x, y, n_nearest: int = 0, radius: float = 0.0, interp: int = capi.INTERP_SPLINE):
        """Met stations and each face's station list (core.cpp:168-205)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        rc = self._lib.pbsm3d_set_stations(self._ctx, x.size, capi.ptr(x), capi.ptr(y), int(n_nearest),
                                           float(radius), int(interp))
        if rc != 0:
            self._error(rc, "pbsm3d_set_stations")

    def uniform_wind(self, station_U_R, station_vw_dir):
        """Per-face U_R and vw_dir interpolated from one time step of the
        stations (interp_met/uniform_wind.cpp:58-127)."""
        u = np.ascontiguousarray(station_U_R, dtype=np.float64)
        d = np.ascontiguousarray(station_vw_dir, dtype=np.float64)
        U, D = np.empty(self.n_faces), np.empty(self.n_faces)
        rc = self._lib.pbsm3d_uniform_wind(self._ctx, capi.ptr(u), capi.ptr(d), capi.ptr(U), capi.ptr(D), 0)
        if rc != 0:
            self._error(rc, "pbsm3d_uniform_wind")
        return U, D

    def debug(self, name: str) -> np.ndarray:
        """A diagnostic of the last step by its debug_output name ("hs",
        "ustar", "u*_th", "csalt", "z0", "is_drifting", "c<z>", "csubl<z>",
        "u_z<z>", "cz<z>")."""
        out = np.empty(self.n_faces)
        rc = self._lib.pbsm3d_get_debug(self._ctx, name.encode(), capi.ptr(out), 0)
        if rc != 0:
            self._error(rc, "pbsm3d_get_debug")
        return out

    def output_keys(self) -> tuple:
        """The per-face outputs a step writes: the provides list of
        PBSM3D.cpp:188-218 that carries values (test_err is provided but never
        written by the reference)."""
        keys = list(OUTPUT_KEYS)
        if self.use_subgrid_topo:
            keys += ["frac_contrib", "frac_contrib_nosnw", "hold_topo"]
        if self.use_subgrid_topo_V2:
            keys += [k for k in ("frac_contrib", "hold_topo", "tpi_lim", "test_int") if k not in keys]
        return tuple(keys)

    def set_snow(self, swe, depth, drift_density: float = 300.0):
        """Keep swe and snow depth on the device: later run() calls without
        swe/snowdepthavg read them from the context, and each step applies
        its drift_mass to them (include/pbsm3d.h, pbsm3d_set_snow)."""
        swe = np.ascontiguousarray(swe, dtype=np.float64)
        depth = np.ascontiguousarray(depth, dtype=np.float64)
        if swe.shape != (self.n_faces,) or depth.shape != (self.n_faces,):
            raise ModuleError("set_snow: swe and depth need one value per face")
        rc = self._lib.pbsm3d_set_snow(self._ctx, capi.ptr(swe), capi.ptr(depth), float(drift_density), 0)
        if rc != 0:
            self._error(rc, "pbsm3d_set_snow")

    def get_snow(self):
        swe = np.empty(self.n_faces)
        depth = np.empty(self.n_faces)
        rc = self._lib.pbsm3d_get_snow(self._ctx, capi.ptr(swe), capi.ptr(depth), 0)
        if rc != 0:
            self._error(rc, "pbsm3d_get_snow")
        return swe, depth

    def export_system(self, which: str):
        n, L = self.n_faces, self.nLayer
        rows = n * L if which == "suspension" else n
        cols = np.empty(rows * 6, np.int32)
        vals = np.empty(rows * 6)
        rhs = np.empty(rows)
        x = np.empty(rows)
        fn = self._lib.pbsm3d_export_suspension if which == "suspension" else self._lib.pbsm3d_export_deposition
        rc = fn(self._ctx, capi.ptr(cols, C.c_int32), capi.ptr(vals), capi.ptr(rhs), capi.ptr(x))
        if rc != 0:
            self._error(rc, "export")
        return cols.reshape(rows, 6), vals.reshape(rows, 6), rhs, x

    # PBSM3D::checkpoint / load_checkpoint (PBSM3D.cpp:1753-1773)
    def checkpoint(self) -> dict:
        sd = np.empty(self.n_faces)
        self._lib.pbsm3d_get_state(self._ctx, capi.ptr(sd), None, None, None)
        return {"PBSM3D:sum_drift": sd}

    def load_checkpoint(self, chk: dict):
        sd = np.ascontiguousarray(chk["PBSM3D:sum_drift"], dtype=np.float64)
        rc = self._lib.pbsm3d_set_state(self._ctx, capi.ptr(sd), None, None, None)
        if rc != 0:
            self._error(rc, "load_checkpoint")

    def state(self) -> dict:
        a = {k: np.empty(self.n_faces) for k in ("sum_drift", "sum_subl", "drift_mass", "more")}
        self._lib.pbsm3d_get_state(self._ctx, capi.ptr(a["sum_drift"]), capi.ptr(a["sum_subl"]),
                                   capi.ptr(a["drift_mass"]), capi.ptr(a["more"]))
        return a

    def close(self):
        if self._ctx is not None and self._lib is not None:
            self._lib.pbsm3d_destroy(self._ctx)
        self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
