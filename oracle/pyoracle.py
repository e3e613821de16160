"""ctypes bindings of the CPU oracle (oracle/liboracle_pbsm3d.so).

TEST INFRASTRUCTURE ONLY: imported by the tests, the smoke check and the
CPU-baseline leg of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
from chm_gb300 import capi  # noqa: E402  (struct definitions of the shared C ABI)

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)


class SolverCfg(C.Structure):
    _fields_ = [("restart", C.c_int32), ("maxit", C.c_int32), ("tol", C.c_double), ("ilut_drop", C.c_double),
                ("ilut_fill", C.c_double), ("nblocks", C.c_int32), ("dep_maxit", C.c_int32),
                ("dep_tol", C.c_double)]


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    from . import build_oracle  # type: ignore
    p = build_oracle.ORACLE_LIB
    if not p.exists():
        build_oracle.build_oracle()
    lib = C.CDLL(str(p))
    vp = C.c_void_p
    lib.oracle_create.argtypes = [C.POINTER(capi.MeshDesc), C.POINTER(capi.Config), C.POINTER(vp)]
    lib.oracle_destroy.argtypes = [vp]
    lib.oracle_destroy.restype = None
    lib.oracle_solver_defaults.argtypes = [C.POINTER(SolverCfg)]
    lib.oracle_solver_defaults.restype = None
    lib.oracle_set_solver.argtypes = [vp, C.POINTER(SolverCfg)]
    lib.oracle_set_threads.argtypes = [C.c_int]
    lib.oracle_set_threads.restype = C.c_int
    lib.oracle_last_error.argtypes = [vp]
    lib.oracle_last_error.restype = C.c_char_p
    lib.oracle_step.argtypes = [vp, C.POINTER(capi.ForcingDesc), C.c_double, C.POINTER(capi.Outputs),
                                C.POINTER(capi.Stats)]
    lib.oracle_stage_assemble_suspension.argtypes = [vp, C.POINTER(capi.ForcingDesc), C.c_double]
    for n in ("oracle_stage_solve_suspension", "oracle_stage_post_and_assemble_deposition",
              "oracle_stage_solve_deposition"):
        getattr(lib, n).argtypes = [vp]
    lib.oracle_stage_set_suspension_solution.argtypes = [vp, _dp]
    lib.oracle_stage_set_deposition_solution.argtypes = [vp, _dp]
    lib.oracle_stage_update.argtypes = [vp, C.POINTER(capi.Outputs), C.POINTER(capi.Stats)]
    lib.oracle_rows.argtypes = [vp, C.c_int32]
    lib.oracle_rows.restype = C.c_int64
    lib.oracle_nnz.argtypes = [vp, C.c_int32]
    lib.oracle_nnz.restype = C.c_int64
    lib.oracle_get_system.argtypes = [vp, C.c_int32, _i64p, _i32p, _dp, _dp, _dp]
    lib.oracle_get_face_fields.argtypes = [vp] + [_dp] * 8
    lib.oracle_get_state.argtypes = [vp] + [_dp] * 4
    lib.oracle_set_state.argtypes = [vp] + [_dp] * 4
    lib.oracle_log_scale_wind.argtypes = [C.c_double] * 5
    lib.oracle_log_scale_wind.restype = C.c_double
    lib.oracle_saturated_vapour_pressure.argtypes = [C.c_double]
    lib.oracle_saturated_vapour_pressure.restype = C.c_double
    lib.oracle_bearing_to_cartesian.argtypes = [C.c_double, _dp]
    lib.oracle_bearing_to_cartesian.restype = None
    lib.oracle_std_dry_air_density.argtypes = [C.c_double, C.c_double]
    lib.oracle_std_dry_air_density.restype = C.c_double
    lib.oracle_coupled_ustar.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_double)]
    lib.oracle_coupled_ustar.restype = C.c_int
    lib.oracle_ice_bulb_temperature.argtypes = [C.c_double] * 6
    lib.oracle_ice_bulb_temperature.restype = C.c_double
    lib.oracle_incomplete_gamma.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.oracle_incomplete_gamma.restype = None
    lib.oracle_gamma_pdf.argtypes = [C.c_double] * 3
    lib.oracle_gamma_pdf.restype = C.c_double
    lib.oracle_subgrid_face.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.oracle_subgrid_face.restype = None
    lib.oracle_scale_wind_vert.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                           C.POINTER(C.c_double)]
    lib.oracle_fetchr.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]
    lib.oracle_uniform_wind.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int,
                                        C.c_double, C.c_int] + [C.POINTER(C.c_double)] * 4
    lib.oracle_uniform_wind.restype = C.c_int
    lib.oracle_expint_e1.argtypes = [C.c_double]
    lib.oracle_expint_e1.restype = C.c_double
    lib.oracle_tps.argtypes = [C.POINTER(C.c_double)] * 3 + [C.c_int, C.c_double, C.c_double]
    lib.oracle_tps.restype = C.c_double
    lib.oracle_face_geometry.argtypes = [C.c_int64, _dp, C.c_int64, _i32p, _dp, _dp, _dp, _dp]
    lib.oracle_face_geometry.restype = None
    lib.oracle_face_neighbors.argtypes = [C.c_int64, C.c_int64, _i32p, _i32p]
    lib.oracle_mlp_loss_grad.argtypes = [C.c_int64, _fp, _fp] + [_fp] * 8 + [_dp] * 9
    lib.oracle_mlp_loss_grad.restype = C.c_double
    _lib = lib
    return lib


def ptr(a, t=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


class Oracle:
    """The CPU restatement of PBSM3D over one mesh (same C ABI structs)."""

    def __init__(self, mesh, nLayer=10, cfg: dict | None = None, solver: dict | None = None):
        self.lib = load()
        self.keep = []
        c = capi.Config()
        # oracle takes the same config struct; defaults identical to the library's
        _fill_defaults(c)
        c.nLayer = nLayer
        for k, v in (cfg or {}).items():
            setattr(c, k, v)
        self.cfg = c
        self.L = nLayer
        self.n = mesh.n_faces
        desc = capi.mesh_desc(mesh, self.keep)
        self.ctx = C.c_void_p()
        rc = self.lib.oracle_create(C.byref(desc), C.byref(c), C.byref(self.ctx))
        if rc != 0:
            raise RuntimeError(f"oracle_create {rc}: {self.lib.oracle_last_error(None).decode()}")
        s = SolverCfg()
        self.lib.oracle_solver_defaults(C.byref(s))
        for k, v in (solver or {}).items():
            setattr(s, k, v)
        self.lib.oracle_set_solver(self.ctx, C.byref(s))
        self.solver = s

    def set_solver(self, **kw):
        for k, v in kw.items():
            setattr(self.solver, k, v)
        self.lib.oracle_set_solver(self.ctx, C.byref(self.solver))

    def _forcing(self, forcing):
        f = capi.ForcingDesc()
        src = forcing if isinstance(forcing, dict) else forcing.arrays()
        for k, a in src.items():
            a = np.ascontiguousarray(a, dtype=np.float64)
            self.keep.append(a)
            setattr(f, k, ptr(a))
        return f

    def _outputs(self, want_c=True):
        from chm_gb300.pbsm3d import OUTPUT_KEYS
        out = {k: np.empty(self.n) for k in OUTPUT_KEYS}
        if self.cfg.use_subgrid_topo or self.cfg.use_subgrid_topo_V2:
            out.update({k: np.empty(self.n) for k in capi.SUBGRID_OUTPUTS})
        if want_c:
            out["c"] = np.empty(self.n * self.L)
        o = capi.Outputs()
        for k, a in out.items():
            setattr(o, k, ptr(a))
        return o, out

    def step(self, forcing, dt, want_c=True):
        f = self._forcing(forcing)
        o, out = self._outputs(want_c)
        st = capi.Stats()
        rc = self.lib.oracle_step(self.ctx, C.byref(f), float(dt), C.byref(o), C.byref(st))
        if rc != 0:
            raise RuntimeError(f"oracle_step {rc}: {self.lib.oracle_last_error(self.ctx).decode()}")
        self.keep.clear()
        return out, st.as_dict()

    def step_exact(self, forcing, dt, want_c=True):
        """The step with both systems solved directly (scipy SuperLU) -- the
        tight solution the GPU is compared against on small meshes."""
        import scipy.sparse as sp
        import scipy.sparse.linalg as spl
        f = self._forcing(forcing)
        lib, ctx = self.lib, self.ctx
        rc = lib.oracle_stage_assemble_suspension(ctx, C.byref(f), float(dt))
        if rc != 0:
            raise RuntimeError(lib.oracle_last_error(ctx).decode())
        A, b, _ = self.system(0)
        x = np.zeros_like(b)
        if np.abs(b).max() > 1e-12:
            x = spl.spsolve(A.tocsc(), b)
        lib.oracle_stage_set_suspension_solution(ctx, ptr(np.ascontiguousarray(x)))
        lib.oracle_stage_post_and_assemble_deposition(ctx)
        D, bd, _ = self.system(1)
        q = spl.spsolve(D.tocsc(), bd) if np.abs(bd).max() > 1e-12 else np.zeros_like(bd)
        lib.oracle_stage_set_deposition_solution(ctx, ptr(np.ascontiguousarray(q)))
        o, out = self._outputs(want_c)
        st = capi.Stats()
        lib.oracle_stage_update(ctx, C.byref(o), C.byref(st))
        self.keep.clear()
        return out, st.as_dict()

    def assemble(self, forcing, dt):
        """Stage 1 only: zero both systems, saltation, coefficients, suspension rows."""
        f = self._forcing(forcing)
        rc = self.lib.oracle_stage_assemble_suspension(self.ctx, C.byref(f), float(dt))
        if rc != 0:
            raise RuntimeError(self.lib.oracle_last_error(self.ctx).decode())

    def set_suspension_solution(self, x):
        self.lib.oracle_stage_set_suspension_solution(self.ctx, ptr(np.ascontiguousarray(x, dtype=np.float64)))

    def post_and_assemble_deposition(self):
        rc = self.lib.oracle_stage_post_and_assemble_deposition(self.ctx)
        if rc != 0:
            raise RuntimeError(self.lib.oracle_last_error(self.ctx).decode())

    def system(self, which: int):
        import scipy.sparse as sp
        rows = self.lib.oracle_rows(self.ctx, which)
        nnz = self.lib.oracle_nnz(self.ctx, which)
        rp = np.empty(rows + 1, np.int64)
        cols = np.empty(nnz, np.int32)
        vals = np.empty(nnz)
        rhs = np.empty(rows)
        x = np.empty(rows)
        self.lib.oracle_get_system(self.ctx, which, ptr(rp, C.c_int64), ptr(cols, C.c_int32), ptr(vals), ptr(rhs),
                                   ptr(x))
        return sp.csr_matrix((vals, cols, rp), shape=(rows, rows)), rhs, x

    def raw_system(self, which: int):
        rows = self.lib.oracle_rows(self.ctx, which)
        nnz = self.lib.oracle_nnz(self.ctx, which)
        rp = np.empty(rows + 1, np.int64)
        cols = np.empty(nnz, np.int32)
        vals = np.empty(nnz)
        rhs = np.empty(rows)
        x = np.empty(rows)
        self.lib.oracle_get_system(self.ctx, which, ptr(rp, C.c_int64), ptr(cols, C.c_int32), ptr(vals), ptr(rhs),
                                   ptr(x))
        return rp, cols, vals, rhs, x

    def scale_wind_vert(self, U_R, snowdepthavg=None, ignore_canopy=False):
        u = np.ascontiguousarray(U_R, dtype=np.float64)
        sd = None if snowdepthavg is None else np.ascontiguousarray(snowdepthavg, dtype=np.float64)
        out = np.empty(self.n)
        self.lib.oracle_scale_wind_vert(self.ctx, int(ignore_canopy), ptr(u), ptr(sd) if sd is not None else None,
                                        ptr(out))
        return out

    def fetchr(self, vw_dir, steps=10, max_distance=1000.0, I=0.06, incl_veg=True):
        d = np.ascontiguousarray(vw_dir, dtype=np.float64)
        out = np.empty(self.n)
        self.lib.oracle_fetchr(self.ctx, int(steps), float(max_distance), float(I), int(incl_veg), ptr(d), ptr(out))
        return out

    def uniform_wind(self, sx, sy, st_U, st_dir, n_nearest=5, radius=0.0, interp=0):
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (sx, sy, st_U, st_dir)]
        U, D = np.empty(self.n), np.empty(self.n)
        rc = self.lib.oracle_uniform_wind(self.ctx, a[0].size, ptr(a[0]), ptr(a[1]), int(n_nearest), float(radius),
                                          int(interp), ptr(a[2]), ptr(a[3]), ptr(U), ptr(D))
        if rc != 0:
            raise RuntimeError("oracle_uniform_wind: a face has no valid station")
        return U, D

    def face_fields(self):
        n, L = self.n, self.L
        d = {k: np.empty(n) for k in ("saltation", "hs", "z0", "ustar", "c_salt", "ustar_th")}
        d["u_z"] = np.empty(n * L)
        d["csubl"] = np.empty(n * L)
        self.lib.oracle_get_face_fields(self.ctx, *(ptr(d[k]) for k in ("saltation", "hs", "z0", "ustar", "c_salt",
                                                                         "ustar_th", "u_z", "csubl")))
        return d

    def state(self):
        a = {k: np.empty(self.n) for k in ("sum_drift", "sum_subl", "drift_mass", "more")}
        self.lib.oracle_get_state(self.ctx, *(ptr(a[k]) for k in ("sum_drift", "sum_subl", "drift_mass", "more")))
        return a

    def set_state(self, sum_drift=None, sum_subl=None, drift_mass=None, more=None):
        keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                for a in (sum_drift, sum_subl, drift_mass, more)]
        self.lib.oracle_set_state(self.ctx, *(ptr(a) for a in keep))

    def close(self):
        if self.ctx:
            self.lib.oracle_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _fill_defaults(c):
    """pbsm3d_config_defaults restated (the oracle must not need the GPU library)."""
    c.abi_version = capi.ABI_VERSION
    c.nLayer = 10
    c.do_fixed_settling = 0
    c.do_sublimation = 1
    c.do_lateral_diff = 1
    c.rouault_diffusion_coef = 0
    c.enable_veg = 1
    c.use_exp_fetch = 0
    c.use_tanh_fetch = 1
    c.use_PomLi_probability = 0
    c.use_R94_lambda = 1
    c.settling_velocity = 0.5
    c.smooth_coeff = 820.0
    c.min_sd_trans = 0.1
    c.cutoff = 0.3
    c.snow_diffusion_const = 0.3
    c.ustar_th_scale = 1.0
    c.z0_snow = 0.01
    c.settling_scale = 1.0
    c.gmres_restart = 30
    c.susp_maxit = 1000
    c.dep_maxit = 1000
    c.susp_tol = 1e-8
    c.dep_tol = 1e-10
    c.inner_tol = 1e-4


def ref_atmosphere():
    """The reference's own Atmosphere.cpp (oracle/_ref), or None when not built."""
    from . import build_oracle  # type: ignore
    p = build_oracle.REF_LIB
    if not p.exists():
        return None
    lib = C.CDLL(str(p))
    lib.ref_log_scale_wind.argtypes = [C.c_double] * 5
    lib.ref_log_scale_wind.restype = C.c_double
    lib.ref_saturated_vapour_pressure.argtypes = [C.c_double]
    lib.ref_saturated_vapour_pressure.restype = C.c_double
    return lib
