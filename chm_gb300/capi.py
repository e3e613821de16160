"""ctypes view of include/pbsm3d.h (libpbsm3d_cuda).

``load()`` returns the in-tree library and raises if it has not been built:
there is no CPU fallback for the step.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libpbsm3d_cuda.so"

ABI_VERSION = 3
OK, ERR_INVALID_ARG, ERR_BAD_MESH, ERR_NAN_INPUT, ERR_NOT_CONVERGED, ERR_CUDA, ERR_UNSUPPORTED, ERR_OOM = (
    0, -1, -2, -3, -4, -5, -6, -7)
STATUS_NAMES = {0: "OK", -1: "INVALID_ARG", -2: "BAD_MESH", -3: "NAN_INPUT", -4: "NOT_CONVERGED", -5: "CUDA",
                -6: "UNSUPPORTED", -7: "OUT_OF_MEMORY"}
SOLVER_BICGSTAB, SOLVER_GMRES = 0, 1
FP64, MIXED = 0, 1
INTERP_SPLINE, INTERP_IDW, INTERP_NEAREST = 0, 1, 2
X0_ZERO, X0_PREVIOUS, X0_LEARNED = 0, 1, 2
KERNELS = ["ASSEMBLE", "BICG_P", "BICG_V", "BICG_S", "BICG_T", "BICG_X", "RESIDUAL", "POST", "DEP_ASSEMBLE", "CG",
           "UPDATE", "OTHER", "MLP", "NEUMANN"]

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)


class Config(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("nLayer", C.c_int32), ("do_fixed_settling", C.c_int32),
        ("do_sublimation", C.c_int32), ("do_lateral_diff", C.c_int32), ("rouault_diffusion_coef", C.c_int32),
        ("enable_veg", C.c_int32), ("iterative_subl", C.c_int32), ("use_exp_fetch", C.c_int32),
        ("use_tanh_fetch", C.c_int32), ("use_PomLi_probability", C.c_int32), ("z0_ustar_coupling", C.c_int32),
        ("use_subgrid_topo", C.c_int32), ("use_subgrid_topo_V2", C.c_int32), ("use_R94_lambda", C.c_int32),
        ("debug_output", C.c_int32),
        ("settling_velocity", C.c_double), ("smooth_coeff", C.c_double), ("min_sd_trans", C.c_double),
        ("cutoff", C.c_double), ("snow_diffusion_const", C.c_double),
        ("ustar_th_scale", C.c_double), ("z0_snow", C.c_double), ("settling_scale", C.c_double),
        ("solver", C.c_int32), ("precision", C.c_int32), ("warm_start", C.c_int32), ("gmres_restart", C.c_int32),
        ("susp_maxit", C.c_int32), ("dep_maxit", C.c_int32),
        ("susp_tol", C.c_double), ("dep_tol", C.c_double), ("inner_tol", C.c_double),
        ("warm_flags", C.c_int32), ("graph", C.c_int32),
        ("autotune", C.c_int32), ("neumann", C.c_int32), ("derive_wind", C.c_int32),
        ("wind_ignore_canopy", C.c_int32), ("derive_fetch", C.c_int32), ("fetch_steps", C.c_int32),
        ("fetch_incl_veg", C.c_int32), ("dep_neumann", C.c_int32),
        ("reserved", C.c_int32 * 2), ("fetch_max_distance", C.c_double),
        ("fetch_I", C.c_double),
    ]


TPI_FIELDS = ("tpi_mean", "tpi_std", "tpi_neg_frac", "tpi_neg_mean", "tpi_neg_std")
SUBGRID_OUTPUTS = ("frac_contrib", "frac_contrib_nosnw", "hold_topo", "tpi_lim", "test_int")


class MeshError(RuntimeError):
    """A mesh file the native reader refused."""


class MeshDesc(C.Structure):
    _fields_ = [
        ("n_faces", C.c_int64), ("neighbor", _i32p), ("edge_length", _dp), ("edge_normal", _dp), ("area", _dp),
        ("center", _dp), ("has_vegetation", _u8p), ("canopy_height", _dp), ("lai", _dp), ("stalk_number", _dp),
        ("stalk_diameter", _dp), ("is_water", _u8p), ("tpi_mean", _dp), ("tpi_std", _dp), ("tpi_neg_frac", _dp),
        ("tpi_neg_mean", _dp), ("tpi_neg_std", _dp),
    ]


class Member(C.Structure):
    _fields_ = [("ustar_th_scale", C.c_double), ("z0_snow", C.c_double), ("settling_scale", C.c_double)]


class ForcingDesc(C.Structure):
    _fields_ = [(n, _dp) for n in ("U_R", "U_2m_above_srf", "vw_dir", "swe", "t", "rh", "snowdepthavg", "fetch",
                                   "p_snow_hours")] + [("on_device", C.c_int32)]


class Outputs(C.Structure):
    _fields_ = [(n, _dp) for n in ("Qsalt", "Qsusp", "Qsubl", "Qsubl_mass", "sum_subl", "drift_mass", "sum_drift",
                                   "pbsm_more_than_avail", "blowingsnow_probability", "c", "frac_contrib",
                                   "frac_contrib_nosnw", "hold_topo", "tpi_lim", "test_int")] + [
                   ("on_device", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [
        ("suspension_present", C.c_int32), ("deposition_present", C.c_int32), ("susp_iters", C.c_int32),
        ("susp_matvecs", C.c_int32), ("susp_refinements", C.c_int32), ("dep_iters", C.c_int32),
        ("susp_rel_residual", C.c_double), ("dep_rel_residual", C.c_double), ("susp_rhs_max", C.c_double),
        ("dep_rhs_max", C.c_double), ("ms_coefficients", C.c_double), ("ms_susp_solve", C.c_double),
        ("ms_post", C.c_double), ("ms_dep_assembly", C.c_double), ("ms_dep_solve", C.c_double),
        ("ms_update", C.c_double), ("ms_total", C.c_double), ("ledger_divergence", C.c_double),
        ("ledger_deposited", C.c_double), ("ledger_clipped", C.c_double), ("ledger_snow_mass", C.c_double),
        ("ledger_residual", C.c_double), ("bytes_moved", C.c_int64), ("gpu_launches", C.c_int32),
        ("profiled", C.c_int32), ("kern_ms", C.c_double * 16), ("kern_bytes", C.c_int64 * 16),
        ("kern_launches", C.c_int32 * 16), ("dep_refinements", C.c_int32), ("n_slow_faces", C.c_int32),
    ]

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            if isinstance(v, C.Array):
                v = list(v)
            d[name] = v
        return d


EXPORTS = [
    "pbsm3d_config_defaults", "pbsm3d_create", "pbsm3d_step", "pbsm3d_get_state", "pbsm3d_set_state",
    "pbsm3d_export_suspension", "pbsm3d_export_deposition", "pbsm3d_set_mlp", "pbsm3d_set_profiling",
    "pbsm3d_timer_mark", "pbsm3d_timer_elapsed", "pbsm3d_last_error", "pbsm3d_destroy",
    "pbsm3d_deposition_solve_noalloc", "pbsm3d_mlp_num_params", "pbsm3d_mlp_features", "pbsm3d_mlp_trainer_create",
    "pbsm3d_mlp_train", "pbsm3d_mlp_grad", "pbsm3d_mlp_get_params", "pbsm3d_mlp_trainer_destroy",
    "pbsm3d_mlp_gemm_bf16", "pbsm3d_mlp_predict", "pbsm3d_ensemble_create", "pbsm3d_member_offsets",
    "pbsm3d_set_snow", "pbsm3d_get_snow", "pbsm3d_scale_wind_vert", "pbsm3d_fetchr", "pbsm3d_mesh_read",
    "pbsm3d_mesh_describe", "pbsm3d_mesh_arrays", "pbsm3d_mesh_free", "pbsm3d_mesh_last_error", "pbsm3d_get_debug",
    "pbsm3d_set_stations", "pbsm3d_uniform_wind", "pbsm3d_math_eval", "pbsm3d_fp64_rate",
    "pbsm3d_arm_wait_timeout_test", "pbsm3d_set_column_geometry", "pbsm3d_get_column_geometry",
]

_lib = None


def load(path: Path | None = None):
    """Load libpbsm3d_cuda.so (built by chm_gb300.build) and declare its signatures."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with chm_gb300.build.build_cuda() (no CPU fallback exists)")
    lib = C.CDLL(str(p))
    vp = C.c_void_p
    lib.pbsm3d_config_defaults.argtypes = [C.POINTER(Config)]
    lib.pbsm3d_config_defaults.restype = None
    lib.pbsm3d_create.argtypes = [C.POINTER(MeshDesc), C.POINTER(Config), C.POINTER(vp)]
    lib.pbsm3d_create.restype = C.c_int
    lib.pbsm3d_ensemble_create.argtypes = [C.c_int32, C.POINTER(MeshDesc), C.POINTER(Member), C.POINTER(Config),
                                           C.POINTER(vp)]
    lib.pbsm3d_ensemble_create.restype = C.c_int
    lib.pbsm3d_member_offsets.argtypes = [vp, C.POINTER(C.c_int64)]
    lib.pbsm3d_member_offsets.restype = C.c_int
    dp = C.POINTER(C.c_double)
    lib.pbsm3d_set_snow.argtypes = [vp, dp, dp, C.c_double, C.c_int]
    lib.pbsm3d_set_snow.restype = C.c_int
    lib.pbsm3d_get_snow.argtypes = [vp, dp, dp, C.c_int]
    lib.pbsm3d_get_snow.restype = C.c_int
    lib.pbsm3d_scale_wind_vert.argtypes = [vp, dp, dp, dp, C.c_int]
    lib.pbsm3d_scale_wind_vert.restype = C.c_int
    lib.pbsm3d_fetchr.argtypes = [vp, dp, dp, C.c_int]
    lib.pbsm3d_fetchr.restype = C.c_int
    lib.pbsm3d_set_stations.argtypes = [vp, C.c_int64, dp, dp, C.c_int32, C.c_double, C.c_int32]
    lib.pbsm3d_set_stations.restype = C.c_int
    lib.pbsm3d_uniform_wind.argtypes = [vp, dp, dp, dp, dp, C.c_int]
    lib.pbsm3d_uniform_wind.restype = C.c_int
    lib.pbsm3d_get_debug.argtypes = [vp, C.c_char_p, dp, C.c_int]
    lib.pbsm3d_get_debug.restype = C.c_int
    lib.pbsm3d_mesh_read.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(vp)]
    lib.pbsm3d_mesh_read.restype = C.c_int
    lib.pbsm3d_mesh_describe.argtypes = [vp, C.POINTER(MeshDesc)]
    lib.pbsm3d_mesh_describe.restype = C.c_int
    lib.pbsm3d_mesh_arrays.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(dp), C.POINTER(C.POINTER(C.c_int32))]
    lib.pbsm3d_mesh_arrays.restype = C.c_int
    lib.pbsm3d_mesh_free.argtypes = [vp]
    lib.pbsm3d_mesh_free.restype = None
    lib.pbsm3d_mesh_last_error.argtypes = []
    lib.pbsm3d_mesh_last_error.restype = C.c_char_p
    lib.pbsm3d_step.argtypes = [vp, C.POINTER(ForcingDesc), C.c_double, C.POINTER(Outputs), C.POINTER(Stats)]
    lib.pbsm3d_step.restype = C.c_int
    lib.pbsm3d_get_state.argtypes = [vp, _dp, _dp, _dp, _dp]
    lib.pbsm3d_get_state.restype = C.c_int
    lib.pbsm3d_set_state.argtypes = [vp, _dp, _dp, _dp, _dp]
    lib.pbsm3d_set_state.restype = C.c_int
    for n in ("pbsm3d_export_suspension", "pbsm3d_export_deposition"):
        getattr(lib, n).argtypes = [vp, _i32p, _dp, _dp, _dp]
        getattr(lib, n).restype = C.c_int
    lib.pbsm3d_set_mlp.argtypes = [vp, _fp, _fp, _fp]
    lib.pbsm3d_set_mlp.restype = C.c_int
    lib.pbsm3d_mlp_num_params.argtypes = []
    lib.pbsm3d_mlp_num_params.restype = C.c_int
    lib.pbsm3d_mlp_features.argtypes = [vp, vp, vp, C.c_int32]
    lib.pbsm3d_mlp_features.restype = C.c_int
    lib.pbsm3d_mlp_trainer_create.argtypes = [C.c_int32, _fp, _fp, _fp, C.POINTER(vp)]
    lib.pbsm3d_mlp_trainer_create.restype = C.c_int
    lib.pbsm3d_mlp_train.argtypes = [vp, vp, vp, C.c_int64, C.c_int32, C.c_float, C.c_uint64, _fp]
    lib.pbsm3d_mlp_train.restype = C.c_int
    lib.pbsm3d_mlp_grad.argtypes = [vp, _fp, _fp, _fp, _fp, _fp]
    lib.pbsm3d_mlp_grad.restype = C.c_int
    lib.pbsm3d_mlp_get_params.argtypes = [vp, _fp]
    lib.pbsm3d_mlp_get_params.restype = C.c_int
    lib.pbsm3d_mlp_trainer_destroy.argtypes = [vp]
    lib.pbsm3d_mlp_trainer_destroy.restype = None
    lib.pbsm3d_mlp_gemm_bf16.argtypes = [C.POINTER(C.c_uint16), C.POINTER(C.c_uint16), _fp, C.c_int32, C.c_int32,
                                         C.c_int32]
    lib.pbsm3d_mlp_gemm_bf16.restype = C.c_int
    lib.pbsm3d_mlp_predict.argtypes = [vp, _dp]
    lib.pbsm3d_mlp_predict.restype = C.c_int
    lib.pbsm3d_set_profiling.argtypes = [vp, C.c_int32]
    lib.pbsm3d_set_profiling.restype = C.c_int
    lib.pbsm3d_timer_mark.argtypes = [vp, C.c_int32]
    lib.pbsm3d_timer_mark.restype = C.c_int
    lib.pbsm3d_timer_elapsed.argtypes = [vp, C.c_int32, C.c_int32, _dp]
    lib.pbsm3d_timer_elapsed.restype = C.c_int
    lib.pbsm3d_deposition_solve_noalloc.argtypes = [C.c_int64, vp, vp, vp, vp, vp, C.c_double, C.c_int32,
                                                    C.POINTER(C.c_int32), _dp]
    lib.pbsm3d_deposition_solve_noalloc.restype = C.c_int
    lib.pbsm3d_set_column_geometry.argtypes = [vp, C.c_int32, C.c_int32]
    lib.pbsm3d_set_column_geometry.restype = C.c_int
    lib.pbsm3d_get_column_geometry.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    lib.pbsm3d_get_column_geometry.restype = C.c_int
    lib.pbsm3d_arm_wait_timeout_test.argtypes = [vp, C.c_int32, C.c_double]
    lib.pbsm3d_arm_wait_timeout_test.restype = C.c_int
    lib.pbsm3d_math_eval.argtypes = [C.c_int32, C.c_int64, vp, vp, vp]
    lib.pbsm3d_math_eval.restype = C.c_int
    lib.pbsm3d_fp64_rate.argtypes = [C.POINTER(C.c_double)]
    lib.pbsm3d_fp64_rate.restype = C.c_int
    lib.pbsm3d_last_error.argtypes = [vp]
    lib.pbsm3d_last_error.restype = C.c_char_p
    lib.pbsm3d_destroy.argtypes = [vp]
    lib.pbsm3d_destroy.restype = None
    if path is None:
        _lib = lib
    return lib


def ptr(a, ctype=C.c_double):
    """Pointer to a contiguous numpy array (None stays NULL)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def default_config(lib=None, **overrides) -> Config:
    lib = lib or load()
    cfg = Config()
    lib.pbsm3d_config_defaults(C.byref(cfg))
    for k, v in overrides.items():
        if not hasattr(cfg, k):
            raise KeyError(k)
        setattr(cfg, k, v)
    return cfg


def mesh_desc(mesh, keep: list) -> MeshDesc:
    """MeshDesc over a chm_gb300.synth.Mesh; arrays are appended to keep (lifetime)."""
    def c64(a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        return a
    nb = np.ascontiguousarray(mesh.neighbor, dtype=np.int32)
    keep.append(nb)
    d = MeshDesc()
    d.n_faces = mesh.n_faces
    d.neighbor = ptr(nb, C.c_int32)
    d.edge_length = ptr(c64(mesh.edge_length))
    d.edge_normal = ptr(c64(mesh.edge_normal))
    d.area = ptr(c64(mesh.area))
    d.center = ptr(c64(mesh.center))
    if mesh.canopy_height is not None:
        d.canopy_height = ptr(c64(mesh.canopy_height))
    if mesh.lai is not None:
        d.lai = ptr(c64(mesh.lai))
    for k in TPI_FIELDS:
        a = getattr(mesh, k, None)
        if a is not None:
            setattr(d, k, ptr(c64(a)))
    return d
