"""The wind-input modules on the device against the oracle:
scale_wind_vert (U_2m_above_srf, scale_wind_vert.cpp:53-227) and fetchr
(fetch, fetchr.cpp:55-117), stand-alone, per ensemble member, and derived
inside the step (derive_wind / derive_fetch) against a step given the
oracle's inputs.

Bars: U_2m within relative 1e-12 (libm vs CUDA exp/log, and the 4x4
full-pivot solve); fetch identical (a discrete distance: both pick the
nearest face centre, lowest index on a tie); step fields within relative
1e-6 as in the parity tests."""
import numpy as np
import pytest

from chm_gb300 import capi, synth
from chm_gb300.ensemble import Ensemble, MemberParams
from chm_gb300.pbsm3d import PBSM3D

pytestmark = pytest.mark.gpu

FIELDS = ("c", "Qsalt", "Qsusp", "Qsubl", "drift_mass", "sum_drift")


def relerr(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def terrain_workload(seed, veg=True, n_points=1200, side=2500.0):
    """A seeded mesh with the benchmark's relief; vegetation from 0 to 3 m on
    part of it (some taller than the 1 m of fetchr's own-face test)."""
    w = synth.Workload(n_points, side, seed=seed)
    if veg:
        rng = np.random.default_rng(seed + 500)
        n = w.mesh.n_faces
        ch = np.where(rng.random(n) < 0.4, rng.uniform(0.0, 3.0, n), 0.0)
        w.mesh.canopy_height = ch
        w.mesh.lai = rng.uniform(0.2, 4.0, n)
    return w


@pytest.mark.parametrize("veg", [False, True])
@pytest.mark.parametrize("ignore_canopy", [0, 1])
def test_scale_wind_vert(cuda_lib, oracle_lib, veg, ignore_canopy):
    from oracle import pyoracle
    w = terrain_workload(31, veg)
    f = w.forcing(0)
    sd = f.snowdepthavg.copy()
    sd[::17] = -9999.0   # CHM's missing value reads as 0
    m = PBSM3D({"nLayer": "3"})
    m.init(w.mesh, wind_ignore_canopy=ignore_canopy)
    o = pyoracle.Oracle(w.mesh, nLayer=3)
    for depth in (sd, None):
        got = m.scale_wind_vert(f.U_R, depth)
        ref = o.scale_wind_vert(f.U_R, depth, ignore_canopy=bool(ignore_canopy))
        assert relerr(got, ref) < 1e-12, relerr(got, ref)
        assert (got >= 0.1).all()
    m.close()


@pytest.mark.parametrize("veg", [False, True])
@pytest.mark.parametrize("settings", [{}, {"fetch_steps": 25, "fetch_max_distance": 600.0, "fetch_I": 0.02},
                                      {"fetch_incl_veg": 0}], ids=["default", "fine", "no_veg"])
def test_fetchr(cuda_lib, oracle_lib, veg, settings):
    from oracle import pyoracle
    w = terrain_workload(32, veg)
    f = w.forcing(0)
    m = PBSM3D({"nLayer": "3"})
    m.init(w.mesh, **settings)
    o = pyoracle.Oracle(w.mesh, nLayer=3)
    got = m.fetchr(f.vw_dir)
    ref = o.fetchr(f.vw_dir, steps=settings.get("fetch_steps", 10),
                   max_distance=settings.get("fetch_max_distance", 1000.0), I=settings.get("fetch_I", 0.06),
                   incl_veg=bool(settings.get("fetch_incl_veg", 1)))
    np.testing.assert_array_equal(got, ref)
    assert 0 < (got < settings.get("fetch_max_distance", 1000.0)).mean() < 1
    m.close()


def test_fetchr_queries_outside_the_mesh(cuda_lib, oracle_lib):
    """Search points beyond the domain take the nearest boundary face."""
    from oracle import pyoracle
    w = terrain_workload(33, veg=False, n_points=400, side=800.0)
    n = w.mesh.n_faces
    m = PBSM3D({"nLayer": "3"})
    m.init(w.mesh, fetch_max_distance=5000.0, fetch_steps=7)
    o = pyoracle.Oracle(w.mesh, nLayer=3)
    for d in (0.0, 45.0, 137.0, 270.0, 359.0):
        dirs = np.full(n, d)
        np.testing.assert_array_equal(m.fetchr(dirs), o.fetchr(dirs, steps=7, max_distance=5000.0))
    m.close()


def test_ensemble_members_search_their_own_mesh(cuda_lib, oracle_lib):
    """fetchr in a batched context: each face's nearest-face queries stay in
    its member's mesh (the members overlap in space)."""
    from oracle import pyoracle
    ws = [terrain_workload(34, veg=True), terrain_workload(35, veg=True, n_points=800)]
    ens = Ensemble({"nLayer": "3"})
    ens.init([w.mesh for w in ws], [MemberParams(1.0, 0.01, 1.0)] * 2)
    fs = [w.forcing(0) for w in ws]
    dirs = np.concatenate([f.vw_dir for f in fs])
    got = ens.fetchr(dirs)
    u2 = ens.scale_wind_vert(np.concatenate([f.U_R for f in fs]), np.concatenate([f.snowdepthavg for f in fs]))
    off = ens.offsets
    for k, (w, f) in enumerate(zip(ws, fs)):
        o = pyoracle.Oracle(w.mesh, nLayer=3)
        np.testing.assert_array_equal(got[off[k]:off[k + 1]], o.fetchr(f.vw_dir))
        assert relerr(u2[off[k]:off[k + 1]], o.scale_wind_vert(f.U_R, f.snowdepthavg)) < 1e-12
    ens.close()


@pytest.mark.parametrize("solver", [{}, {"precision": capi.MIXED, "warm_start": capi.X0_PREVIOUS, "graph": 1,
                                         "neumann": 5}], ids=["host", "graph"])
def test_step_derives_its_wind_inputs(cuda_lib, oracle_lib, solver):
    """derive_wind / derive_fetch: the step computes U_2m_above_srf and fetch
    itself; the result matches the oracle step given the oracle's modules'
    outputs, over steps with the snow state on the device."""
    from oracle import pyoracle
    cfg = {"nLayer": "5", "use_tanh_fetch": "false", "use_exp_fetch": "true"}
    wg, wo = terrain_workload(36), terrain_workload(36)
    m = PBSM3D(cfg)
    m.init(wg.mesh, derive_wind=1, derive_fetch=1, **solver)
    m.set_snow(wg.swe, wg.depth)
    o = pyoracle.Oracle(wo.mesh, nLayer=5, cfg={"use_tanh_fetch": 0, "use_exp_fetch": 1})
    for s in range(3):
        fg = wg.forcing(s).arrays()
        for k in ("U_2m_above_srf", "fetch", "swe", "snowdepthavg"):
            fg.pop(k)
        fo = wo.forcing(s).arrays()
        fo["U_2m_above_srf"] = o.scale_wind_vert(fo["U_R"], fo["snowdepthavg"])
        fo["fetch"] = o.fetchr(fo["vw_dir"])
        assert (fo["fetch"] < 500).any()   # the exp fetch branch is exercised
        # the stand-alone modules agree on this step's inputs
        np.testing.assert_array_equal(m.fetchr(fo["vw_dir"]), fo["fetch"])
        assert relerr(m.scale_wind_vert(fo["U_R"], fo["snowdepthavg"]), fo["U_2m_above_srf"]) < 1e-12
        out = m.run(fg, 3600.0, want_c=True)
        ref, _ = o.step_exact(fo, 3600.0)
        for k in FIELDS:
            assert relerr(out[k], ref[k]) < 1e-6, (s, k, relerr(out[k], ref[k]))
        # both fed the oracle's drift (the forcing generator's U_R depends on
        # the depth); the device state applied the GPU's, so it is reset too
        wo.apply_drift(ref["drift_mass"])
        wg.apply_drift(ref["drift_mass"])
        m.set_snow(wo.swe, wo.depth)
    m.close()


def _stations(seed, n, side):
    rng = np.random.default_rng(seed)
    return rng.uniform(-0.1 * side, 1.1 * side, n), rng.uniform(-0.1 * side, 1.1 * side, n)


@pytest.mark.parametrize("interp,n_nearest,radius", [(capi.INTERP_SPLINE, 5, 0.0), (capi.INTERP_SPLINE, 2, 0.0),
                                                     (capi.INTERP_IDW, 4, 0.0), (capi.INTERP_NEAREST, 1, 0.0),
                                                     (capi.INTERP_SPLINE, 0, 0.0), (capi.INTERP_IDW, 0, 1400.0)],
                         ids=["spline5", "spline2", "idw4", "nearest", "spline_default", "idw_radius"])
def test_uniform_wind(cuda_lib, oracle_lib, interp, n_nearest, radius):
    """uniform_wind (interp_met/uniform_wind.cpp:58-127) from 12 stations, the
    station lists built as CHM's core does, against the oracle; one station
    missing its data this step (except with the nearest station alone, where
    that leaves faces without a station: an error, as in the reference)."""
    from oracle import pyoracle
    w = terrain_workload(37, veg=False)
    sx, sy = _stations(5, 12, 2500.0)
    rng = np.random.default_rng(6)
    su, sd = rng.uniform(2, 15, 12), rng.uniform(0, 360, 12)
    if interp != capi.INTERP_NEAREST:
        su[3] = -9999.0  # the faces whose only station it is would be left without one
    m = PBSM3D({"nLayer": "3"})
    m.init(w.mesh)
    o = pyoracle.Oracle(w.mesh, nLayer=3)
    m.set_stations(sx, sy, n_nearest, radius, interp)
    eff_n = n_nearest or (1 if interp == capi.INTERP_NEAREST else 5)
    U, D = m.uniform_wind(su, sd)
    Ur, Dr = o.uniform_wind(sx, sy, su, sd, eff_n if not radius else 0, radius, interp)
    assert relerr(U, Ur) < 1e-12, relerr(U, Ur)
    # bearings: compare on the circle
    dd = np.abs((D - Dr + 180.0) % 360.0 - 180.0)
    assert dd.max() < 1e-9
    assert (U >= 0.1).all() and ((D >= 0) & (D <= 360)).all()
    m.close()


def test_uniform_wind_errors(cuda_lib):
    from chm_gb300.pbsm3d import ModuleError
    w = terrain_workload(38, veg=False, n_points=300, side=800.0)
    sx, sy = _stations(7, 4, 800.0)
    m = PBSM3D({"nLayer": "3"})
    m.init(w.mesh)
    with pytest.raises(ModuleError, match="both"):
        m.set_stations(sx, sy, 3, 100.0)
    with pytest.raises(ModuleError, match=">= 2"):
        m.set_stations(sx, sy, 1, 0.0, capi.INTERP_IDW)
    with pytest.raises(ModuleError, match="exactly 1"):
        m.set_stations(sx, sy, 2, 0.0, capi.INTERP_NEAREST)
    with pytest.raises(ModuleError, match="no stations"):
        m.uniform_wind(np.ones(4), np.ones(4))
    m.set_stations(sx, sy, 2, 0.0, capi.INTERP_IDW)
    with pytest.raises(ModuleError, match="NAN_INPUT"):
        m.uniform_wind(np.full(4, np.nan), np.ones(4))
    U, D = m.uniform_wind(np.full(4, 5.0), np.full(4, 90.0))
    assert np.allclose(U, 5.0) and np.allclose(D, 90.0)
    m.close()
