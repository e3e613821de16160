"""Non-default configuration branches of PBSM3D: the CUDA step through the C
ABI against the oracle's exact solve.

z0_ustar_coupling (PBSM3D.cpp:691-737) and iterative_subl
(PBSM3D.cpp:1062-1100) alone, together, and over steps with the snow state
fed back, on a mesh whose vegetation ranges from buried to just above the
snow (so the coupling's lambda is non-zero); and every other switch of the
module's config block on that mesh.  Bars as in the default-branch parity
tests: fields within relative 1e-6, Qsalt to rounding, the erosion flags
bit-exact."""
import numpy as np
import pytest

from chm_gb300 import capi, synth
from chm_gb300.pbsm3d import PBSM3D

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-6
FIELDS = ("c", "Qsalt", "Qsusp", "Qsubl", "Qsubl_mass", "drift_mass", "sum_drift", "sum_subl",
          "blowingsnow_probability")
L = 6


def relerr(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def veg_workload(seed, wind=10.0):
    w = synth.Workload(1536, 3000.0, seed=seed, wind_scale=wind)
    n = w.mesh.n_faces
    rng = np.random.default_rng(seed + 1000)
    # canopy from 0.3 m below to 0.25 m above the snow surface (cutoff 0.3 m)
    w.mesh.canopy_height = np.maximum(0.0, w.depth + rng.uniform(-0.3, 0.25, n))
    w.mesh.lai = rng.uniform(0.5, 3.0, n)
    # subgrid TPI statistics, a tenth of each undefined (-9999)
    w.mesh.tpi_mean = rng.uniform(-3.0, 3.0, n)
    w.mesh.tpi_std = 10 ** rng.uniform(-1.0, 0.5, n)
    w.mesh.tpi_neg_frac = rng.uniform(0.0, 0.8, n)
    w.mesh.tpi_neg_mean = rng.uniform(-3.0, -0.02, n)
    w.mesh.tpi_neg_std = 10 ** rng.uniform(-1.2, 0.4, n)
    for k in ("tpi_mean", "tpi_std", "tpi_neg_frac", "tpi_neg_mean", "tpi_neg_std"):
        getattr(w.mesh, k)[rng.random(n) < 0.1] = -9999.0
    return w


def forcing(w, step, seed=0):
    f = w.forcing(step).arrays()
    rng = np.random.default_rng([seed, step])
    f["fetch"] = rng.uniform(50.0, 1500.0, w.mesh.n_faces)
    f["p_snow_hours"] = rng.uniform(1.0, 48.0, w.mesh.n_faces)
    return f


def module_cfg(cfg):
    return {"nLayer": str(L), **{k: ("true" if v is True else "false" if v is False else str(v))
                                 for k, v in cfg.items()}}


def oracle_cfg(cfg):
    return {k: (int(v) if isinstance(v, bool) else float(v)) for k, v in cfg.items()}


def check(out, ref, tag):
    for k in FIELDS:
        assert relerr(out[k], ref[k]) < FIELD_TOL, (tag, k, relerr(out[k], ref[k]))
    assert relerr(out["Qsalt"], ref["Qsalt"]) < 1e-12, tag
    np.testing.assert_array_equal(out["pbsm_more_than_avail"], ref["pbsm_more_than_avail"])
    # subgrid diagnostics: quadrature, special functions and root to ~1e-13
    for k in capi.SUBGRID_OUTPUTS:
        if k in out:
            assert relerr(out[k], ref[k]) < 1e-10, (tag, k, relerr(out[k], ref[k]))


BRANCHES = {
    "z0_ustar_coupling": {"z0_ustar_coupling": True},
    "iterative_subl": {"iterative_subl": True},
    "both": {"z0_ustar_coupling": True, "iterative_subl": True},
    "coupling_pomeroy_lambda": {"z0_ustar_coupling": True, "use_R94_lambda": False},
    "exp_fetch": {"use_exp_fetch": True, "use_tanh_fetch": False},
    "no_fetch": {"use_tanh_fetch": False},
    "pomli_probability": {"use_PomLi_probability": True, "use_tanh_fetch": False},
    "rouault": {"rouault_diffusion_coef": True},
    "no_lateral_diff": {"do_lateral_diff": False},
    "no_sublimation": {"do_sublimation": False},
    "fixed_settling": {"do_fixed_settling": True, "settling_velocity": 0.3},
    "pomeroy_lambda": {"use_R94_lambda": False},
    "no_veg": {"enable_veg": False},
    "thresholds": {"cutoff": 0.15, "min_sd_trans": 0.3, "snow_diffusion_const": 0.5, "smooth_coeff": 2000.0},
    "subgrid_topo": {"use_subgrid_topo": True},
    "subgrid_topo_V2": {"use_subgrid_topo_V2": True},
    "subgrid_both": {"use_subgrid_topo": True, "use_subgrid_topo_V2": True, "min_sd_trans": 0.25},
    "everything": {"use_subgrid_topo": True, "use_subgrid_topo_V2": True, "z0_ustar_coupling": True,
                   "iterative_subl": True, "use_PomLi_probability": True, "use_tanh_fetch": False},
}


@pytest.mark.parametrize("name", list(BRANCHES))
def test_branch_matches_oracle(cuda_lib, oracle_lib, name):
    from oracle import pyoracle
    cfg = BRANCHES[name]
    w = veg_workload(71)
    f = forcing(w, 0)
    m = PBSM3D(module_cfg(cfg))
    m.init(w.mesh)
    out = m.run(f, 3600.0, want_c=True)
    assert m.last_stats["susp_rel_residual"] <= 1e-8
    ref, _ = pyoracle.Oracle(w.mesh, nLayer=L, cfg=oracle_cfg(cfg)).step_exact(f, 3600.0)
    check(out, ref, name)
    m.close()


def test_subgrid_outputs_and_effect(cuda_lib):
    """With the subgrid branches the module provides their variables, the
    contributing fraction lies in [0, 1] and scales the saltation flux."""
    w = veg_workload(74)
    f = forcing(w, 0)
    res = {}
    for name, cfg in (("off", {}), ("on", {"use_subgrid_topo": True, "use_subgrid_topo_V2": True})):
        m = PBSM3D(module_cfg(cfg))
        m.init(w.mesh)
        res[name] = m.run(f, 3600.0)
        keys = m.output_keys()
        m.close()
    assert set(capi.SUBGRID_OUTPUTS) <= set(keys)
    on = res["on"]
    assert ((on["frac_contrib"] >= 0) & (on["frac_contrib"] <= 1)).all()
    assert (on["Qsalt"] <= res["off"]["Qsalt"] + 1e-15).all()
    assert relerr(on["Qsalt"], res["off"]["Qsalt"]) > 1e-3
    # faces without TPI_std keep tpi_lim at -min_sd_trans and test_int at -9999
    undefined = np.asarray(w.mesh.tpi_std) == -9999.0
    assert (on["tpi_lim"][undefined] == -0.1).all() and (on["test_int"][undefined] == -9999.0).all()


def test_subgrid_ensemble(cuda_lib, oracle_lib):
    """Members' TPI parameters travel with their meshes into the batched context."""
    from oracle import pyoracle
    from chm_gb300.ensemble import Ensemble, MemberParams
    cfg = {"use_subgrid_topo": True, "use_subgrid_topo_V2": True}
    ws = [veg_workload(75), veg_workload(76, wind=12.0)]
    members = [MemberParams(1.0, 0.01, 1.0), MemberParams(0.9, 0.005, 1.1)]
    ens = Ensemble(module_cfg(cfg))
    ens.init([w.mesh for w in ws], members)
    fs = [forcing(w, 0) for w in ws]
    outs = ens.run_members(fs, 3600.0, want_c=True)
    for m, (w, p, f) in enumerate(zip(ws, members, fs)):
        ocfg = {**oracle_cfg(cfg), "ustar_th_scale": p.ustar_th_scale, "z0_snow": p.z0_snow,
                "settling_scale": p.settling_scale}
        ref, _ = pyoracle.Oracle(w.mesh, nLayer=L, cfg=ocfg).step_exact(f, 3600.0)
        for k in ("c", "Qsalt", "Qsusp", "Qsubl", "drift_mass"):
            assert relerr(outs[m][k], ref[k]) < FIELD_TOL, (m, k)
    ens.close()


def test_coupling_changes_the_answer(cuda_lib):
    """The coupled branch is taken: with vegetation in the snow, u* and z0
    from Li and Pomeroy eqns 4-5 move the saltation flux off the default's."""
    w = veg_workload(72)
    f = forcing(w, 0)
    res = []
    for cfg in ({}, {"z0_ustar_coupling": True}):
        m = PBSM3D(module_cfg(cfg))
        m.init(w.mesh)
        res.append(m.run(f, 3600.0, want_c=True))
        m.close()
    assert relerr(res[1]["Qsalt"], res[0]["Qsalt"]) > 1e-3
    assert relerr(res[1]["c"], res[0]["c"]) > 1e-3


@pytest.mark.parametrize("solver", [{}, {"precision": capi.MIXED, "warm_start": capi.X0_PREVIOUS, "graph": 1}],
                         ids=["host", "graph_mixed"])
def test_branches_over_steps(cuda_lib, oracle_lib, solver):
    """Both branches on, three hourly steps with drift_mass fed back into the
    snow state and the module's sums carried."""
    from oracle import pyoracle
    cfg = {"z0_ustar_coupling": True, "iterative_subl": True}
    wg, wo = veg_workload(73), veg_workload(73)
    m = PBSM3D(module_cfg(cfg))
    m.init(wg.mesh, **solver)
    o = pyoracle.Oracle(wo.mesh, nLayer=L, cfg=oracle_cfg(cfg))
    for s in range(3):
        fg, fo = forcing(wg, s), forcing(wo, s)
        out = m.run(fg, 3600.0, want_c=True)
        ref, _ = o.step_exact(fo, 3600.0)
        check(out, ref, s)
        # both fed the oracle's drift, so that the inputs stay identical
        wg.apply_drift(ref["drift_mass"])
        wo.apply_drift(ref["drift_mass"])
    m.close()


@pytest.mark.parametrize("cfg", [{}, {"z0_ustar_coupling": True}], ids=["default", "coupling"])
def test_debug_diagnostics(cuda_lib, oracle_lib, cfg):
    """debug_output's variables kept by the library (pbsm3d_get_debug)
    against the oracle's per-face and per-layer values of the same step."""
    from oracle import pyoracle
    w = veg_workload(77)
    f = forcing(w, 0)
    m = PBSM3D(module_cfg({**cfg, "debug_output": True}))
    m.init(w.mesh)
    assert "hs" in m.provides and f"c{L - 1}" in m.provides
    out = m.run(f, 3600.0, want_c=True)
    o = pyoracle.Oracle(w.mesh, nLayer=L, cfg=oracle_cfg(cfg))
    ref, _ = o.step_exact(f, 3600.0)
    ff = o.face_fields()
    n = w.mesh.n_faces
    for name, key in (("hs", "hs"), ("ustar", "ustar"), ("u*_th", "ustar_th"), ("csalt", "c_salt"), ("z0", "z0")):
        assert relerr(m.debug(name), ff[key]) < 1e-12, name
    np.testing.assert_array_equal(m.debug("is_drifting"), ff["saltation"])
    dz = 5.0 / L
    for z in (0, L - 1):
        assert relerr(m.debug(f"c{z}"), out["c"][z * n:(z + 1) * n]) == 0.0
        assert relerr(m.debug(f"c{z}"), ref["c"][z * n:(z + 1) * n]) < FIELD_TOL
        assert relerr(m.debug(f"u_z{z}"), ff["u_z"][z * n:(z + 1) * n]) < 1e-12
        assert relerr(m.debug(f"csubl{z}"), ff["csubl"][z * n:(z + 1) * n]) < 1e-12
        assert relerr(m.debug(f"cz{z}"), z * dz + ff["hs"] + dz / 2.0) < 1e-14
    from chm_gb300.pbsm3d import ModuleError
    with pytest.raises(ModuleError, match="unknown diagnostic"):
        m.debug(f"c{L}")
    m.close()


def test_everything_in_one_graph_ensemble(cuda_lib, oracle_lib):
    """A two-member ensemble with every switch on: one CUDA-graph launch per
    step, FP32-inner/FP64-refined order-5 polynomial-preconditioned solve,
    previous-step start, the coupled u* and iterative sublimation, both
    subgrid branches, the PomLi probability, the exp fetch, U_2m and fetch
    derived on the device, and the snow state kept there.  Each member
    against the oracle given that member's constants and the oracle's wind
    modules' outputs, over two steps."""
    from oracle import pyoracle
    from chm_gb300.ensemble import Ensemble, MemberParams
    keys = {"z0_ustar_coupling": True, "iterative_subl": True, "use_subgrid_topo": True, "use_subgrid_topo_V2": True,
            "use_PomLi_probability": True, "use_tanh_fetch": False, "use_exp_fetch": True}
    ws = [veg_workload(81), veg_workload(82, wind=12.0)]
    members = [MemberParams(1.05, 0.01, 1.0), MemberParams(0.9, 0.003, 1.1)]
    ens = Ensemble(module_cfg(keys))
    ens.init([w.mesh for w in ws], members, precision=capi.MIXED, warm_start=capi.X0_PREVIOUS, graph=1, neumann=5,
             derive_wind=1, derive_fetch=1)
    ens.set_snow(np.concatenate([w.swe for w in ws]), np.concatenate([w.depth for w in ws]))
    orcs = [pyoracle.Oracle(w.mesh, nLayer=L, cfg={**oracle_cfg(keys), "ustar_th_scale": p.ustar_th_scale,
                                                  "z0_snow": p.z0_snow, "settling_scale": p.settling_scale})
            for w, p in zip(ws, members)]
    off = ens.offsets
    for s in range(2):
        fs = [forcing(w, s) for w in ws]
        fg = ens.concat_forcing(fs)
        for k in ("U_2m_above_srf", "fetch", "swe", "snowdepthavg"):
            fg.pop(k)
        out = ens.run(fg, 3600.0, want_c=True)
        assert ens.last_stats["susp_rel_residual"] <= 1e-8
        for m, (o, f, w) in enumerate(zip(orcs, fs, ws)):
            fo = dict(f)
            fo["U_2m_above_srf"] = o.scale_wind_vert(fo["U_R"], fo["snowdepthavg"])
            fo["fetch"] = o.fetchr(fo["vw_dir"])
            ref, _ = o.step_exact(fo, 3600.0)
            n = w.mesh.n_faces
            for k in ("Qsalt", "Qsusp", "Qsubl", "drift_mass", "frac_contrib", "hold_topo"):
                assert relerr(out[k][off[m]:off[m + 1]], ref[k]) < FIELD_TOL, (s, m, k)
            c = out["c"].reshape(L, -1)[:, off[m]:off[m + 1]].ravel()
            assert relerr(c, ref["c"]) < FIELD_TOL, (s, m, "c")
            w.apply_drift(ref["drift_mass"])
        ens.set_snow(np.concatenate([w.swe for w in ws]), np.concatenate([w.depth for w in ws]))
    ens.close()
