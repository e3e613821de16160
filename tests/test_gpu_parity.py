"""Parity of the CUDA step (through the C ABI) with the CPU oracle.

Bars: mesh adjacency/indexing of the assembled systems bit-exact; matrix and
RHS entries within 1e-12 of the row scale; fields (c, Qsusp, Qsalt, Qsubl,
drift_mass, sum_drift) within relative 1e-6 (max-norm, relative to the
field's max) of the oracle's exact solve; mass ledger closed to 1e-10 of the
domain snow mass.
"""
import numpy as np
import pytest

from chm_gb300 import synth
from chm_gb300.pbsm3d import PBSM3D, ModuleError

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-6
FIELDS = ("c", "Qsalt", "Qsusp", "Qsubl", "Qsubl_mass", "drift_mass", "sum_drift", "sum_subl")


def relerr(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def gpu_module(mesh, nLayer, cfg=None, **solver):
    m = PBSM3D({"nLayer": str(nLayer), **(cfg or {})})
    m.init(mesh, **solver)
    return m


def oracle(mesh, nLayer, cfg=None):
    from oracle import pyoracle
    return pyoracle.Oracle(mesh, nLayer=nLayer, cfg=cfg)


@pytest.fixture(scope="module")
def small():
    return synth.Workload(2048, 3500.0, seed=3)


def _compare_system(o, which, gcols, gvals, grhs, name):
    rp, cols, vals, rhs, _ = o.raw_system(which)
    rows = rhs.size
    assert gcols.shape[0] == rows
    for r in range(rows):
        oc = cols[rp[r]:rp[r + 1]]
        ov = vals[rp[r]:rp[r + 1]]
        n = oc.size
        # identical graph: same columns in the same slot order
        np.testing.assert_array_equal(gcols[r, :n], oc)
        assert (gcols[r, n:] == -1).all()
        scale = max(np.abs(ov).max(), 1e-300)
        assert np.abs(gvals[r, :n] - ov).max() <= 1e-12 * scale, (name, r, gvals[r, :n], ov)
    rscale = max(np.abs(rhs).max(), 1e-300)
    assert np.abs(grhs - rhs).max() <= 1e-12 * rscale, name


def test_assembled_systems_match_oracle(cuda_lib, oracle_lib, small):
    """Both systems entry by entry.  The deposition RHS depends on the
    suspension solution, so the oracle is given the GPU's solution first."""
    L = 5
    f = small.forcing(0)
    m = gpu_module(small.mesh, L)
    m.run(f, 3600.0)
    o = oracle(small.mesh, L)
    o.assemble(f, 3600.0)
    gcols, gvals, grhs, gx = m.export_system("suspension")
    _compare_system(o, 0, gcols, gvals, grhs, "suspension")
    o.set_suspension_solution(gx)
    o.post_and_assemble_deposition()
    gcols, gvals, grhs, _ = m.export_system("deposition")
    _compare_system(o, 1, gcols, gvals, grhs, "deposition")
    m.close()


@pytest.mark.parametrize("neumann", [0, 5])
def test_step_matches_exact_oracle(cuda_lib, oracle_lib, small, neumann):
    L = 5
    f = small.forcing(0)
    m = gpu_module(small.mesh, L, neumann=neumann)
    out = m.run(f, 3600.0, want_c=True)
    st = m.last_stats
    assert st["suspension_present"] == 1 and st["deposition_present"] == 1
    assert st["susp_rel_residual"] <= 1e-8
    ref, _ = oracle(small.mesh, L).step_exact(f, 3600.0)
    for k in FIELDS:
        assert relerr(out[k], ref[k]) < FIELD_TOL, (k, relerr(out[k], ref[k]))
    # Qsalt has no solve in it: agreement to rounding
    assert relerr(out["Qsalt"], ref["Qsalt"]) < 1e-12
    np.testing.assert_array_equal(out["pbsm_more_than_avail"], ref["pbsm_more_than_avail"])
    m.close()


def test_golden_oracle_fixture(cuda_lib):
    from conftest import GOLDEN
    d = np.load(GOLDEN / "oracle_small.npz")
    w = synth.Workload(int(d["n_points"]), float(d["side"]), seed=int(d["seed"]))
    f = {k[3:]: d[k] for k in d.files if k.startswith("in_")}
    m = gpu_module(w.mesh, int(d["nLayer"]))
    out = m.run(f, 3600.0, want_c=True)
    for k in FIELDS:
        assert relerr(out[k], d["out_" + k]) < FIELD_TOL, k
    m.close()


def test_multi_step_snow_loop(cuda_lib, oracle_lib):
    """Three hourly steps with the snow state fed back (drift_mass -> swe,
    depth) and the module state (sum_drift, sum_subl) carried, GPU vs oracle."""
    L = 5
    wg = synth.Workload(1536, 3000.0, seed=5)
    wo = synth.Workload(1536, 3000.0, seed=5)
    m = gpu_module(wg.mesh, L)
    o = oracle(wo.mesh, L)
    for s in range(3):
        fg, fo = wg.forcing(s), wo.forcing(s)
        np.testing.assert_array_equal(fg.swe, fo.swe)
        out = m.run(fg, 3600.0, want_c=True)
        ref, _ = o.step_exact(fo, 3600.0)
        for k in FIELDS:
            assert relerr(out[k], ref[k]) < FIELD_TOL, (s, k, relerr(out[k], ref[k]))
        # feed both with the oracle's drift so the inputs stay identical
        wg.apply_drift(ref["drift_mass"])
        wo.apply_drift(ref["drift_mass"])
    m.close()


def test_mass_ledger_closes(cuda_lib, small):
    L = 5
    m = gpu_module(small.mesh, L)
    m.run(small.forcing(0), 3600.0)
    st = m.last_stats
    snow = st["ledger_snow_mass"]
    assert snow > 0
    assert abs(st["ledger_deposited"] - st["ledger_divergence"]) <= 1e-10 * snow
    assert abs(st["ledger_residual"]) <= 1e-10 * snow
    m.close()


@pytest.mark.parametrize("neumann", [0, 1, 2, 3, 5, 9])
def test_mixed_precision_matches(cuda_lib, oracle_lib, small, neumann):
    L = 5
    f = small.forcing(0)
    m = gpu_module(small.mesh, L, precision=1, neumann=neumann)
    out = m.run(f, 3600.0, want_c=True)
    st = m.last_stats
    assert st["susp_rel_residual"] <= 1e-8
    assert st["susp_refinements"] >= 1
    ref, _ = oracle(small.mesh, L).step_exact(f, 3600.0)
    for k in FIELDS:
        assert relerr(out[k], ref[k]) < FIELD_TOL, (k, relerr(out[k], ref[k]))
    m.close()


@pytest.mark.parametrize("solver", [{}, {"precision": 1}, {"graph": 1}, {"precision": 1, "graph": 1}],
                         ids=["fp64", "mixed", "fp64_graph", "mixed_graph"])
def test_polynomial_deposition_preconditioner(cuda_lib, oracle_lib, solver):
    """dep_neumann = 1 (the order-1 Neumann preconditioner of the deposition
    CG, in the cooperative kernel and in the tile kernels of graph mode) gives
    the exact oracle's fields over coupled steps, closes the mass ledger, and
    needs fewer CG iterations than Jacobi on the same systems."""
    L = 5
    wg, wj, wo = (synth.Workload(1536, 3000.0, seed=5) for _ in range(3))
    m = gpu_module(wg.mesh, L, dep_neumann=1, **solver)
    mj = gpu_module(wj.mesh, L, **solver)
    o = oracle(wo.mesh, L)
    for s in range(3):
        out = m.run(wg.forcing(s), 3600.0, want_c=True)
        st = m.last_stats
        mj.run(wj.forcing(s), 3600.0)
        sj = mj.last_stats
        assert st["deposition_present"] == 1
        assert st["dep_rel_residual"] <= 1e-10
        assert st["dep_iters"] <= 0.75 * sj["dep_iters"], (st["dep_iters"], sj["dep_iters"])
        snow = st["ledger_snow_mass"]
        assert abs(st["ledger_residual"]) <= 1e-10 * snow
        ref, _ = o.step_exact(wo.forcing(s), 3600.0)
        for k in FIELDS:
            assert relerr(out[k], ref[k]) < FIELD_TOL, (s, k, relerr(out[k], ref[k]))
        for w in (wg, wj, wo):
            w.apply_drift(ref["drift_mass"])
    m.close()
    mj.close()


@pytest.mark.parametrize("wind", [4.0, 14.0])
@pytest.mark.parametrize("neumann", [0, 5])
def test_wind_regimes(cuda_lib, oracle_lib, wind, neumann):
    L = 5
    w = synth.Workload(1024, 2500.0, seed=9, wind_scale=wind)
    f = w.forcing(0)
    m = gpu_module(w.mesh, L, neumann=neumann)
    out = m.run(f, 3600.0, want_c=True)
    ref, _ = oracle(w.mesh, L).step_exact(f, 3600.0)
    for k in FIELDS:
        assert relerr(out[k], ref[k]) < FIELD_TOL, (k, relerr(out[k], ref[k]))
    m.close()


def test_reference_mesh_slope(cuda_lib, oracle_lib):
    """CHM's functional-test mesh with its PBSM3D config block
    (functional_tests/mesh_versioning/json_mesh.json:82-99)."""
    from conftest import load_golden_mesh
    mesh, _ = load_golden_mesh("slope_mesh.npz")
    cfg = {"nLayer": "10", "smooth_coeff": "6500", "do_fixed_settling": "true", "settling_velocity": "0.5",
           "use_R94_lambda": "false", "enable_veg": "true"}
    n = mesh.n_faces
    rng = np.random.default_rng(2)
    f = {"U_R": rng.uniform(8, 20, n), "U_2m_above_srf": rng.uniform(5, 12, n),
         "vw_dir": np.full(n, 250.0) + rng.normal(0, 10, n), "swe": rng.uniform(20, 200, n),
         "t": rng.uniform(-15, -2, n), "rh": rng.uniform(60, 95, n), "snowdepthavg": rng.uniform(0.2, 1.0, n),
         "fetch": np.full(n, 1000.0)}
    m = PBSM3D(cfg)
    m.init(mesh)
    out = m.run(f, 3600.0, want_c=True)
    ocfg = {"smooth_coeff": 6500.0, "do_fixed_settling": 1, "use_R94_lambda": 0}
    ref, _ = oracle(mesh, 10, ocfg).step_exact(f, 3600.0)
    for k in FIELDS:
        assert relerr(out[k], ref[k]) < FIELD_TOL, (k, relerr(out[k], ref[k]))
    m.close()


def test_deterministic(cuda_lib, small):
    f = small.forcing(0)
    outs = []
    for _ in range(2):
        m = gpu_module(small.mesh, 5)
        outs.append(m.run(f, 3600.0, want_c=True))
        m.close()
    for k in outs[0]:
        np.testing.assert_array_equal(outs[0][k], outs[1][k])


def test_no_suspension_keeps_drift_mass(cuda_lib):
    """Calm air: no solve, and drift_mass keeps its previous value (-9999 at
    start, PBSM3D.cpp:1742-1745)."""
    w = synth.Workload(512, 1500.0, seed=4, wind_scale=0.3)
    m = gpu_module(w.mesh, 5)
    out = m.run(w.forcing(0), 3600.0)
    st = m.last_stats
    assert st["suspension_present"] == 0 and st["deposition_present"] == 0
    assert (out["drift_mass"] == -9999.0).all()
    assert (out["Qsusp"] == 0).all()
    m.close()


def test_checkpoint_roundtrip(cuda_lib, small):
    m = gpu_module(small.mesh, 5)
    m.run(small.forcing(0), 3600.0)
    chk = m.checkpoint()
    assert np.abs(chk["PBSM3D:sum_drift"]).max() > 0
    m2 = gpu_module(small.mesh, 5)
    m2.load_checkpoint(chk)
    np.testing.assert_array_equal(m2.checkpoint()["PBSM3D:sum_drift"], chk["PBSM3D:sum_drift"])
    a = m.run(small.forcing(1), 3600.0)
    b = m2.run(small.forcing(1), 3600.0)
    np.testing.assert_array_equal(a["sum_drift"], b["sum_drift"])
    m.close()
    m2.close()


def test_nan_temperature_is_an_error(cuda_lib, oracle_lib):
    """A NaN air temperature reaches the matrix (rho, D, lambda_t); the
    reference's Belos solve would throw, here the step returns NAN_INPUT."""
    w = synth.Workload(512, 1500.0, seed=4)
    f = w.forcing(0).arrays()
    f["t"] = f["t"].copy()
    f["t"][10] = np.nan
    m = gpu_module(w.mesh, 5)
    with pytest.raises(ModuleError, match="NAN_INPUT"):
        m.run(f, 3600.0)
    m.close()
    with pytest.raises(RuntimeError):
        oracle(w.mesh, 5).step(f, 3600.0)


def test_nan_wind_is_clamped_like_the_reference(cuda_lib, oracle_lib):
    """NaN U_R is absorbed by std::max(0.01, .) in u* and u_z
    (PBSM3D.cpp:752, 976-981): the step succeeds and matches the oracle."""
    w = synth.Workload(512, 1500.0, seed=4)
    f = w.forcing(0).arrays()
    f["U_R"] = f["U_R"].copy()
    f["U_R"][10] = np.nan
    m = gpu_module(w.mesh, 5)
    out = m.run(f, 3600.0, want_c=True)
    ref, _ = oracle(w.mesh, 5).step_exact(f, 3600.0)
    for k in FIELDS:
        assert relerr(out[k], ref[k]) < FIELD_TOL, k
    m.close()


def test_maxit_cap_reports_not_converged(cuda_lib, small):
    m = gpu_module(small.mesh, 5, susp_maxit=1)
    with pytest.raises(ModuleError, match="NOT_CONVERGED"):
        m.run(small.forcing(0), 3600.0)
    m.close()


def test_full_size_properties(cuda_lib):
    """1M faces x 10 layers: FP64 residual recomputed on the host from the
    exported system, the mass ledger, non-negative clamped concentrations."""
    import scipy.sparse as sp
    cfg = synth.CONFIGS["tri1m"]
    w = synth.Workload(cfg["n_points"], cfg["side"], seed=1)
    m = gpu_module(w.mesh, 10)
    out = m.run(w.forcing(0), 3600.0, want_c=True)
    st = m.last_stats
    assert st["susp_rel_residual"] <= 1e-8
    cols, vals, rhs, x = m.export_system("suspension")
    rows = rhs.size
    mask = cols >= 0
    ri = np.repeat(np.arange(rows), 6).reshape(rows, 6)
    A = sp.csr_matrix((vals[mask], (ri[mask], cols[mask])), shape=(rows, rows))
    res = np.linalg.norm(rhs - A @ x) / np.linalg.norm(rhs)
    assert res <= 1.5e-8, res
    assert abs(st["ledger_deposited"] - st["ledger_divergence"]) <= 1e-10 * st["ledger_snow_mass"]
    assert (out["Qsusp"] >= 0).all()
    m.close()


def test_device_snow_state(cuda_lib, oracle_lib):
    """The drift consumer on the device: swe and depth stay in the context
    between steps and take each step's drift_mass exactly as the host rule
    (chm_gb300.synth.consume_drift) does; the physics matches the oracle fed
    the same snow state."""
    L = 5
    w = synth.Workload(1536, 3000.0, seed=5)
    m = gpu_module(w.mesh, L)
    o = oracle(w.mesh, L)
    swe, depth = w.swe.copy(), w.depth.copy()
    m.set_snow(swe, depth)
    moved = 0.0
    for s in range(3):
        fa = w.forcing(s).arrays()
        own = {k: v for k, v in fa.items() if k not in ("swe", "snowdepthavg")}
        out = m.run(own, 3600.0, want_c=True)
        ref, _ = o.step_exact({**fa, "swe": swe, "snowdepthavg": depth}, 3600.0)
        for k in FIELDS:
            assert relerr(out[k], ref[k]) < FIELD_TOL, (s, k, relerr(out[k], ref[k]))
        swe, depth = synth.consume_drift(swe, depth, out["drift_mass"])
        gswe, gdepth = m.get_snow()
        np.testing.assert_array_equal(gswe, swe)
        np.testing.assert_array_equal(gdepth, depth)
        moved += np.abs(out["drift_mass"]).sum()
    assert moved > 0
    # without a snow state the step needs swe and snow depth from the caller
    m2 = gpu_module(w.mesh, L)
    with pytest.raises(ModuleError):
        m2.run(own, 3600.0)
    m.close()
    m2.close()


@pytest.mark.parametrize("solver", [{}, {"precision": 1}, {"precision": 1, "warm_start": 1},
                                    {"precision": 1, "warm_start": 1, "autotune": 1},
                                    {"precision": 1, "warm_start": 1, "neumann": 5}, {"neumann": 1}],
                         ids=["fp64", "mixed", "mixed_previous", "autotuned", "mixed_previous_neumann5",
                              "fp64_neumann1"])
def test_graph_mode_matches_oracle(cuda_lib, oracle_lib, solver):
    """The whole step as one CUDA-graph launch (device-side control of the
    Krylov and refinement loops) against the exact oracle over coupled steps."""
    L = 5
    wg = synth.Workload(1536, 3000.0, seed=5)
    wo = synth.Workload(1536, 3000.0, seed=5)
    m = gpu_module(wg.mesh, L, graph=1, **solver)
    o = oracle(wo.mesh, L)
    for s in range(3):
        fg, fo = wg.forcing(s), wo.forcing(s)
        out = m.run(fg, 3600.0, want_c=True)
        st = m.last_stats
        # one graph launch (after the autotuner's host-driven first steps);
        # the count is the kernels it executed
        assert st["susp_rel_residual"] <= 1e-8 and st["susp_iters"] > 0 and st["gpu_launches"] > 5 * st["susp_iters"]
        ref, _ = o.step_exact(fo, 3600.0)
        for k in FIELDS:
            assert relerr(out[k], ref[k]) < FIELD_TOL, (s, k, relerr(out[k], ref[k]))
        assert relerr(out["Qsalt"], ref["Qsalt"]) < 1e-12
        wg.apply_drift(ref["drift_mass"])
        wo.apply_drift(ref["drift_mass"])
    m.close()


def test_graph_mode_errors_and_state(cuda_lib, small):
    """Graph mode reports the host path's errors and, like it, leaves the
    module state untouched by a failed step; the device snow state works."""
    f = small.forcing(0).arrays()
    bad = dict(f)
    bad["t"] = f["t"].copy()
    bad["t"][10] = np.nan
    m = gpu_module(small.mesh, 5, graph=1)
    with pytest.raises(ModuleError, match="NAN_INPUT"):
        m.run(bad, 3600.0)
    assert np.all(m.state()["sum_subl"] == 0.0)
    m.close()
    m = gpu_module(small.mesh, 5, graph=1, susp_maxit=1)
    with pytest.raises(ModuleError, match="NOT_CONVERGED"):
        m.run(f, 3600.0)
    assert np.all(m.state()["sum_subl"] == 0.0)
    m.close()
    # device snow state inside the graph, against the host path
    outs = []
    for graph in (0, 1):
        m = gpu_module(small.mesh, 5, graph=graph)
        m.set_snow(small.swe, small.depth)
        own = {k: v for k, v in f.items() if k not in ("swe", "snowdepthavg")}
        for s in range(2):
            m.run(own, 3600.0)
        outs.append(m.get_snow())
        m.close()
    for a, b in zip(outs[0], outs[1]):
        assert relerr(b, a) < 1e-6


def test_native_mesh_reader_end_to_end(cuda_lib, oracle_lib, tmp_path):
    """The reference's slope mesh in CHM's JSON layout, read by the library's
    native reader and stepped on the GPU, against the oracle on the same
    mesh."""
    from conftest import GOLDEN
    from chm_gb300.meshio import ChmMesh, write_chm_mesh
    d = np.load(GOLDEN / "slope_mesh.npz")
    write_chm_mesh(tmp_path / "slope.mesh", d["vertex"], d["elem"], d["neigh"], {"area": d["area"]},
                   tmp_path / "slope.param")
    mesh = ChmMesh(tmp_path / "slope.mesh", tmp_path / "slope.param")
    n = mesh.n_faces
    rng = np.random.default_rng(3)
    f = {"U_R": rng.uniform(8, 20, n), "U_2m_above_srf": rng.uniform(5, 12, n),
         "vw_dir": np.full(n, 250.0) + rng.normal(0, 10, n), "swe": rng.uniform(20, 200, n),
         "t": rng.uniform(-15, -2, n), "rh": rng.uniform(60, 95, n), "snowdepthavg": rng.uniform(0.2, 1.0, n),
         "fetch": np.full(n, 1000.0)}
    m = gpu_module(mesh, 6)
    out = m.run(f, 3600.0, want_c=True)
    ref, _ = oracle(mesh, 6).step_exact(f, 3600.0)
    for k in FIELDS:
        assert relerr(out[k], ref[k]) < FIELD_TOL, (k, relerr(out[k], ref[k]))
    m.close()


@pytest.mark.parametrize("solver", [{}, {"precision": 1, "warm_start": 1, "neumann": 5, "dep_neumann": 1}],
                         ids=["fp64", "mixed_previous_neumann5"])
def test_graph_phase_times(cuda_lib, solver):
    """With profiling on, a graph-mode step (one launch) reports its phases --
    assembly, suspension solve, post with the deposition assembly, deposition
    solve, update -- from device-clock stamps at the phase boundaries; they
    are positive and add up to about the step."""
    w = synth.Workload(2048, 3500.0, seed=9)
    m = gpu_module(w.mesh, 5, graph=1, **solver)
    m.set_profiling(True)
    for s in range(5):
        m.run(w.forcing(s), 3600.0)
        w.apply_drift(m.state()["drift_mass"])
    st = m.last_stats
    assert st["susp_iters"] > 0 and st["deposition_present"]
    phases = [st[k] for k in ("ms_coefficients", "ms_susp_solve", "ms_post", "ms_dep_solve", "ms_update")]
    assert all(p > 0 for p in phases), phases
    assert 0.5 * st["ms_total"] <= sum(phases) <= 1.05 * st["ms_total"], (phases, st["ms_total"])
    m.close()


@pytest.mark.parametrize("solver", [{}, {"precision": 1, "warm_start": 1, "neumann": 5, "dep_neumann": 1},
                                    {"graph": 1, "neumann": 5, "dep_neumann": 1},
                                    {"graph": 1, "precision": 1, "warm_start": 1, "neumann": 5, "dep_neumann": 1}],
                         ids=["fp64", "mixed_previous_neumann5", "graph_fp64_neumann5", "graph_mixed_previous_neumann5"])
def test_pinned_host_outputs(cuda_lib, solver):
    """Host outputs in page-locked memory: the outputs final after the column
    post (and c) go to the host on a second stream while the deposition solve
    runs (host-driven), or between the step graph's two launches (graph
    mode).  Every output equals, bit for bit, the one a twin context writes
    to pageable memory after the step, over coupled steps with the device
    snow state."""
    torch = pytest.importorskip("torch")
    w = synth.Workload(2048, 3500.0, seed=21)
    L = 5
    mods = [gpu_module(w.mesh, L, **solver) for _ in range(2)]
    n = mods[0].n_faces
    keys = list(mods[0].output_keys())
    pinned = {k: torch.empty(n, dtype=torch.float64).pin_memory().numpy() for k in keys}
    pinned["c"] = torch.empty(L * n, dtype=torch.float64).pin_memory().numpy()
    for m in mods:
        m.set_snow(w.swe.copy(), w.depth.copy())
    for s in range(5):
        fa = {k: v for k, v in w.forcing(s).arrays().items() if k not in ("swe", "snowdepthavg")}
        a = mods[0].run(fa, 3600.0, outputs=pinned)
        b = mods[1].run(fa, 3600.0, want_c=True)
        assert mods[0].last_stats["deposition_present"] == 1
        for k in keys + ["c"]:
            np.testing.assert_array_equal(a[k], b[k], err_msg=f"step {s} {k}")
    for m in mods:
        m.close()
