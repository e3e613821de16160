"""Batched ensembles: every member of one ensemble context against the exact
oracle run with that member's constants, and against its own single-domain
context; members whose suspension or deposition is absent; mixed precision
and warm starts across several steps.  Bars as in the single-domain parity
tests: fields within relative 1e-6 of the oracle's exact solve, Qsalt to
rounding, the erosion flags bit-exact."""
import numpy as np
import pytest

from chm_gb300 import capi, synth
from chm_gb300.ensemble import Ensemble, MemberParams
from chm_gb300.pbsm3d import PBSM3D

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-6
FIELDS = ("c", "Qsalt", "Qsusp", "Qsubl", "Qsubl_mass", "drift_mass", "sum_drift", "sum_subl")
L = 5


def relerr(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def member_cfg(p: MemberParams) -> dict:
    return {"ustar_th_scale": p.ustar_th_scale, "z0_snow": p.z0_snow, "settling_scale": p.settling_scale}


def workloads():
    # uneven sizes, one calm member (no saltation: suspension absent)
    return [synth.Workload(1024, 2500.0, seed=41), synth.Workload(700, 2000.0, seed=42),
            synth.Workload(1536, 3000.0, seed=43, wind_scale=0.3), synth.Workload(400, 1500.0, seed=44)]


MEMBERS = [MemberParams(1.15, 3e-3, 0.9), MemberParams(0.82, 2e-4, 1.12), MemberParams(1.0, 0.01, 1.0),
           MemberParams(0.9, 1e-4, 0.87)]


def _check_member(out, ref, tag):
    for k in FIELDS:
        assert relerr(out[k], ref[k]) < FIELD_TOL, (tag, k, relerr(out[k], ref[k]))
    assert relerr(out["Qsalt"], ref["Qsalt"]) < 1e-12, tag
    np.testing.assert_array_equal(out["pbsm_more_than_avail"], ref["pbsm_more_than_avail"])


@pytest.mark.parametrize("solver", [{}, {"precision": capi.MIXED}, {"warm_start": capi.X0_PREVIOUS},
                                    {"precision": capi.MIXED, "warm_start": capi.X0_PREVIOUS, "graph": 1},
                                    {"precision": capi.MIXED, "warm_start": capi.X0_PREVIOUS, "graph": 1,
                                     "neumann": 5},
                                    {"dep_neumann": 1}, {"precision": capi.MIXED, "dep_neumann": 1},
                                    {"precision": capi.MIXED, "warm_start": capi.X0_PREVIOUS, "graph": 1,
                                     "neumann": 5, "dep_neumann": 1}],
                         ids=["fp64", "mixed", "warm", "graph", "graph_neumann5", "fp64_dep_neumann",
                              "mixed_dep_neumann", "graph_neumann5_dep_neumann"])
def test_members_match_oracle_over_steps(cuda_lib, oracle_lib, solver):
    from oracle import pyoracle
    ws = workloads()
    ens = Ensemble({"nLayer": str(L)})
    ens.init([w.mesh for w in ws], MEMBERS, **solver)
    assert list(np.diff(ens.offsets)) == [w.mesh.n_faces for w in ws]
    orc = [pyoracle.Oracle(w.mesh, nLayer=L, cfg=member_cfg(p)) for w, p in zip(ws, MEMBERS)]
    saw_absent = False
    for s in range(3):
        fs = [w.forcing(s) for w in ws]
        outs = ens.run_members(fs, 3600.0, want_c=True)
        st = ens.last_stats
        assert st["susp_rel_residual"] <= 1e-8
        for m, (o, f, w) in enumerate(zip(orc, fs, ws)):
            ref, _ = o.step_exact(f, 3600.0)
            if np.abs(ref["c"]).max() == 0.0:
                saw_absent = True
                assert np.abs(outs[m]["c"]).max() == 0.0
            _check_member(outs[m], ref, (s, m))
            w.apply_drift(ref["drift_mass"])
    assert saw_absent, "the calm member should have no suspension"
    ens.close()


def test_members_match_single_domain_contexts(cuda_lib):
    """The same members run one by one through pbsm3d_create with the
    constants in the config."""
    ws = workloads()
    ens = Ensemble({"nLayer": str(L)})
    ens.init([w.mesh for w in ws], MEMBERS)
    fs = [w.forcing(0) for w in ws]
    outs = ens.run_members(fs, 3600.0, want_c=True)
    for m, (w, p, f) in enumerate(zip(ws, MEMBERS, fs)):
        single = PBSM3D({"nLayer": str(L)})
        single.init(w.mesh, **member_cfg(p))
        ref = single.run(f, 3600.0, want_c=True)
        for k in FIELDS:
            # both stop at relative residual 1e-8: agreement well inside the field bar
            assert relerr(outs[m][k], ref[k]) < FIELD_TOL, (m, k)
        np.testing.assert_array_equal(outs[m]["Qsalt"], ref["Qsalt"])
        single.close()
    ens.close()


def test_all_members_calm(cuda_lib):
    """No member saltates: nothing is solved and drift_mass keeps its value."""
    ws = [synth.Workload(600, 2000.0, seed=51, wind_scale=0.2), synth.Workload(500, 2000.0, seed=52, wind_scale=0.2)]
    ens = Ensemble({"nLayer": str(L)})
    ens.init([w.mesh for w in ws], MEMBERS[:2])
    outs = ens.run_members([w.forcing(0) for w in ws], 3600.0, want_c=True)
    assert ens.last_stats["suspension_present"] == 0
    for o in outs:
        assert np.abs(o["c"]).max() == 0.0
    ens.close()


def test_single_member_ensemble_equals_plain_context(cuda_lib):
    """A one-member ensemble runs exactly the single-domain kernels."""
    w = synth.Workload(1024, 2500.0, seed=61)
    p = MEMBERS[1]
    ens = Ensemble({"nLayer": str(L)})
    ens.init([w.mesh], [p])
    single = PBSM3D({"nLayer": str(L)})
    single.init(w.mesh, **member_cfg(p))
    f = w.forcing(0)
    a = ens.run(f.arrays(), 3600.0, want_c=True)
    b = single.run(f, 3600.0, want_c=True)
    for k in FIELDS:
        np.testing.assert_array_equal(a[k], b[k])
    ens.close()
    single.close()
