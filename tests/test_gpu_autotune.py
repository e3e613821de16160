"""The launch-geometry autotuner of the suspension solve's column kernels.

The column kernels (vector update fused with the column Thomas solve, and
the polynomial-preconditioner step) run at nine geometries: slices of 256,
128 or 64 faces a block, with 1, 2 or 4 threads a face column.  Which thread
does a row's work changes with the geometry, the arithmetic does not: every
geometry must give bit-identical fields, so the tuner (on by default) can
pick any of them without changing a result.  Checked over coupled steps, in
FP64 and mixed precision, with the column and the order-5 polynomial
preconditioner, host-driven and as one CUDA-graph launch, and for a two-
member ensemble of uneven meshes.
"""
import ctypes as C

import numpy as np
import pytest

from chm_gb300 import capi, synth
from chm_gb300.ensemble import Ensemble, perturbed_members
from chm_gb300.pbsm3d import PBSM3D

pytestmark = pytest.mark.gpu

GEOMS = [(w, l) for l in (1, 2, 4) for w in (256, 128, 64)]
FIELDS = ("c", "Qsalt", "Qsusp", "Qsubl", "drift_mass", "sum_drift", "sum_subl")
FORMS = {
    "fp64": {},
    "fp64_neumann5": {"neumann": 5, "dep_neumann": 1},
    "mixed_previous_neumann5": {"precision": capi.MIXED, "warm_start": capi.X0_PREVIOUS, "neumann": 5},
    "graph_mixed_previous_neumann5": {"precision": capi.MIXED, "warm_start": capi.X0_PREVIOUS, "neumann": 5,
                                      "graph": 1},
}


def geometry(lib, m):
    w, l, t = C.c_int32(), C.c_int32(), C.c_int32()
    assert lib.pbsm3d_get_column_geometry(m._ctx, C.byref(w), C.byref(l), C.byref(t)) == capi.OK
    return w.value, l.value, t.value


def run_steps(mesh_w, L, solver, geom, lib, steps=3):
    m = PBSM3D({"nLayer": str(L)})
    m.init(mesh_w.mesh, autotune=0, **solver)
    if geom is not None:
        assert lib.pbsm3d_set_column_geometry(m._ctx, *geom) == capi.OK
        assert geometry(lib, m) == (geom[0], geom[1], 1)
    m.set_snow(mesh_w.swe.copy(), mesh_w.depth.copy())
    outs = []
    for s in range(steps):
        fa = {k: v for k, v in mesh_w.forcing(s).arrays().items() if k not in ("swe", "snowdepthavg")}
        outs.append(m.run(fa, 3600.0, want_c=True))
        assert m.last_stats["susp_rel_residual"] <= 1e-8
    m.close()
    return outs


@pytest.mark.parametrize("form", list(FORMS))
def test_every_geometry_gives_identical_bits(cuda_lib, form):
    w = synth.Workload(4096, 5000.0, seed=31)  # ~8k faces: 32 tiles of 256 faces
    L = 5
    ref = run_steps(w, L, FORMS[form], (256, 1), cuda_lib)
    for g in GEOMS[1:]:
        outs = run_steps(w, L, FORMS[form], g, cuda_lib)
        for s, (a, b) in enumerate(zip(outs, ref)):
            for k in FIELDS:
                np.testing.assert_array_equal(a[k], b[k], err_msg=f"{form} {g} step {s} {k}")


def test_tuned_context_equals_fixed_one(cuda_lib):
    """autotune = 1 (the default): the first solves time the candidates, a
    choice is made and kept, and every step's fields equal those of a context
    at the fixed default geometry, bit for bit."""
    w = synth.Workload(4096, 5000.0, seed=32)
    L = 5
    solver = {"precision": capi.MIXED, "warm_start": capi.X0_PREVIOUS, "neumann": 5, "dep_neumann": 1}
    cfg = capi.default_config(cuda_lib)
    assert cfg.autotune == 1
    tuned = PBSM3D({"nLayer": str(L)})
    tuned.init(w.mesh, **solver)
    ref = run_steps(w, L, solver, (256, 1), cuda_lib, steps=8)
    tuned.set_snow(w.swe.copy(), w.depth.copy())
    for s in range(8):
        fa = {k: v for k, v in w.forcing(s).arrays().items() if k not in ("swe", "snowdepthavg")}
        out = tuned.run(fa, 3600.0, want_c=True)
        for k in FIELDS:
            np.testing.assert_array_equal(out[k], ref[s][k], err_msg=f"step {s} {k}")
    gw, gl, done = geometry(cuda_lib, tuned)
    assert done == 1 and (gw, gl) in GEOMS
    print(f"tuned column geometry: {gw} faces a block, {gl} lane(s) a column")
    tuned.close()


def test_ensemble_geometries_identical(cuda_lib):
    ws = [synth.Workload(1500, 3000.0, seed=41), synth.Workload(3000, 4200.0, seed=42)]
    members = perturbed_members(2, 5)
    L = 5
    res = {}
    for g in [(256, 1), (64, 4), (128, 2)]:
        ens = Ensemble({"nLayer": str(L)})
        ens.init([w.mesh for w in ws], members, precision=capi.MIXED, neumann=5, autotune=0)
        assert cuda_lib.pbsm3d_set_column_geometry(ens._ctx, *g) == capi.OK
        out = ens.run_members([w.forcing(0) for w in ws], 3600.0, want_c=True)
        res[g] = out
        ens.close()
    for g in [(64, 4), (128, 2)]:
        for a, b in zip(res[g], res[(256, 1)]):
            for k in FIELDS:
                np.testing.assert_array_equal(a[k], b[k], err_msg=f"{g} {k}")


def test_geometry_argument_checks(cuda_lib):
    w = synth.Workload(512, 1500.0, seed=43)
    m = PBSM3D({"nLayer": "5"})
    m.init(w.mesh)
    for bad in ((32, 1), (256, 3), (512, 1), (128, 8)):
        assert cuda_lib.pbsm3d_set_column_geometry(m._ctx, *bad) == capi.ERR_INVALID_ARG
    m.close()
