"""The device-side wait limits end a stuck solve with an error, not a hang.

The persistent deposition CG is one cooperative launch whose blocks
synchronise through flags in global memory; every wait is bounded (2 s by
default).  pbsm3d_arm_wait_timeout_test makes one block of the next launch
publish no flag at all (a flag that nothing sets) and shortens the limit:
the other blocks' waits must run out, every block must leave, the step must
return PBSM3D_ERR_CUDA within about the armed limit, and the context must
stay usable: the next step gives the fields of a context that never failed.
The failure is made by a flag that is never set; nothing faults or traps.
"""
import time

import numpy as np
import pytest

from chm_gb300 import capi, synth
from chm_gb300.pbsm3d import PBSM3D, ModuleError

pytestmark = pytest.mark.gpu

# fields a step computes from its inputs alone (sum_subl and sum_drift
# accumulate, and the failed step has already added its sublimation)
FIELDS = ("Qsalt", "Qsusp", "Qsubl", "drift_mass", "c")


@pytest.mark.parametrize("solver", [{}, {"precision": capi.MIXED}, {"dep_neumann": 1}],
                         ids=["fp64", "mixed", "fp64_dep_neumann"])
@pytest.mark.parametrize("withhold", [0, 7])
def test_withheld_flag_times_out_cleanly(cuda_lib, solver, withhold):
    torch = pytest.importorskip("torch")
    w = synth.Workload(4096, 5000.0, seed=11)  # ~8k faces: 16 blocks in the CG grid
    L = 5
    m = PBSM3D({"nLayer": str(L)})
    m.init(w.mesh, **solver)
    ref = PBSM3D({"nLayer": str(L)})
    ref.init(w.mesh, **solver)
    for mod in (m, ref):
        mod.run(w.forcing(0), 3600.0)
        assert mod.last_stats["deposition_present"] == 1
    limit_ms = 20.0
    assert cuda_lib.pbsm3d_arm_wait_timeout_test(m._ctx, withhold, limit_ms) == capi.OK
    t0 = time.perf_counter()
    with pytest.raises(ModuleError, match="timed out"):
        m.run(w.forcing(1), 3600.0)
    dt = time.perf_counter() - t0
    # every block left after about the armed limit, far inside the 2 s default
    assert dt < 1.0, dt
    # the context (and the CUDA context) stays usable
    x = torch.ones(1024, device="cuda")
    assert float((x * 2).sum()) == 2048.0
    out = m.run(w.forcing(1), 3600.0, want_c=True)
    exp = ref.run(w.forcing(1), 3600.0, want_c=True)
    for k in FIELDS:
        np.testing.assert_array_equal(out[k], exp[k], err_msg=k)
    m.close()
    ref.close()


def test_arming_is_refused_where_there_is_no_persistent_cg(cuda_lib):
    w = synth.Workload(1024, 2500.0, seed=12)
    m = PBSM3D({"nLayer": "5"})
    m.init(w.mesh, graph=1)
    assert cuda_lib.pbsm3d_arm_wait_timeout_test(m._ctx, 0, 20.0) == capi.ERR_INVALID_ARG
    m.close()
    m = PBSM3D({"nLayer": "5"})
    m.init(w.mesh)
    for args in ((-1, 20.0), (0, 0.0), (0, 5000.0)):
        assert cuda_lib.pbsm3d_arm_wait_timeout_test(m._ctx, *args) == capi.ERR_INVALID_ARG
    m.close()
