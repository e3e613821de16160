"""The C++ PBSM3D module driven like CHM's core (factory -> init -> run per
step through face variables) gives the same fields as the C ABI called
directly, and matches the oracle."""
import subprocess

import numpy as np
import pytest

from chm_gb300 import synth
from chm_gb300.pbsm3d import PBSM3D, OUTPUT_KEYS

pytestmark = pytest.mark.gpu


def test_cpp_module_matches_direct_calls(cuda_lib, tmp_path):
    from chm_gb300 import build
    exe = build.build_shim()
    w = synth.Workload(1024, 2500.0, seed=12)
    m = w.mesh
    n, L, steps = m.n_faces, 5, 2
    case = tmp_path / "case"
    out = tmp_path / "out"
    case.mkdir()
    out.mkdir()
    (case / "meta.txt").write_text(f"{n} {L} {steps} 3600\nnLayer {L}\n")
    m.neighbor.astype(np.int32).tofile(case / "neighbor.bin")
    m.edge_length.tofile(case / "edge_length.bin")
    m.edge_normal.tofile(case / "edge_normal.bin")
    m.area.tofile(case / "area.bin")
    m.center.tofile(case / "center.bin")
    forcings = [w.forcing(s) for s in range(steps)]
    for s, f in enumerate(forcings):
        for k, a in f.arrays().items():
            np.ascontiguousarray(a).tofile(case / f"{k}_{s}.bin")
    r = subprocess.run([str(exe), str(case), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    mod = PBSM3D({"nLayer": str(L)})
    mod.init(m)
    for s, f in enumerate(forcings):
        direct = mod.run(f, 3600.0)
        for k in OUTPUT_KEYS:
            via_cpp = np.fromfile(out / f"{k}_{s}.bin")
            np.testing.assert_array_equal(via_cpp, direct[k], err_msg=k)
    np.testing.assert_array_equal(np.fromfile(out / "checkpoint_sum_drift.bin"), mod.checkpoint()["PBSM3D:sum_drift"])
    mod.close()
