"""Regenerate the golden fixtures of tests/golden from the reference tree.

* slope_mesh.npz     <- functional_tests/mesh_versioning/slope.mesh + slope.param
* granger1m_mesh.npz <- test_data/meshes/granger1m.mesh + granger1m.param
  (vertex xyz, elem vertex ids, the mesher's neigh lists, the 'area'
  parameter): the reference's own adjacency and geometry inputs, used to
  pin the adjacency convention and to run the step on real CHM meshes.
* oracle_small.npz   <- one step of the CPU oracle (exact solves) on a small
  seeded synthetic mesh, frozen so a change in the oracle is noticed.

Run in a container that has the reference tree:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
REFERENCE = Path(os.environ.get("CHM_REFERENCE", "/root/reference"))

MESHES = {
    "slope_mesh.npz": ("functional_tests/mesh_versioning/slope.mesh", "functional_tests/mesh_versioning/slope.param"),
    "granger1m_mesh.npz": ("test_data/meshes/granger1m.mesh", "test_data/meshes/granger1m.param"),
}


def mesh_fixture(mesh_path: Path, param_path: Path, out: Path):
    m = json.loads(mesh_path.read_text())["mesh"]
    p = json.loads(param_path.read_text())
    np.savez_compressed(out, vertex=np.asarray(m["vertex"], np.float64), elem=np.asarray(m["elem"], np.int32),
                        neigh=np.asarray(m["neigh"], np.int32), area=np.asarray(p["area"], np.float64))


def oracle_fixture(out: Path):
    from chm_gb300 import synth
    from oracle import pyoracle
    w = synth.Workload(512, 1500.0, seed=11)
    f = w.forcing(0)
    o = pyoracle.Oracle(w.mesh, nLayer=5)
    res, st = o.step_exact(f, 3600.0)
    arrays = {f"in_{k}": v for k, v in f.arrays().items()}
    arrays.update({f"out_{k}": v for k, v in res.items()})
    np.savez_compressed(out, seed=11, n_points=512, side=1500.0, nLayer=5, **arrays)


if __name__ == "__main__":
    for name, (mp, pp) in MESHES.items():
        mesh_fixture(REFERENCE / mp, REFERENCE / pp, HERE / name)
        print("wrote", name)
    oracle_fixture(HERE / "oracle_small.npz")
    print("wrote oracle_small.npz")
