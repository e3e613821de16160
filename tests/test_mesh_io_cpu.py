"""CHM's JSON mesh files through the library's native reader (no GPU
needed): the reference's slope mesh written back in CHM's layout reads with
its own neighbour lists and with the geometry CHM's face class computes
(bit for bit against the numpy restatement), parameters included; malformed
and geographic meshes are refused with the reason."""
import json

import numpy as np
import pytest

from chm_gb300 import capi, synth
from chm_gb300.meshio import ChmMesh, write_chm_mesh


def test_reads_reference_mesh(cuda_lib, tmp_path):
    from conftest import GOLDEN
    d = np.load(GOLDEN / "slope_mesh.npz")
    rng = np.random.default_rng(0)
    nt = d["elem"].shape[0]
    params = {"area": d["area"], "TPI_mean": rng.normal(size=nt), "TPI_std": rng.uniform(0.1, 2, nt),
              "CanopyHeight": rng.uniform(0, 2, nt), "LAI": rng.uniform(0, 3, nt)}
    write_chm_mesh(tmp_path / "slope.mesh", d["vertex"], d["elem"], d["neigh"], params, tmp_path / "slope.param")
    m = ChmMesh(tmp_path / "slope.mesh", tmp_path / "slope.param")
    ref = synth.mesh_from_arrays(d["vertex"], d["elem"], d["neigh"], area=d["area"])
    np.testing.assert_array_equal(m.tri, d["elem"])
    np.testing.assert_array_equal(m.neighbor, d["neigh"])
    np.testing.assert_array_equal(m.xyz, d["vertex"])
    for k in ("edge_length", "edge_normal", "area", "center"):
        np.testing.assert_array_equal(getattr(m, k), getattr(ref, k), err_msg=k)
    np.testing.assert_array_equal(m.tpi_mean, params["TPI_mean"])
    np.testing.assert_array_equal(m.canopy_height, params["CanopyHeight"])
    assert m.tpi_neg_frac is None
    # without a .param file the area is the 2-D triangle area
    m2 = ChmMesh(tmp_path / "slope.mesh")
    a2 = synth.face_geometry(d["vertex"], d["elem"])[2]
    np.testing.assert_array_equal(m2.area, a2)
    assert m2.canopy_height is None


def test_refuses_bad_meshes(cuda_lib, tmp_path):
    w = synth.make_mesh(64, 300.0, 0)
    good = {"vertex": w.xyz.tolist(), "nvertex": len(w.xyz), "elem": w.tri.tolist(), "neigh": w.neighbor.tolist(),
            "nelem": len(w.tri), "is_geographic": 0}
    cases = {
        "missing_neigh": {k: v for k, v in good.items() if k != "neigh"},
        "count": {**good, "nelem": len(w.tri) + 1},
        "range": {**good, "neigh": [[len(w.tri) + 3, -1, -1]] + w.neighbor.tolist()[1:]},
        "ragged": {**good, "elem": [[0, 1]] + w.tri.tolist()[1:]},
    }
    for name, mesh in cases.items():
        (tmp_path / f"{name}.mesh").write_text(json.dumps({"mesh": mesh}))
        with pytest.raises(capi.MeshError, match="BAD_MESH"):
            ChmMesh(tmp_path / f"{name}.mesh")
    (tmp_path / "geo.mesh").write_text(json.dumps({"mesh": {**good, "is_geographic": 1}}))
    with pytest.raises(capi.MeshError, match="UNSUPPORTED"):
        ChmMesh(tmp_path / "geo.mesh")
    (tmp_path / "trunc.mesh").write_text(json.dumps({"mesh": good})[:-40])
    with pytest.raises(capi.MeshError, match="BAD_MESH"):
        ChmMesh(tmp_path / "trunc.mesh")
    (tmp_path / "ok.mesh").write_text(json.dumps({"mesh": good}))
    (tmp_path / "bad.param").write_text(json.dumps({"area": [1.0, 2.0]}))
    with pytest.raises(capi.MeshError, match="one number per face"):
        ChmMesh(tmp_path / "ok.mesh", tmp_path / "bad.param")
    with pytest.raises(capi.MeshError, match="cannot open"):
        ChmMesh(tmp_path / "nope.mesh")


def test_synthetic_round_trip(cuda_lib, tmp_path):
    """A synthetic mesh written in CHM's layout reads back to the same arrays."""
    w = synth.make_mesh(2000, 3000.0, 4)
    write_chm_mesh(tmp_path / "s.mesh", w.xyz, w.tri, w.neighbor, {"area": w.area}, tmp_path / "s.param")
    m = ChmMesh(tmp_path / "s.mesh", tmp_path / "s.param")
    for k in ("tri", "neighbor", "edge_length", "edge_normal", "area", "center"):
        np.testing.assert_array_equal(getattr(m, k), getattr(w, k), err_msg=k)


# ---------------------------------------------------------------- HDF5
# CHM's HDF5 mesh and parameter files (triangulation.cpp:724-1035, 1237-1383)
# through the same reader: the file's signature selects the format.

def test_hdf5_mesh_matches_json(cuda_lib, tmp_path):
    """The same mesh and parameters written in CHM's HDF5 layout (root
    attributes "/mesh/...", /mesh/vertex|elem|neighbor as 3-element arrays,
    big-endian cell_global_id, /parameters/<name>) and in its JSON layout read
    to identical arrays."""
    from h5_writer import write_mesh_h5, write_params_h5
    from conftest import GOLDEN
    d = np.load(GOLDEN / "slope_mesh.npz")
    rng = np.random.default_rng(3)
    nt = d["elem"].shape[0]
    params = {"area": d["area"], "TPI_mean": rng.normal(size=nt), "CanopyHeight": rng.uniform(0, 2, nt),
              "LAI": rng.uniform(0, 3, nt), "id": np.arange(nt, dtype=float)}
    write_chm_mesh(tmp_path / "s.mesh", d["vertex"], d["elem"], d["neigh"], params, tmp_path / "s.param")
    write_mesh_h5(tmp_path / "s_mesh.h5", d["vertex"], d["elem"], d["neigh"])
    write_params_h5(tmp_path / "s_param.h5", params)
    a = ChmMesh(tmp_path / "s_mesh.h5", tmp_path / "s_param.h5")
    b = ChmMesh(tmp_path / "s.mesh", tmp_path / "s.param")
    for k in ("xyz", "tri", "neighbor", "edge_length", "edge_normal", "area", "center", "canopy_height", "lai",
              "tpi_mean"):
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=k)
    assert a.tpi_std is None
    # a JSON mesh with HDF5 parameters, and the other way round
    c = ChmMesh(tmp_path / "s.mesh", tmp_path / "s_param.h5")
    np.testing.assert_array_equal(c.area, b.area)
    e = ChmMesh(tmp_path / "s_mesh.h5", tmp_path / "s.param")
    np.testing.assert_array_equal(e.lai, b.lai)


def test_hdf5_refusals(cuda_lib, tmp_path):
    from h5_writer import write_mesh_h5, write_params_h5
    w = synth.make_mesh(64, 300.0, 1)
    write_mesh_h5(tmp_path / "part.h5", w.xyz, w.tri, w.neighbor, is_partition=1)
    with pytest.raises(capi.MeshError, match="partitioned"):
        ChmMesh(tmp_path / "part.h5")
    write_mesh_h5(tmp_path / "geo.h5", w.xyz, w.tri, w.neighbor, is_geographic=1)
    with pytest.raises(capi.MeshError, match="UNSUPPORTED"):
        ChmMesh(tmp_path / "geo.h5")
    gid = np.arange(len(w.tri))[::-1]
    write_mesh_h5(tmp_path / "perm.h5", w.xyz, w.tri, w.neighbor, global_ids=gid)
    with pytest.raises(capi.MeshError, match="cell_global_id"):
        ChmMesh(tmp_path / "perm.h5")
    bad = w.neighbor.copy()
    bad[0, 0] = len(w.tri) + 5
    write_mesh_h5(tmp_path / "range.h5", w.xyz, w.tri, bad)
    with pytest.raises(capi.MeshError, match="out of range"):
        ChmMesh(tmp_path / "range.h5")
    write_mesh_h5(tmp_path / "ok.h5", w.xyz, w.tri, w.neighbor)
    write_params_h5(tmp_path / "short.h5", {"area": np.ones(len(w.tri) - 1)})
    with pytest.raises(capi.MeshError, match="one number per face"):
        ChmMesh(tmp_path / "ok.h5", tmp_path / "short.h5")
    raw = (tmp_path / "ok.h5").read_bytes()
    (tmp_path / "trunc.h5").write_bytes(raw[:len(raw) // 2])
    with pytest.raises(capi.MeshError, match="BAD_MESH"):
        ChmMesh(tmp_path / "trunc.h5")


def test_reference_hdf5_mesh(cuda_lib):
    """The reference's own HDF5 slope mesh and parameters (its METIS-ordered
    copy of the functional-test mesh) against its JSON slope.mesh/.param:
    under the face permutation between the two files, every face's vertices
    (in order), its neighbours and the area parameter are identical.  Runs
    where the reference tree is present."""
    import os
    from pathlib import Path
    ref = Path(os.environ.get("CHM_REFERENCE", "/root/reference")) / "functional_tests" / "mesh_versioning"
    if not (ref / "slope.metis_mesh.h5").exists():
        pytest.skip("reference tree not present")
    a = ChmMesh(ref / "slope.metis_mesh.h5", ref / "slope.metis_param.h5")
    b = ChmMesh(ref / "slope.mesh", ref / "slope.param")
    np.testing.assert_array_equal(a.xyz, b.xyz)
    index = {tuple(sorted(t)): i for i, t in enumerate(b.tri.tolist())}
    perm = np.array([index[tuple(sorted(t))] for t in a.tri.tolist()])
    np.testing.assert_array_equal(np.sort(perm), np.arange(len(perm)))
    np.testing.assert_array_equal(a.tri, b.tri[perm])
    nb = np.where(a.neighbor >= 0, perm[np.maximum(a.neighbor, 0)], -1)
    np.testing.assert_array_equal(nb, b.neighbor[perm])
    np.testing.assert_array_equal(a.area, b.area[perm])
