"""CHM's JSON mesh files read by the library's native reader
(pbsm3d_mesh_read, triangulation.cpp:206-356) into the attributes the rest of
the package uses (those of chm_gb300.synth.Mesh)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi


class ChmMesh:
    """A mesh read from a .mesh (+ .param) pair.  Arrays are numpy copies of
    the reader's: xyz [nv, 3], tri [nt, 3], neighbor [nt, 3], edge_length
    [nt, 3], edge_normal [nt, 3, 2], area [nt], center [nt, 3], and when the
    .param file has them canopy_height, lai and the tpi_* statistics."""

    def __init__(self, mesh_path: str, param_path: str | None = None):
        lib = capi.load()
        h = C.c_void_p()
        rc = lib.pbsm3d_mesh_read(str(mesh_path).encode(), str(param_path).encode() if param_path else None,
                                  C.byref(h))
        if rc != 0:
            raise capi.MeshError(f"pbsm3d_mesh_read: {capi.STATUS_NAMES.get(rc, rc)}: "
                                 f"{lib.pbsm3d_mesh_last_error().decode(errors='replace')}")
        try:
            d = capi.MeshDesc()
            lib.pbsm3d_mesh_describe(h, C.byref(d))
            nv = C.c_int64()
            vp = C.POINTER(C.c_double)()
            ep = C.POINTER(C.c_int32)()
            lib.pbsm3d_mesh_arrays(h, C.byref(nv), C.byref(vp), C.byref(ep))
            nt = int(d.n_faces)

            def arr(p, n, shape=None):
                if not p:
                    return None
                a = np.ctypeslib.as_array(p, shape=(n,)).copy()
                return a.reshape(shape) if shape else a
            self.xyz = arr(vp, 3 * nv.value, (nv.value, 3))
            self.tri = arr(ep, 3 * nt, (nt, 3))
            self.neighbor = arr(d.neighbor, 3 * nt, (nt, 3))
            self.edge_length = arr(d.edge_length, 3 * nt, (nt, 3))
            self.edge_normal = arr(d.edge_normal, 6 * nt, (nt, 3, 2))
            self.area = arr(d.area, nt)
            self.center = arr(d.center, 3 * nt, (nt, 3))
            self.canopy_height = arr(d.canopy_height, nt)
            self.lai = arr(d.lai, nt)
            for k in capi.TPI_FIELDS:
                setattr(self, k, arr(getattr(d, k), nt))
        finally:
            lib.pbsm3d_mesh_free(h)

    @property
    def n_faces(self) -> int:
        return int(self.tri.shape[0])


def write_chm_mesh(path, xyz, tri, neighbor, params: dict | None = None, param_path=None, is_geographic=0):
    """Write a mesh in CHM's JSON layout (the inverse of ChmMesh, for tests
    and for meshes made by chm_gb300.synth)."""
    import json
    m = {"mesh": {"vertex": np.asarray(xyz, float).tolist(), "nvertex": int(len(xyz)),
                  "elem": np.asarray(tri, int).tolist(), "neigh": np.asarray(neighbor, int).tolist(),
                  "nelem": int(len(tri)), "is_geographic": int(is_geographic), "proj4": "+proj=utm +zone=8"}}
    with open(path, "w") as f:
        json.dump(m, f)
    if params is not None and param_path is not None:
        with open(param_path, "w") as f:
            json.dump({k: np.asarray(v, float).tolist() for k, v in params.items()}, f)
