"""pbsm3d_deposition_solve_noalloc: the deposition solve for hosts that do
not let a library allocate device memory (they own every device
allocation themselves).  It must give the same deposition flux as the
solve inside pbsm3d_step, call after call, without allocating: its work
space is a fixed static device array (at most 1,048,576 faces).

This file is collected last so that a run stopping at the first failure
has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from chm_gb300 import capi, synth
from chm_gb300.pbsm3d import PBSM3D

pytestmark = pytest.mark.gpu

TOL = 1e-6  # the field tolerance of the parity tests


def _soa(mesh, cols, vals):
    """Deposition rows (self, present neighbours in face order) -> SoA
    [3][n] neighbour ids and off-diagonals, diagonal [n]."""
    n = mesh.n_faces
    nb = mesh.neighbor
    present = nb >= 0
    slot = np.cumsum(present, axis=1)  # entry index of neighbour j in the row (self at 0)
    nbr = np.where(present, nb, -1).T.astype(np.int32).copy()
    rows = np.arange(n)[:, None]
    off = np.where(present, vals[rows, np.where(present, slot, 0)], 0.0).T.copy()
    assert (np.where(present, cols[rows, np.where(present, slot, 0)], -1) == np.where(present, nb, -1)).all()
    return nbr, vals[:, 0].copy(), off


def test_noalloc_deposition_solve_matches_step(cuda_lib):
    torch = pytest.importorskip("torch")
    lib = cuda_lib
    w = synth.Workload(2048, 3500.0, seed=21)
    n = w.mesh.n_faces
    m = PBSM3D({"nLayer": "5"})
    m.init(w.mesh)
    m.run(w.forcing(0), 3600.0)
    assert m.last_stats["deposition_present"] == 1
    cols, vals, rhs, x_step = m.export_system("deposition")
    m.close()
    nbr, diag, off = _soa(w.mesh, cols, vals)
    dev = torch.device("cuda")
    t_nbr = torch.from_numpy(nbr).to(dev)
    t_diag = torch.from_numpy(diag).to(dev)
    t_off = torch.from_numpy(off).to(dev)
    t_rhs = torch.from_numpy(rhs).to(dev)
    t_x = torch.empty(n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    vp = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    scale = np.abs(x_step).max()
    for call in range(2):  # the shared scratch keeps the last call's contents
        t_x.fill_(float("nan"))
        torch.cuda.synchronize()
        it = C.c_int32()
        rr = C.c_double()
        rc = lib.pbsm3d_deposition_solve_noalloc(n, vp(t_nbr), vp(t_diag), vp(t_off), vp(t_rhs), vp(t_x), 1e-10,
                                                 1000, C.byref(it), C.byref(rr))
        assert rc == capi.OK, lib.pbsm3d_last_error(None).decode()
        x = t_x.cpu().numpy()
        assert rr.value <= 1e-10 and it.value > 0
        assert np.abs(x - x_step).max() <= TOL * scale, (call, np.abs(x - x_step).max() / scale)


def _oracle_soa(mesh, o):
    """The oracle's own deposition system (CSR) as the entry point's SoA."""
    rp, cols, vals, rhs, _ = o.raw_system(1)
    n = mesh.n_faces
    nbr = np.where(mesh.neighbor >= 0, mesh.neighbor, -1).T.astype(np.int32).copy()
    diag = np.zeros(n)
    off = np.zeros((3, n))
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            c = cols[k]
            if c == i:
                diag[i] = vals[k]
            else:
                j = int(np.nonzero(nbr[:, i] == c)[0][0])
                off[j, i] = vals[k]
    return nbr, diag, off, rhs


def test_noalloc_matches_oracle_deposition_solve(cuda_lib, oracle_lib):
    """The oracle's deposition system, solved by the entry point, against a
    direct solve of the same system (independent of the GPU assembly)."""
    torch = pytest.importorskip("torch")
    import scipy.sparse.linalg as spl
    from oracle import pyoracle
    w = synth.Workload(2048, 3500.0, seed=22)
    o = pyoracle.Oracle(w.mesh, nLayer=5)
    o.step_exact(w.forcing(0), 3600.0, want_c=False)
    D, bd, _ = o.system(1)
    q_ref = spl.spsolve(D.tocsc(), bd)
    nbr, diag, off, rhs = _oracle_soa(w.mesh, o)
    o.close()
    n = w.mesh.n_faces
    dev = torch.device("cuda")
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (nbr, diag, off, rhs)]
    t_x = torch.empty(n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    vp = lambda a: C.c_void_p(a.data_ptr())  # noqa: E731
    it, rr = C.c_int32(), C.c_double()
    rc = cuda_lib.pbsm3d_deposition_solve_noalloc(n, *(vp(a) for a in t), vp(t_x), 1e-12, 2000, C.byref(it),
                                                  C.byref(rr))
    assert rc == capi.OK, cuda_lib.pbsm3d_last_error(None).decode()
    x = t_x.cpu().numpy()
    assert rr.value <= 1e-11  # the true residual, checked after the recursive one met 1e-12
    assert np.abs(x - q_ref).max() <= TOL * np.abs(q_ref).max()
    # the CG stops at one iteration when maxit = 1: NOT_CONVERGED, with the
    # iteration count and a finite relative residual reported
    it, rr = C.c_int32(), C.c_double(-1.0)
    rc = cuda_lib.pbsm3d_deposition_solve_noalloc(n, *(vp(a) for a in t), vp(t_x), 1e-12, 1, C.byref(it),
                                                  C.byref(rr))
    assert rc == capi.ERR_NOT_CONVERGED
    assert it.value == 1 and np.isfinite(rr.value) and rr.value > 1e-12
    assert b"did not converge" in cuda_lib.pbsm3d_last_error(None)


def test_noalloc_rejects_invalid_arguments(cuda_lib):
    torch = pytest.importorskip("torch")
    t = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(t.data_ptr())
    for args in ((0, p, p, p, p, p, 1e-10, 10), (8, None, p, p, p, p, 1e-10, 10), (8, p, p, p, p, None, 1e-10, 10),
                 (8, p, p, p, p, p, 0.0, 10), (8, p, p, p, p, p, 1e-10, 0)):
        assert cuda_lib.pbsm3d_deposition_solve_noalloc(*args, None, None) == capi.ERR_INVALID_ARG


def test_noalloc_rejects_sizes_beyond_its_limit(cuda_lib):
    torch = pytest.importorskip("torch")
    t = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(t.data_ptr())
    rc = cuda_lib.pbsm3d_deposition_solve_noalloc((1 << 20) + 1, p, p, p, p, p, 1e-10, 10, None, None)
    assert rc == capi.ERR_INVALID_ARG
    assert b"1048576" in cuda_lib.pbsm3d_last_error(None)
