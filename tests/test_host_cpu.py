"""Host-side logic on CPU: the module/factory mirror, config parsing, the
C-ABI library's exports, and the replica reduction of bench.py under a
2-rank gloo group."""
import ctypes as C
import os
import re
from pathlib import Path

import numpy as np
import pytest

from chm_gb300 import capi
from chm_gb300.pbsm3d import ModuleError, ModuleNotFound, PBSM3D, create, registered_keys

ROOT = Path(__file__).resolve().parent.parent


def test_factory_and_depends_provides():
    assert "PBSM3D" in registered_keys()
    m = create("PBSM3D", {"nLayer": "10"})
    assert isinstance(m, PBSM3D)
    assert m.parallel == "domain"
    for v in ("U_2m_above_srf", "vw_dir", "swe", "t", "rh", "U_R", "fetch"):
        assert v in m.depends
    for v in ("Qsubl", "Qsubl_mass", "sum_subl", "drift_mass", "Qsusp", "Qsalt", "sum_drift",
              "pbsm_more_than_avail", "blowingsnow_probability", "global_cell_id"):
        assert v in m.provides
    m2 = create("PBSM3D", {"use_tanh_fetch": "false"})
    assert "p_snow_hours" in m2.depends and "fetch" not in m2.depends
    with pytest.raises(ModuleNotFound):
        create("NotAModule", {})


def test_config_errors_match_reference():
    with pytest.raises(ModuleError, match="Cannot specify both"):
        PBSM3D({"use_exp_fetch": "true", "use_tanh_fetch": "true"})
    with pytest.raises(ModuleError, match="positive"):
        PBSM3D({"settling_velocity": "-1"}).init(None)
    with pytest.raises(ModuleError):
        PBSM3D({"use_exp_fetch": "maybe"})


def _header_functions():
    text = (ROOT / "include" / "pbsm3d.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pbsm3d_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_header_symbol(cuda_lib):
    names = _header_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(cuda_lib, n), n
    assert set(names) == set(capi.EXPORTS)


def test_struct_layout_matches_header(cuda_lib):
    """The config defaults filled by the library read back through ctypes."""
    cfg = capi.default_config(cuda_lib)
    assert cfg.abi_version == capi.ABI_VERSION
    assert cfg.nLayer == 10 and cfg.use_tanh_fetch == 1 and cfg.use_R94_lambda == 1
    assert cfg.settling_velocity == 0.5 and cfg.smooth_coeff == 820 and cfg.susp_tol == 1e-8
    assert cfg.gmres_restart == 30 and cfg.susp_maxit == 1000 and cfg.z0_snow == 0.01


def test_create_without_gpu_is_an_error(cuda_lib):
    """No CPU fallback: without a device the library refuses to create a context."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from chm_gb300 import synth
    m = synth.make_mesh(64, 300.0, 0)
    keep = []
    desc = capi.mesh_desc(m, keep)
    cfg = capi.default_config(cuda_lib)
    ctx = C.c_void_p()
    rc = cuda_lib.pbsm3d_create(C.byref(desc), C.byref(cfg), C.byref(ctx))
    assert rc == capi.ERR_CUDA
    assert cuda_lib.pbsm3d_last_error(None)


def test_create_rejects_bad_configs(cuda_lib):
    from chm_gb300 import synth
    m = synth.make_mesh(64, 300.0, 0)
    keep = []
    desc = capi.mesh_desc(m, keep)
    ctx = C.c_void_p()
    for bad in (dict(use_exp_fetch=1, use_tanh_fetch=1), dict(settling_velocity=-0.1), dict(nLayer=0),
                dict(abi_version=99), dict(neumann=10), dict(neumann=-1), dict(dep_neumann=2)):
        cfg = capi.default_config(cuda_lib, **bad)
        assert cuda_lib.pbsm3d_create(C.byref(desc), C.byref(cfg), C.byref(ctx)) == capi.ERR_INVALID_ARG
    bad_nb = m.neighbor.copy()
    bad_nb[0, 0] = m.n_faces + 5
    m.neighbor = bad_nb
    desc = capi.mesh_desc(m, keep)
    cfg = capi.default_config(cuda_lib)
    assert cuda_lib.pbsm3d_create(C.byref(desc), C.byref(cfg), C.byref(ctx)) == capi.ERR_BAD_MESH


def test_ensemble_create_rejects_bad_members(cuda_lib):
    """Argument checks of pbsm3d_ensemble_create run before any device call."""
    from chm_gb300 import synth
    meshes = [synth.make_mesh(64, 300.0, 0), synth.make_mesh(48, 250.0, 1)]
    keep = []
    descs = (capi.MeshDesc * 2)(*[capi.mesh_desc(m, keep) for m in meshes])
    cfg = capi.default_config(cuda_lib)
    ctx = C.c_void_p()
    good = capi.Member(1.0, 0.01, 1.0)
    for bad in (capi.Member(1.0, 0.0, 1.0), capi.Member(-1.0, 0.01, 1.0), capi.Member(1.0, 0.01, -0.5),
                capi.Member(1.0, float("nan"), 1.0)):
        mem = (capi.Member * 2)(good, bad)
        assert cuda_lib.pbsm3d_ensemble_create(2, descs, mem, C.byref(cfg), C.byref(ctx)) == capi.ERR_INVALID_ARG
        assert b"positive" in cuda_lib.pbsm3d_last_error(None)
    mem = (capi.Member * 2)(good, good)
    assert cuda_lib.pbsm3d_ensemble_create(0, descs, mem, C.byref(cfg), C.byref(ctx)) == capi.ERR_INVALID_ARG
    assert cuda_lib.pbsm3d_ensemble_create(257, descs, mem, C.byref(cfg), C.byref(ctx)) == capi.ERR_INVALID_ARG
    # vegetation is a per-domain switch: members must agree on it
    meshes[1].canopy_height = None
    descs = (capi.MeshDesc * 2)(*[capi.mesh_desc(m, keep) for m in meshes])
    assert cuda_lib.pbsm3d_ensemble_create(2, descs, mem, C.byref(cfg), C.byref(ctx)) == capi.ERR_INVALID_ARG
    assert b"vegetation" in cuda_lib.pbsm3d_last_error(None)
    # a neighbour index outside its own member's mesh
    meshes[1].canopy_height = np.zeros(meshes[1].n_faces)
    nb = meshes[1].neighbor.copy()
    nb[0, 0] = meshes[1].n_faces
    meshes[1].neighbor = nb
    descs = (capi.MeshDesc * 2)(*[capi.mesh_desc(m, keep) for m in meshes])
    assert cuda_lib.pbsm3d_ensemble_create(2, descs, mem, C.byref(cfg), C.byref(ctx)) == capi.ERR_BAD_MESH


def test_ensemble_forcing_split_and_members(cuda_lib):
    """Host side of the ensemble wrapper: forcing concatenation and output split."""
    from chm_gb300 import ensemble, synth
    e = ensemble.Ensemble({"nLayer": "3"})
    e.nLayer, e.n_members, e.offsets = 3, 2, np.array([0, 4, 7])
    e.n_faces = 7
    c = np.arange(21.0)
    out = {"drift_mass": np.arange(7.0), "c": c}
    parts = e.split(out)
    np.testing.assert_array_equal(parts[1]["drift_mass"], [4, 5, 6])
    np.testing.assert_array_equal(parts[0]["c"], [0, 1, 2, 3, 7, 8, 9, 10, 14, 15, 16, 17])
    np.testing.assert_array_equal(parts[1]["c"], [4, 5, 6, 11, 12, 13, 18, 19, 20])
    f = e.concat_forcing([{"t": np.zeros(4), "rh": np.ones(4)}, {"t": np.ones(3), "rh": np.ones(3)}])
    assert f["t"].shape == (7,) and f["rh"].shape == (7,)
    with pytest.raises(ModuleError):
        e.concat_forcing([{"t": np.zeros(4)}, {"rh": np.ones(3)}])
    ms = ensemble.perturbed_members(200, 0)
    u = np.array([m.ustar_th_scale for m in ms])
    z = np.array([m.z0_snow for m in ms])
    s = np.array([m.settling_scale for m in ms])
    assert u.min() >= 0.8 and u.max() <= 1.2 and z.min() >= 1e-4 and z.max() <= 1e-2
    assert s.min() >= 0.85 and s.max() <= 1.15


def _replica_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import sys
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist(world)
    d.barrier()
    mx = d.max(float(rank + 1))
    tot = d.sum(float(10 * (rank + 1)))
    q.put((rank, mx, tot))
    d.dist.destroy_process_group()


def test_replica_reduction_two_ranks_gloo():
    """bench.py --gpus N runs independent replicas: time = max over ranks,
    element-steps = sum over ranks (gloo, world size 2)."""
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert res == [(0, 2.0, 30.0), (1, 2.0, 30.0)]


def test_cpp_module_shim_selftest(cuda_lib):
    """The C++ module (CHM module_base/factory replica + PBSM3D over the C
    ABI) builds and passes its host-side checks without a GPU."""
    import subprocess
    from chm_gb300 import build
    exe = build.build_shim()
    r = subprocess.run([str(exe), "--selftest"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "selftest ok" in r.stdout


def test_consume_drift_rule():
    """snobal's use of drift_mass (snobal.cpp:363-387): erosion at the pack's
    bulk density, deposition at drift_density, removal at zero, NaN/-9999 as 0."""
    from chm_gb300.synth import consume_drift
    swe = np.array([100.0, 100.0, 10.0, 50.0, 0.0, 80.0])
    depth = np.array([0.5, 0.5, 0.05, 0.2, 0.0, 0.4])
    dm = np.array([-20.0, 30.0, -10.0, -9999.0, 6.0, np.nan])
    s, d = consume_drift(swe, depth, dm, 300.0)
    np.testing.assert_allclose(s, [80.0, 130.0, 0.0, 50.0, 6.0, 80.0])
    np.testing.assert_allclose(d, [0.5 - 20.0 / 200.0, 0.5 + 30.0 / 300.0, 0.0, 0.2, 6.0 / 300.0, 0.4])


def _deposition_like_system(n_points=3000, seed=5):
    """A deposition-shaped SPD system on a synthetic mesh: diag = area +
    eps sum E/dx, off = -eps E/dx across each shared edge (PBSM3D.cpp:1546-1592)."""
    from chm_gb300 import synth
    w = synth.Workload(n_points, 6000.0, seed=seed)
    m = w.mesh
    nb = np.asarray(m.neighbor)
    E = np.asarray(m.edge_length)
    c = np.asarray(m.center)[:, :2]
    area = np.asarray(m.area)
    off = np.zeros((m.n_faces, 3))
    diag = area.copy()
    for j in range(3):
        k = nb[:, j]
        ok = k >= 0
        wgt = 820.0 * E[ok, j] / np.linalg.norm(c[ok] - c[k[ok]], axis=1)
        diag[ok] += wgt
        off[ok, j] = -wgt
    return nb, diag, off, np.random.default_rng(seed).standard_normal(m.n_faces) * area


def _apply(nb, d, off, v):
    y = d * v
    for j in range(3):
        ok = nb[:, j] >= 0
        y[ok] += off[ok, j] * v[nb[ok, j]]
    return y


@pytest.mark.parametrize("poly", [False, True])
def test_scaled_recurrence_cg_is_the_preconditioned_cg(poly):
    """The persistent deposition CG runs on S A S (S = D^-1/2) with the
    polynomial preconditioner's z carried by z -= alpha M^-1 q.  In exact
    arithmetic its iterates are those of the unscaled preconditioned CG
    (Jacobi, or M^-1 = D^-1 + D^-1 R D^-1); in FP64 both stop at the same
    iteration of the unscaled-residual test and agree to rounding."""
    nb, d, off, b = _deposition_like_system()
    tol = 1e-10
    dinv = 1.0 / d

    def M(r):  # unscaled preconditioner
        if not poly:
            return dinv * r
        acc = r.copy()
        for j in range(3):
            ok = nb[:, j] >= 0
            acc[ok] -= off[ok, j] * dinv[nb[ok, j]] * r[nb[ok, j]]
        return dinv * acc

    x = np.zeros_like(b); r = b.copy(); z = M(r); p = z.copy(); rho = r @ z; bb = b @ b
    for it_ref in range(1, 500):
        q = _apply(nb, d, off, p); al = rho / (p @ q)
        x += al * p; r -= al * q
        if r @ r <= tol * tol * bb:
            break
        z = M(r); rn = r @ z; p = z + rn / rho * p; rho = rn

    s = 1.0 / np.sqrt(d)
    offs = np.zeros_like(off)
    for j in range(3):
        ok = nb[:, j] >= 0
        offs[ok, j] = s[ok] * off[ok, j] * s[nb[ok, j]]

    def shifted(v, sign):  # v + sign * (offs gathered)
        y = v.copy()
        for j in range(3):
            ok = nb[:, j] >= 0
            y[ok] += sign * offs[ok, j] * v[nb[ok, j]]
        return y

    y = np.zeros_like(b); rh = s * b
    zh = shifted(rh, -1.0) if poly else rh.copy()
    ph = zh.copy(); rho = rh @ zh; qh = shifted(ph, 1.0); al = rho / (ph @ qh)
    for it in range(1, 500):
        y += al * ph; rh = rh - al * qh
        zh = zh - al * shifted(qh, -1.0) if poly else rh
        if (rh * rh) @ d <= tol * tol * bb:
            break
        rz = rh @ zh; be = rz / rho; rho = rz
        ph = zh + be * ph; qh = shifted(zh, 1.0) + be * qh; al = rho / (ph @ qh)
    assert it == it_ref
    np.testing.assert_allclose(s * y, x, rtol=0, atol=1e-12 * np.abs(x).max())
    assert np.linalg.norm(b - _apply(nb, d, off, s * y)) <= 1.01 * tol * np.sqrt(bb)


def test_bicgstab_half_step_test():
    """k_bicg_v's FP64 half-step test (van der Vorst 1992, Alg. 1): with
    s = r - alpha v, ||s||^2 = ||r||^2 - 2 alpha (r, v) + alpha^2 (v, v)
    from the dot products the kernel sums, to rounding of ||r||^2; and the
    half-step iterate x + alpha M^-1 p that the column kernel s then stores
    leaves the true residual s.  Nonsymmetric rows (each face's couplings
    scaled differently), right-preconditioned by Jacobi."""
    nb, d, off, _ = _deposition_like_system()
    rng = np.random.default_rng(11)
    offn = off * (0.3 + 0.7 * rng.random(off.shape))
    b = rng.standard_normal(d.size)

    def A(v):
        return _apply(nb, d, offn, v)

    tol = 1e-8
    bb = b @ b
    x = np.zeros_like(b); r = b.copy(); rh = r.copy(); v = np.zeros_like(b); p = np.zeros_like(b)
    rho = alpha = omega = 1.0
    halves = 0
    for it in range(1, 400):
        rho_new = rh @ r
        beta = (rho_new / rho) * (alpha / omega) if it > 1 else 0.0
        rho = rho_new
        p = r + beta * (p - omega * v)
        y = p / d
        v = A(y)
        alpha = rho / (rh @ v)
        rr = r @ r
        s2 = rr - 2.0 * alpha * (r @ v) + alpha * alpha * (v @ v)
        s = r - alpha * v
        assert abs(s2 - s @ s) <= 1e-13 * rr, (it, s2, s @ s, rr)
        # the stop the kernel would take at this half step: true residual = s
        tr = b - A(x + alpha * y)
        assert abs(tr @ tr - s @ s) <= 1e-3 * (s @ s) + 1e-26 * bb, (it, tr @ tr, s @ s)
        halves += 1
        z = s / d
        t = A(z)
        omega = (t @ s) / (t @ t)
        x += alpha * y + omega * z
        r = s - omega * t
        if r @ r <= tol * tol * bb:
            break
    assert r @ r <= tol * tol * bb and halves >= 5


def test_half_step_norm_of_fp32_vectors():
    """Why the mixed form's FP32 inner solve has no half-step test: near its
    target of ~1e-8 ||r||^2, ||r - alpha v||^2 from FP32 sums of (r, r),
    (r, v), (v, v) is off by more than its own size.  FP64 sums of the same
    FP32 vectors (each FP32 product is exact there) would resolve it, but
    cost the FP32 lateral kernel FP64 operations in nearly every iteration
    (measured: the step 3% slower)."""
    rng = np.random.default_rng(4)
    n = 1 << 20
    r = rng.standard_normal(n).astype(np.float32)
    alpha = 0.37
    v = ((r + (1e-4 * rng.standard_normal(n)).astype(np.float32)) / np.float32(alpha)).astype(np.float32)
    r64, v64 = r.astype(np.float64), v.astype(np.float64)
    exact = float(((r64 - alpha * v64) ** 2).sum())
    rr = float(r64 @ r64)
    assert 1e-9 * rr < exact < 1e-7 * rr
    s2 = rr - 2.0 * alpha * float(r64 @ v64) + alpha * alpha * float(v64 @ v64)
    assert abs(s2 - exact) <= 1e-4 * exact
    # the same difference from FP32 sums (numpy's pairwise ones, more
    # accurate than a thread's running sum) misses it by more than its size
    rr32 = float(np.sum(r * r, dtype=np.float32))
    s2_32 = rr32 - 2.0 * alpha * float(np.sum(r * v, dtype=np.float32)) + \
        alpha * alpha * float(np.sum(v * v, dtype=np.float32))
    assert abs(s2_32 - exact) > exact
