"""CPU tests: the oracle pinned against the reference, its quirks, and the
host-side logic.  No GPU needed."""
import ctypes as C
import math

import numpy as np
import pytest

from chm_gb300 import synth


def test_helpers_pinned_to_reference_source(oracle_lib):
    """log_scale_wind and saturatedVapourPressure against the reference's
    own src/physics/Atmosphere.cpp compiled from source (oracle/_ref)."""
    from oracle import build_oracle, pyoracle
    try:
        build_oracle.build_ref()
    except RuntimeError:
        pass
    ref = pyoracle.ref_atmosphere()
    if ref is None:
        pytest.skip("reference tree not present: helper pin runs where the reference is mounted")
    rng = np.random.default_rng(0)
    for _ in range(2000):
        u = rng.uniform(0, 40)
        sd = rng.uniform(0, 3)
        zout = sd + rng.uniform(0.05, 45)
        z0 = 10 ** rng.uniform(-4, -2)
        a = oracle_lib.oracle_log_scale_wind(u, 50.0, zout, sd, z0)
        b = ref.ref_log_scale_wind(u, 50.0, zout, sd, z0)
        assert a == b or (math.isnan(a) and math.isnan(b))
        T = rng.uniform(230, 300)
        assert oracle_lib.oracle_saturated_vapour_pressure(T) == ref.ref_saturated_vapour_pressure(T)


def test_saturation_vapour_pressure_quirk(oracle_lib):
    """T in K is compared with Tfreeze = 0: the over-water formula always
    applies (Atmosphere.cpp:62-80)."""
    T = 263.15
    expect = 611.21 * math.exp((17.502 * (T - 273.15)) / (240.97 + (T - 273.15)))
    assert oracle_lib.oracle_saturated_vapour_pressure(T) == expect


def test_bearing_to_cartesian(oracle_lib):
    xy = (C.c_double * 2)()
    oracle_lib.oracle_bearing_to_cartesian(0.0, xy)
    assert abs(xy[0]) < 1e-15 and abs(xy[1] - 1) < 1e-15      # north
    oracle_lib.oracle_bearing_to_cartesian(270.0, xy)
    assert abs(xy[0] + 1) < 1e-15 and abs(xy[1]) < 1e-15      # west
    oracle_lib.oracle_bearing_to_cartesian(90.0, xy)
    assert abs(xy[0] - 1) < 1e-15                              # east


def test_std_dry_air_density(oracle_lib):
    rho0 = oracle_lib.oracle_std_dry_air_density(0.0, 288.15)
    assert abs(rho0 - 101325.0 / (287.058 * 288.15)) < 1e-15
    # decreases with altitude; about 1.007 kg m^-3 at 2 km and 15 C
    assert 0.95 < oracle_lib.oracle_std_dry_air_density(2000.0, 288.15) < 1.05


def _random_mesh(seed=0, n=300):
    return synth.make_mesh(n, 1000.0, seed)


def test_face_geometry_matches_numpy(oracle_lib):
    from oracle.pyoracle import ptr
    m = _random_mesh()
    nt, nv = m.n_faces, m.xyz.shape[0]
    E = np.empty(3 * nt)
    N = np.empty(6 * nt)
    A = np.empty(nt)
    Cc = np.empty(3 * nt)
    xyz = np.ascontiguousarray(m.xyz)
    tri = np.ascontiguousarray(m.tri)
    oracle_lib.oracle_face_geometry(nv, ptr(xyz), nt, ptr(tri, C.c_int32), ptr(E), ptr(N), ptr(A), ptr(Cc))
    np.testing.assert_array_equal(E, m.edge_length.ravel())
    np.testing.assert_array_equal(N, m.edge_normal.ravel())
    np.testing.assert_array_equal(A, m.area)
    np.testing.assert_array_equal(Cc, m.center.ravel())
    assert (A > 0).all()
    # outward normals: pointing away from the centroid
    for j in range(3):
        a = m.xyz[m.tri[:, (j + 1) % 3], :2]
        mid = a + 0.5 * (m.xyz[m.tri[:, (j + 2) % 3], :2] - a)
        assert (np.einsum("ij,ij->i", m.edge_normal[:, j], mid - m.center[:, :2]) > 0).all()


def _neighbors(oracle_lib, nv, tri):
    from oracle.pyoracle import ptr
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    out = np.empty(tri.size, np.int32)
    assert oracle_lib.oracle_face_neighbors(nv, tri.shape[0], ptr(tri, C.c_int32), ptr(out, C.c_int32)) == 0
    return out.reshape(-1, 3)


@pytest.mark.parametrize("fixture", ["slope_mesh.npz", "granger1m_mesh.npz"])
def test_adjacency_pinned_to_reference_meshes(oracle_lib, fixture):
    """The neighbour convention (neighbor(j) across the edge opposite vertex
    j, -1 on the boundary) reproduces the reference meshes' own 'neigh'
    lists bit for bit."""
    from conftest import GOLDEN
    d = np.load(GOLDEN / fixture)
    nb = _neighbors(oracle_lib, d["vertex"].shape[0], d["elem"])
    np.testing.assert_array_equal(nb, d["neigh"])


def test_synthetic_neighbors_follow_the_convention(oracle_lib):
    m = _random_mesh(3, 2000)
    nb = _neighbors(oracle_lib, m.xyz.shape[0], m.tri)
    np.testing.assert_array_equal(nb, m.neighbor)


def test_oracle_golden_fixture(oracle_lib):
    from conftest import GOLDEN
    from oracle import pyoracle
    d = np.load(GOLDEN / "oracle_small.npz")
    w = synth.Workload(int(d["n_points"]), float(d["side"]), seed=int(d["seed"]))
    f = {k[3:]: d[k] for k in d.files if k.startswith("in_")}
    np.testing.assert_array_equal(f["U_R"], w.forcing(0).U_R)
    out, _ = pyoracle.Oracle(w.mesh, nLayer=int(d["nLayer"])).step_exact(f, 3600.0)
    for k in out:
        ref = d["out_" + k]
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(out[k] - ref).max() <= 1e-12 * scale, k


def test_reference_solver_settings_reach_exact_solution(oracle_lib):
    """GMRES(30) + ILUT(1e-4, 3), tol 1e-8, x0 = 0 (LinearAlgebra.cpp:164-187)
    lands within 1e-6 of the direct solve."""
    from oracle import pyoracle
    w = synth.Workload(1024, 2500.0, seed=2)
    f = w.forcing(0)
    a, st = pyoracle.Oracle(w.mesh, nLayer=5).step(f, 3600.0)
    b, _ = pyoracle.Oracle(w.mesh, nLayer=5).step_exact(f, 3600.0)
    assert st["susp_rel_residual"] <= 1e-8 and st["susp_iters"] > 0
    for k in ("c", "Qsusp", "drift_mass"):
        assert np.abs(a[k] - b[k]).max() <= 1e-6 * np.abs(b[k]).max(), k


def test_suspension_stencil_and_signs(oracle_lib):
    """Graph: self, present lateral neighbours, below, above; the column is
    an M-matrix pattern (negative diagonal, non-negative off-diagonals)."""
    from oracle import pyoracle
    w = synth.Workload(400, 1200.0, seed=6)
    L = 4
    o = pyoracle.Oracle(w.mesh, nLayer=L)
    o.assemble(w.forcing(0), 3600.0)
    rp, cols, vals, rhs, _ = o.raw_system(0)
    T = w.mesh.n_faces
    for r in range(0, T * L, 37):
        z, i = divmod(r, T)
        c = cols[rp[r]:rp[r + 1]]
        expect = [r] + [z * T + n for n in w.mesh.neighbor[i] if n >= 0]
        if z > 0:
            expect.append(r - T)
        if z < L - 1:
            expect.append(r + T)
        assert list(c) == expect
        v = vals[rp[r]:rp[r + 1]]
        assert v[0] < 0 and (v[1:] >= 0).all()
    # right-hand side only in the bottom layer (saltation boundary)
    assert np.abs(rhs[T:]).max() == 0 and np.abs(rhs[:T]).max() > 0


def test_deposition_matrix_is_spd(oracle_lib):
    import scipy.sparse as sp
    from oracle import pyoracle
    w = synth.Workload(600, 1500.0, seed=8)
    o = pyoracle.Oracle(w.mesh, nLayer=3)
    o.step_exact(w.forcing(0), 3600.0)
    D, b, _ = o.system(1)
    assert abs(D - D.T).max() <= 1e-12 * abs(D).max()
    lap = D - sp.diags(w.mesh.area)
    np.testing.assert_allclose(np.asarray(lap.sum(axis=1)).ravel(), 0.0, atol=1e-9 * abs(D).max())
    assert np.linalg.eigvalsh(D.toarray()).min() > 0


def test_tanh_fetch_quirk(oracle_lib):
    """With fetch <= 300 m c_salt is scaled by the constant
    0.5 tanh(0.01333*300 - 2) + 0.5, not by a function of fetch (PBSM3D.cpp:839-845)."""
    from oracle import pyoracle
    w = synth.Workload(400, 1200.0, seed=1, wind_scale=14.0)
    f = w.forcing(0).arrays()
    lc = 0.5 * math.tanh(0.1333333333e-1 * 300 - 2.0) + 0.5
    res = {}
    for fetch in (1000.0, 250.0, 50.0):
        g = dict(f, fetch=np.full_like(f["fetch"], fetch))
        o = pyoracle.Oracle(w.mesh, nLayer=3)
        o.assemble(g, 3600.0)
        res[fetch] = o.face_fields()["c_salt"]
    on = res[1000.0] > 0
    assert on.sum() > 10
    np.testing.assert_allclose(res[250.0][on] / res[1000.0][on], lc, rtol=1e-14)
    np.testing.assert_array_equal(res[250.0], res[50.0])


def test_hs_set_before_c_salt_reset(oracle_lib):
    """hs comes from u* before c_salt < 0 can clear saltation
    (PBSM3D.cpp:762-824): such faces keep hs > 0 with saltation false."""
    from oracle import pyoracle
    w = synth.Workload(400, 1200.0, seed=1, wind_scale=6.0)
    n = w.mesh.n_faces
    mesh = w.mesh
    mesh.canopy_height = np.full(n, 0.0) + w.depth + 0.2   # vegetation 0.2 m above the snow
    mesh.lai = np.full(n, 3.0)
    o = pyoracle.Oracle(mesh, nLayer=3)
    o.assemble(w.forcing(0), 3600.0)
    ff = o.face_fields()
    quirk = (ff["hs"] > 0) & (ff["saltation"] == 0)
    assert quirk.any()
    assert (ff["c_salt"][quirk] == 0).all()


def test_drift_mass_kept_without_deposition_and_flag_sticky(oracle_lib):
    from oracle import pyoracle
    w = synth.Workload(400, 1200.0, seed=2, wind_scale=12.0)
    o = pyoracle.Oracle(w.mesh, nLayer=3)
    f = w.forcing(0).arrays()
    f["swe"] = np.full_like(f["swe"], 0.5)     # little snow: erosion is capped
    out, st = o.step_exact(f, 3600.0)
    assert st["deposition_present"]
    assert (out["pbsm_more_than_avail"] == 1).any()
    flagged = out["pbsm_more_than_avail"] == 1
    calm = dict(f, U_R=np.full_like(f["U_R"], 0.05), U_2m_above_srf=np.full_like(f["U_R"], 0.05))
    out2, st2 = o.step_exact(calm, 3600.0)
    assert not st2["suspension_present"] and not st2["deposition_present"]
    np.testing.assert_array_equal(out2["drift_mass"], out["drift_mass"])     # not rewritten
    assert (out2["pbsm_more_than_avail"][flagged] == 1).all()                # never reset
    np.testing.assert_array_equal(out2["sum_drift"], out["sum_drift"])


def test_mass_ledger_oracle(oracle_lib):
    from oracle import pyoracle
    w = synth.Workload(800, 2000.0, seed=4)
    _, st = pyoracle.Oracle(w.mesh, nLayer=4).step_exact(w.forcing(0), 3600.0)
    assert abs(st["ledger_deposited"] - st["ledger_divergence"]) <= 1e-10 * st["ledger_snow_mass"]


def test_mlp_oracle_gradients(oracle_lib):
    """The FP64 MLP reference used to check the GPU training kernels:
    analytic gradients against central differences."""
    from oracle.pyoracle import ptr
    rng = np.random.default_rng(0)
    n = 16
    dims = [(128, 14), (128, 128), (128, 128), (1, 128)]
    W = [(rng.normal(size=d) / np.sqrt(d[1])).astype(np.float32) for d in dims]
    B = [rng.normal(size=d[0]).astype(np.float32) * 0.1 for d in dims]
    x = rng.normal(size=(n, 14)).astype(np.float32)
    t = rng.normal(size=n).astype(np.float32)
    G = [np.empty(d) for d in dims]
    GB = [np.empty(d[0]) for d in dims]
    fp = C.c_float

    def loss(Wl, grads=True):
        args = [n, ptr(x, fp), ptr(t, fp)]
        for w, b in zip(Wl, B):
            args += [ptr(w, fp), ptr(b, fp)]
        args += sum(([ptr(g), ptr(gb)] if grads else [None, None] for g, gb in zip(G, GB)), [])
        args.append(None)
        return oracle_lib.oracle_mlp_loss_grad(*args)

    loss(W)
    for li, (o_, k_) in [(0, (3, 5)), (1, (7, 9)), (3, (0, 11))]:
        h = 1e-2
        Wp = [w.copy() for w in W]
        Wm = [w.copy() for w in W]
        Wp[li][o_, k_] += h
        Wm[li][o_, k_] -= h
        fd = (loss(Wp, False) - loss(Wm, False)) / (2 * h)
        assert abs(fd - G[li][o_, k_]) <= 1e-3 * max(1.0, abs(fd)), (li, fd, G[li][o_, k_])


def _ustar_g(u2, lam, u):
    return u2 * 0.4 / math.log(2.0 / (0.6131702345e-2 * u * u + 0.5 * lam)) - u


def test_coupled_ustar_root(oracle_lib):
    """z0_ustar_coupling's u* (Li and Pomeroy 2000 eqn 5, PBSM3D.cpp:691-712)
    against scipy's brentq on the physical root: the first sign change of the
    falling g(u) = u2 kappa / log(2/(c u^2 + lambda/2)) - u above 0.  The
    reference's TOMS 748 midpoint lies within 5e-9 of the same root."""
    from scipy.optimize import brentq
    out = C.c_double()
    for u2 in (0.3, 1.0, 3.0, 7.5, 12.0, 20.0, 30.0):
        for lam in (0.0, 0.01, 0.2, 1.0):
            assert oracle_lib.oracle_coupled_ustar(u2, lam, C.byref(out)) == 1
            # bracket the first sign change on a fine grid below the pole of g
            grid = np.geomspace(1e-6, 50.0, 20000)
            vals = np.array([_ustar_g(u2, lam, u) for u in grid])
            k = int(np.argmax(vals < 0))
            r = brentq(lambda u: _ustar_g(u2, lam, u), grid[k - 1], grid[k], xtol=1e-15, rtol=1e-15)
            assert abs(out.value - r) <= 1e-13 * r, (u2, lam, out.value, r)


def test_coupled_ustar_edges(oracle_lib):
    out = C.c_double()
    # no wind: g(u) = -u everywhere, the walk descends to the root 0
    assert oracle_lib.oracle_coupled_ustar(0.0, 0.1, C.byref(out)) == 1
    assert 0.0 <= out.value < 1e-300
    # lambda/2 > 2: the logarithm is negative everywhere, g < 0, root 0
    assert oracle_lib.oracle_coupled_ustar(5.0, 5.0, C.byref(out)) == 1
    assert 0.0 <= out.value < 1e-300
    # NaN wind: no sign change within the 500 evaluations, u* keeps its placeholder
    assert oracle_lib.oracle_coupled_ustar(float("nan"), 0.1, C.byref(out)) == 0


def _ice_bulb_newton(T, t, ea, D, lt, L):
    """The Newton iteration of iterative_subl restated in Python: start at T,
    stop after the first step no larger than |Ti| 2^-5."""
    mw, R = 18.01528, 0.00831441
    rho = mw * ea / (R * t)
    x, lo, hi = T, -50.0, 0.0
    for _ in range(100):
        e = math.exp(17.3 * x / (237.3 + x))
        sat = 0.611 * mw * e / (R * (x + 273.15) * 1000.0)
        f = T + D * L * (rho / 1000.0 - sat) / lt - x
        if f == 0:
            break
        df = -D * L * sat * (17.3 * 237.3 / (237.3 + x) ** 2 - 1.0 / (x + 273.15)) / lt - 1.0
        frm = x
        step = f / df
        x = frm - step
        if x <= lo:
            step = 0.5 * (frm - lo)
            x = frm - step
        elif x >= hi:
            step = 0.5 * (frm - hi)
            x = frm - step
        if step > 0:
            hi = frm
        else:
            lo = frm
        if not abs(x / 32.0) < abs(step):
            break
    return x


def test_ice_bulb_temperature(oracle_lib):
    """iterative_subl's Ti (PBSM3D.cpp:1062-1096): the oracle against the
    Newton restatement above, and within |Ti|/32 of scipy's root (the loose
    stopping rule of 6 binary digits)."""
    from scipy.optimize import brentq
    rng = np.random.default_rng(3)
    for _ in range(300):
        T = rng.uniform(-30, -0.5)
        rh = rng.uniform(0.4, 1.0)
        t = T + 273.15
        es = oracle_lib.oracle_saturated_vapour_pressure(t)
        ea = rh * es / 1000.0
        D = 2.06e-5 * (t / 273.15) ** 1.75
        lt = 0.000063 * t + 0.00673
        L = 2.838e6
        Ti = oracle_lib.oracle_ice_bulb_temperature(T, t, ea, D, lt, L)
        ref = _ice_bulb_newton(T, t, ea, D, lt, L)
        assert abs(Ti - ref) <= 1e-12 * abs(ref), (T, Ti, ref)
        mw, R = 18.01528, 0.00831441

        def f(x):
            return T + D * L * (mw * ea / (R * t) / 1000.0
                                - 0.611 * mw * math.exp(17.3 * x / (237.3 + x)) / (R * (x + 273.15) * 1000.0)) / lt - x
        root = brentq(f, -60.0, 5.0)
        assert abs(Ti - root) <= abs(Ti) / 32.0


def test_incomplete_gamma_and_density(oracle_lib):
    """use_subgrid_topo's gamma functions (gsl_cdf_gamma_P/Q,
    gsl_ran_gamma_pdf; PBSM3D.cpp:615-639) against scipy.special over the
    shapes the branch produces (TPI_neg_mean^2 / TPI_neg_std^2 in [1e-4, 1e4])."""
    from scipy import special
    rng = np.random.default_rng(5)
    P, Q = C.c_double(), C.c_double()
    for _ in range(3000):
        a = 10 ** rng.uniform(-4, 4)
        x = a * 10 ** rng.uniform(-2, 0.7) if rng.random() < 0.8 else 10 ** rng.uniform(-3, 3)
        oracle_lib.oracle_incomplete_gamma(a, x, C.byref(P), C.byref(Q))
        assert abs(P.value - special.gammainc(a, x)) < 5e-12, (a, x)
        assert abs(Q.value - special.gammaincc(a, x)) < 5e-12, (a, x)
    for _ in range(1000):
        a, b, x = 10 ** rng.uniform(-4, 4), 10 ** rng.uniform(-3, 1), 10 ** rng.uniform(-3, 1)
        ref = np.exp(special.xlogy(a - 1, x) - x / b - special.gammaln(a) - a * np.log(b))
        if ref > 1e-250:
            assert abs(oracle_lib.oracle_gamma_pdf(x, a, b) - ref) <= 1e-10 * ref


def _v2_reference(sd, m, s, min_sd, epsrel):
    """use_subgrid_topo_V2 (PBSM3D.cpp:486-597) with scipy's QUADPACK QAGS
    (the algorithm gsl_integration_qags implements) and brentq."""
    from scipy import integrate, optimize
    a1, b1, a2, b2, fac = 1.5, 0.3, 0.6, 0.55, 0.8
    m = max(-5.0, min(5.0, m))
    s = min(5.0, max(0.1, s))

    def pdf(x):
        return math.exp(-((x - m) / s) ** 2 / 2) / (math.sqrt(2 * math.pi) * s)

    def F(x):
        return (1 - a1 * math.tanh(b1 * (x + 0.25))) if x + 0.25 <= 0 else (1 - a2 * math.tanh(b2 * (x + 0.25)))

    q = dict(epsabs=0, epsrel=epsrel, limit=5000)
    res = integrate.quad(lambda x: F(x) * pdf(x), -50, 50, points=[-0.25, m], **q)[0]

    def fr(xx):
        return (1 - a1 * math.tanh(b1 * (xx + 0.25))) * sd / res + fac * xx
    lo = -1.0
    while fr(lo) > 0:
        lo *= 2
    tl = optimize.brentq(fr, lo, 0.0, xtol=1e-15)
    pts = [p for p in (-0.25, m) if -50 < p < tl]
    h1 = integrate.quad(lambda x: F(x) * sd / res * pdf(x), -50, tl, points=pts or None, **q)[0]
    h2 = integrate.quad(lambda x: -fac * x * pdf(x), tl, -min_sd / fac, **q)[0]
    h3 = min_sd * 0.5 * math.erfc((-min_sd / fac - m) / (s * math.sqrt(2)))
    return min(h1 + h2 + h3, sd), 0.5 * math.erfc((tl - m) / (s * math.sqrt(2))), tl, res


def test_subgrid_v2_face(oracle_lib):
    """The oracle's V2 holding capacity, contributing fraction, threshold and
    normalisation integral against QUADPACK run tight; the reference's QAGS at
    its relative 1e-7 stays within a few 1e-7 of them."""
    from chm_gb300 import capi
    lib = capi.load()
    cfg = capi.default_config(lib, use_subgrid_topo_V2=1)
    out, tpi = (C.c_double * 5)(), (C.c_double * 5)()
    rng = np.random.default_rng(6)
    for _ in range(150):
        sd, m, s = rng.uniform(0.11, 3.0), rng.uniform(-6, 6), 10 ** rng.uniform(-1.2, 0.8)
        tpi[0], tpi[1] = m, s
        tpi[2] = tpi[3] = tpi[4] = float("nan")
        oracle_lib.oracle_subgrid_face(C.byref(cfg), sd, tpi, out)
        got = (out[0], out[1], out[3], out[4])
        tight = _v2_reference(sd, m, s, 0.1, 2e-14)
        for g, r in zip(got, tight):
            assert abs(g - r) <= 1e-10 * max(abs(r), 1e-3), (sd, m, s, got, tight)
        loose = _v2_reference(sd, m, s, 0.1, 1e-7)
        for g, r in zip(got, loose):
            assert abs(g - r) <= 5e-7 * max(abs(r), 1e-3)
    # undefined TPI_std: defaults; snow at most min_sd_trans: no integrals
    tpi[1] = -9999.0
    oracle_lib.oracle_subgrid_face(C.byref(cfg), 1.0, tpi, out)
    assert (out[0], out[1], out[3], out[4]) == (0.1, 1.0, -0.1, -9999.0)
    tpi[0], tpi[1] = 0.5, 1.0
    oracle_lib.oracle_subgrid_face(C.byref(cfg), 0.05, tpi, out)
    assert out[0] == 0.1 and out[4] == -9999.0
    assert abs(out[1] - 0.5 * math.erfc((-0.1 - 0.5) / math.sqrt(2))) < 1e-15


def test_subgrid_v1_face(oracle_lib):
    """use_subgrid_topo (PBSM3D.cpp:604-645) against the same closed forms
    evaluated with scipy.special."""
    from scipy import special
    from chm_gb300 import capi
    cfg = capi.default_config(capi.load(), use_subgrid_topo=1)
    out, tpi = (C.c_double * 5)(), (C.c_double * 5)()
    rng = np.random.default_rng(7)
    msd = 0.1
    for _ in range(500):
        sd = rng.uniform(0, 3.0)
        fn, mn, sn = rng.uniform(0, 1), rng.uniform(-12, 0), 10 ** rng.uniform(-1.3, 0.8)
        tpi[0] = tpi[1] = float("nan")
        tpi[2], tpi[3], tpi[4] = fn, mn, sn
        oracle_lib.oracle_subgrid_face(C.byref(cfg), sd, tpi, out)
        mn_c, sn_c = max(-10.0, min(-0.05, mn)), min(5.0, max(0.1, sn))
        k, th = mn_c ** 2 / sn_c ** 2, -sn_c ** 2 / mn_c

        def gP(x):
            return special.gammainc(k, x / th)

        def gQ(x):
            return special.gammaincc(k, x / th)

        def pdf(x):
            return np.exp(special.xlogy(k - 1, x / th) - x / th - special.gammaln(k)) / th
        frac = (1 - fn) + fn * gP(sd)
        hold = msd
        if sd > msd:
            hint = k * th - th * (sd * pdf(sd) - msd * pdf(msd) + k * gP(msd) + k * gQ(sd))
            hold = (1 - fn) * msd + fn * (msd * gP(msd) + hint + sd * gQ(sd))
        assert abs(out[1] - frac) < 1e-11 and abs(out[2] - (1 - fn)) < 1e-15
        assert abs(out[0] - hold) <= 1e-9 * max(1.0, abs(hold)), (sd, fn, mn, sn, out[0], hold)


def test_expint_e1(oracle_lib):
    """The exponential integral of the thin-plate-spline basis against scipy."""
    from scipy import special
    for x in np.concatenate([np.geomspace(1e-8, 700, 400), [0.5, 1.0, 1.0000001, 2.0]]):
        ref = special.exp1(x)
        assert abs(oracle_lib.oracle_expint_e1(x) - ref) <= 1e-14 * ref + 1e-300, x


def _tps_numpy(sx, sy, sz, qx, qy):
    """interpolation/TPSpline.cpp:55-157 with numpy (dense solve)."""
    from scipy import special
    n = len(sx)

    def basis(dx, dy):
        d = math.hypot(dx, dy)
        d = (d * 0.01 / 2.0) ** 2
        return -(math.log(d) + 0.577215 + special.exp1(d))
    A = np.zeros((n + 1, n + 1))
    for i in range(n):
        for j in range(i + 1, n):
            A[i, j + 1] = A[j, i + 1] = basis(sx[i] - sx[j], sy[i] - sy[j])
    A[:, 0] = 1
    A[n, :] = 1
    A[n, 0] = 0
    b = np.append(np.asarray(sz, float), 0.0)
    x = np.linalg.solve(A, b)
    return x[0] + sum(x[i + 1] * basis(sx[i] - qx, sy[i] - qy) for i in range(n))


def test_thin_plate_spline(oracle_lib):
    rng = np.random.default_rng(8)
    dp = C.POINTER(C.c_double)
    for n in (1, 2, 3):
        for _ in range(200):
            sx, sy = rng.uniform(0, 300, n), rng.uniform(0, 300, n)
            sz = rng.uniform(0.1, 15, n)
            qx, qy = rng.uniform(0, 300), rng.uniform(0, 300)
            a = [np.ascontiguousarray(v) for v in (sx, sy, sz)]
            got = oracle_lib.oracle_tps(*[v.ctypes.data_as(dp) for v in a], n, qx, qy)
            ref = _tps_numpy(sx, sy, sz, qx, qy)
            assert abs(got - ref) <= 1e-9 * max(1.0, abs(ref)), (n, got, ref)
    # interpolates its samples
    sx, sy, sz = np.array([0., 100., 30.]), np.array([0., 10., 90.]), np.array([3., 5., 7.])
    a = [np.ascontiguousarray(v) for v in (sx, sy, sz)]
    for k in range(3):
        got = oracle_lib.oracle_tps(*[v.ctypes.data_as(dp) for v in a], 3, sx[k] + 1e-9, sy[k])
        assert abs(got - sz[k]) < 1e-5


def test_wind_modules_oracle(oracle_lib):
    """scale_wind_vert keeps U_2m within the neighbours' range and at least
    0.1 m/s; fetchr is max_distance on flat open ground, 0 under tall canopy,
    and shortens upwind of a ridge."""
    from oracle import pyoracle
    w = synth.Workload(600, 1500.0, seed=2)
    o = pyoracle.Oracle(w.mesh, nLayer=3)
    f = w.forcing(0)
    u2 = o.scale_wind_vert(f.U_R, f.snowdepthavg)
    assert (u2 >= 0.1).all() and np.isfinite(u2).all()
    n = w.mesh.n_faces
    flat = synth.Workload(600, 1500.0, seed=2)
    flat.mesh.center = flat.mesh.center.copy()
    flat.mesh.center[:, 2] = 0.0
    of = pyoracle.Oracle(flat.mesh, nLayer=3)
    fe = of.fetchr(np.full(n, 270.0), incl_veg=False)
    assert (fe == 1000.0).all()
    tall = synth.Workload(600, 1500.0, seed=2)
    tall.mesh.canopy_height = np.full(n, 2.0)
    ot = pyoracle.Oracle(tall.mesh, nLayer=3)
    assert (ot.fetchr(np.full(n, 270.0)) == 0.0).all()
    # a ridge to the west: faces east of it see a short fetch from 270 deg
    ridge = synth.Workload(600, 1500.0, seed=2)
    ridge.mesh.center = ridge.mesh.center.copy()
    x = ridge.mesh.center[:, 0]
    ridge.mesh.center[:, 2] = np.where(np.abs(x - 500.0) < 60.0, 100.0, 0.0)
    orr = pyoracle.Oracle(ridge.mesh, nLayer=3)
    fr = orr.fetchr(np.full(n, 270.0), incl_veg=False)
    east = (x > 600) & (x < 900)
    assert (fr[east] < 1000.0).mean() > 0.9
    assert (fr[x < 400] == 1000.0).mean() > 0.9
