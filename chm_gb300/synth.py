"""Seeded synthetic PBSM3D workloads: Delaunay meshes, per-face geometry and
hourly forcing.

The reference quotes no public dataset; its workloads are synthetic meshes
built as follows from one master seed (one numpy stream per quantity):

* points uniform in a square, Delaunay-triangulated (scipy/Qhull), each
  triangle re-oriented counter-clockwise with its neighbour list permuted with
  it, so ``neighbor[3*i+j]`` is the face across the edge opposite vertex j
  (CGAL's ``neighbor(j)``, the convention of CHM's ``.mesh`` files read at
  src/mesh/triangulation.cpp:318-356);
* faces renumbered along a Morton (Z-order) curve of their centroids, so
  neighbouring faces sit close in memory (CHM's mesh permutation tools do the
  same job for its own meshes);
* elevation = sum of 8 random-phase sinusoids (wavelengths log-uniform
  300 m - 3 km, random directions, amplitudes summing to 200 m) + N(0, 5 m);
* forcing per face: 10 m wind ~ Weibull(k=2, scale), converted to the 50 m
  reference height by inverting PBSM3D.cpp:449-463; U_2m_above_srf from the
  no-canopy branch of scale_wind_vert.cpp:131-139; wind direction 270 deg +
  a smooth N(0, 30 deg) field; t ~ U(-15, -2) C; rh ~ U(60, 95) %; snow depth
  lognormal (mean 0.5 m, sigma_log 0.5); swe = 250 kg m^-3 x depth;
  fetch = 1000 m; open terrain (CanopyHeight = 0, LAI = 0).
* step s: t and rh redrawn, wind speed x (1 + 0.2 sin(2 pi s / 24)), wind
  direction rotated +3 deg per step.

Geometry follows src/mesh/triangulation.hpp:1443-1498 (edges, outward unit
normals, lengths), :1577-1589 (centroid) and :1830-1856 (2-D area).
"""
from __future__ import annotations

import dataclasses

import numpy as np

Z_U_R = 50.0
Z0_SNOW = 0.01


@dataclasses.dataclass
class Mesh:
    xyz: np.ndarray        # [nv, 3] float64
    tri: np.ndarray        # [nt, 3] int32, CCW
    neighbor: np.ndarray   # [nt, 3] int32, -1 = none
    edge_length: np.ndarray  # [nt, 3]
    edge_normal: np.ndarray  # [nt, 3, 2]
    area: np.ndarray       # [nt]
    center: np.ndarray     # [nt, 3]
    canopy_height: np.ndarray | None = None
    lai: np.ndarray | None = None
    # subgrid TPI statistics (mesh parameters TPI_mean, TPI_std, TPI_neg_frac,
    # TPI_neg_mean, TPI_neg_std), None = undefined
    tpi_mean: np.ndarray | None = None
    tpi_std: np.ndarray | None = None
    tpi_neg_frac: np.ndarray | None = None
    tpi_neg_mean: np.ndarray | None = None
    tpi_neg_std: np.ndarray | None = None

    @property
    def n_faces(self) -> int:
        return int(self.tri.shape[0])


def face_geometry(xyz: np.ndarray, tri: np.ndarray):
    """Per-face geometry with the operation order of triangulation.hpp."""
    p = [xyz[tri[:, k]] for k in range(3)]
    ex = np.empty((tri.shape[0], 3))
    ey = np.empty((tri.shape[0], 3))
    for i in range(3):
        a = p[(i + 1) % 3]
        b = p[(i + 2) % 3]
        ex[:, i] = b[:, 0] - a[:, 0]
        ey[:, i] = b[:, 1] - a[:, 1]
    normal = np.empty((tri.shape[0], 3, 2))
    length = np.empty((tri.shape[0], 3))
    for i in range(3):
        nx = ey[:, i].copy()
        ny = -ex[:, i]
        i1 = (i + 1) % 3
        D = ex[:, i1] * nx + ey[:, i1] * ny
        flip = D > 0
        nx = np.where(flip, -nx, nx)
        ny = np.where(flip, -ny, ny)
        ln = np.sqrt(nx * nx + ny * ny)
        normal[:, i, 0] = nx / ln
        normal[:, i, 1] = ny / ln
        length[:, i] = np.sqrt(ex[:, i] * ex[:, i] + ey[:, i] * ey[:, i])
    area = ((p[1][:, 0] - p[0][:, 0]) * (p[2][:, 1] - p[0][:, 1])
            - (p[1][:, 1] - p[0][:, 1]) * (p[2][:, 0] - p[0][:, 0])) / 2.0
    center = (p[0] + p[1] + p[2]) / 3.0
    return length, normal, area, center


def _morton_key(x: np.ndarray, y: np.ndarray, bits: int = 16) -> np.ndarray:
    def spread(v):
        v = v.astype(np.uint64)
        out = np.zeros_like(v)
        for b in range(bits):
            out |= ((v >> np.uint64(b)) & np.uint64(1)) << np.uint64(2 * b)
        return out
    scale = (1 << bits) - 1
    xs = (x - x.min()) / max(float(np.ptp(x)), 1e-30) * scale
    ys = (y - y.min()) / max(float(np.ptp(y)), 1e-30) * scale
    return spread(np.round(xs)) | (spread(np.round(ys)) << np.uint64(1))


def streams(seed: int, n: int = 16):
    ss = np.random.SeedSequence(seed)
    return [np.random.default_rng(s) for s in ss.spawn(n)]


# stream ids
S_POINTS, S_ELEV, S_SPEED, S_DIR, S_TRH, S_DEPTH = range(6)


def make_mesh(n_points: int, side: float, seed: int, morton: bool = True) -> Mesh:
    from scipy.spatial import Delaunay

    rs = streams(seed)
    pts = rs[S_POINTS].uniform(0.0, side, size=(n_points, 2))
    # elevation: 8 sinusoids + noise
    re = rs[S_ELEV]
    lam = np.exp(re.uniform(np.log(300.0), np.log(3000.0), 8))
    ang = re.uniform(0, 2 * np.pi, 8)
    phase = re.uniform(0, 2 * np.pi, 8)
    amp = re.uniform(0.5, 1.0, 8)
    amp = amp / amp.sum() * 200.0
    z = np.zeros(n_points)
    for k in range(8):
        proj = pts[:, 0] * np.cos(ang[k]) + pts[:, 1] * np.sin(ang[k])
        z += amp[k] * np.sin(2 * np.pi * proj / lam[k] + phase[k])
    z += re.normal(0.0, 5.0, n_points)
    xyz = np.column_stack([pts, z]).astype(np.float64)

    d = Delaunay(pts)
    tri = d.simplices.astype(np.int64).copy()
    nb = d.neighbors.astype(np.int64).copy()
    # CCW orientation; swapping vertices 1,2 swaps neighbours 1,2
    p0, p1, p2 = xyz[tri[:, 0]], xyz[tri[:, 1]], xyz[tri[:, 2]]
    cross = (p1[:, 0] - p0[:, 0]) * (p2[:, 1] - p0[:, 1]) - (p1[:, 1] - p0[:, 1]) * (p2[:, 0] - p0[:, 0])
    cw = cross < 0
    tri[cw, 1], tri[cw, 2] = tri[cw, 2].copy(), tri[cw, 1].copy()
    nb[cw, 1], nb[cw, 2] = nb[cw, 2].copy(), nb[cw, 1].copy()
    # drop degenerate slivers (zero area) is not needed for random points
    if morton:
        c = (xyz[tri[:, 0]] + xyz[tri[:, 1]] + xyz[tri[:, 2]]) / 3.0
        order = np.argsort(_morton_key(c[:, 0], c[:, 1]), kind="stable")
        inv = np.empty_like(order)
        inv[order] = np.arange(order.size)
        tri = tri[order]
        nb = nb[order]
        nb = np.where(nb >= 0, inv[np.maximum(nb, 0)], -1)
    tri = tri.astype(np.int32)
    nb = nb.astype(np.int32)
    length, normal, area, center = face_geometry(xyz, tri)
    nt = tri.shape[0]
    return Mesh(xyz=xyz, tri=tri, neighbor=nb, edge_length=length, edge_normal=normal, area=area,
                center=center, canopy_height=np.zeros(nt), lai=np.zeros(nt))


def mesh_from_arrays(xyz, tri, neighbor, area=None, canopy_height=None, lai=None) -> Mesh:
    """A mesh as CHM reads it from a .mesh/.param pair (triangulation.cpp:206-356):
    the neighbour list is taken as given; area comes from the 'area' parameter
    when present (triangulation.hpp:1830-1838)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    length, normal, a2, center = face_geometry(xyz, tri)
    if area is None:
        area = a2
    nt = tri.shape[0]
    return Mesh(xyz=xyz, tri=tri, neighbor=np.ascontiguousarray(neighbor, dtype=np.int32), edge_length=length,
                edge_normal=normal, area=np.ascontiguousarray(area, dtype=np.float64), center=center,
                canopy_height=np.zeros(nt) if canopy_height is None else canopy_height,
                lai=np.zeros(nt) if lai is None else lai)


def log_scale_wind(u, z_in, z_out, sd, z0=Z0_SNOW):
    """Atmosphere.cpp:32-38."""
    return u * np.log((z_out - (sd + z0)) / z0) / np.log((z_in - (sd + z0)) / z0)


def _smooth_direction_field(rng, side: float, n: int = 128, sigma_cells: float = 4.0, std_deg: float = 30.0):
    from scipy.ndimage import gaussian_filter

    g = gaussian_filter(rng.normal(size=(n, n)), sigma=sigma_cells, mode="wrap")
    g = (g - g.mean()) / g.std() * std_deg
    return g


def _bilinear(grid: np.ndarray, side: float, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    n = grid.shape[0]
    gx = np.clip(x / side * (n - 1), 0, n - 1 - 1e-9)
    gy = np.clip(y / side * (n - 1), 0, n - 1 - 1e-9)
    i0 = np.floor(gx).astype(np.int64)
    j0 = np.floor(gy).astype(np.int64)
    fx = gx - i0
    fy = gy - j0
    return ((1 - fx) * (1 - fy) * grid[j0, i0] + fx * (1 - fy) * grid[j0, i0 + 1]
            + (1 - fx) * fy * grid[j0 + 1, i0] + fx * fy * grid[j0 + 1, i0 + 1])


@dataclasses.dataclass
class Forcing:
    U_R: np.ndarray
    U_2m_above_srf: np.ndarray
    vw_dir: np.ndarray
    swe: np.ndarray
    t: np.ndarray
    rh: np.ndarray
    snowdepthavg: np.ndarray
    fetch: np.ndarray

    def arrays(self):
        return {k: getattr(self, k) for k in
                ("U_R", "U_2m_above_srf", "vw_dir", "swe", "t", "rh", "snowdepthavg", "fetch")}


class Workload:
    """A mesh plus the forcing generator of one seeded configuration.

    ``forcing(step)`` gives step ``step``'s forcing; ``swe``/``snowdepthavg``
    are the current snow state, which ``apply_drift`` advances like CHM's snow
    models consume ``drift_mass`` (snobal.cpp:363-387: density 250 kg m^-3 on
    erosion, drift_density 300 on deposition)."""

    def __init__(self, n_points: int, side: float, seed: int, wind_scale: float = 8.0, mesh: Mesh | None = None):
        self.seed = seed
        self.side = side
        self.mesh = mesh if mesh is not None else make_mesh(n_points, side, seed)
        nt = self.mesh.n_faces
        rs = streams(seed)
        self.speed10 = rs[S_SPEED].weibull(2.0, nt) * wind_scale
        grid = _smooth_direction_field(rs[S_DIR], side)
        c = self.mesh.center
        self.dir0 = 270.0 + _bilinear(grid, side, c[:, 0], c[:, 1])
        mu = np.log(0.5) - 0.125
        self.depth = rs[S_DEPTH].lognormal(mu, 0.5, nt)
        self.swe = 250.0 * self.depth
        self.trh_seed = rs[S_TRH].integers(0, 2**63 - 1)

    def forcing(self, step: int = 0) -> Forcing:
        nt = self.mesh.n_faces
        r = np.random.default_rng(np.random.SeedSequence([int(self.trh_seed), step]))
        t = r.uniform(-15.0, -2.0, nt)
        rh = r.uniform(60.0, 95.0, nt)
        u10 = self.speed10 * (1.0 + 0.2 * np.sin(2 * np.pi * step / 24.0))
        u10 = np.maximum(u10, 0.05)
        sd = self.depth
        # invert u10 = log_scale_wind(U_R, 50, 10+sd, sd) (PBSM3D.cpp:449-463)
        U_R = u10 * np.log((Z_U_R - (sd + Z0_SNOW)) / Z0_SNOW) / np.log((10.0 + sd - (sd + Z0_SNOW)) / Z0_SNOW)
        U2 = np.maximum(0.1, log_scale_wind(U_R, Z_U_R, sd + 2.0, sd))
        vw_dir = np.mod(self.dir0 + 3.0 * step, 360.0)
        return Forcing(U_R=np.ascontiguousarray(U_R), U_2m_above_srf=np.ascontiguousarray(U2),
                       vw_dir=np.ascontiguousarray(vw_dir), swe=self.swe.copy(), t=t, rh=rh,
                       snowdepthavg=self.depth.copy(), fetch=np.full(nt, 1000.0))

    def apply_drift(self, drift_mass: np.ndarray, drift_density: float = 300.0):
        self.swe, self.depth = consume_drift(self.swe, self.depth, drift_mass, drift_density)


def consume_drift(swe, depth, drift_mass, drift_density: float = 300.0):
    """How CHM's snobal consumes PBSM3D's drift_mass (snobal.cpp:363-387 and
    its _adj_snow): mass 0 when NaN/-9999; the depth change is mass / rho,
    rho the pack's bulk density swe/depth for erosion and drift_density for
    deposition; a pack whose depth or mass reaches 0 is removed."""
    m = np.asarray(drift_mass, dtype=np.float64)
    m = np.where(np.isnan(m) | (np.abs(m + 9999.0) < 1e-5), 0.0, m)
    swe = np.asarray(swe, dtype=np.float64)
    depth = np.asarray(depth, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        rho = np.where((m < 0) & (depth > 0), swe / np.where(depth > 0, depth, 1.0), drift_density)
    new_depth = depth + m / rho
    new_swe = swe + m
    gone = (new_depth <= 0) | (new_swe <= 0)
    return np.where(gone, 0.0, new_swe), np.where(gone, 0.0, new_depth)


# Named configurations of the measurement plan.
CONFIGS = {
    # ~8.1k faces in a 5 km square, 5 layers (CPU reference case)
    "tri8k": dict(n_points=4096, side=5000.0, nLayer=5),
    # ~1.05M faces in a 70 km square, 10 layers
    "tri1m": dict(n_points=524288, side=70000.0, nLayer=10),
    # the same point density at a quarter of the size (~262k faces), for
    # profiler captures that must stay small
    "tri262k": dict(n_points=131072, side=35000.0, nLayer=10),
    # the learned-warm-start configuration's size: ~4.2M faces at the same
    # point density, 10 layers
    "tri4m": dict(n_points=2097152, side=140000.0, nLayer=10),
}
