"""Seeded synthetic scenarios (the reference ships no benchmark inputs).

Each builder returns a :class:`Scenario`: a Morton-ordered :class:`Mesh`,
per-triangle initial values in ANUGA's layout, the boundary objects per tag
and the run length.  The same arrays feed the GPU domain and the CPU oracle.

* :func:`dam_break`      100 x 100 rectangular_cross cells on 100 m x 100 m
  (40,000 triangles), flat bed, stage 1.0 m for x < 50 else 0.5 m, Manning
  n = 0.03, reflective walls, evolve to t = 5 s.
* :func:`tidal_harbour`  Poisson-disk points in 2 km x 1 km, Delaunay
  (~45,000 triangles); bed a Gaussian random field (mean -5 m, sd 3 m,
  correlation length 100 m) clipped at +1 m; stage 0 (dry land at the bed);
  west edge stage 0.5 sin(2 pi t / 600) m, reflective elsewhere; n = 0.025;
  2,000 steps.
* :func:`wet_dry`        1000 x 1000 rectangular_cross cells on 10 km x 10 km
  (4,000,000 triangles); bed a 1:100 beach slope plus Gaussian bumps
  (amplitude 2 m, sigma 200 m); stage 0 with a 2 m Gaussian hump at the
  centre; n uniform in [0.02, 0.04] per triangle; 1,000 steps.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from .boundaries import Reflective_boundary, Time_stage_sine_boundary
from .mesh import Mesh, rectangular_cross

__all__ = ["Scenario", "dam_break", "tidal_harbour", "wet_dry", "poisson_disk",
           "poisson_disk_grid", "harbour_points", "gaussian_random_field", "small_basin"]


@dataclasses.dataclass
class Scenario:
    name: str
    mesh: Mesh
    elevation_vertex: np.ndarray        # (N,3)
    stage_centroid: np.ndarray          # (N,)
    xmom_centroid: np.ndarray
    ymom_centroid: np.ndarray
    friction: np.ndarray                # (N,)
    boundaries: dict                    # tag -> boundary object
    steps: int | None = None
    finaltime: float | None = None

    @property
    def N(self):
        return self.mesh.number_of_elements

    def elevation_arrays(self):
        v = self.elevation_vertex
        c = (v[:, 0] + v[:, 1] + v[:, 2]) / 3.0
        e = np.stack([0.5 * (v[:, 1] + v[:, 2]), 0.5 * (v[:, 0] + v[:, 2]),
                      0.5 * (v[:, 0] + v[:, 1])], axis=1)
        return c, v, e

    def apply_to(self, domain):
        """Load this scenario's initial state into a GPU_domain built on
        ``self.mesh`` (internal order == caller order when the domain was
        built from the Mesh object)."""
        from . import _lib
        from ._lib import check, f64p, lib
        zc, zv, ze = self.elevation_arrays()
        h = domain._h

        def up(q, c, v=None, e=None):
            c = np.ascontiguousarray(c, dtype=np.float64)
            vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
            ee = None if e is None else np.ascontiguousarray(e, dtype=np.float64)
            check(lib().swgpu_set_quantity(h, q, f64p(c), None if vv is None else f64p(vv),
                                           None if ee is None else f64p(ee)), h)

        up(_lib.ELEVATION, zc, zv, ze)
        up(_lib.FRICTION, self.friction)
        for q, c in ((_lib.STAGE, self.stage_centroid), (_lib.XMOMENTUM, self.xmom_centroid),
                     (_lib.YMOMENTUM, self.ymom_centroid)):
            rep = np.repeat(np.asarray(c, dtype=np.float64)[:, None], 3, axis=1)
            up(q, c, rep, rep)
        domain.set_boundary(self.boundaries)

    def apply_to_oracle(self, od, tag_names=None):
        zc, zv, ze = self.elevation_arrays()
        od.set_quantity("elevation", zc, zv, ze)
        od.set_quantity("friction", self.friction)
        for name, c in (("stage", self.stage_centroid), ("xmomentum", self.xmom_centroid),
                        ("ymomentum", self.ymom_centroid)):
            rep = np.repeat(np.asarray(c, dtype=np.float64)[:, None], 3, axis=1)
            od.set_quantity(name, c, rep, rep)

    def oracle_tags(self):
        out = []
        for t in self.mesh.tag_names:
            b = self.boundaries.get(t) or Reflective_boundary()
            out.append((int(b.type), tuple(b.params(self.mesh, t))))
        return out


# ------------------------------------------------------------- generators

def poisson_disk(width, height, r, seed, k=30):
    """Bridson's Poisson-disk sampling in [0,width] x [0,height] with
    minimum spacing r, plus evenly spaced points on the rectangle's edges."""
    rng = np.random.default_rng(seed)
    cell = r / np.sqrt(2.0)
    gw, gh = int(np.ceil(width / cell)), int(np.ceil(height / cell))
    grid = -np.ones((gw, gh), dtype=np.int64)
    pts = []

    def put(p):
        i, j = min(int(p[0] / cell), gw - 1), min(int(p[1] / cell), gh - 1)
        grid[i, j] = len(pts)
        pts.append(p)

    # boundary points first (spacing r), then the interior
    nx_, ny_ = max(int(round(width / r)), 1), max(int(round(height / r)), 1)
    bpts = []
    for t in np.linspace(0, width, nx_ + 1):
        bpts += [(t, 0.0), (t, height)]
    for t in np.linspace(0, height, ny_ + 1)[1:-1]:
        bpts += [(0.0, t), (width, t)]
    for p in bpts:
        put(np.array(p))
    active = list(range(len(pts)))
    margin = 0.5 * r
    while active:
        a = active[rng.integers(len(active))]
        base = pts[a]
        ang = rng.uniform(0, 2 * np.pi, k)
        rad = rng.uniform(r, 2 * r, k)
        cand = base + np.stack([rad * np.cos(ang), rad * np.sin(ang)], axis=1)
        ok = ((cand[:, 0] > margin) & (cand[:, 0] < width - margin) &
              (cand[:, 1] > margin) & (cand[:, 1] < height - margin))
        placed = False
        for c in cand[ok]:
            i, j = int(c[0] / cell), int(c[1] / cell)
            i0, i1 = max(i - 2, 0), min(i + 3, gw)
            j0, j1 = max(j - 2, 0), min(j + 3, gh)
            near = grid[i0:i1, j0:j1]
            near = near[near >= 0]
            if near.size:
                d = np.asarray([pts[q] for q in near]) - c
                if np.min(np.einsum("ij,ij->i", d, d)) < r * r:
                    continue
            put(c)
            active.append(len(pts) - 1)
            placed = True
            break
        if not placed:
            active.remove(a)
    return np.asarray(pts)


def poisson_disk_grid(width, height, r, seed, rounds=30):
    """Poisson-disk points (minimum spacing r) in [0,width] x [0,height] by
    phased dart throwing on a background grid of cells r/sqrt(2) wide, which
    hold at most one point each: every round visits the nine cell classes
    (i mod 3, j mod 3) in turn and throws one uniform dart into every empty
    cell of the class, keeping the darts with no point within r (cells of one
    class lie three cells apart, so the darts of one phase never conflict;
    a point within r lies at most two cells away).  Evenly spaced points on
    the rectangle's edges come first, as in :func:`poisson_disk`.  Vectorised
    over cells: about a second for 10^5 points."""
    rng = np.random.default_rng(seed)
    cell = r / np.sqrt(2.0)
    gw, gh = int(np.ceil(width / cell)), int(np.ceil(height / cell))
    px = np.full((gw + 4, gh + 4), np.nan)   # two guard cells on every side
    py = np.full((gw + 4, gh + 4), np.nan)
    nx_, ny_ = max(int(round(width / r)), 1), max(int(round(height / r)), 1)
    bx = np.linspace(0.0, width, nx_ + 1)
    by = np.linspace(0.0, height, ny_ + 1)[1:-1]
    edge = np.concatenate([np.stack([bx, np.zeros_like(bx)], 1),
                           np.stack([bx, np.full_like(bx, height)], 1),
                           np.stack([np.zeros_like(by), by], 1),
                           np.stack([np.full_like(by, width), by], 1)])
    ei = np.minimum((edge[:, 0] / cell).astype(np.int64), gw - 1) + 2
    ej = np.minimum((edge[:, 1] / cell).astype(np.int64), gh - 1) + 2
    px[ei, ej], py[ei, ej] = edge[:, 0], edge[:, 1]
    margin = 0.5 * r
    offsets = [(di, dj) for di in range(-2, 3) for dj in range(-2, 3) if di or dj]
    for _ in range(rounds):
        for ci in range(3):
            for cj in range(3):
                I, J = np.meshgrid(np.arange(ci, gw) [::3], np.arange(cj, gh)[::3],
                                   indexing="ij")
                I, J = I.ravel() + 2, J.ravel() + 2
                empty = np.isnan(px[I, J])
                I, J = I[empty], J[empty]
                x = (I - 2 + rng.random(I.size)) * cell
                y = (J - 2 + rng.random(J.size)) * cell
                ok = (x > margin) & (x < width - margin) & (y > margin) & (y < height - margin)
                for di, dj in offsets:
                    dx = px[I + di, J + dj] - x
                    dy = py[I + di, J + dj] - y
                    ok &= ~(dx * dx + dy * dy < r * r)   # NaN (empty): no conflict
                px[I[ok], J[ok]], py[I[ok], J[ok]] = x[ok], y[ok]
    inner = ~np.isnan(px)
    inner[ei, ej] = False
    return np.concatenate([edge, np.stack([px[inner], py[inner]], axis=1)])


def gaussian_random_field(shape, spacing, corr, mean, sd, seed):
    """Stationary Gaussian random field on a grid by spectral synthesis with
    a Gaussian covariance of correlation length ``corr``."""
    rng = np.random.default_rng(seed)
    nx, ny = shape
    noise = rng.standard_normal((nx, ny))
    kx = np.fft.fftfreq(nx, d=spacing) * 2 * np.pi
    ky = np.fft.fftfreq(ny, d=spacing) * 2 * np.pi
    K2 = kx[:, None] ** 2 + ky[None, :] ** 2
    filt = np.exp(-K2 * corr * corr / 4.0)
    f = np.real(np.fft.ifft2(np.fft.fft2(noise) * filt))
    f = (f - f.mean()) / (f.std() + 1e-300)
    return mean + sd * f


def _bilinear(field, spacing, x, y):
    nx, ny = field.shape
    fx = np.clip(x / spacing, 0, nx - 1 - 1e-9)
    fy = np.clip(y / spacing, 0, ny - 1 - 1e-9)
    i, j = np.floor(fx).astype(int), np.floor(fy).astype(int)
    tx, ty = fx - i, fy - j
    return ((1 - tx) * (1 - ty) * field[i, j] + tx * (1 - ty) * field[i + 1, j] +
            (1 - tx) * ty * field[i, j + 1] + tx * ty * field[i + 1, j + 1])


def dam_break(m=100, n=100):
    pts, tris, bnd = rectangular_cross(m, n, 100.0, 100.0)
    mesh = Mesh(pts, tris, bnd)
    N = mesh.number_of_elements
    c = mesh.centroid_coordinates
    return Scenario(
        name=f"dam_break_{m}x{n}", mesh=mesh, elevation_vertex=np.zeros((N, 3)),
        stage_centroid=np.where(c[:, 0] < 50.0, 1.0, 0.5), xmom_centroid=np.zeros(N),
        ymom_centroid=np.zeros(N), friction=np.full(N, 0.03),
        boundaries={t: Reflective_boundary() for t in mesh.tag_names}, finaltime=5.0)


def harbour_points(width, height, target_triangles, seed, points="grid"):
    """Seeded Poisson-disk points whose Delaunay triangulation has about
    ``target_triangles`` triangles: ``points="grid"`` the vectorised
    :func:`poisson_disk_grid` (about 0.68 r^-2 points per unit area, 1.96
    triangles per point), ``"bridson"`` the serial :func:`poisson_disk` with
    the spacing rule of the committed golden fixtures (0.70 r^-2, 2 triangles
    per point; about 10% fewer triangles than the target)."""
    if points == "bridson":
        return poisson_disk(width, height, np.sqrt(0.70 * width * height /
                                                    (target_triangles / 2.0)), seed)
    if points != "grid":
        raise ValueError(f"points={points!r}: 'grid' or 'bridson'")
    r = np.sqrt(0.68 * width * height * 1.96 / target_triangles)
    return poisson_disk_grid(width, height, r, seed)


def tidal_harbour(target_triangles=45000, seed=2, width=2000.0, height=1000.0, points="grid"):
    # Delaunay of the Poisson-disk points (~2 triangles per point)
    pts = harbour_points(width, height, target_triangles, seed, points)
    r = np.sqrt(width * height * 1.4 / target_triangles)   # the mean spacing
    from scipy.spatial import Delaunay
    tri = Delaunay(pts).simplices
    V = pts[tri]
    area = 0.5 * np.abs((V[:, 1, 0] - V[:, 0, 0]) * (V[:, 2, 1] - V[:, 0, 1]) -
                        (V[:, 2, 0] - V[:, 0, 0]) * (V[:, 1, 1] - V[:, 0, 1]))
    tri = tri[area > 1e-9 * r * r]
    tmp = Mesh(pts, tri, None, reorder=False)
    # west edge: boundary edges with both end points on x == 0
    boundary = {}
    for (k, e), _ in tmp.boundary.items():
        a, b = tmp.triangles[k, (e + 1) % 3], tmp.triangles[k, (e + 2) % 3]
        boundary[(k, e)] = "west" if pts[a, 0] == 0.0 and pts[b, 0] == 0.0 else "wall"
    mesh = Mesh(pts, tmp.triangles, boundary)
    spacing = 10.0
    field = gaussian_random_field((int(width / spacing) + 2, int(height / spacing) + 2), spacing,
                                  100.0, -5.0, 3.0, seed)
    V = mesh.vertex_coordinates.reshape(-1, 3, 2)
    z = np.minimum(_bilinear(field, spacing, V[..., 0], V[..., 1]), 1.0)
    zc = z.mean(axis=1)
    N = mesh.number_of_elements
    return Scenario(
        name="tidal_harbour", mesh=mesh, elevation_vertex=z,
        stage_centroid=np.maximum(0.0, zc), xmom_centroid=np.zeros(N),
        ymom_centroid=np.zeros(N), friction=np.full(N, 0.025),
        boundaries={"west": Time_stage_sine_boundary(amplitude=0.5, period=600.0),
                    "wall": Reflective_boundary()}, steps=2000)


def wet_dry_bed(rng, length=10000.0):
    """The wet/dry bed as a function of (x, y): a 1:100 beach rising in x
    (the shoreline at 0.8 length) plus 40 Gaussian bumps of +-2 m (sigma 200
    m at 10 km), their centres and signs drawn from ``rng``."""
    nb = 40
    bx, by = rng.uniform(0, length, nb), rng.uniform(0, length, nb)
    amp = 2.0 * rng.choice([-1.0, 1.0], nb)
    sig = 200.0
    scale = length / 10000.0

    def bed(x, y):
        # each bump evaluated only within 6 sigma of its centre
        z = (x - 0.8 * length) / 100.0
        s = sig * scale
        for i in range(nb):
            near = (np.abs(x - bx[i]) < 6 * s) & (np.abs(y - by[i]) < 6 * s)
            dx, dy = x[near] - bx[i], y[near] - by[i]
            z[near] += amp[i] * np.exp(-(dx * dx + dy * dy) / (2 * s * s))
        return z

    return bed


def wet_dry(m=1000, n=None, seed=3, length=10000.0):
    n = m if n is None else n
    pts, tris, bnd = rectangular_cross(m, n, length, length)
    mesh = Mesh(pts, tris, bnd)
    rng = np.random.default_rng(seed)
    bed = wet_dry_bed(rng, length)
    scale = length / 10000.0
    zp = bed(mesh.points[:, 0].copy(), mesh.points[:, 1].copy())
    z = zp[mesh.triangles]
    zc = z.mean(axis=1)
    c = mesh.centroid_coordinates
    r2 = (c[:, 0] - 0.5 * length) ** 2 + (c[:, 1] - 0.5 * length) ** 2
    hump = 2.0 * np.exp(-r2 / (2 * (250.0 * scale) ** 2))
    w = np.maximum(zc, hump)
    N = mesh.number_of_elements
    return Scenario(
        name=f"wet_dry_{m}x{n}", mesh=mesh, elevation_vertex=z, stage_centroid=w,
        xmom_centroid=np.zeros(N), ymom_centroid=np.zeros(N),
        friction=rng.uniform(0.02, 0.04, N),
        boundaries={t: Reflective_boundary() for t in mesh.tag_names}, steps=1000)


def small_basin(m=12, n=10, seed=0, wet_dry_front=True):
    """A small rectangular_cross basin with a sloping, bumpy bed, a partly
    dry beach, random initial momentum and random friction: every branch of
    the limiter, the balance and the flux (wet, dry, shallow) is hit."""
    rng = np.random.default_rng(seed)
    pts, tris, bnd = rectangular_cross(m, n, float(m), float(n))
    bnd = {kk: ("inflow" if t == "left" else t) for kk, t in bnd.items()}
    mesh = Mesh(pts, tris, bnd)
    V = mesh.vertex_coordinates.reshape(-1, 3, 2)
    z = 0.3 * V[..., 0] / m - 0.2 + 0.05 * np.sin(3 * V[..., 1]) * np.cos(2 * V[..., 0])
    zc = z.mean(axis=1)
    N = mesh.number_of_elements
    level = 0.1 if wet_dry_front else 1.0
    w = np.maximum(zc, level + 0.02 * rng.standard_normal(N))
    h = w - zc
    uh = 0.05 * rng.standard_normal(N) * h
    vh = 0.05 * rng.standard_normal(N) * h
    from .boundaries import Dirichlet_boundary
    return Scenario(
        name=f"small_basin_{m}x{n}", mesh=mesh, elevation_vertex=z, stage_centroid=w,
        xmom_centroid=uh, ymom_centroid=vh, friction=rng.uniform(0.0, 0.05, N),
        boundaries={"inflow": Dirichlet_boundary([0.15, 0.0, 0.0]), "right": Reflective_boundary(),
                    "top": Reflective_boundary(), "bottom": Reflective_boundary()}, steps=50)


def channel_inflow(m=14, n=5, seed=0, peak=0.5, rise=2.0):
    """A sloping rectangular_cross channel fed by a triangular inflow
    hydrograph on the left, draining through a transmissive boundary on the
    right, with a transmissive-stage, zero-momentum top and a reflective
    bottom; dry upstream, a shallow pool downstream."""
    from .boundaries import (Inflow_hydrograph_boundary, Transmissive_boundary,
                             Transmissive_stage_zero_momentum_boundary)
    rng = np.random.default_rng(seed)
    pts, tris, bnd = rectangular_cross(m, n, float(m), float(n))
    mesh = Mesh(pts, tris, bnd)
    V = mesh.vertex_coordinates.reshape(-1, 3, 2)
    z = 0.4 - 0.05 * V[..., 0] + 0.02 * np.cos(1.3 * V[..., 1]) * np.sin(0.7 * V[..., 0])
    zc = z.mean(axis=1)
    N = mesh.number_of_elements
    w = np.maximum(zc, 0.05 + 0.01 * rng.standard_normal(N))
    return Scenario(
        name=f"channel_inflow_{m}x{n}", mesh=mesh, elevation_vertex=z, stage_centroid=w,
        xmom_centroid=np.zeros(N), ymom_centroid=np.zeros(N),
        friction=rng.uniform(0.01, 0.04, N),
        boundaries={"left": Inflow_hydrograph_boundary(peak=peak, rise=rise),
                    "right": Transmissive_boundary(),
                    "top": Transmissive_stage_zero_momentum_boundary(),
                    "bottom": Reflective_boundary()}, steps=50)


def inflow_harbour(target_triangles=45000, seed=4, peak=200.0, rise=900.0, friction=0.025,
                   width=2000.0, height=1000.0, points="grid"):
    """The tidal harbour's extent, Delaunay mesh and Gaussian-random-field
    bed (mean -5 m, sd 3 m, correlation 100 m, clipped at +1 m), water at
    rest at level 0, fed through its west edge by a triangular inflow
    hydrograph (``peak`` m^3/s after ``rise`` s, back to 0 after another
    2*rise s), walls elsewhere, uniform Manning ``friction``.  Seeded
    Poisson-disk points (:func:`harbour_points`)."""
    from scipy.spatial import Delaunay
    from .boundaries import Inflow_hydrograph_boundary
    pts = harbour_points(width, height, target_triangles, seed, points)
    tri = Delaunay(pts).simplices
    V = pts[tri]
    area = 0.5 * np.abs((V[:, 1, 0] - V[:, 0, 0]) * (V[:, 2, 1] - V[:, 0, 1]) -
                        (V[:, 2, 0] - V[:, 0, 0]) * (V[:, 1, 1] - V[:, 0, 1]))
    tri = tri[area > 1e-6 * np.median(area)]
    tmp = Mesh(pts, tri, None, reorder=False)
    keys = list(tmp.boundary)
    kk = np.array(keys, dtype=np.int64).reshape(-1, 2)
    a = tmp.triangles[kk[:, 0], (kk[:, 1] + 1) % 3]
    b = tmp.triangles[kk[:, 0], (kk[:, 1] + 2) % 3]
    west = (pts[a, 0] == 0.0) & (pts[b, 0] == 0.0)
    boundary = {k: ("west" if w else "wall") for k, w in zip(keys, west.tolist())}
    mesh = Mesh(pts, tmp.triangles, boundary)
    spacing = 10.0
    field = gaussian_random_field((int(width / spacing) + 2, int(height / spacing) + 2), spacing,
                                  100.0, -5.0, 3.0, seed)
    V = mesh.vertex_coordinates.reshape(-1, 3, 2)
    z = np.minimum(_bilinear(field, spacing, V[..., 0], V[..., 1]), 1.0)
    zc = z.mean(axis=1)
    N = mesh.number_of_elements
    return Scenario(
        name=f"inflow_harbour_{N}", mesh=mesh, elevation_vertex=z,
        stage_centroid=np.maximum(0.0, zc), xmom_centroid=np.zeros(N),
        ymom_centroid=np.zeros(N), friction=np.full(N, float(friction)),
        boundaries={"west": Inflow_hydrograph_boundary(peak=peak, rise=rise),
                    "wall": Reflective_boundary()}, finaltime=3600.0)


def _inflow_harbour_args(args):
    i, seed, n, p, r, f = args
    return inflow_harbour(int(n), seed=int(seed * 100003 + i), peak=p, rise=r, friction=f)


def ensemble_harbour_specs(count=256, seed=4, nmin=5000, nmax=200000):
    """The parameters of ``ensemble_harbours`` without building meshes:
    (index, seed, triangles, peak, rise, friction) per scenario."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(nmin), np.log(nmax), count))
    peaks = rng.uniform(50.0, 500.0, count)
    rises = rng.uniform(300.0, 1800.0, count)
    frics = rng.uniform(0.01, 0.05, count)
    return [(i, seed, n, p, r, f) for i, (n, p, r, f) in
            enumerate(zip(sizes, peaks, rises, frics))]


def ensemble_harbours(count=256, seed=4, nmin=5000, nmax=200000, processes=1, only=None):
    """Ensemble scenarios: ``count`` inflow harbours with triangle counts
    log-uniform in [nmin, nmax], hydrograph peak U[50, 500] m^3/s, rise
    U[300, 1800] s and Manning n U[0.01, 0.05], all drawn from ``seed``.
    ``only`` restricts to those scenario indices (one rank's shard);
    ``processes`` > 1 builds the meshes in a pool of spawned processes."""
    args = ensemble_harbour_specs(count, seed, nmin, nmax)
    if only is not None:
        args = [args[i] for i in only]
    count = len(args)
    if processes and processes > 1 and count > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(min(processes, count)) as pool:
            return pool.map(_inflow_harbour_args, args, chunksize=1)
    return [_inflow_harbour_args(a) for a in args]
