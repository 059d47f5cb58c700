"""BF16 surrogate of the solver's maximum depth and arrival time, with the
solver as its fallback and its check.

The scenario family shares one mesh and bed: the wet/dry beach with bumps
(a 1:100 beach rising to the east, the shoreline at x = 8 km, 40 seeded
bumps of +-2 m) on ``cells`` x ``cells`` rectangular_cross cells over
10 km x 10 km (200,704 triangles at 224).  Scenarios differ in 9
parameters:

* an inflow hydrograph through a 1 km segment of the east (land) edge: peak
  discharge, rise time and total duration (a triangular hydrograph);
* Manning's n, uniform over the mesh;
* five coefficients c0..c4 of the stage on the west (sea) edge,
  c0 + c1 sin(wt) + c2 cos(wt) + c3 sin(2wt) + c4 cos(2wt) with the period
  of the principal lunar tide, 12.42 h (the tide and its first overtide):
  over the one-hour run a slowly changing sea level; the sea starts at rest
  at the boundary's stage at t = 0.

The solver (an ``Ensemble`` with per-triangle tracking) gives, per scenario
and triangle, the maximum depth and the first time the depth exceeded a
threshold.  The network (``libswgpu`` ``swgpu_mlp_*``: 16 -> 256 -> 256 ->
256 -> 3, BF16 on tcgen05 tensor cores) learns both from the scenario
parameters and the triangle's centroid, bed and distance to the inflow (the
depth as its excess over the still-water depth at the highest tide, which
the parameters fix), and a third output learns the absolute error
of its depth.

``fallback`` turns predictions into an answer within a depth tolerance:
blocks of 256 triangles (Morton order: compact patches of the mesh) whose
calibrated error estimate exceeds the tolerance are re-solved by the solver
on a window of the mesh: east of the westmost flagged block and, in y, the
span of the flagged blocks and the inflow segment, each with a margin.  The
window's west cut carries the tide delayed by the long-wave travel time to
it (the sea's still level there, the tide being slow), its north and south
cuts are walls.  Leaving out the deep sea, which sets the solver's CFL
step, the window needs several times fewer steps as well as fewer
triangles.  The window's values replace the predictions in the flagged
blocks.  ``evaluate`` reports the
time to the answer against the solver alone, and the answer's error against
the full solve.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import lib
from .boundaries import (Inflow_hydrograph_boundary, Reflective_boundary,
                         Time_stage_fourier_boundary)
from .config import DEFAULT
from .ensemble import ALIGN, Ensemble
from .mesh import Mesh, rectangular_cross
from .scenarios import Scenario, wet_dry_bed

__all__ = ["PARAM_NAMES", "PARAM_RANGES", "FamilyMesh", "sample_params", "family_scenario",
           "solve", "Surrogate", "init_params", "initial_depth", "static_depth", "max_tide",
           "targets_from",
           "block_index", "calibrate", "window_scenarios", "shifted_tide", "fallback", "evaluate",
           "FINALTIME", "TIDE_PERIOD", "THRESHOLD", "DEPTH_SCALE", "NEVER"]

PARAM_NAMES = ("peak", "rise", "duration", "manning", "c0", "c1", "c2", "c3", "c4")
PARAM_RANGES = np.array([(50.0, 500.0), (300.0, 1800.0), (450.0, 5400.0), (0.01, 0.05),
                         (-0.5, 0.5), (-0.4, 0.4), (-0.4, 0.4), (-0.4, 0.4), (-0.4, 0.4)])
DURATION_RATIO = (1.5, 3.0)     # duration / rise
TIDE_PERIOD = 44712.0           # s: the M2 tide (12.42 h)
FINALTIME = 3600.0              # s
THRESHOLD = 0.02                # m: depth that counts as arrival
INFLOW_Y = (4500.0, 5500.0)     # the inflow segment of the east edge, m
F, H, OUT = 16, 256, 3
DEPTH_SCALE = 1.0   # depth target: (max depth - still depth at the highest tide) / DEPTH_SCALE
NEVER = 1.25        # arrival target (arrival / finaltime) of a triangle that stays dry


def _f32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class FamilyMesh:
    """The shared mesh and bed, and the per-triangle feature table."""

    def __init__(self, cells=224, seed=3, length=10000.0):
        pts, tris, bnd = rectangular_cross(cells, cells, length, length)
        y0, y1 = (v * length / 10000.0 for v in INFLOW_Y)
        for (t, e), tag in list(bnd.items()):
            if tag == "right":
                a, b = [tris[t][j] for j in range(3) if j != e]
                ym = 0.5 * (pts[a, 1] + pts[b, 1])
                if y0 <= ym <= y1:
                    bnd[(t, e)] = "inflow"
        self.length = float(length)
        self.mesh = Mesh(pts, tris, bnd)
        bed = wet_dry_bed(np.random.default_rng(seed), length)
        zp = bed(self.mesh.points[:, 0].copy(), self.mesh.points[:, 1].copy())
        self.elevation_vertex = zp[self.mesh.triangles]
        self.zc = self.elevation_vertex.mean(axis=1)
        self.N = self.mesh.number_of_elements
        c = self.mesh.centroid_coordinates.reshape(-1, 2)
        self.xy = c
        dx = length - c[:, 0]
        dy = np.maximum(np.maximum(y0 - c[:, 1], c[:, 1] - y1), 0.0)
        self.d_inflow = np.hypot(dx, dy)
        self.tri = np.stack([c[:, 0], c[:, 1], self.zc, self.d_inflow],
                            axis=1).astype(np.float32)
        self.inflow_y = (y0, y1)


def sample_params(count, seed):
    """Seeded parameter vectors [count][9] (PARAM_NAMES order)."""
    rng = np.random.default_rng(seed)
    th = np.empty((count, 9))
    th[:, 0] = rng.uniform(*PARAM_RANGES[0], count)
    th[:, 1] = rng.uniform(*PARAM_RANGES[1], count)
    th[:, 2] = th[:, 1] * rng.uniform(*DURATION_RATIO, count)
    th[:, 3] = rng.uniform(*PARAM_RANGES[3], count)
    th[:, 4] = rng.uniform(*PARAM_RANGES[4], count)
    th[:, 5:9] = rng.uniform(-0.4, 0.4, (count, 4))
    return th


def tide(theta, t):
    c0, c1, c2, c3, c4 = (float(v) for v in theta[4:9])
    wt = 2.0 * np.pi * np.asarray(t, np.float64) / TIDE_PERIOD
    return c0 + c1 * np.sin(wt) + c2 * np.cos(wt) + c3 * np.sin(2 * wt) + c4 * np.cos(2 * wt)


def _boundaries(theta):
    peak, rise, dur, _n = (float(v) for v in theta[:4])
    return {"left": Time_stage_fourier_boundary(coefficients=tuple(float(v) for v in theta[4:9]),
                                                period=TIDE_PERIOD),
            "inflow": Inflow_hydrograph_boundary(peak=peak, rise=rise, fall=dur - rise),
            "right": Reflective_boundary(), "top": Reflective_boundary(),
            "bottom": Reflective_boundary(), "exterior": Reflective_boundary()}


def family_scenario(fm: FamilyMesh, theta, finaltime=FINALTIME, mesh=None, zv=None):
    """The scenario of one parameter vector (on a sub-mesh when mesh and its
    vertex bed zv are given)."""
    mesh = fm.mesh if mesh is None else mesh
    zv = fm.elevation_vertex if zv is None else zv
    zc = zv.mean(axis=1)
    w = np.maximum(zc, float(tide(theta, 0.0)))
    N = mesh.number_of_elements
    b = {t: v for t, v in _boundaries(theta).items() if t in mesh.tag_names}
    return Scenario(name="surrogate_family", mesh=mesh, elevation_vertex=zv,
                    stage_centroid=w, xmom_centroid=np.zeros(N), ymom_centroid=np.zeros(N),
                    friction=np.full(N, float(theta[3])), boundaries=b, finaltime=finaltime)


def _run(scenarios, finaltime, threshold, precision):
    ens = Ensemble(scenarios, DEFAULT, precision)
    ens.set_tracking(threshold)
    ms = ens.run_timed(finaltime)
    out = ens.get_tracking()
    del ens
    return out, ms


def solve(fm: FamilyMesh, thetas, finaltime=FINALTIME, threshold=THRESHOLD, batch=32,
          precision="mixed"):
    """Solver fields for each parameter vector: (max_depth [S][N],
    arrival [S][N] (-1: never), device milliseconds)."""
    S = len(thetas)
    hmax = np.empty((S, fm.N), np.float32)
    tarr = np.empty((S, fm.N), np.float32)
    ms = 0.0
    for b0 in range(0, S, batch):
        scs = [family_scenario(fm, th, finaltime) for th in thetas[b0:b0 + batch]]
        out, t = _run(scs, finaltime, threshold, precision)
        ms += t
        for i, (hm, ta) in enumerate(out):
            hmax[b0 + i], tarr[b0 + i] = hm, ta
    return hmax, tarr, ms


def initial_depth(fm: FamilyMesh, thetas):
    """Depth of each scenario's initial state, [S][N]: the sea at rest at the
    west boundary's stage at t = 0."""
    th = np.asarray(thetas, np.float64)
    w0 = th[:, 4] + th[:, 6] + th[:, 8]   # c0 + c2 + c4: the series at t = 0
    return np.maximum(w0[:, None] - fm.zc[None, :], 0.0).astype(np.float32)


def max_tide(thetas, finaltime=FINALTIME, samples=3601):
    """Highest stage of each scenario's west boundary over [0, finaltime]."""
    t = np.linspace(0.0, finaltime, samples)
    return np.array([tide(th, t).max() for th in np.asarray(thetas, np.float64)])


def wave_lag(fm: FamilyMesh, c0, g=9.8):
    """Travel time [N] of a long wave from the west boundary to each
    triangle's x over the beach profile (bed (x - 0.8 L)/100, bumps left
    out) with the sea at rest at level c0: the integral of dx / sqrt(g h),
    h = a - x/100, a = c0 + 0.008 L; constant beyond the still shoreline."""
    a = float(c0) + 0.008 * fm.length
    x = np.minimum(fm.xy[:, 0], 100.0 * a)
    return 200.0 / np.sqrt(g) * (np.sqrt(a) - np.sqrt(np.maximum(a - x / 100.0, 0.0)))


def static_depth(fm: FamilyMesh, thetas, finaltime=FINALTIME, dt=2.0):
    """Still-water depth under each scenario's highest lagged tide, [S][N]:
    a triangle the tide reaches after tau (wave_lag) sees the boundary's
    stage tau late, and the initial stage before that, so its still level
    is the highest of the initial stage and the boundary's stage over
    [0, finaltime - tau].  This is the part of the maximum depth that the
    tide alone sets in a sea far shorter than the tide's wavelength and
    forced far more slowly than its own seiche period (about half an
    hour); the network learns the rest (the river flood, and the sea's
    departures from the still level)."""
    th = np.asarray(thetas, np.float64)
    t = np.arange(0.0, finaltime + 0.5 * dt, dt)
    out = np.empty((len(th), fm.N), np.float32)
    for s, p in enumerate(th):
        run = np.maximum.accumulate(tide(p, t))   # highest stage over [0, t]
        tau = wave_lag(fm, p[4])
        k = np.clip(((finaltime - tau) / dt).astype(np.int64), 0, len(t) - 1)
        level = np.maximum(run[k], run[0])        # run[0]: the initial stage
        out[s] = np.maximum(level - fm.zc, 0.0)
    return out


def targets_from(fm: FamilyMesh, thetas, hmax, tarr, finaltime=FINALTIME):
    """Normalised targets [S][N][2]: the maximum depth in excess of the
    still-water depth at the highest tide, and the arrival time."""
    t = np.empty(hmax.shape + (2,), np.float32)
    t[..., 0] = (hmax - static_depth(fm, thetas, finaltime)) / DEPTH_SCALE
    t[..., 1] = np.where(tarr >= 0, tarr / finaltime, NEVER)
    return t


def init_params(seed=0):
    """He-normal weights, zero biases, flat in the library's order."""
    rng = np.random.default_rng(seed)
    W1 = rng.standard_normal((F, H)) * np.sqrt(2.0 / 13)
    W1[13:] = 0.0
    parts = [W1, np.zeros(H), rng.standard_normal((H, H)) * np.sqrt(2.0 / H), np.zeros(H),
             rng.standard_normal((H, H)) * np.sqrt(2.0 / H), np.zeros(H),
             rng.standard_normal((H, OUT)) * np.sqrt(1.0 / H), np.zeros(OUT)]
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)


def feature_normalisation(fm: FamilyMesh):
    """(mean, inv_std) of the 16 features: parameters by their ranges,
    bed, coordinates and distance by the mesh."""
    mu = np.zeros(F, np.float32)
    isd = np.zeros(F, np.float32)
    lo, hi = PARAM_RANGES[:, 0], PARAM_RANGES[:, 1]
    mu[:9] = 0.5 * (lo + hi)
    isd[:9] = 2.0 / (hi - lo)
    for j, col in ((9, fm.tri[:, 2]), (10, fm.tri[:, 0]), (11, fm.tri[:, 1]),
                   (12, fm.tri[:, 3])):
        mu[j] = col.mean()
        isd[j] = 1.0 / max(col.std(), 1e-6)
    return mu, isd


class Surrogate:
    def __init__(self, fm: FamilyMesh, seed=0):
        self.fm = fm
        self.mu, self.isd = feature_normalisation(fm)
        p = init_params(seed)
        h = C.c_void_p()
        st = lib().swgpu_mlp_create(_f32p(p), _f32p(self.mu), _f32p(self.isd), C.byref(h))
        self._check(st, None)
        self._h = h
        self._data = None

    def _check(self, st, h):
        if st != 0:
            msg = lib().swgpu_mlp_last_error(h)
            raise _lib.SwgpuError(st, msg.decode() if msg else "")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().swgpu_mlp_destroy(h)
            except Exception:
                pass
            self._h = None

    def set_data(self, thetas, targets=None):
        scen = np.ascontiguousarray(thetas, dtype=np.float32)
        tri = np.ascontiguousarray(self.fm.tri, dtype=np.float32)
        tg = None if targets is None else np.ascontiguousarray(targets, dtype=np.float32)
        self._check(lib().swgpu_mlp_set_data(self._h, _f32p(tri), tri.shape[0], _f32p(scen),
                                             scen.shape[0], None if tg is None else _f32p(tg)),
                    self._h)
        self._data = (scen, tg)

    def params(self):
        out = np.empty(lib().swgpu_mlp_num_params(), np.float32)
        self._check(lib().swgpu_mlp_get_params(self._h, _f32p(out)), self._h)
        return out

    def gradients(self, rows, w_depth=1.0, w_arrival=1.0, w_error=1.0):
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        y = np.empty((len(rows), OUT), np.float32)
        g = np.empty(lib().swgpu_mlp_num_params(), np.float32)
        loss = np.empty(1, np.float32)
        self._check(lib().swgpu_mlp_gradients(self._h, rows.ctypes.data_as(C.POINTER(C.c_int64)),
                                              len(rows), w_depth, w_arrival, w_error, _f32p(y),
                                              _f32p(g), _f32p(loss)), self._h)
        return y, float(loss[0]), g

    def fit(self, thetas, targets, steps=4000, batch=32768, lr=1e-3, seed=1, w_depth=1.0,
            w_arrival=0.25, w_error=0.02, chunk=250):
        """Adam training on random (scenario, triangle) rows with a cosine
        learning-rate decay; returns {"loss", "samples_per_s", "seconds",
        "tflops"} (device time)."""
        self.set_data(thetas, targets)
        loss = np.empty(1, np.float32)
        ms = np.empty(1, np.float32)
        done, total_ms = 0, 0.0
        while done < steps:
            n = min(chunk, steps - done)
            lr_now = lr * 0.5 * (1 + np.cos(np.pi * done / steps))
            self._check(lib().swgpu_mlp_train(self._h, n, batch, seed + done, float(lr_now),
                                              w_depth, w_arrival, w_error, _f32p(loss),
                                              _f32p(ms)), self._h)
            total_ms += float(ms[0])
            done += n
        flop = 3 * 2 * (F * H + 2 * H * H + H * OUT) * batch * steps   # forward + backward
        return {"loss": float(loss[0]), "samples_per_s": steps * batch / (total_ms / 1000.0),
                "seconds": total_ms / 1000.0, "steps": steps, "batch": batch,
                "tflops": flop / (total_ms / 1000.0) / 1e12}

    def predict_raw(self, thetas):
        """Network outputs [S][N][3] and device milliseconds."""
        import torch  # device buffer for the outputs
        self.set_data(thetas)
        S, N = len(thetas), self.fm.N
        out = torch.empty((S * N, OUT), dtype=torch.float32, device="cuda")
        ms = np.empty(1, np.float32)
        self._check(lib().swgpu_mlp_predict(self._h, 0, S * N, C.c_void_p(out.data_ptr()),
                                            _f32p(ms)), self._h)
        return out.cpu().numpy().reshape(S, N, OUT), float(ms[0])

    def predict(self, thetas):
        """(max_depth [S][N], arrival [S][N] (-1: never), estimated absolute
        depth error [S][N] in m, device ms)."""
        y, ms = self.predict_raw(thetas)
        depth = np.maximum(static_depth(self.fm, thetas) + y[..., 0] * DEPTH_SCALE, 0.0)
        arr = np.where(y[..., 1] > 0.5 * (1.0 + NEVER), -1.0,
                       np.clip(y[..., 1], 0, 1) * FINALTIME)
        err = np.maximum(y[..., 2], 0.0) * DEPTH_SCALE
        return depth, arr, err, ms


# ---- the solver as fallback ----------------------------------------------------

def block_index(N, block=ALIGN):
    """Block of each triangle (blocks of ``block`` consecutive triangles of
    the mesh's Morton order)."""
    return np.arange(N) // block


def _block_max(a, block=ALIGN):
    S, N = a.shape
    nb = (N + block - 1) // block
    pad = nb * block - N
    if pad:
        a = np.concatenate([a, np.zeros((S, pad), a.dtype)], axis=1)
    return a.reshape(S, nb, block).max(axis=2)


def calibrate(err_est, err_true, tol=0.05, miss_rate=0.01, block=ALIGN):
    """Scale k of the error estimate such that, over these (calibration)
    scenarios, at most ``miss_rate`` of the blocks whose true maximum depth
    error exceeds ``tol`` have k * (estimated block maximum) <= tol, i.e. go
    unflagged.  Returns (k, stats)."""
    est = _block_max(np.asarray(err_est, np.float64), block).ravel()
    tru = _block_max(np.asarray(err_true, np.float64), block).ravel()
    bad = tru > tol
    if not bad.any():
        return 1.0, {"bad_blocks": 0, "blocks": int(est.size)}
    # flagged when k * est > tol: the bad blocks with the smallest estimates
    # decide k
    q = np.quantile(est[bad], miss_rate)
    k = tol / max(q, 1e-9)
    return float(k), {"bad_blocks": int(bad.sum()), "blocks": int(est.size),
                      "flagged_frac": float((k * est > tol).mean())}


def shifted_tide(theta, tau):
    """Parameter vector whose boundary stage is this one's delayed by tau:
    tide(t - tau) as the same five-term series (each harmonic's sine and
    cosine coefficients rotated by its phase lag)."""
    th = np.array(theta, np.float64, copy=True)
    for j, m in ((5, 1.0), (7, 2.0)):
        phi = m * 2.0 * np.pi * tau / TIDE_PERIOD
        a, b = th[j], th[j + 1]
        th[j] = a * np.cos(phi) + b * np.sin(phi)
        th[j + 1] = -a * np.sin(phi) + b * np.cos(phi)
    return th


def window_mesh(fm: FamilyMesh, xlo, ylo, yhi):
    """The sub-mesh of triangles with centroid x >= xlo and y in [ylo, yhi]:
    (mesh, vertex bed, family index of each sub-mesh triangle).  Boundary
    edges keep their family tags; cut edges facing west (toward the sea) are
    tagged "cut_west", the other cut edges "exterior" (reflective walls)."""
    sel = (fm.xy[:, 0] >= xlo) & (fm.xy[:, 1] >= ylo) & (fm.xy[:, 1] <= yhi)
    idx = np.nonzero(sel)[0]
    local = -np.ones(fm.N, np.int64)
    local[idx] = np.arange(len(idx))
    bnd = {}
    for (k, e), tag in fm.mesh.boundary.items():
        if local[k] >= 0:
            bnd[(int(local[k]), e)] = tag
    nb = fm.mesh.neighbours[idx]
    for j, k in enumerate(idx):
        for e in range(3):
            n = nb[j, e]
            if n >= 0 and not sel[n] and fm.xy[n, 0] < xlo:
                bnd[(j, e)] = "cut_west"
    sub = Mesh(fm.mesh.points, fm.mesh.triangles[idx], bnd)
    fam_idx = idx[sub.permutation]
    return sub, fm.elevation_vertex[fam_idx], fam_idx


def window_scenario(fm: FamilyMesh, theta, xlo, ylo, yhi, cache=None):
    """The scenario of one parameter vector on a window of the mesh: east of
    xlo (the whole width when xlo is 0) and within [ylo, yhi], with the sea
    at rest at the boundary's initial stage.  Its west cut carries the
    boundary's stage delayed by the long-wave travel time to xlo (wave_lag),
    the sea's still level there; the north and south cuts are walls, far
    enough (the margin) from the flagged blocks that their reflections stay
    small there."""
    cache = {} if cache is None else cache
    key = (xlo, ylo, yhi)
    if key not in cache:
        cache[key] = window_mesh(fm, xlo, ylo, yhi)
    sub, zv, fam_idx = cache[key]
    sc = family_scenario(fm, theta, FINALTIME, sub, zv)
    if "cut_west" in sub.tag_names:
        a = float(theta[4]) + 0.008 * fm.length
        tau = 200.0 / np.sqrt(9.8) * (np.sqrt(a) - np.sqrt(max(a - xlo / 100.0, 0.0)))
        sh = shifted_tide(theta, tau)
        sc.boundaries = dict(sc.boundaries)
        sc.boundaries["cut_west"] = Time_stage_fourier_boundary(
            coefficients=tuple(float(v) for v in sh[4:9]), period=TIDE_PERIOD)
    return sc, fam_idx


def window_scenarios(fm: FamilyMesh, thetas, flagged, margin=1500.0, quantum=500.0,
                     block=ALIGN, cache=None):
    """For each scenario with flagged blocks ([S][nblocks] bool): its window
    (east of the westmost flagged block, and in y the span of the flagged
    blocks and the inflow segment; each widened by ``margin`` and rounded
    outward to ``quantum``) as (scenario index, Scenario, family index).
    Sub-meshes are cached by window."""
    cache = {} if cache is None else cache
    blk = block_index(fm.N, block)
    out = []
    for s in np.nonzero(np.asarray(flagged).any(axis=1))[0]:
        tri = np.isin(blk, np.nonzero(flagged[s])[0])
        x, y = fm.xy[tri, 0], fm.xy[tri, 1]
        xlo = max(0.0, np.floor((float(x.min()) - margin) / quantum) * quantum)
        if xlo < 2.0 * quantum:
            xlo = 0.0   # the whole width: no west cut
        lo = min(float(y.min()), fm.inflow_y[0]) - margin
        hi = max(float(y.max()), fm.inflow_y[1]) + margin
        lo = max(0.0, np.floor(lo / quantum) * quantum)
        hi = min(fm.length, np.ceil(hi / quantum) * quantum)
        sc, fam_idx = window_scenario(fm, thetas[s], xlo, lo, hi, cache)
        out.append((int(s), sc, fam_idx))
    return out


def fallback(fm: FamilyMesh, thetas, depth, err_est, k, tol=0.05, margin=1500.0, batch=32,
             block=ALIGN, precision="mixed"):
    """The answer within ``tol``: predictions where the calibrated error
    estimate allows, window re-solves elsewhere.  Returns (depth [S][N],
    flagged blocks [S][nblocks], solver device ms, window triangles solved)."""
    est = _block_max(np.asarray(err_est, np.float64), block)
    flagged = k * est > tol
    answer = np.array(depth, np.float32, copy=True)
    wins = window_scenarios(fm, thetas, flagged, margin=margin, block=block)
    blk = block_index(fm.N, block)
    ms, tri_solved = 0.0, 0
    for b0 in range(0, len(wins), batch):
        part = wins[b0:b0 + batch]
        out, t = _run([sc for _, sc, _ in part], FINALTIME, THRESHOLD, precision)
        ms += t
        for (s, sc, fam_idx), (hm, _ta) in zip(part, out):
            tri_solved += sc.N
            take = flagged[s][blk[fam_idx]]
            answer[s, fam_idx[take]] = hm[take]
    return answer, flagged, ms, tri_solved


def evaluate(fm: FamilyMesh, thetas, true_depth, solver_ms, pred_depth, err_est, infer_ms, k,
             tol=0.05, margin=1500.0, block=ALIGN):
    """Time to an answer within ``tol`` (inference + window re-solves, device
    time) against the solver alone on the same scenarios, and the answer's
    error against the full solve."""
    answer, flagged, win_ms, tri_solved = fallback(fm, thetas, pred_depth, err_est, k, tol,
                                                    margin, block=block)
    true_depth = np.asarray(true_depth, np.float64)
    err_pred = _block_max(np.abs(np.asarray(pred_depth) - true_depth), block)
    err_ans = _block_max(np.abs(answer - true_depth), block)
    over = err_ans > tol
    t_answer = infer_ms + win_ms
    S = len(thetas)
    return {"scenarios": S, "tol_m": tol,
            "blocks_flagged_pct": 100.0 * float(flagged.mean()),
            "scenarios_with_window_solve": int(flagged.any(axis=1).sum()),
            "window_triangle_fraction": tri_solved / float(S * fm.N),
            "prediction_mean_abs_error_m": float(np.abs(pred_depth - true_depth).mean()),
            "prediction_max_abs_error_m": float(err_pred.max()),
            "prediction_blocks_over_tol_pct": 100.0 * float((err_pred > tol).mean()),
            "answer_max_abs_error_m": float(err_ans.max()),
            "answer_blocks_over_tol_pct": 100.0 * float(over.mean()),
            "answer_blocks_over_tol_unflagged_pct": 100.0 * float((over & ~flagged).mean()),
            "answer_blocks_over_tol_window_pct": 100.0 * float((over & flagged).mean()),
            "inference_ms": float(infer_ms), "window_solve_ms": float(win_ms),
            "time_to_answer_ms": float(t_answer), "solver_only_ms": float(solver_ms),
            "gain": float(solver_ms / t_answer) if t_answer > 0 else None}
