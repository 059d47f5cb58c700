"""BF16 MLP surrogate of the solver's maximum depth and arrival time.

A family of flood scenarios shares one mesh and bed (the wet/dry beach
with bumps) and differs in 9 parameters: height, centre x and y, radius
and aspect of an initial hump of water, Manning n, sea level, and the
hump's initial x and y velocity.  The solver (an ``Ensemble`` with
per-triangle tracking) gives, per scenario and triangle, the maximum depth
and the first time the depth exceeded a threshold.  The surrogate
(``libswgpu`` ``swgpu_mlp_*``: 16 -> 128 -> 128 -> 2, BF16 tensor cores)
learns both from the scenario parameters and the triangle's bed,
coordinates and distance to the hump centre (the depth as its excess over
the initial depth, which the parameters fix exactly), and predicts them
for new parameters in one pass over all (scenario, triangle) rows.

``fallback_report`` compares predictions with solver fields on held-out
scenarios: the blocks of 256 triangles whose maximum-depth error exceeds a
tolerance (5 cm) are counted, and a scenario containing any such block is
counted as rerun by the solver; time to answer is the surrogate's inference
time plus the solver time of the rerun scenarios, against solver-only.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib
from ._lib import lib
from .config import DEFAULT
from .ensemble import ALIGN, Ensemble
from .scenarios import Scenario, wet_dry

__all__ = ["PARAM_NAMES", "PARAM_RANGES", "FamilyMesh", "sample_params", "family_scenario",
           "solve", "Surrogate", "init_params", "fallback_report", "still_depth", "initial_depth",
           "targets_from"]

PARAM_NAMES = ("height", "x0", "y0", "radius", "manning", "sea_level", "aspect", "u0", "v0")
PARAM_RANGES = np.array([(0.5, 3.0), (3000.0, 7000.0), (3000.0, 7000.0), (150.0, 500.0),
                         (0.01, 0.05), (-0.5, 0.5), (0.5, 1.5), (-0.5, 0.5), (-0.5, 0.5)])
F, H, OUT = 16, 128, 2
DEPTH_SCALE = 2.0        # depth target: (max depth - still-water depth) / DEPTH_SCALE
NEVER = 1.25             # arrival target (arrival / finaltime) of a triangle that stays dry


def _f32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class FamilyMesh:
    """The shared mesh and bed (wet_dry with ``cells`` x ``cells`` cells on
    10 km x 10 km)."""

    def __init__(self, cells=224, seed=3):
        base = wet_dry(m=cells, seed=seed)
        self.mesh = base.mesh
        self.elevation_vertex = base.elevation_vertex
        self.zc = base.elevation_arrays()[0]
        self.N = base.N
        c = self.mesh.centroid_coordinates.reshape(-1, 2)
        self.xy = c
        self.tri = np.stack([c[:, 0], c[:, 1], self.zc], axis=1).astype(np.float32)


def sample_params(count, seed):
    rng = np.random.default_rng(seed)
    lo, hi = PARAM_RANGES[:, 0], PARAM_RANGES[:, 1]
    return lo + (hi - lo) * rng.uniform(size=(count, len(lo)))


def family_scenario(fm: FamilyMesh, theta, finaltime=600.0):
    A, x0, y0, rad, n, eta, asp, u0, v0 = (float(v) for v in theta)
    dx, dy = fm.xy[:, 0] - x0, fm.xy[:, 1] - y0
    shape = np.exp(-(dx * dx / (2 * rad * rad) + dy * dy / (2 * (asp * rad) ** 2)))
    w = np.maximum(fm.zc, eta + A * shape)
    h = w - fm.zc
    N = fm.N
    from .boundaries import Reflective_boundary
    return Scenario(name="surrogate_family", mesh=fm.mesh, elevation_vertex=fm.elevation_vertex,
                    stage_centroid=w, xmom_centroid=h * u0 * shape, ymom_centroid=h * v0 * shape,
                    friction=np.full(N, n),
                    boundaries={t: Reflective_boundary() for t in fm.mesh.tag_names},
                    finaltime=finaltime)


def solve(fm: FamilyMesh, thetas, finaltime=600.0, threshold=0.05, batch=32,
          precision="mixed"):
    """Solver fields for each parameter vector: (max_depth [S][N],
    arrival [S][N] (-1: never), device milliseconds)."""
    S = len(thetas)
    hmax = np.empty((S, fm.N), np.float32)
    tarr = np.empty((S, fm.N), np.float32)
    ms = 0.0
    for b0 in range(0, S, batch):
        scs = [family_scenario(fm, th, finaltime) for th in thetas[b0:b0 + batch]]
        ens = Ensemble(scs, DEFAULT, precision)
        ens.set_tracking(threshold)
        ms += ens.run_timed(finaltime)
        for i, (hm, ta) in enumerate(ens.get_tracking()):
            hmax[b0 + i], tarr[b0 + i] = hm, ta
        del ens
    return hmax, tarr, ms


def still_depth(fm: FamilyMesh, thetas):
    """Depth of the sea at rest at each scenario's sea level, [S][N]: the
    part of the maximum depth that the bathymetry alone fixes."""
    eta = np.asarray(thetas, np.float64)[:, 5:6]
    return np.maximum(eta - fm.zc[None, :], 0.0).astype(np.float32)


def initial_depth(fm: FamilyMesh, thetas):
    """Depth of each scenario's initial state, [S][N]: the hump over the sea
    at rest (as family_scenario builds it).  The maximum depth is at least
    this, and the part the network learns is its excess: the sharp Gaussian
    of the hump itself is known exactly from the parameters."""
    th = np.asarray(thetas, np.float64)
    x, y = fm.xy[:, 0], fm.xy[:, 1]
    out = np.empty((len(th), fm.N), np.float32)
    for s, (A, x0, y0, rad, _n, eta, asp, _u, _v) in enumerate(th):
        dx, dy = x - x0, y - y0
        shape = np.exp(-(dx * dx / (2 * rad * rad) + dy * dy / (2 * (asp * rad) ** 2)))
        out[s] = np.maximum(eta + A * shape - fm.zc, 0.0)
    return out


def targets_from(fm: FamilyMesh, thetas, hmax, tarr, finaltime):
    """Normalised targets [S][N][2]: the maximum depth in excess of the
    initial depth, and the arrival time."""
    t = np.empty(hmax.shape + (2,), np.float32)
    t[..., 0] = (hmax - initial_depth(fm, thetas)) / DEPTH_SCALE
    t[..., 1] = np.where(tarr >= 0, tarr / finaltime, NEVER)
    return t


def init_params(seed=0):
    """He-normal weights, zero biases, flat in the library's order."""
    rng = np.random.default_rng(seed)
    W1 = rng.standard_normal((F, H)) * np.sqrt(2.0 / 13)
    W1[13:] = 0.0
    parts = [W1, np.zeros(H), rng.standard_normal((H, H)) * np.sqrt(2.0 / H), np.zeros(H),
             rng.standard_normal((H, OUT)) * np.sqrt(1.0 / H), np.zeros(OUT)]
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)


def feature_normalisation(fm: FamilyMesh):
    """(mean, inv_std) of the 16 features: parameters by their ranges,
    bed and coordinates by the mesh, distance by the domain size."""
    mu = np.zeros(F, np.float32)
    isd = np.zeros(F, np.float32)
    lo, hi = PARAM_RANGES[:, 0], PARAM_RANGES[:, 1]
    mu[:9] = 0.5 * (lo + hi)
    isd[:9] = 2.0 / (hi - lo)
    for j, col in ((9, fm.tri[:, 2]), (10, fm.tri[:, 0]), (11, fm.tri[:, 1])):
        mu[j] = col.mean()
        isd[j] = 1.0 / max(col.std(), 1e-6)
    mu[12] = 3000.0
    isd[12] = 1.0 / 2000.0
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
        self.set_tensor_path("tcgen05")   # 1.2x the mma.sync inference at 200k x 256 rows

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

    def gradients(self, rows, w_depth=1.0, w_arrival=1.0):
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        y = np.empty((len(rows), 2), np.float32)
        g = np.empty(lib().swgpu_mlp_num_params(), np.float32)
        loss = np.empty(1, np.float32)
        self._check(lib().swgpu_mlp_gradients(self._h, rows.ctypes.data_as(C.POINTER(C.c_int64)),
                                              len(rows), w_depth, w_arrival, _f32p(y), _f32p(g),
                                              _f32p(loss)), self._h)
        return y, float(loss[0]), g

    def fit(self, thetas, targets, steps=2000, batch=16384, lr=2e-3, seed=1,
            w_depth=1.0, w_arrival=0.25):
        """Adam training on random (scenario, triangle) rows; returns
        {"loss", "samples_per_s", "seconds"} (device time)."""
        self.set_data(thetas, targets)
        loss = np.empty(1, np.float32)
        ms = np.empty(1, np.float32)
        done, total_ms, chunk = 0, 0.0, 250
        while done < steps:
            n = min(chunk, steps - done)
            lr_now = lr * 0.5 * (1 + np.cos(np.pi * done / steps))   # cosine decay
            self._check(lib().swgpu_mlp_train(self._h, n, batch, seed + done, float(lr_now),
                                              w_depth, w_arrival, _f32p(loss), _f32p(ms)),
                        self._h)
            total_ms += float(ms[0])
            done += n
        return {"loss": float(loss[0]), "samples_per_s": steps * batch / (total_ms / 1000.0),
                "seconds": total_ms / 1000.0, "steps": steps, "batch": batch}

    def set_tensor_path(self, path):
        """Inference on "mma.sync" (default) or "tcgen05" tensor cores."""
        code = {"mma.sync": 0, "tcgen05": 1}[path]
        self._check(lib().swgpu_mlp_set_tensor_path(self._h, code), self._h)

    def predict(self, thetas):
        """(max_depth [S][N], arrival [S][N] (-1: never), device ms) for the
        parameter vectors."""
        import torch  # device buffer for the outputs
        self.set_data(thetas)
        S, N = len(thetas), self.fm.N
        out = torch.empty((S * N, 2), dtype=torch.float32, device="cuda")
        ms = np.empty(1, np.float32)
        self._check(lib().swgpu_mlp_predict(self._h, 0, S * N, C.c_void_p(out.data_ptr()),
                                            _f32p(ms)), self._h)
        y = out.cpu().numpy().reshape(S, N, 2)
        depth = np.maximum(initial_depth(self.fm, thetas) + y[..., 0] * DEPTH_SCALE, 0.0)
        arr = np.where(y[..., 1] > 0.5 * (1.0 + NEVER), -1.0, np.clip(y[..., 1], 0, 1))
        return depth, arr, float(ms[0])


def fallback_report(pred_depth, true_depth, solver_ms_per_scenario, infer_ms, tol=0.05,
                    block=ALIGN):
    """Blocks of ``block`` triangles whose max-depth error exceeds ``tol``;
    scenarios with any such block are rerun by the solver."""
    S, N = true_depth.shape
    nb = (N + block - 1) // block
    pad = nb * block - N
    err = np.abs(np.asarray(pred_depth) - np.asarray(true_depth))
    if pad:
        err = np.concatenate([err, np.zeros((S, pad), err.dtype)], axis=1)
    berr = err.reshape(S, nb, block).max(axis=2)
    bad = berr > tol
    rerun = bad.any(axis=1)
    t_fallback = infer_ms + rerun.sum() * solver_ms_per_scenario
    t_solver = S * solver_ms_per_scenario
    return {"blocks_over_tol_pct": 100.0 * bad.mean(), "scenarios_rerun": int(rerun.sum()),
            "scenarios": S, "max_abs_error_m": float(err.max()),
            "mean_abs_error_m": float(np.abs(np.asarray(pred_depth) - true_depth).mean()),
            "time_to_answer_ms": float(t_fallback), "solver_only_ms": float(t_solver),
            "gain": float(t_solver / t_fallback) if t_fallback > 0 else None}
