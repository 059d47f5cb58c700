"""Batched ensembles: many independent scenarios advanced by one handle.

A scenario is a mesh with its initial state, friction and boundary
conditions (an ``anuga_cuda.scenarios.Scenario``).  ``Ensemble``
concatenates the meshes into one (scenario s owns a 256-aligned triangle
range; each range is padded with isolated, dry triangles), hands it to
``swgpu_create_ensemble`` and runs all scenarios in one device-resident loop:
one graph of fused steps over every triangle of every scenario, each
scenario with its own time, CFL timestep, finaltime and stop state kept in
its own control block.  A scenario that reaches its finaltime stops; its
blocks return at entry while the others continue.  Small meshes, which
alone would leave most of the GPU idle between launches, share every
launch with the rest.

There is no counterpart in the reference, which runs one domain per
process; each scenario's result equals its own single-domain run (every
per-triangle operation and the per-scenario timestep reduction are the
same).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, f64p, i64p, lib
from .boundaries import Reflective_boundary
from .config import DEFAULT, Parameters
from .mesh import Mesh

__all__ = ["Ensemble", "ALIGN", "shard"]

ALIGN = 256   # scenario ranges start on multiples of this many triangles

_MESH_INT = ("neighbours", "neighbour_edges", "surrogate_neighbours", "number_of_boundaries",
             "tri_full_flag")
_MESH_FLOAT = ("normals", "edgelengths", "radii", "areas", "vertex_coordinates",
               "centroid_coordinates")


def shard(work, rank, world):
    """Scenario indices of one rank when ``world`` processes (one per GPU)
    split an ensemble: longest-processing-time-first assignment of the
    per-scenario work estimates to the least loaded rank, deterministic, so
    every rank computes the same partition without communicating.  The
    ensemble path needs no exchange between ranks (weak in scenarios)."""
    load = [0.0] * world
    mine = []
    for i in sorted(range(len(work)), key=lambda j: (-work[j], j)):
        r = min(range(world), key=lambda q: (load[q], q))
        load[r] += float(work[i])
        if r == rank:
            mine.append(i)
    return sorted(mine)


def _pad_mesh():
    """One isolated right triangle (all three edges boundary)."""
    return Mesh(np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]]), np.array([[0, 1, 2]]),
                {(0, 0): "pad", (0, 1): "pad", (0, 2): "pad"}, reorder=False)


def _initial_timestep(sc, g=9.8):
    """The scenario's CFL timestep at rest, min over wet triangles of
    radius / sqrt(g h) (over all triangles with h = 1 m when none is wet):
    a proxy for its number of steps to a common finaltime (on the inflow
    harbours its rank order equals that of the steps actually taken)."""
    r = np.asarray(sc.mesh.radii, dtype=np.float64)
    h = np.asarray(sc.stage_centroid, dtype=np.float64) - sc.elevation_arrays()[0]
    wet = h > 0.01
    if not wet.any():
        return float(np.min(r) / np.sqrt(g))
    return float(np.min(r[wet] / np.sqrt(g * h[wet])))


class Ensemble:
    """``scenarios``: a list of Scenario objects (mesh, initial state,
    friction, boundaries).  ``precision`` "mixed" (default) or "fp64"."""

    def __init__(self, scenarios, parameters: Parameters | None = None, precision="mixed"):
        if not scenarios:
            raise ValueError("an ensemble needs at least one scenario")
        scenarios = list(scenarios)
        # Internally the scenarios expected to run longest (the smallest
        # initial CFL timestep, i.e. the most steps) come first, so that the
        # launches can stop short of the finished ones at the end; every
        # per-scenario input and output is in the caller's order.
        dt0 = [_initial_timestep(sc) for sc in scenarios]
        self.order = sorted(range(len(scenarios)), key=lambda i: (dt0[i], -scenarios[i].N, i))
        self.scenarios = [scenarios[i] for i in self.order]
        self.parameters = parameters or DEFAULT
        self.precision = precision
        self._build_arrays()
        self._h = None
        self._create()

    # -- concatenation -------------------------------------------------
    def _build_arrays(self):
        pad = _pad_mesh()
        parts, offsets, tri_off, bnd_off, tag_off = [], [0], 0, 0, 0
        tags = []   # global list of boundary objects
        self.ranges = []
        for sc in self.scenarios:
            m = sc.mesh
            n = m.number_of_elements
            npad = (-n) % ALIGN
            parts.append((m, tri_off, bnd_off, tag_off))
            self.ranges.append((tri_off, tri_off + n))
            tri_off += n
            bnd_off += m.number_of_boundary_elements
            tag_off += len(m.tag_names)
            tags.extend(sc.boundaries.get(t) or Reflective_boundary() for t in m.tag_names)
            for _ in range(npad):
                parts.append((pad, tri_off, bnd_off, -1))
                tri_off += 1
                bnd_off += 3
            offsets.append(tri_off)
        self.pad_tag = tag_off
        tags.append(Reflective_boundary())
        self.offsets = np.array(offsets, dtype=np.int64)
        self.N = tri_off
        self.Nb = bnd_off
        A = {k: [] for k in _MESH_INT + _MESH_FLOAT +
             ("boundary_cells", "boundary_edges", "boundary_tag")}
        for m, t0, b0, g0 in parts:
            nbr = np.asarray(m.neighbours, dtype=np.int64).reshape(-1, 3)
            A["neighbours"].append(np.where(nbr >= 0, nbr + t0, nbr - b0))
            A["neighbour_edges"].append(np.asarray(m.neighbour_edges, np.int64).reshape(-1, 3))
            A["surrogate_neighbours"].append(
                np.asarray(m.surrogate_neighbours, np.int64).reshape(-1, 3) + t0)
            A["number_of_boundaries"].append(np.asarray(m.number_of_boundaries, np.int64))
            A["tri_full_flag"].append(np.asarray(m.tri_full_flag, np.int64))
            for k in _MESH_FLOAT:
                a = np.asarray(getattr(m, k), dtype=np.float64)
                A[k].append(a.reshape(m.number_of_elements, -1) if a.ndim > 1 or a.size !=
                            m.number_of_elements else a)
            A["boundary_cells"].append(np.asarray(m.boundary_cells, np.int64) + t0)
            A["boundary_edges"].append(np.asarray(m.boundary_edges, np.int64))
            bt = np.asarray(m.boundary_tag, np.int64)
            A["boundary_tag"].append(bt + g0 if g0 >= 0 else np.full_like(bt, self.pad_tag))
        self.arrays = {k: np.ascontiguousarray(np.concatenate(v)) for k, v in A.items()}
        self.tags = tags
        # initial state, padded with dry flat triangles
        zv, w, uh, vh, fr = [], [], [], [], []
        for sc, (a, b), o1 in zip(self.scenarios, self.ranges, self.offsets[1:]):
            npad = o1 - b
            zv.append(np.asarray(sc.elevation_vertex, np.float64).reshape(-1, 3))
            zv.append(np.zeros((npad, 3)))
            for lst, src in ((w, sc.stage_centroid), (uh, sc.xmom_centroid),
                             (vh, sc.ymom_centroid), (fr, sc.friction)):
                lst.append(np.asarray(src, np.float64))
                lst.append(np.zeros(npad))
        self.elevation_vertex = np.concatenate(zv)
        self.stage_centroid = np.concatenate(w)
        self.xmom_centroid = np.concatenate(uh)
        self.ymom_centroid = np.concatenate(vh)
        self.friction = np.concatenate(fr)

    def _create(self):
        A = self.arrays
        ms = _lib.Mesh_t()
        ms.number_of_elements = self.N
        ms.number_of_boundary_elements = self.Nb
        for name, arr in A.items():
            setattr(ms, name, i64p(arr) if arr.dtype == np.int64 else f64p(arr))
        ps = _lib.Params_t(*self.parameters.as_tuple())
        h = C.c_void_p()
        prec = {"fp64": _lib.FP64, "mixed": _lib.MIXED}[self.precision]
        check(lib().swgpu_create_ensemble(C.byref(ms), i64p(self.offsets), len(self.scenarios),
                                          C.byref(ps), prec, C.byref(h)), None)
        self._h = h
        arr = (_lib.BoundaryTag_t * len(self.tags))()
        for i, b in enumerate(self.tags):
            owner = self._tag_owner(i)
            arr[i] = b.tag_struct(*owner) if owner else b.tag_struct()
        check(lib().swgpu_set_boundary_tags(self._h, arr, len(self.tags)), self._h)
        self._upload_state()

    def _tag_owner(self, g):
        """(mesh, tag name) of global tag index g (None for the pad tag)."""
        base = 0
        for sc in self.scenarios:
            names = sc.mesh.tag_names
            if g < base + len(names):
                return sc.mesh, names[g - base]
            base += len(names)
        return None

    def _upload_state(self):
        v = self.elevation_vertex
        zc = (v[:, 0] + v[:, 1] + v[:, 2]) / 3.0
        ze = np.stack([0.5 * (v[:, 1] + v[:, 2]), 0.5 * (v[:, 0] + v[:, 2]),
                       0.5 * (v[:, 0] + v[:, 1])], axis=1)

        def up(q, c, vv=None, ee=None):
            c = np.ascontiguousarray(c, dtype=np.float64)
            vv = None if vv is None else np.ascontiguousarray(vv, dtype=np.float64)
            ee = None if ee is None else np.ascontiguousarray(ee, dtype=np.float64)
            check(lib().swgpu_set_quantity(self._h, q, f64p(c), None if vv is None else f64p(vv),
                                           None if ee is None else f64p(ee)), self._h)

        up(_lib.ELEVATION, zc, v, ze)
        up(_lib.FRICTION, self.friction)
        for q, c in ((_lib.STAGE, self.stage_centroid), (_lib.XMOMENTUM, self.xmom_centroid),
                     (_lib.YMOMENTUM, self.ymom_centroid)):
            rep = np.repeat(c[:, None], 3, axis=1)
            up(q, c, rep, rep)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().swgpu_destroy(h)
            except Exception:
                pass
            self._h = None

    # -- running -------------------------------------------------------
    def __len__(self):
        return len(self.scenarios)

    def evolve(self, finaltime, starttime=0.0, max_steps=None):
        """Run every scenario from ``starttime`` to its finaltime (a scalar
        or one per scenario), or for at most ``max_steps`` steps; returns
        the per-scenario states."""
        ft = self._internal(np.broadcast_to(np.asarray(finaltime, dtype=np.float64),
                                            (len(self),)))
        big = float(ft.max())
        check(lib().swgpu_evolve_start(self._h, float(starttime), big, big), self._h)
        check(lib().swgpu_ensemble_set_finaltimes(self._h, f64p(ft)), self._h)
        st = _lib.State_t()
        budget = 0 if max_steps is None else int(max_steps)
        check(lib().swgpu_evolve_run(self._h, budget, C.byref(st)), self._h)
        return self.states()

    def run_timed(self, finaltime, starttime=0.0):
        """As evolve (to finaltime), returning the device time of the run in
        milliseconds (CUDA events around the graph launches)."""
        ft = self._internal(np.broadcast_to(np.asarray(finaltime, dtype=np.float64),
                                            (len(self),)))
        big = float(ft.max())
        check(lib().swgpu_evolve_start(self._h, float(starttime), big, big), self._h)
        check(lib().swgpu_ensemble_set_finaltimes(self._h, f64p(ft)), self._h)
        st = _lib.State_t()
        ms = C.c_double()
        check(lib().swgpu_evolve_run_timed(self._h, 0, C.byref(st), C.byref(ms)), self._h)
        return ms.value

    def _internal(self, per_scenario):
        """A per-scenario array in the caller's order -> internal order."""
        a = np.asarray(per_scenario)
        return np.ascontiguousarray(a[self.order])

    def _user(self, items):
        """A per-scenario list in internal order -> the caller's order."""
        out = [None] * len(items)
        for j, i in enumerate(self.order):
            out[i] = items[j]
        return out

    def states(self):
        out = []
        for s in range(len(self)):
            st = _lib.State_t()
            check(lib().swgpu_ensemble_get_state(self._h, s, C.byref(st)), self._h)
            out.append(st)
        return self._user(out)

    def set_tracking(self, threshold=0.01, on=True):
        """Maximum depth and arrival time tracking for every scenario."""
        check(lib().swgpu_set_tracking(self._h, int(bool(on)), float(threshold)), self._h)

    def get_tracking(self):
        """Per scenario, (max_depth, arrival_time) arrays of its triangles."""
        hm = np.empty(self.N, dtype=np.float32)
        ta = np.empty(self.N, dtype=np.float32)
        check(lib().swgpu_get_tracking(self._h, hm.ctypes.data_as(C.POINTER(C.c_float)),
                                       ta.ctypes.data_as(C.POINTER(C.c_float))), self._h)
        return self._user([(hm[a:b].copy(), ta[a:b].copy()) for a, b in self.ranges])

    def masses(self):
        m = np.empty(len(self))
        check(lib().swgpu_ensemble_mass(self._h, f64p(m)), self._h)
        return np.array(self._user(list(m)))

    def centroid_values(self, name):
        """Centroid values of quantity ``name`` for every scenario (a list of
        arrays in each scenario mesh's own triangle order)."""
        qid = {"stage": _lib.STAGE, "xmomentum": _lib.XMOMENTUM, "ymomentum": _lib.YMOMENTUM,
               "elevation": _lib.ELEVATION, "friction": _lib.FRICTION, "height": _lib.HEIGHT,
               "xvelocity": _lib.XVELOCITY, "yvelocity": _lib.YVELOCITY}[name]
        c = np.empty(self.N)
        check(lib().swgpu_get_quantity(self._h, qid, f64p(c), None, None), self._h)
        return self._user([c[a:b].copy() for a, b in self.ranges])
