"""GPU_domain: the reference's GPU Domain API on libswgpu.

The reference exposes ANUGA's shallow-water evolve step on the GPU as a
subclass of ``anuga.Domain`` whose per-step methods launch PyCUDA kernels
(``CUDA_advanced_domain``, src/anuga_cuda/gpu_domain_advanced.py:47;
exported as ``anuga_cuda.GPU_domain``, src/anuga_cuda/__init__.py:25).  This
class keeps those method names, argument meanings and call order, and runs
them through the C ABI of libswgpu.so (include/swgpu.h).  All state lives on
the GPU for the lifetime of the domain; arrays cross to the host only when a
quantity is read or set.

Triangles are stored internally in Morton order; every array a caller passes
in or reads out uses the caller's own triangle order.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import check, f64p, i64p, lib
from .boundaries import Boundary
from .config import DEFAULT, Parameters
from .mesh import Mesh

__all__ = ["GPU_domain", "Quantity"]

_QID = {
    "stage": _lib.STAGE, "xmomentum": _lib.XMOMENTUM, "ymomentum": _lib.YMOMENTUM,
    "elevation": _lib.ELEVATION, "friction": _lib.FRICTION, "height": _lib.HEIGHT,
    "xvelocity": _lib.XVELOCITY, "yvelocity": _lib.YVELOCITY,
}
_PRECISION = {"fp64": _lib.FP64, "double": _lib.FP64, "mixed": _lib.MIXED}


class Quantity:
    """Host view of one quantity; values are downloaded on access."""

    def __init__(self, domain: "GPU_domain", name: str):
        self.domain = domain
        self.name = name
        self.qid = _QID[name]

    def _get(self, which):
        d = self.domain
        N = d.number_of_elements
        c = np.empty(N)
        v = np.empty((N, 3)) if which in ("vertex", "edge") else None
        e = np.empty((N, 3)) if which == "edge" else None
        if which == "edge":
            check(lib().swgpu_get_quantity(d._h, self.qid, f64p(c), f64p(v), f64p(e)), d._h)
            return d._to_user(e)
        if which == "vertex":
            check(lib().swgpu_get_quantity(d._h, self.qid, f64p(c), f64p(v), None), d._h)
            return d._to_user(v)
        check(lib().swgpu_get_quantity(d._h, self.qid, f64p(c), None, None), d._h)
        return d._to_user(c)

    @property
    def centroid_values(self):
        return self._get("centroid")

    @property
    def vertex_values(self):
        return self._get("vertex")

    @property
    def edge_values(self):
        return self._get("edge")

    @property
    def boundary_values(self):
        d = self.domain
        out = np.empty(d.number_of_boundary_elements)
        check(lib().swgpu_get_boundary_values(d._h, self.qid, f64p(out)), d._h)
        return out

    @property
    def explicit_update(self):
        d = self.domain
        out = np.empty(d.number_of_elements)
        check(lib().swgpu_get_explicit_update(d._h, self.qid, f64p(out)), d._h)
        return d._to_user(out)

    @property
    def semi_implicit_update(self):
        d = self.domain
        out = np.empty(d.number_of_elements)
        check(lib().swgpu_get_semi_implicit_update(d._h, self.qid, f64p(out)), d._h)
        return d._to_user(out)

    def get_values(self, location="centroids"):
        return {"centroids": self.centroid_values, "vertices": self.vertex_values,
                "edges": self.edge_values}[location]

    def set_values(self, *args, **kw):
        self.domain.set_quantity(self.name, *args, **kw)


class GPU_domain:
    """ANUGA shallow-water domain whose evolve step runs on one GB300.

    Constructor arguments follow the reference (``coordinates``,
    ``vertices``, ``boundary``, ``starttime``, ``using_gpu``, ``cotesting``,
    ``stream``, ``rearranged``, ``domain``); ANUGA's parallel arguments are
    accepted and must describe a single full domain.  Added: ``mesh`` (a
    prebuilt :class:`Mesh`), ``precision`` ('fp64' or 'mixed') and
    ``parameters`` (a :class:`Parameters`, or keyword overrides).
    """

    conserved_quantities = ["stage", "xmomentum", "ymomentum"]
    evolved_quantities = ["stage", "xmomentum", "ymomentum"]
    other_quantities = ["elevation", "friction", "height", "xvelocity", "yvelocity"]

    def __init__(self, coordinates=None, vertices=None, boundary=None, mesh=None,
                 precision="fp64", parameters: Parameters | None = None, reorder=True,
                 starttime=0.0, using_gpu=True, cotesting=False, stream=False, rearranged=True,
                 domain=None, processor=0, numproc=1, full_send_dict=None,
                 ghost_recv_dict=None, **param_overrides):
        if numproc != 1 or processor != 0 or full_send_dict or ghost_recv_dict:
            raise NotImplementedError("one full domain per GPU_domain (no ghost exchange)")
        if not using_gpu:
            raise ValueError("GPU_domain has no CPU implementation; using_gpu must be True")
        if domain is not None:
            mesh = domain.mesh if isinstance(domain, GPU_domain) else domain
        built_here = mesh is None
        if built_here:
            if coordinates is None or vertices is None:
                raise ValueError("give coordinates and vertices, or a Mesh")
            mesh = Mesh(coordinates, vertices, boundary, reorder=reorder)
        self.mesh = mesh
        self.precision = precision
        params = parameters or DEFAULT
        if param_overrides:
            params = params.replace(**param_overrides)
        self.parameters = params
        self.cotesting = cotesting
        self.using_stream = stream
        self.rearranged_domain = rearranged
        self.starttime = float(starttime)
        self.number_of_elements = mesh.number_of_elements
        self.number_of_boundary_elements = mesh.number_of_boundary_elements
        # caller's triangle order: the coordinates/vertices given here, or the
        # Mesh's own order when a Mesh is passed in
        self._perm = mesh.permutation if built_here else np.arange(mesh.number_of_elements)
        self._identity = bool(np.all(self._perm == np.arange(len(self._perm))))
        # triangles the Mesh turned counter-clockwise (vertices, and so edges,
        # 1 and 2 swapped) in the caller's order
        flip = getattr(mesh, "flipped", None) if built_here else None
        self._flip = np.nonzero(flip)[0] if flip is not None and np.any(flip) else None
        self.boundary_map = {t: None for t in mesh.tag_names}
        self.quantities = {n: Quantity(self, n) for n in _QID}
        self.flux_timestep = None
        self.timestep = None
        self.yieldstep = None
        self.finaltime = None
        self._timestepping_method = "euler"
        self.protect_against_isolated_degenerate_timesteps = False
        self.name = "domain"
        self.datadir = "."
        self.store = False
        self.smooth = True           # SWW values averaged onto mesh nodes
        self.writer = None
        self._h = None
        self._create()

    # -- construction ---------------------------------------------------
    def _create(self):
        m = self.mesh
        self._keep = keep = {
            "neighbours": np.ascontiguousarray(m.neighbours, dtype=np.int64),
            "neighbour_edges": np.ascontiguousarray(m.neighbour_edges, dtype=np.int64),
            "surrogate_neighbours": np.ascontiguousarray(m.surrogate_neighbours, dtype=np.int64),
            "number_of_boundaries": np.ascontiguousarray(m.number_of_boundaries, dtype=np.int64),
            "tri_full_flag": np.ascontiguousarray(m.tri_full_flag, dtype=np.int64),
            "normals": np.ascontiguousarray(m.normals, dtype=np.float64),
            "edgelengths": np.ascontiguousarray(m.edgelengths, dtype=np.float64),
            "radii": np.ascontiguousarray(m.radii, dtype=np.float64),
            "areas": np.ascontiguousarray(m.areas, dtype=np.float64),
            "vertex_coordinates": np.ascontiguousarray(m.vertex_coordinates, dtype=np.float64),
            "centroid_coordinates": np.ascontiguousarray(m.centroid_coordinates, dtype=np.float64),
            "boundary_cells": np.ascontiguousarray(m.boundary_cells, dtype=np.int64),
            "boundary_edges": np.ascontiguousarray(m.boundary_edges, dtype=np.int64),
            "boundary_tag": np.ascontiguousarray(m.boundary_tag, dtype=np.int64),
        }
        ms = _lib.Mesh_t()
        ms.number_of_elements = m.number_of_elements
        ms.number_of_boundary_elements = m.number_of_boundary_elements
        for name, arr in keep.items():
            setattr(ms, name, i64p(arr) if arr.dtype == np.int64 else f64p(arr))
        ps = _lib.Params_t(*self.parameters.as_tuple())
        h = C.c_void_p()
        prec = _PRECISION[self.precision]
        st = lib().swgpu_create(C.byref(ms), C.byref(ps), prec, C.byref(h))
        check(st, None)
        self._h = h
        self._keep = None
        # ANUGA's defaults before set_quantity / set_boundary
        z = np.zeros(self.number_of_elements)
        for name in ("elevation", "friction", "stage", "xmomentum", "ymomentum"):
            self._upload(name, z, np.zeros((self.number_of_elements, 3)))
        self._install_tags()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().swgpu_destroy(h)
            except Exception:
                pass
            self._h = None

    # -- index order ----------------------------------------------------
    def _swap12(self, a):
        """Swap columns 1 and 2 of the flipped rows of a caller-order (N, 3)
        array (vertex or edge values, triangle vertex indices)."""
        if self._flip is None or a.ndim != 2 or a.shape[1] != 3:
            return a
        a = a.copy()
        a[self._flip, 1], a[self._flip, 2] = a[self._flip, 2].copy(), a[self._flip, 1].copy()
        return a

    def _to_user(self, a):
        if self._identity:
            return self._swap12(a)
        out = np.empty_like(a)
        out[self._perm] = a
        return self._swap12(out)

    def _to_internal(self, a):
        a = self._swap12(np.asarray(a))
        if self._identity:
            return np.ascontiguousarray(a)
        return np.ascontiguousarray(a[self._perm])

    # -- quantities -----------------------------------------------------
    def _upload(self, name, centroid, vertex=None, edge=None):
        c = np.ascontiguousarray(centroid, dtype=np.float64)
        v = None if vertex is None else np.ascontiguousarray(vertex, dtype=np.float64)
        e = None if edge is None else np.ascontiguousarray(edge, dtype=np.float64)
        check(lib().swgpu_set_quantity(self._h, _QID[name], f64p(c),
                                       None if v is None else f64p(v),
                                       None if e is None else f64p(e)), self._h)

    def set_quantity(self, name, value=None, function=None, numeric=None,
                     location="vertices", indices=None, **kw):
        """Quantity.set_values semantics: a scalar, a function f(x, y), or an
        array of centroid values (N,) or vertex values (N, 3) in the
        caller's triangle order.  Vertex values give centroids as their mean
        and edges as the mean of the two adjacent vertices."""
        if name not in ("stage", "xmomentum", "ymomentum", "elevation", "friction"):
            raise KeyError(f"cannot set quantity {name!r}")
        if indices is not None:
            raise NotImplementedError("indices= is not supported")
        if value is None and function is None and numeric is not None:
            value = numeric
        N = self.number_of_elements
        m = self.mesh
        if function is not None or callable(value):
            f = function or value
            if location == "centroids":
                c = m.centroid_values(f)
                vert = None
            else:
                vert = m.vertex_values(f)
                c = None
        else:
            a = np.asarray(value, dtype=np.float64)
            if a.ndim == 0:
                c = np.full(N, float(a))
                vert = None if location == "centroids" else np.full((N, 3), float(a))
            elif a.shape == (N,):
                c = self._to_internal(a)
                vert = None
            elif a.shape == (N, 3):
                vert = self._to_internal(a)
                c = None
            else:
                raise ValueError(f"bad shape {a.shape} for {name}")
        if vert is not None:
            c = (vert[:, 0] + vert[:, 1] + vert[:, 2]) / 3.0
            edge = np.stack([0.5 * (vert[:, 1] + vert[:, 2]), 0.5 * (vert[:, 0] + vert[:, 2]),
                             0.5 * (vert[:, 0] + vert[:, 1])], axis=1)
        else:
            vert = np.repeat(c[:, None], 3, axis=1)
            edge = vert
        self._upload(name, c, vert, edge)

    def get_quantity(self, name):
        return self.quantities[name]

    # -- boundaries ------------------------------------------------------
    def set_boundary(self, boundary_map):
        """Map each boundary tag to a boundary object (Domain.set_boundary)."""
        for tag, b in boundary_map.items():
            if tag not in self.boundary_map:
                raise KeyError(f"tag {tag!r} not in mesh (tags: {list(self.boundary_map)})")
            if b is not None and not isinstance(b, Boundary):
                raise TypeError(f"unsupported boundary object {b!r} for tag {tag!r}")
            self.boundary_map[tag] = b
        self._install_tags()

    def _install_tags(self):
        from .boundaries import Reflective_boundary
        names = self.mesh.tag_names
        arr = (_lib.BoundaryTag_t * max(len(names), 1))()
        for i, t in enumerate(names):
            b = self.boundary_map.get(t) or Reflective_boundary(self)
            arr[i] = b.tag_struct(self.mesh, t)
        check(lib().swgpu_set_boundary_tags(self._h, arr, len(names)), self._h)

    # -- time -------------------------------------------------------------
    def _state(self):
        s = _lib.State_t()
        check(lib().swgpu_get_state(self._h, C.byref(s)), self._h)
        return s

    def _set_state(self, s):
        check(lib().swgpu_set_state(self._h, C.byref(s)), self._h)

    def get_time(self):
        return self._state().time

    def set_time(self, time=0.0):
        s = self._state()
        s.time = float(time)
        self._set_state(s)

    def get_starttime(self):
        return self.starttime

    def set_starttime(self, t):
        self.starttime = float(t)

    @property
    def _order_(self):
        return int(self._state().order)

    @_order_.setter
    def _order_(self, v):
        s = self._state()
        s.order = int(v)
        self._set_state(s)

    def set_default_order(self, n):
        if n not in (1, 2):
            raise ValueError("order must be 1 or 2")
        self.parameters = self.parameters.replace(default_order=n)
        self._order_ = n

    _TIMESTEPPING = {"euler": _lib.EULER, "rk2": _lib.RK2, "rk3": _lib.RK3}

    def get_timestepping_method(self):
        return self._timestepping_method

    def set_timestepping_method(self, method):
        """'euler', 'rk2' or 'rk3' (or 1, 2, 3): the step that evolve runs."""
        if isinstance(method, int):
            names = {v: k for k, v in self._TIMESTEPPING.items()}
            if method not in names:
                raise ValueError(f"timestepping method {method}")
            method = names[method]
        if method not in self._TIMESTEPPING:
            raise ValueError(f"timestepping method {method!r}: euler, rk2 or rk3")
        check(lib().swgpu_set_timestepping_method(self._h, self._TIMESTEPPING[method]),
              self._h)
        self._timestepping_method = method

    def set_name(self, name):
        self.name = name
        self.writer = None

    def get_name(self):
        return self.name

    def set_store(self, flag=True):
        """Write an SWW time slice at every yield of evolve."""
        self.store = bool(flag)

    def set_datadir(self, path):
        self.datadir = path
        self.writer = None

    def get_datadir(self):
        return self.datadir

    def set_store_vertices_uniquely(self, flag=True):
        """SWW points per triangle vertex (True) or smoothed onto the mesh
        nodes (False, the default)."""
        self.smooth = not flag
        self.writer = None

    def store_timestep(self):
        """Copy the vertex values back and append one SWW time slice
        (gpu_domain_advanced.py:2167-2172).  The file is
        <datadir>/<name>.sww, created at the first call."""
        from .io import SWWWriter, sww_path
        if self.writer is None:
            os.makedirs(self.datadir or ".", exist_ok=True)
            tris = self._to_user(np.asarray(self.mesh.triangles))
            fric = np.repeat(self.quantities["friction"].centroid_values[:, None], 3, axis=1)
            self.writer = SWWWriter(sww_path(self.datadir, self.name), self.mesh.points, tris,
                                    self.quantities["elevation"].vertex_values, fric,
                                    smooth=self.smooth, starttime=self.starttime)
        self.writer.store_timestep(self.get_time(), {
            n: self.quantities[n].vertex_values for n in ("stage", "xmomentum", "ymomentum")})

    def check_integrity(self):
        return True

    def __len__(self):
        return self.number_of_elements

    # -- per-method entry points (gpu_domain_advanced.py) ----------------
    def protect_against_infinitesimal_and_negative_heights(self):
        check(lib().swgpu_protect(self._h), self._h)

    def distribute_to_vertices_and_edges(self):
        check(lib().swgpu_distribute_to_vertices_and_edges(self._h), self._h)

    def update_boundary(self):
        check(lib().swgpu_update_boundary(self._h), self._h)

    def compute_fluxes(self):
        ft = C.c_double()
        check(lib().swgpu_compute_fluxes(self._h, C.byref(ft)), self._h)
        self.flux_timestep = ft.value
        return ft.value

    def compute_forcing_terms(self):
        check(lib().swgpu_compute_forcing_terms(self._h), self._h)

    manning_friction_implicit = compute_forcing_terms

    def manning_friction_explicit(self):
        """gpu_domain_advanced.py:1330-1388: Manning friction added to the
        explicit updates of the momenta."""
        check(lib().swgpu_manning_friction_explicit(self._h), self._h)

    def extrapolate_second_order_sw(self):
        """gpu_domain_advanced.py:1061-1161: the limited second-order
        reconstruction of stage and momentum (through velocity when
        extrapolate_velocity_second_order) at the vertices; no protect, no
        balance."""
        check(lib().swgpu_extrapolate_second_order_sw(self._h), self._h)

    def balance_deep_and_shallow(self):
        """gpu_domain_advanced.py:957-995 on the current vertex values."""
        check(lib().swgpu_balance_deep_and_shallow(self._h), self._h)

    @property
    def max_speed(self):
        """Per-triangle max_speed of the last compute_fluxes (FP64)."""
        out = np.empty(self.number_of_elements)
        check(lib().swgpu_get_max_speed(self._h, f64p(out)), self._h)
        return self._to_user(out)

    def apply_protection_against_isolated_degenerate_timesteps(self):
        """gpu_domain_advanced.py:914-951: when the fastest triangle exceeds
        10 m/s and stands alone at the top of a 10-bin histogram of max_speed
        (bins 4..8 empty), zero the momentum of the triangles above the last
        bin edge.  Bins and counts as ANUGA's numerical_tools.create_bins /
        histogram: edges arange(min, max, (max-min)/10), counts between
        consecutive edges of the sorted speeds, the last bin open-ended."""
        if not self.protect_against_isolated_degenerate_timesteps:
            return
        ms = self.max_speed
        if ms.max() < 10.0:
            return
        mx, mn = float(ms.max()), float(ms.min())
        bins = np.array([mn]) if mx == mn else np.arange(mn, mx, (mx - mn) / 10.0)
        n = np.searchsorted(np.sort(ms), bins)
        hist = np.diff(np.concatenate([n, [len(ms)]]))
        if len(hist) > 1 and hist[-1] > 0 and (hist[4:9] == 0).all():
            sel = ms > bins[-1]
            for name in ("xmomentum", "ymomentum"):
                q = self.quantities[name]
                c, v, e = q.centroid_values, q.vertex_values, q.edge_values
                c[sel] = 0.0
                self._upload(name, self._to_internal(c), self._to_internal(v),
                             self._to_internal(e))

    def update_timestep(self, yieldstep, finaltime):
        """Generic_Domain.update_timestep (restated in
        src/anuga_HMPP/evolve.c:115-160) on the device-held time state,
        after the degenerate-timestep protection when it is switched on."""
        self.apply_protection_against_isolated_degenerate_timesteps()
        p = self.parameters
        s = self._state()
        dt = min(p.CFL * self.flux_timestep, p.evolve_max_timestep)
        s.recorded_max_timestep = max(dt, s.recorded_max_timestep)
        s.recorded_min_timestep = min(dt, s.recorded_min_timestep)
        if dt < p.evolve_min_timestep:
            s.smallsteps += 1
            if s.smallsteps > p.max_smallsteps:
                s.smallsteps = 0
                if s.order == 1:
                    raise RuntimeError(f"Too small timestep {dt:.16f} reached even after "
                                       f"{p.max_smallsteps} steps of 1 order scheme")
                s.order = 1
        else:
            s.smallsteps = 0
            if s.order == 1 and p.default_order == 2:
                s.order = 2
        if finaltime is not None and s.time + dt > finaltime:
            dt = finaltime - s.time
        if s.time + dt > s.yieldtime:
            dt = s.yieldtime - s.time
        s.timestep = dt
        s.flux_timestep = self.flux_timestep
        self._set_state(s)
        self.timestep = dt
        return dt

    def update_conserved_quantities(self):
        check(lib().swgpu_update_conserved_quantities(self._h, float(self.timestep)), self._h)

    def evolve_one_euler_step(self, yieldstep, finaltime):
        """gpu_domain_advanced.py:2178-2191, one method at a time."""
        self.compute_fluxes()
        self.compute_forcing_terms()
        self.update_timestep(yieldstep, finaltime)
        self.update_conserved_quantities()

    def backup_conserved_quantities(self):
        check(lib().swgpu_backup_conserved_quantities(self._h), self._h)

    def saxpy_conserved_quantities(self, a, b):
        check(lib().swgpu_saxpy_conserved_quantities(self._h, float(a), float(b)), self._h)

    def _rk_stage(self):
        self.compute_fluxes()
        self.compute_forcing_terms()
        self.update_conserved_quantities()

    def evolve_one_rk2_step(self, yieldstep, finaltime):
        """ANUGA Generic_Domain.evolve_one_rk2_step (called at
        gpu_domain_advanced.py:2198-2204), one method at a time: the second
        stage reuses the first stage's timestep."""
        self.backup_conserved_quantities()
        self.evolve_one_euler_step(yieldstep, finaltime)
        self.set_time(self.get_time() + self.timestep)
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self._rk_stage()
        self.saxpy_conserved_quantities(0.5, 0.5)

    def evolve_one_rk3_step(self, yieldstep, finaltime):
        """ANUGA Generic_Domain.evolve_one_rk3_step (called at
        gpu_domain_advanced.py:2248-2254), one method at a time."""
        initial_time = self.get_time()
        self.backup_conserved_quantities()
        self.evolve_one_euler_step(yieldstep, finaltime)
        self.set_time(self.get_time() + self.timestep)
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self._rk_stage()
        self.saxpy_conserved_quantities(0.25, 0.75)
        self.set_time(initial_time + self.timestep * 0.5)
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self._rk_stage()
        self.saxpy_conserved_quantities(2.0 / 3.0, 1.0 / 3.0)

    def update_other_quantities(self):
        check(lib().swgpu_update_other_quantities(self._h), self._h)

    def update_centroids_of_velocities_and_height(self):
        self.update_other_quantities()

    def update_ghosts(self):
        pass

    def update_extrema(self):
        pass

    def apply_fractional_steps(self):
        pass

    def set_tracking(self, threshold=0.01, on=True):
        """Track, per triangle over the following evolve steps, the maximum
        depth and the first time the depth exceeds ``threshold``."""
        check(lib().swgpu_set_tracking(self._h, int(bool(on)), float(threshold)), self._h)

    def get_tracking(self):
        """(max_depth, arrival_time) per triangle in the caller's order
        (arrival -1 where the depth never exceeded the threshold)."""
        n = self.number_of_elements
        hm = np.empty(n, dtype=np.float32)
        ta = np.empty(n, dtype=np.float32)
        check(lib().swgpu_get_tracking(self._h, hm.ctypes.data_as(C.POINTER(C.c_float)),
                                       ta.ctypes.data_as(C.POINTER(C.c_float))), self._h)
        return self._to_user(hm), self._to_user(ta)

    def get_water_volume(self):
        m = C.c_double()
        check(lib().swgpu_mass(self._h, C.byref(m)), self._h)
        return m.value

    # -- evolve -----------------------------------------------------------
    def evolve(self, yieldstep=None, finaltime=None, duration=None, skip_initial_step=False,
               max_steps=None):
        """Domain.evolve as a generator (gpu_domain_advanced.py:2296-2697).

        The time loop runs on the device: each Euler stage is three kernels
        (flux, update, distribute; the mixed path adds a one-thread-per-
        scenario kernel for the step's clock; an RK2 step is two stages,
        an RK3 step three; set_timestepping_method),
        the timestep is reduced on the device, and steps are issued as CUDA
        graphs; the host synchronises only between graphs and at yields.
        ``max_steps`` (added) stops after that many steps in total."""
        if finaltime is not None and duration is not None:
            raise ValueError("give finaltime or duration, not both")
        if self.protect_against_isolated_degenerate_timesteps:
            raise NotImplementedError(
                "the degenerate-timestep protection runs on the host between per-method "
                "steps (evolve_one_euler_step); the device-resident evolve does not call it")
        start = self.starttime
        if duration is not None:
            finaltime = start + float(duration)
        if finaltime is not None and finaltime < start:
            raise ValueError("finaltime before starttime")
        if yieldstep is None:
            yieldstep = self.parameters.evolve_max_timestep
        self.yieldstep = float(yieldstep)
        self.finaltime = None if finaltime is None else float(finaltime)
        check(lib().swgpu_evolve_start(self._h, start, self.yieldstep,
                                       -1.0 if finaltime is None else float(finaltime)), self._h)
        if not skip_initial_step:
            if self.store:
                self.store_timestep()
            yield self.get_time()
        remaining = max_steps
        st = _lib.State_t()
        while True:
            budget = 0 if remaining is None else int(remaining)
            if remaining is not None and remaining <= 0:
                return
            steps_before = self._state().total_steps
            check(lib().swgpu_evolve_run(self._h, budget, C.byref(st)), self._h)
            if remaining is not None:
                remaining -= st.total_steps - steps_before
            if st.stop_reason in (_lib.STOP_FINAL, _lib.STOP_YIELD) and self.store:
                self.store_timestep()
            if st.stop_reason == _lib.STOP_FINAL:
                yield st.time
                return
            if st.stop_reason == _lib.STOP_YIELD:
                yield st.time
            elif st.stop_reason == _lib.STOP_BUDGET:
                return

    def evolve_steps(self, nsteps, yieldstep=None, finaltime=None):
        """Start an evolve and run exactly ``nsteps`` steps with no
        yields in between (unless finaltime comes first); returns the final
        device state."""
        if yieldstep is None:
            yieldstep = 1.0e300
        if nsteps < 0:
            raise ValueError("nsteps must be >= 0")
        check(lib().swgpu_evolve_start(self._h, self.starttime, float(yieldstep),
                                       -1.0 if finaltime is None else float(finaltime)), self._h)
        st = _lib.State_t()
        if nsteps == 0:  # the library reads a zero budget as "no limit"
            check(lib().swgpu_get_state(self._h, C.byref(st)), self._h)
            return st
        check(lib().swgpu_evolve_run(self._h, int(nsteps), C.byref(st)), self._h)
        return st

    def step(self):
        """One Euler step plus distribute and boundary, issued without a
        graph (after evolve_start / evolve_steps)."""
        st = _lib.State_t()
        check(lib().swgpu_evolve_one_step(self._h, C.byref(st)), self._h)
        return st

    def synchronize(self):
        check(lib().swgpu_synchronize(self._h), self._h)

    def timestepping_statistics(self):
        s = self._state()
        return (f"Time = {s.time:.4f}, delta t in [{s.recorded_min_timestep:.8f}, "
                f"{s.recorded_max_timestep:.8f}], steps={s.number_of_steps}")

    # -- convenience -------------------------------------------------------
    def get_conserved(self):
        """(stage, xmomentum, ymomentum) centroid values, caller's order."""
        return tuple(self.quantities[n].centroid_values for n in self.conserved_quantities)

    @staticmethod
    def device_info():
        buf = C.create_string_buffer(256)
        check(lib().swgpu_device_info(buf, 256))
        return buf.value.decode()
