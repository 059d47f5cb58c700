"""CPU oracle for the ANUGA shallow-water evolve step -- TEST INFRASTRUCTURE.

Two CPU implementations, used only by tests/, the smoke check and the CPU
baseline leg of bench.py (never by the product, which has no CPU path):

* :class:`OracleDomain` drives ``oracle/swcpu.c`` (built by ``oracle/Makefile``
  into ``oracle/_build/libswcpu.so``), a plain-C restatement of the
  reference's ANUGA C path; it exists wherever gcc does, including the GPU
  box.
* :class:`ReferenceKernels` drives the reference's own vendored ANUGA C
  kernels, compiled from ``src/anuga_HMPP/shallow_water_ext.c`` and
  ``quantity.c`` where the reference sources are present (``make -C oracle
  ref`` -> ``oracle/_ref/``).  It pins the restatement: tests compare the two
  kernel by kernel, and ``tests/golden/make_golden.py`` stores its outputs as
  fixtures for machines without the reference.

All arrays use ANUGA's layout ([3k+i], [6k+2i]) and int64 indices.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SWCPU_SO = os.path.join(HERE, "_build", "libswcpu.so")
REF_SW_SO = os.path.join(HERE, "_ref", "libref_sw.so")
REF_Q_SO = os.path.join(HERE, "_ref", "libref_quantity.so")
REF_SWB2_SO = os.path.join(HERE, "_ref", "libref_swb2.so")
# the reference project's root (its vendored ANUGA C kernels are compiled
# from there when present): $ANUGA_CUDA_REFERENCE, default /root/reference
REFERENCE_ROOT = os.environ.get("ANUGA_CUDA_REFERENCE", "/root/reference")
REFERENCE_SRC = os.path.join(REFERENCE_ROOT, "src", "anuga_HMPP")

BC_REFLECTIVE, BC_DIRICHLET, BC_TIME_STAGE_SINE = 0, 1, 2

_d = C.POINTER(C.c_double)
_l = C.POINTER(C.c_long)
_u8 = C.POINTER(C.c_ubyte)


def build(ref: bool | None = None, quiet: bool = True) -> None:
    """make the oracle; also the reference kernels when their sources exist."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", HERE], check=True, stdout=out)
    if ref is None:
        ref = os.path.isdir(REFERENCE_SRC)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True, stdout=out)


def reference_available() -> bool:
    return all(os.path.exists(p) for p in (REF_SW_SO, REF_Q_SO, REF_SWB2_SO))


# --------------------------------------------------------------- swcpu.h
class OrcParams(C.Structure):
    _fields_ = [
        ("g", C.c_double), ("epsilon", C.c_double), ("H0", C.c_double),
        ("minimum_allowed_height", C.c_double), ("maximum_allowed_speed", C.c_double),
        ("beta_w", C.c_double), ("beta_w_dry", C.c_double), ("beta_uh", C.c_double),
        ("beta_uh_dry", C.c_double), ("beta_vh", C.c_double), ("beta_vh_dry", C.c_double),
        ("alpha_balance", C.c_double), ("CFL", C.c_double),
        ("evolve_max_timestep", C.c_double), ("evolve_min_timestep", C.c_double),
        ("tight_slope_limiters", C.c_long), ("use_centroid_velocities", C.c_long),
        ("optimise_dry_cells", C.c_long), ("extrapolate_velocity_second_order", C.c_long),
        ("use_sloped_mannings", C.c_long), ("max_smallsteps", C.c_long),
        ("default_order", C.c_long), ("optimised_gradient_limiter", C.c_long),
        ("use_edge_limiter", C.c_long), ("flow_algorithm", C.c_long),
    ]


class OrcTag(C.Structure):
    _fields_ = [("type", C.c_long), ("p", C.c_double * 8)]


_MESH_L = ["neighbours", "neighbour_edges", "surrogate_neighbours", "number_of_boundaries",
           "tri_full_flag"]
_MESH_D = ["normals", "edgelengths", "radii", "areas", "vertex_coordinates",
           "centroid_coordinates"]
_QNAMES = [
    "stage_centroid_values", "xmom_centroid_values", "ymom_centroid_values",
    "bed_centroid_values", "friction_centroid_values",
    "stage_vertex_values", "xmom_vertex_values", "ymom_vertex_values", "bed_vertex_values",
    "stage_edge_values", "xmom_edge_values", "ymom_edge_values", "bed_edge_values",
    "stage_boundary_values", "xmom_boundary_values", "ymom_boundary_values",
    "bed_boundary_values",
    "stage_explicit_update", "xmom_explicit_update", "ymom_explicit_update",
    "stage_semi_implicit_update", "xmom_semi_implicit_update", "ymom_semi_implicit_update",
    "max_speed",
]


_BACKUPS = ["stage_centroid_backup", "xmom_centroid_backup", "ymom_centroid_backup"]


class OrcDomain(C.Structure):
    _fields_ = (
        [("params", C.POINTER(OrcParams)), ("number_of_elements", C.c_long),
         ("number_of_boundary_elements", C.c_long)]
        + [(n, _l) for n in ["neighbours", "neighbour_edges", "surrogate_neighbours"]]
        + [(n, _l) for n in ["number_of_boundaries", "tri_full_flag"]]
        + [(n, _d) for n in ["normals", "edgelengths", "radii", "areas"]]
        + [(n, _d) for n in ["vertex_coordinates", "centroid_coordinates"]]
        + [(n, _l) for n in ["boundary_cells", "boundary_edges", "boundary_tag"]]
        + [("tags", C.POINTER(OrcTag))]
        + [(n, _d) for n in _QNAMES]
        + [("work_flags", _u8), ("work_a", _d), ("work_b", _d)]
        + [(n, C.c_double) for n in ["time", "starttime", "yieldtime", "timestep",
                                     "flux_timestep", "recorded_max_timestep",
                                     "recorded_min_timestep"]]
        + [(n, C.c_long) for n in ["order", "smallsteps", "number_of_steps", "status"]]
        + [("timestepping_method", C.c_long)]
        + [(n, _d) for n in _BACKUPS]
        + [("edge_coordinates", _d)]
    )


_SWCPU = None


def swcpu():
    global _SWCPU
    if _SWCPU is None:
        if not os.path.exists(SWCPU_SO):
            build(ref=False)
        L = C.CDLL(SWCPU_SO)
        P = C.POINTER(OrcDomain)
        for name in ["swcpu_gravity_wb", "swcpu_manning_friction",
                     "swcpu_manning_friction_explicit", "swcpu_protect",
                     "swcpu_extrapolate_second_order_sw", "swcpu_extrapolate_first_order",
                     "swcpu_balance_deep_and_shallow", "swcpu_interpolate_to_edges",
                     "swcpu_distribute_to_vertices_and_edges", "swcpu_update_boundary"]:
            getattr(L, name).argtypes = [P]
            getattr(L, name).restype = None
        L.swcpu_compute_fluxes.argtypes = [P]
        L.swcpu_compute_fluxes.restype = C.c_double
        L.swcpu_edge_speeds.argtypes = [P, _d]
        L.swcpu_edge_speeds.restype = C.c_int
        L.swcpu_update_conserved_quantities.argtypes = [P, C.c_double]
        L.swcpu_update_conserved_quantities.restype = C.c_int
        L.swcpu_update_timestep.argtypes = [P, C.c_double]
        L.swcpu_update_timestep.restype = None
        L.swcpu_evolve_one_euler_step.argtypes = [P, C.c_double]
        L.swcpu_evolve_one_euler_step.restype = C.c_int
        for name in ["swcpu_evolve_one_rk2_step", "swcpu_evolve_one_rk3_step"]:
            getattr(L, name).argtypes = [P, C.c_double]
            getattr(L, name).restype = C.c_int
        L.swcpu_protect_swb2.argtypes = [P]
        L.swcpu_protect_swb2.restype = None
        L.swcpu_extrapolate_second_order_edge_sw.argtypes = [P]
        L.swcpu_extrapolate_second_order_edge_sw.restype = C.c_int
        L.swcpu_extrapolate_and_limit_by_neighbours.argtypes = [P, C.c_int]
        L.swcpu_extrapolate_and_limit_by_neighbours.restype = C.c_int
        L.swcpu_backup_conserved_quantities.argtypes = [P]
        L.swcpu_backup_conserved_quantities.restype = None
        L.swcpu_saxpy_conserved_quantities.argtypes = [P, C.c_double, C.c_double]
        L.swcpu_saxpy_conserved_quantities.restype = None
        L.swcpu_evolve_start.argtypes = [P, C.c_double]
        L.swcpu_evolve_start.restype = None
        L.swcpu_evolve_steps.argtypes = [P, C.c_double, C.c_double, C.c_long, C.c_double]
        L.swcpu_evolve_steps.restype = C.c_int
        L.swcpu_mass.argtypes = [P]
        L.swcpu_mass.restype = C.c_double
        L.swcpu_velocities_and_height.argtypes = [P, _d, _d, _d]
        L.swcpu_velocities_and_height.restype = None
        L.swcpu_boundary_velocities_and_height.argtypes = [P, _d, _d, _d]
        L.swcpu_boundary_velocities_and_height.restype = None
        L.swcpu_set_libm_ulps.argtypes = [C.c_int]
        L.swcpu_set_libm_ulps.restype = None
        _SWCPU = L
    return _SWCPU


def set_libm_ulps(n: int) -> None:
    """Move every pow and sin result of the oracle by n ulps (0 restores
    the host libm's results): a one-ulp libm difference, the kind CUDA's pow
    and sin have against the host's, applied to the oracle alone."""
    swcpu().swcpu_set_libm_ulps(int(n))


def _params_struct(p) -> OrcParams:
    import dataclasses
    vals = {f.name: getattr(p, f.name) for f in dataclasses.fields(p)}
    return OrcParams(**vals)


def edge_midpoints(V):
    """(N, 3, 2) midpoints of the edges of triangles with vertex coordinates
    V (N, 3, 2); edge i is opposite vertex i: 0.5 * (v_j + v_k)."""
    return np.stack([0.5 * (V[:, 1] + V[:, 2]), 0.5 * (V[:, 2] + V[:, 0]),
                     0.5 * (V[:, 0] + V[:, 1])], axis=1)


class OracleDomain:
    """One mesh plus all quantity arrays, driven through libswcpu.so.

    ``mesh`` is an anuga_cuda.mesh.Mesh (or anything with its arrays),
    ``params`` an anuga_cuda.config.Parameters, ``tags`` a list of
    (type, (p0, p1, p2, p3)) per boundary tag index."""

    def __init__(self, mesh, params, tags=None):
        N = mesh.number_of_elements
        Nb = mesh.number_of_boundary_elements
        self.N, self.Nb = N, Nb
        self.params = params
        self._p = _params_struct(params)
        self.arrays = {}
        for n in _MESH_L:
            self.arrays[n] = np.ascontiguousarray(getattr(mesh, n), dtype=np.int64).ravel()
        for n in _MESH_D:
            self.arrays[n] = np.ascontiguousarray(getattr(mesh, n), dtype=np.float64).ravel()
        for n in ["boundary_cells", "boundary_edges", "boundary_tag"]:
            a = np.ascontiguousarray(getattr(mesh, n), dtype=np.int64).ravel()
            self.arrays[n] = a if a.size else np.zeros(1, np.int64)
        for n in _QNAMES:
            size = 3 * N if ("vertex" in n or "edge" in n) else (max(Nb, 1) if "boundary" in n else N)
            self.arrays[n] = np.zeros(size)
        self.arrays["work_flags"] = np.zeros(3 * N, np.uint8)
        self.arrays["work_a"] = np.zeros(N)
        self.arrays["work_b"] = np.zeros(N)
        for n in _BACKUPS:
            self.arrays[n] = np.zeros(N)
        V = np.asarray(mesh.vertex_coordinates, dtype=np.float64).reshape(N, 3, 2)
        self.arrays["edge_coordinates"] = edge_midpoints(V).reshape(-1)
        ntag = max(int(mesh.boundary_tag.max()) + 1 if Nb else 1, len(tags or []), 1)
        self._tags = (OrcTag * ntag)()
        for i, (t, p) in enumerate(tags or []):
            self._tags[i].type = t
            for j, v in enumerate(p):
                self._tags[i].p[j] = v
        D = OrcDomain()
        D.params = C.pointer(self._p)
        D.number_of_elements = N
        D.number_of_boundary_elements = Nb
        for n, a in self.arrays.items():
            if a.dtype == np.int64:
                setattr(D, n, a.ctypes.data_as(_l))
            elif a.dtype == np.uint8:
                setattr(D, n, a.ctypes.data_as(_u8))
            else:
                setattr(D, n, a.ctypes.data_as(_d))
        D.tags = self._tags
        D.order = params.default_order
        D.timestepping_method = 1
        D.recorded_min_timestep = params.evolve_max_timestep
        D.recorded_max_timestep = params.evolve_min_timestep
        self.D = D
        self.L = swcpu()

    # -- data ------------------------------------------------------------
    _PREFIX = {"stage": "stage", "xmomentum": "xmom", "ymomentum": "ymom",
               "elevation": "bed", "friction": "friction"}

    def set_quantity(self, name, centroid, vertex=None, edge=None):
        p = self._PREFIX[name]
        self.arrays[p + "_centroid_values"][:] = np.asarray(centroid, dtype=np.float64).ravel()
        if vertex is not None and p + "_vertex_values" in self.arrays:
            self.arrays[p + "_vertex_values"][:] = np.asarray(vertex, dtype=np.float64).ravel()
        if edge is not None and p + "_edge_values" in self.arrays:
            self.arrays[p + "_edge_values"][:] = np.asarray(edge, dtype=np.float64).ravel()

    def get(self, name):
        return self.arrays[name]

    def centroid(self, name):
        return self.arrays[self._PREFIX[name] + "_centroid_values"]

    def vertex(self, name):
        return self.arrays[self._PREFIX[name] + "_vertex_values"].reshape(-1, 3)

    def edge(self, name):
        return self.arrays[self._PREFIX[name] + "_edge_values"].reshape(-1, 3)

    @property
    def status(self):
        return self.D.status

    @property
    def time(self):
        return self.D.time

    # -- methods ---------------------------------------------------------
    def _ref(self):
        return C.byref(self.D)

    def compute_fluxes(self):
        return self.L.swcpu_compute_fluxes(self._ref())

    def edge_speeds(self):
        """Maximum wave speed of each (triangle, edge) from the triangle's own
        side, [N, 3]; -1 where the dry-cell optimisation skips the edge."""
        out = np.empty(3 * self.N)
        if self.L.swcpu_edge_speeds(self._ref(), out.ctypes.data_as(_d)):
            raise RuntimeError("discontinuous bed")
        return out.reshape(-1, 3)

    def gravity_wb(self):
        self.L.swcpu_gravity_wb(self._ref())

    def manning_friction(self):
        self.L.swcpu_manning_friction(self._ref())

    def manning_friction_explicit(self):
        self.L.swcpu_manning_friction_explicit(self._ref())

    def update_other_quantities(self):
        """Height and velocities at centroids and boundary slots
        (update_other_quantities' kernel): dict name -> (centroid, boundary)."""
        N, Nb = self.N, max(self.Nb, 1)
        c = [np.zeros(N) for _ in range(3)]
        b = [np.zeros(Nb) for _ in range(3)]
        self.L.swcpu_velocities_and_height(self._ref(), *(a.ctypes.data_as(_d) for a in c))
        self.L.swcpu_boundary_velocities_and_height(self._ref(),
                                                    *(a.ctypes.data_as(_d) for a in b))
        return {n: (c[i], b[i][:self.Nb]) for i, n in
                enumerate(("height", "xvelocity", "yvelocity"))}

    def update_conserved_quantities(self, dt):
        return self.L.swcpu_update_conserved_quantities(self._ref(), dt)

    def protect(self):
        self.L.swcpu_protect(self._ref())

    def extrapolate_second_order_sw(self):
        self.L.swcpu_extrapolate_second_order_sw(self._ref())

    def extrapolate_first_order(self):
        self.L.swcpu_extrapolate_first_order(self._ref())

    def protect_swb2(self):
        self.L.swcpu_protect_swb2(self._ref())

    def extrapolate_second_order_edge_sw(self):
        return self.L.swcpu_extrapolate_second_order_edge_sw(self._ref())

    def extrapolate_and_limit_by_neighbours(self, by_edge):
        return self.L.swcpu_extrapolate_and_limit_by_neighbours(self._ref(), int(by_edge))

    def balance_deep_and_shallow(self):
        self.L.swcpu_balance_deep_and_shallow(self._ref())

    def interpolate_to_edges(self):
        self.L.swcpu_interpolate_to_edges(self._ref())

    def distribute_to_vertices_and_edges(self):
        self.L.swcpu_distribute_to_vertices_and_edges(self._ref())

    def update_boundary(self):
        self.L.swcpu_update_boundary(self._ref())

    def update_timestep(self, finaltime=-1.0):
        self.L.swcpu_update_timestep(self._ref(), finaltime)
        return self.D.timestep

    def evolve_one_euler_step(self, finaltime=-1.0):
        return self.L.swcpu_evolve_one_euler_step(self._ref(), finaltime)

    _METHODS = {"euler": 1, "rk2": 2, "rk3": 3}

    def set_timestepping_method(self, method):
        self.D.timestepping_method = self._METHODS[method]

    def backup_conserved_quantities(self):
        self.L.swcpu_backup_conserved_quantities(self._ref())

    def saxpy_conserved_quantities(self, a, b):
        self.L.swcpu_saxpy_conserved_quantities(self._ref(), a, b)

    def evolve_one_rk2_step(self, finaltime=-1.0):
        return self.L.swcpu_evolve_one_rk2_step(self._ref(), finaltime)

    def evolve_one_rk3_step(self, finaltime=-1.0):
        return self.L.swcpu_evolve_one_rk3_step(self._ref(), finaltime)

    def evolve_start(self, yieldstep, starttime=0.0):
        self.D.starttime = starttime
        self.L.swcpu_evolve_start(self._ref(), yieldstep)

    def evolve_steps(self, yieldstep, finaltime, max_steps):
        return self.L.swcpu_evolve_steps(self._ref(), yieldstep,
                                         -1.0 if finaltime is None else finaltime,
                                         int(max_steps), self.params.epsilon)

    def run_steps(self, nsteps, yieldstep=1.0e300, finaltime=None):
        """evolve_start then exactly nsteps steps (no yields)."""
        self.evolve_start(yieldstep)
        rc = self.evolve_steps(yieldstep, finaltime, nsteps)
        return rc

    def mass(self):
        return self.L.swcpu_mass(self._ref())


# ------------------------------------------- the reference's own kernels
class RefDomain(C.Structure):
    """struct domain of src/anuga_HMPP/sw_domain.h:16-180, field for field."""
    _fields_ = (
        [(n, C.c_long) for n in ["number_of_elements", "number_of_boundary_elements",
                                 "boundary_number"]]
        + [(n, C.c_double) for n in ["epsilon", "H0", "h0", "limiting_threshold", "g"]]
        + [("optimise_dry_cells", C.c_long)]
        + [(n, C.c_double) for n in ["evolve_max_timestep", "evolve_min_timestep"]]
        + [("extrapolate_velocity_second_order", C.c_long)]
        + [(n, C.c_double) for n in ["minimum_allowed_height", "time", "starttime",
                                     "finaltime", "yieldtime", "timestep"]]
        + [(n, C.c_int) for n in ["smallsteps", "max_smallsteps", "number_of_steps",
                                  "number_of_first_order_steps", "_order_", "default_order",
                                  "use_sloped_mannings", "use_centroid_velocities",
                                  "use_edge_limiter", "flow_algorithm",
                                  "compute_fluxes_method", "timestepping_method"]]
        + [("boundary_cells", _l), ("boundary_edges", _l), ("boundary_map", C.c_void_p)]
        + [(n, C.c_double) for n in ["CFL", "flux_timestep", "recorded_max_timestep",
                                     "recorded_min_timestep", "maximum_allowed_speed",
                                     "optimised_gradient_limiter", "alpha_balance",
                                     "tight_slope_limiters", "beta_w", "beta_w_dry",
                                     "beta_uh", "beta_uh_dry", "beta_vh", "beta_vh_dry",
                                     "stage_beta", "xmom_beta", "ymom_beta"]]
        + [("neighbours", _l), ("neighbour_edges", _l), ("surrogate_neighbours", _l)]
        + [(n, _d) for n in ["normals", "edgelengths", "radii", "areas"]]
        + [("tri_full_flag", _l), ("already_computed_flux", _l)]
        + [(n, _d) for n in ["max_speed", "timestep_array", "vertex_coordinates",
                             "edge_coordinates", "centroid_coordinates"]]
        + [("number_of_boundaries", _l)]
        + [(q + "_edge_values", _d) for q in ["stage", "xmom", "ymom", "bed", "height",
                                               "xvelocity", "yvelocity"]]
        + [(q + "_centroid_values", _d) for q in ["stage", "xmom", "ymom", "bed", "friction",
                                                   "height", "xvelocity", "yvelocity"]]
        + [(q + "_centroid_store", _d) for q in ["stage", "xmom", "ymom"]]
        + [(q + "_centroid_backup", _d) for q in ["stage", "xmom", "ymom"]]
        + [(q + "_vertex_values", _d) for q in ["stage", "xmom", "ymom", "bed", "height",
                                                 "xvelocity", "yvelocity"]]
        + [(q + "_explicit_update", _d) for q in ["stage", "xmom", "ymom"]]
        + [(q + "_semi_implicit_update", _d) for q in ["stage", "xmom", "ymom"]]
        + [(q + "_x_gradient", _d) for q in ["stage", "xmom", "ymom", "height", "xvelocity",
                                              "yvelocity"]]
        + [(q + "_y_gradient", _d) for q in ["stage", "xmom", "ymom", "height", "xvelocity",
                                              "yvelocity"]]
        + [("min_bed_edge_values", _d), ("max_bed_edge_values", _d),
           ("count_wet_neighbours", C.POINTER(C.c_int))]
        + [(q + "_boundary_values", _d) for q in ["stage", "xmom", "ymom", "bed", "height",
                                                   "xvelocity", "yvelocity"]]
    )


class ReferenceKernels:
    """The reference's own ANUGA C kernels (oracle/_ref), applied in place to
    the arrays of an :class:`OracleDomain`, so that each restated oracle
    routine can be compared with the code it restates."""

    def __init__(self):
        if not reference_available():
            raise FileNotFoundError("oracle/_ref not built (make -C oracle ref)")
        # PyDLL keeps the GIL: the reference reports some errors through
        # PyErr_SetString
        self.sw = C.PyDLL(REF_SW_SO, mode=os.RTLD_LAZY)
        self.q = C.PyDLL(REF_Q_SO, mode=os.RTLD_LAZY)
        self.sw._compute_fluxes_central_structure.argtypes = [C.POINTER(RefDomain)]
        self.sw._compute_fluxes_central_structure.restype = C.c_double
        self.sw._extrapolate_second_order_sw.argtypes = [C.POINTER(RefDomain)]
        self.sw._extrapolate_second_order_sw.restype = C.c_int
        self.sw._balance_deep_and_shallow.argtypes = (
            [C.c_int] + [_d] * 9 + [C.c_double, C.c_int, C.c_int, C.c_double])
        self.sw._balance_deep_and_shallow.restype = C.c_int
        self.sw._protect.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double] + [_d] * 4
        self.sw._protect.restype = C.c_int
        self.sw._manning_friction_flat.argtypes = (
            [C.c_double, C.c_double, C.c_int] + [_d] * 7)
        self.sw._manning_friction_flat.restype = None
        self.sw._manning_friction_sloped.argtypes = (
            [C.c_double, C.c_double, C.c_int] + [_d] * 8)
        self.sw._manning_friction_sloped.restype = None
        self.q._update.argtypes = [C.c_int, C.c_double, _d, _d, _d]
        self.q._update.restype = C.c_int
        self.q._interpolate_from_vertices_to_edges.argtypes = [C.c_int, _d, _d]
        self.q._interpolate_from_vertices_to_edges.restype = C.c_int
        self.q._saxpy_centroid_values.argtypes = [C.c_int, C.c_double, C.c_double, _d, _d]
        self.q._saxpy_centroid_values.restype = C.c_int
        self.q._compute_gradients.argtypes = [C.c_int, _d, _d, _l, _l, _d, _d]
        self.q._compute_gradients.restype = C.c_int
        self.q._extrapolate_from_gradient.argtypes = [C.c_int] + [_d] * 7
        self.q._extrapolate_from_gradient.restype = C.c_int
        for name in ("_limit_vertices_by_all_neighbours", "_limit_edges_by_all_neighbours"):
            getattr(self.q, name).argtypes = [C.c_int, C.c_double, _d, _d, _d, _l, _d, _d]
            getattr(self.q, name).restype = C.c_int
        # gravity_wb exists in the reference only as a Python-C entry point
        # taking a domain object; the module's numpy C API is set up by its
        # init function.
        self.sw._extrapolate_second_order_edge_sw.argtypes = [C.POINTER(RefDomain)]
        self.sw._extrapolate_second_order_edge_sw.restype = C.c_int
        self.swb2 = C.CDLL(REF_SWB2_SO, mode=os.RTLD_LAZY)
        self.swb2.protect_swb2.argtypes = [C.c_long, C.c_long] + [C.c_double] * 3 + [_d] * 7
        self.swb2.protect_swb2.restype = None
        self.sw.initshallow_water_ext.argtypes = []
        self.sw.initshallow_water_ext.restype = None
        self.sw.initshallow_water_ext()
        self.sw.gravity_wb.argtypes = [C.py_object, C.py_object]
        self.sw.gravity_wb.restype = C.py_object

    @staticmethod
    def _ptr(a):
        return a.ctypes.data_as(_l if a.dtype == np.int64 else _d)

    def _struct(self, od: OracleDomain):
        p = od.params
        N = od.N
        R = RefDomain()
        A = od.arrays
        keep = [A]
        R.number_of_elements = N
        R.number_of_boundary_elements = od.Nb
        R.epsilon, R.H0, R.g = p.epsilon, p.H0, p.g
        R.h0 = p.H0 * p.H0
        R.limiting_threshold = 10 * p.H0
        R.optimise_dry_cells = p.optimise_dry_cells
        R.evolve_max_timestep, R.evolve_min_timestep = p.evolve_max_timestep, p.evolve_min_timestep
        R.extrapolate_velocity_second_order = p.extrapolate_velocity_second_order
        R.minimum_allowed_height = p.minimum_allowed_height
        R.beta_w, R.beta_w_dry = p.beta_w, p.beta_w_dry
        R.beta_uh, R.beta_uh_dry = p.beta_uh, p.beta_uh_dry
        R.beta_vh, R.beta_vh_dry = p.beta_vh, p.beta_vh_dry
        for n in ["neighbours", "neighbour_edges", "surrogate_neighbours", "normals",
                  "edgelengths", "radii", "areas", "tri_full_flag", "vertex_coordinates",
                  "centroid_coordinates", "number_of_boundaries", "max_speed",
                  "edge_coordinates"]:
            setattr(R, n, self._ptr(A[n]))
        flags = np.zeros(3 * N, np.int64)
        keep.append(flags)
        R.already_computed_flux = self._ptr(flags)
        for q in ["stage", "xmom", "ymom", "bed"]:
            setattr(R, q + "_edge_values", self._ptr(A[q + "_edge_values"]))
            setattr(R, q + "_centroid_values", self._ptr(A[q + "_centroid_values"]))
            setattr(R, q + "_vertex_values", self._ptr(A[q + "_vertex_values"]))
            setattr(R, q + "_boundary_values", self._ptr(A[q + "_boundary_values"]))
        for q in ["stage", "xmom", "ymom"]:
            setattr(R, q + "_explicit_update", self._ptr(A[q + "_explicit_update"]))
        self._keep = keep
        return R

    @staticmethod
    def _python_domain(od: OracleDomain):
        """The attribute set get_python_domain reads
        (src/anuga_HMPP/sw_domain_fun.h:57-330), backed by od's arrays."""
        from types import SimpleNamespace
        p, A, N = od.params, od.arrays, od.N
        dom = SimpleNamespace(
            number_of_elements=N, epsilon=p.epsilon, H0=p.H0, g=p.g,
            optimise_dry_cells=int(p.optimise_dry_cells),
            evolve_max_timestep=p.evolve_max_timestep, evolve_min_timestep=p.evolve_min_timestep,
            extrapolate_velocity_second_order=int(p.extrapolate_velocity_second_order),
            minimum_allowed_height=p.minimum_allowed_height, _order_=int(p.default_order),
            default_order=int(p.default_order), use_sloped_mannings=int(p.use_sloped_mannings),
            use_centroid_velocities=int(p.use_centroid_velocities), use_edge_limiter=0,
            CFL=p.CFL, flux_timestep=0.0, maximum_allowed_speed=p.maximum_allowed_speed,
            optimised_gradient_limiter=1.0, alpha_balance=p.alpha_balance,
            tight_slope_limiters=float(p.tight_slope_limiters), beta_w=p.beta_w,
            beta_w_dry=p.beta_w_dry, beta_uh=p.beta_uh, beta_uh_dry=p.beta_uh_dry,
            beta_vh=p.beta_vh, beta_vh_dry=p.beta_vh_dry,
            already_computed_flux=np.zeros(3 * N, np.int64),
            edge_coordinates=np.zeros(6 * N))
        for n in ["neighbours", "surrogate_neighbours", "neighbour_edges", "normals",
                  "edgelengths", "radii", "areas", "tri_full_flag", "max_speed",
                  "vertex_coordinates", "centroid_coordinates", "number_of_boundaries",
                  "boundary_cells", "boundary_edges"]:
            setattr(dom, n, A[n])
        Nb = max(od.Nb, 1)

        def quantity(prefix):
            def arr(suffix, size):
                key = f"{prefix}_{suffix}" if prefix else None
                return A[key] if key in A else np.zeros(size)
            return SimpleNamespace(
                edge_values=arr("edge_values", 3 * N), centroid_values=arr("centroid_values", N),
                vertex_values=arr("vertex_values", 3 * N),
                boundary_values=arr("boundary_values", Nb),
                explicit_update=arr("explicit_update", N),
                semi_implicit_update=arr("semi_implicit_update", N),
                x_gradient=np.zeros(N), y_gradient=np.zeros(N), beta=1.0)

        dom.quantities = {"stage": quantity("stage"), "xmomentum": quantity("xmom"),
                          "ymomentum": quantity("ymom"), "elevation": quantity("bed"),
                          "friction": quantity("friction"), "height": quantity(None),
                          "xvelocity": quantity(None), "yvelocity": quantity(None)}
        return dom

    def gravity_wb(self, od: OracleDomain) -> None:
        """The reference's gravity_wb (src/anuga_HMPP/shallow_water_ext.c:1942)
        on od's arrays in place."""
        self.sw.gravity_wb(None, (self._python_domain(od),))

    def compute_fluxes(self, od: OracleDomain) -> float:
        R = self._struct(od)
        return self.sw._compute_fluxes_central_structure(C.byref(R))

    def extrapolate_second_order_sw(self, od: OracleDomain) -> int:
        R = self._struct(od)
        return self.sw._extrapolate_second_order_sw(C.byref(R))

    def balance_deep_and_shallow(self, od: OracleDomain) -> int:
        p, A = od.params, od.arrays
        hvbar = np.zeros(3 * od.N)
        return self.sw._balance_deep_and_shallow(
            od.N, *(self._ptr(A[n]) for n in [
                "stage_centroid_values", "bed_centroid_values", "stage_vertex_values",
                "bed_vertex_values"]), self._ptr(hvbar),
            *(self._ptr(A[n]) for n in ["xmom_centroid_values", "ymom_centroid_values",
                                        "xmom_vertex_values", "ymom_vertex_values"]),
            p.H0, int(p.tight_slope_limiters), int(p.use_centroid_velocities), p.alpha_balance)

    def protect_swb2(self, od: OracleDomain) -> None:
        """protect_swb2 of src/anuga_HMPP/swb2_domain_ext.c:7 on od's arrays."""
        p, A = od.params, od.arrays
        self.swb2.protect_swb2(od.N, 3 * od.N, p.minimum_allowed_height,
                               p.maximum_allowed_speed, p.epsilon,
                               *(self._ptr(A[n]) for n in [
                                   "stage_centroid_values", "stage_vertex_values",
                                   "bed_centroid_values", "bed_vertex_values",
                                   "xmom_centroid_values", "ymom_centroid_values", "areas"]))

    def extrapolate_second_order_edge_sw(self, od: OracleDomain) -> int:
        R = self._struct(od)
        return self.sw._extrapolate_second_order_edge_sw(C.byref(R))

    def protect(self, od: OracleDomain) -> int:
        p, A = od.params, od.arrays
        return self.sw._protect(od.N, p.minimum_allowed_height, p.maximum_allowed_speed,
                                p.epsilon, *(self._ptr(A[n]) for n in [
                                    "stage_centroid_values", "bed_centroid_values",
                                    "xmom_centroid_values", "ymom_centroid_values"]))

    def manning_friction(self, od: OracleDomain, explicit: bool = False) -> None:
        """_manning_friction_flat / _sloped into the semi-implicit updates
        (manning_friction_implicit) or, with ``explicit``, into the explicit
        updates (manning_friction_explicit, gpu_domain_advanced.py:1330-1388)."""
        p, A = od.params, od.arrays
        kind = "explicit" if explicit else "semi_implicit"
        names = ["stage_centroid_values", "bed_vertex_values", "xmom_centroid_values",
                 "ymom_centroid_values", "friction_centroid_values",
                 f"xmom_{kind}_update", f"ymom_{kind}_update"]
        if p.use_sloped_mannings:
            self.sw._manning_friction_sloped(p.g, p.minimum_allowed_height, od.N,
                                             self._ptr(A["vertex_coordinates"]),
                                             *(self._ptr(A[n]) for n in names))
        else:
            self.sw._manning_friction_flat(p.g, p.minimum_allowed_height, od.N,
                                           *(self._ptr(A[n]) for n in names))

    def update(self, od: OracleDomain, dt: float) -> int:
        A = od.arrays
        rc = 0
        for q in ["stage", "xmom", "ymom"]:
            rc |= self.q._update(od.N, dt, self._ptr(A[q + "_centroid_values"]),
                                 self._ptr(A[q + "_explicit_update"]),
                                 self._ptr(A[q + "_semi_implicit_update"]))
        return rc

    def saxpy_conserved_quantities(self, od: OracleDomain, a: float, b: float) -> None:
        """_saxpy_centroid_values (src/anuga_HMPP/quantity.c:749) on the three
        conserved quantities and their backups."""
        A = od.arrays
        for q in ["stage", "xmom", "ymom"]:
            self.q._saxpy_centroid_values(od.N, a, b, self._ptr(A[q + "_centroid_values"]),
                                          self._ptr(A[q + "_centroid_backup"]))

    def limit_by_neighbours(self, od: OracleDomain, by_edge: bool) -> int:
        """Quantity.extrapolate_second_order_and_limit_by_vertex / _by_edge on
        stage, xmomentum and ymomentum (betas beta_w, beta_uh, beta_vh):
        _compute_gradients, _extrapolate_from_gradient and
        _limit_vertices_by_all_neighbours / _limit_edges_by_all_neighbours
        (src/anuga_HMPP/quantity.c:24, :130, :298, :363), with each
        quantity's gradients starting from zero."""
        A, N, p = od.arrays, od.N, od.params
        limit = (self.q._limit_edges_by_all_neighbours if by_edge
                 else self.q._limit_vertices_by_all_neighbours)
        rc = 0
        for q, beta in (("stage", p.beta_w), ("xmom", p.beta_uh), ("ymom", p.beta_vh)):
            gx, gy = np.zeros(N), np.zeros(N)
            qc, qv, qe = (A[q + s] for s in ("_centroid_values", "_vertex_values",
                                              "_edge_values"))
            rc |= self.q._compute_gradients(N, self._ptr(A["centroid_coordinates"]),
                                            self._ptr(qc), self._ptr(A["number_of_boundaries"]),
                                            self._ptr(A["surrogate_neighbours"]), self._ptr(gx),
                                            self._ptr(gy))
            rc |= self.q._extrapolate_from_gradient(
                N, self._ptr(A["centroid_coordinates"]), self._ptr(qc),
                self._ptr(A["vertex_coordinates"]), self._ptr(qv), self._ptr(qe),
                self._ptr(gx), self._ptr(gy))
            rc |= limit(N, beta, self._ptr(qc), self._ptr(qv), self._ptr(qe),
                        self._ptr(A["neighbours"]), self._ptr(gx), self._ptr(gy))
        return rc

    def interpolate_to_edges(self, od: OracleDomain) -> None:
        A = od.arrays
        for q in ["stage", "xmom", "ymom"]:
            self.q._interpolate_from_vertices_to_edges(
                od.N, self._ptr(A[q + "_vertex_values"]), self._ptr(A[q + "_edge_values"]))


# ------------------------------------------------- degenerate-timestep guard

def degenerate_timestep_protection(max_speed, xmom, ymom, nbins=10):
    """The reference's `apply_protection_against_isolated_degenerate_timesteps`
    (src/anuga_cuda/gpu_domain_advanced.py:914-951) restated with plain loops:
    when the fastest triangle exceeds 10 m/s and the histogram of max_speed
    over 10 bins has an occupied last bin and empty bins 4 to 8, the momenta
    of the triangles faster than the last bin's lower edge are zeroed (and
    their max_speed).  The bins and counts are those of ANUGA's
    ``numerical_tools.create_bins`` / ``histogram`` (ANUGA is a dependency
    the reference does not vendor, version unpinned; restated from its
    published definition): lower edges mn, mn + w, ... below mx, w = (mx -
    mn) / nbins (the single edge mn when all speeds are equal); bin i counts
    the speeds in [edge i, edge i+1), the last bin every speed from its edge
    up.  Works on copies; returns (xmom, ymom, max_speed, zeroed indices)."""
    ms = [float(v) for v in max_speed]
    xm = [float(v) for v in xmom]
    ym = [float(v) for v in ymom]
    if not ms or max(ms) < 10.0:
        return np.array(xm), np.array(ym), np.array(ms), []
    mx, mn = max(ms), min(ms)
    if mx == mn:
        edges = [mn]
    else:
        w = (mx - mn) / nbins
        # numpy.arange(mn, mx, w): ceil((mx - mn) / w) edges mn + i w
        edges = [mn + i * w for i in range(int(np.ceil((mx - mn) / w)))]
    hist = [0] * len(edges)
    for v in ms:
        b = -1
        for j, e in enumerate(edges):
            if v >= e:
                b = j
        if b >= 0:
            hist[b] += 1
    zeroed = []
    if len(hist) > 1 and hist[-1] > 0 and all(hist[k] == 0 for k in range(4, 9)):
        for k, v in enumerate(ms):
            if v > edges[-1]:
                xm[k] = ym[k] = 0.0
                ms[k] = 0.0
                zeroed.append(k)
    return np.array(xm), np.array(ym), np.array(ms), zeroed
