"""Shared helpers of the test suite: golden fixtures, scenario -> domain,
comparisons."""
import os
from types import SimpleNamespace

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLDEN_CASES = ["four_triangles", "single_triangle", "basin_wetdry", "basin_momentum_limiter",
                "harbour_small", "basin_edge_limiter", "channel_vertex_limiter", "basin_tsunami"]
MESH_KEYS = ["neighbours", "neighbour_edges", "surrogate_neighbours", "number_of_boundaries",
             "tri_full_flag", "normals", "edgelengths", "radii", "areas", "vertex_coordinates",
             "centroid_coordinates", "boundary_cells", "boundary_edges", "boundary_tag"]


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def golden_mesh(g):
    m = SimpleNamespace(**{k: g["mesh/" + k] for k in MESH_KEYS})
    m.number_of_elements = len(m.areas)
    m.number_of_boundary_elements = len(m.boundary_cells)
    m.permutation = np.arange(m.number_of_elements)
    m.tag_names = [f"tag{i}" for i in range(len(g["tags/type"]))]
    return m


def golden_params(g):
    from anuga_cuda.config import Parameters
    import dataclasses
    vals = g["params"]
    fields = dataclasses.fields(Parameters)
    kw = {}
    for f, v in zip(fields, vals):
        kw[f.name] = int(v) if f.type in (int, "int") else float(v)
    return Parameters(**kw)


def golden_tags(g):
    return [(int(t), tuple(float(x) for x in p)) for t, p in zip(g["tags/type"], g["tags/p"])]


def golden_oracle(g, O):
    m = golden_mesh(g)
    od = O.OracleDomain(m, golden_params(g), golden_tags(g))
    for k in ["stage_centroid_values", "xmom_centroid_values", "ymom_centroid_values",
              "bed_centroid_values", "friction_centroid_values", "stage_vertex_values",
              "xmom_vertex_values", "ymom_vertex_values", "bed_vertex_values",
              "bed_edge_values"]:
        od.arrays[k][:] = g["init/" + k]
    # edge values of stage/momentum start as the vertex values' interpolation
    return od


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


def max_rel(a, b, floor=1e-12):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = max(np.max(np.abs(b)), floor)
    return float(np.max(np.abs(a - b)) / scale) if a.size else 0.0


def gpu_from_golden(g, precision="fp64"):
    """A GPU_domain holding a golden case's mesh, parameters, boundary tags
    and initial state."""
    import ctypes
    from anuga_cuda import GPU_domain, _lib
    from anuga_cuda._lib import check, f64p, lib
    m = golden_mesh(g)
    d = GPU_domain(mesh=m, parameters=golden_params(g), precision=precision)
    tags = golden_tags(g)
    arr = (_lib.BoundaryTag_t * len(tags))()
    for i, (t, p) in enumerate(tags):
        arr[i].type = t
        for j, v in enumerate(p):
            arr[i].p[j] = v
    check(lib().swgpu_set_boundary_tags(d._h, arr, len(tags)), d._h)
    N = m.number_of_elements

    def up(q, c, v=None, e=None):
        c = np.ascontiguousarray(c, dtype=np.float64)
        v = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        e = None if e is None else np.ascontiguousarray(e, dtype=np.float64)
        check(lib().swgpu_set_quantity(d._h, q, f64p(c), None if v is None else f64p(v),
                                       None if e is None else f64p(e)), d._h)

    up(_lib.ELEVATION, g["init/bed_centroid_values"], g["init/bed_vertex_values"],
       g["init/bed_edge_values"])
    up(_lib.FRICTION, g["init/friction_centroid_values"])
    zero_edges = np.zeros(3 * N)
    up(_lib.STAGE, g["init/stage_centroid_values"], g["init/stage_vertex_values"], zero_edges)
    up(_lib.XMOMENTUM, g["init/xmom_centroid_values"], g["init/xmom_vertex_values"], zero_edges)
    up(_lib.YMOMENTUM, g["init/ymom_centroid_values"], g["init/ymom_vertex_values"], zero_edges)
    _ = ctypes
    return d


def gpu_from_scenario(sc, params, precision="fp64"):
    from anuga_cuda import GPU_domain
    d = GPU_domain(mesh=sc.mesh, parameters=params, precision=precision)
    sc.apply_to(d)
    return d


def oracle_from_scenario(O, sc, params):
    od = O.OracleDomain(sc.mesh, params, sc.oracle_tags())
    sc.apply_to_oracle(od)
    return od
