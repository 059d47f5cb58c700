"""Argument and mesh validation at the C ABI (no GPU needed).

`swgpu_create` checks its arguments and the whole topology on the host before
it touches the device, so malformed input is refused with SWGPU_EINVAL or
SWGPU_EMESH and a message, as the reference's Python layer raises on what it
cannot run (gpu_domain_advanced.py:1680, :2100).  A well-formed mesh on a
machine without a GPU fails with SWGPU_ECUDA and no handle: there is no CPU
path to fall back to.
"""
import ctypes as C

import numpy as np
import pytest

from anuga_cuda import DEFAULT, Mesh, _lib, rectangular_cross
from anuga_cuda._lib import check, f64p, i64p, lib

EINVAL, ECUDA, EMESH = 1, 2, 10
INT_FIELDS = ("neighbours", "neighbour_edges", "surrogate_neighbours", "number_of_boundaries",
              "tri_full_flag", "boundary_cells", "boundary_edges", "boundary_tag")
F64_FIELDS = ("normals", "edgelengths", "radii", "areas", "vertex_coordinates",
              "centroid_coordinates")


@pytest.fixture
def arrays(swgpu_built):
    p, t, b = rectangular_cross(4, 3, 4.0, 3.0)
    m = Mesh(p, t, b)
    a = {f: np.ascontiguousarray(getattr(m, f), dtype=np.int64).copy() for f in INT_FIELDS}
    a.update({f: np.ascontiguousarray(getattr(m, f), dtype=np.float64).copy()
              for f in F64_FIELDS})
    a["N"], a["Nb"] = m.number_of_elements, m.number_of_boundary_elements
    return a


def _create(a, precision=_lib.FP64, offsets=None, null=()):
    ms = _lib.Mesh_t()
    ms.number_of_elements, ms.number_of_boundary_elements = a["N"], a["Nb"]
    for f in INT_FIELDS + F64_FIELDS:
        if f not in null:
            setattr(ms, f, i64p(a[f]) if f in INT_FIELDS else f64p(a[f]))
    ps = _lib.Params_t(*DEFAULT.as_tuple())
    h = C.c_void_p()
    if offsets is None:
        st = lib().swgpu_create(C.byref(ms), C.byref(ps), precision, C.byref(h))
    else:
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        st = lib().swgpu_create_ensemble(C.byref(ms), i64p(off), len(off) - 1, C.byref(ps),
                                         precision, C.byref(h))
    msg = lib().swgpu_last_error(None)
    if st == 0:
        lib().swgpu_destroy(h)
    else:
        assert not h.value, "a failed create must not hand out a handle"
    return st, (msg.decode() if msg else "")


def test_null_arguments_refused(arrays):
    ps = _lib.Params_t(*DEFAULT.as_tuple())
    h = C.c_void_p()
    assert lib().swgpu_create(None, C.byref(ps), _lib.FP64, C.byref(h)) == EINVAL
    st, msg = _create(arrays, null=("normals",))
    assert st == EINVAL and "null mesh array" in msg


def test_bad_precision_and_sizes_refused(arrays):
    assert _create(arrays, precision=7)[0] == EINVAL
    bad = dict(arrays, N=0)
    st, msg = _create(bad)
    assert st == EINVAL and "bad sizes" in msg
    assert _create(dict(arrays, Nb=3 * arrays["N"] + 1))[0] == EINVAL
    assert _create(dict(arrays, Nb=-1))[0] == EINVAL
    # the largest mesh a handle takes: 2^29 - 1 triangles (int32 packed neighbours)
    st, msg = _create(dict(arrays, N=1 << 29))
    assert st == EINVAL and "bad sizes" in msg


def test_noalloc_volume_refuses_before_touching_memory(swgpu_built):
    # the pointers are never dereferenced: sizes and nulls are checked first
    fake = C.c_void_p(4096)
    L = lib()
    assert L.swgpu_water_volume_noalloc(fake, fake, fake, 4_194_305, fake, None) == EINVAL
    assert b"4194304" in L.swgpu_last_error(None)
    assert L.swgpu_water_volume_noalloc(fake, fake, fake, 0, fake, None) == EINVAL
    assert L.swgpu_water_volume_noalloc(None, fake, fake, 4, fake, None) == EINVAL
    assert b"null" in L.swgpu_last_error(None)


def _wrong_neighbour_edge(a):
    k, i = np.argwhere(a["neighbours"] >= 0)[0]       # the first interior edge
    a["neighbour_edges"][k, i] = (a["neighbour_edges"][k, i] + 1) % 3


def _surrogate_out_of_range(a):
    a["surrogate_neighbours"][1, 2] = a["N"]


def _wrong_boundary_count(a):
    a["number_of_boundaries"][0] += 1


def _boundary_edge_out_of_range(a):
    a["boundary_edges"][0] = 3


def _boundary_cell_out_of_range(a):
    a["boundary_cells"][0] = -1


@pytest.mark.parametrize("corrupt, words", [
    (_wrong_neighbour_edge, "inconsistent"),
    (_surrogate_out_of_range, "surrogate neighbour"),
    (_wrong_boundary_count, "number_of_boundaries"),
    (_boundary_edge_out_of_range, "boundary slot"),
    (_boundary_cell_out_of_range, "boundary slot"),
])
def test_malformed_topology_refused(arrays, corrupt, words):
    corrupt(arrays)
    st, msg = _create(arrays)
    assert st == EMESH and words in msg, (st, msg)


def test_ensemble_offsets_validated(arrays):
    N = arrays["N"]
    assert N % 256 != 0
    assert _create(arrays, offsets=[0, N])[0] == EINVAL            # range end not 256-aligned
    st, msg = _create(arrays, offsets=[1, N])
    assert st == EINVAL and "offsets" in msg


def test_well_formed_mesh_reaches_the_device_or_fails_loudly(arrays):
    st, msg = _create(arrays)
    if st != 0:
        assert st == ECUDA and "CUDA" in msg, (st, msg)
    # and a call on no handle raises instead of running anything
    with pytest.raises(_lib.SwgpuError):
        check(lib().swgpu_evolve_run(None, 1, None), None)
