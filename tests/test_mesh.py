"""Mesh builder: ANUGA's neighbour conventions, exact edge antisymmetry,
Morton locality, and the sizes of the benchmark meshes."""
import numpy as np
import pytest

from anuga_cuda import Mesh, rectangular_cross, scenarios
from anuga_cuda.mesh import morton_order


def check_mesh(m):
    N = m.number_of_elements
    nb, ne = m.neighbours, m.neighbour_edges
    for k in range(N):
        for i in range(3):
            n = nb[k, i]
            if n >= 0:
                j = ne[k, i]
                assert nb[n, j] == k
                # exactly negated normals, identical lengths (flux antisymmetry)
                assert m.normals[k, 2 * i] == -m.normals[n, 2 * j]
                assert m.normals[k, 2 * i + 1] == -m.normals[n, 2 * j + 1]
                assert m.edgelengths[k, i] == m.edgelengths[n, j]
            else:
                slot = -n - 1
                assert m.boundary_cells[slot] == k and m.boundary_edges[slot] == i
                assert m.surrogate_neighbours[k, i] == k
    assert (m.areas > 0).all() and (m.radii > 0).all()
    assert (m.number_of_boundaries == (nb < 0).sum(axis=1)).all()
    keys = list(zip(m.boundary_cells.tolist(), m.boundary_edges.tolist()))
    assert keys == sorted(keys), "boundary slots in sorted (triangle, edge) order"
    # outward normals: pointing from the centroid towards the edge midpoint
    V = m.vertex_coordinates.reshape(-1, 3, 2)
    for i in range(3):
        mid = 0.5 * (V[:, (i + 1) % 3] + V[:, (i + 2) % 3])
        d = mid - m.centroid_coordinates
        assert (d[:, 0] * m.normals[:, 2 * i] + d[:, 1] * m.normals[:, 2 * i + 1] > 0).all()


def test_rectangular_cross_small():
    p, t, b = rectangular_cross(3, 2, 3.0, 2.0)
    m = Mesh(p, t, b)
    assert m.number_of_elements == 24
    assert m.number_of_boundary_elements == 2 * (3 + 2)
    assert sorted(m.tag_names) == ["bottom", "left", "right", "top"]
    check_mesh(m)


def test_orientation_and_unlisted_boundary():
    pts = np.array([[0, 0], [1, 0], [0, 1], [1, 1]], dtype=float)
    m = Mesh(pts, [[0, 2, 1], [1, 2, 3]], None, reorder=False)  # first is clockwise
    assert set(m.tag_names) == {"exterior"}
    assert m.number_of_boundary_elements == 4
    check_mesh(m)


def test_rejects_bad_meshes():
    pts = np.array([[0, 0], [1, 0], [2, 0]], dtype=float)
    with pytest.raises(ValueError):
        Mesh(pts, [[0, 1, 2]])
    with pytest.raises(ValueError):
        Mesh(pts, [[0, 1, 5]])


def test_delaunay_harbour_mesh():
    sc = scenarios.tidal_harbour(target_triangles=2000, seed=9)
    check_mesh(sc.mesh)
    assert set(sc.mesh.tag_names) == {"west", "wall"}
    assert 1500 < sc.mesh.number_of_elements < 2600


def test_morton_locality():
    """Neighbours of a Morton-ordered mesh sit close in memory even when the
    input triangles come in random order."""
    p, t, _ = rectangular_cross(32, 32, 1.0, 1.0)
    shuffled = t[np.random.default_rng(1).permutation(len(t))]
    k = np.repeat(np.arange(len(t))[:, None], 3, axis=1)
    m = Mesh(p, shuffled, None)
    d = np.abs(m.neighbours - k)[m.neighbours >= 0]
    m2 = Mesh(p, shuffled, None, reorder=False)
    d2 = np.abs(m2.neighbours - k)[m2.neighbours >= 0]
    assert np.median(d) * 50 < np.median(d2)
    assert np.percentile(d, 90) < 64


def test_morton_order_is_permutation():
    rng = np.random.default_rng(0)
    x, y = rng.random(1000), rng.random(1000)
    o = morton_order(x, y)
    assert sorted(o.tolist()) == list(range(1000))


def test_benchmark_mesh_sizes():
    sc = scenarios.dam_break()
    assert sc.mesh.number_of_elements == 40000
    assert sc.mesh.number_of_boundary_elements == 400
    sc = scenarios.tidal_harbour()
    assert 40000 < sc.mesh.number_of_elements < 50000
