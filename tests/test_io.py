"""Mesh input (.tsh) and result output (.sww): CPU only."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REF_TSH = os.path.join(os.environ.get("ANUGA_CUDA_REFERENCE", "/root/reference"),
                       "tests", "CUDA", "merimbula", "merimbula_10785.tsh")

SQUARE_TSH = """5 1 # <# of verts> <# of vert attributes>, next lines <vertex #> <x> <y> [attributes] ...Triangulation Vertices...
0 0.0 0.0 -1.0
1 2.0 0.0 -1.5
2 2.0 2.0 -2.0
3 0.0 2.0 -1.5
4 1.0 1.0 -1.25
# attribute column titles ...Triangulation Vertex Titles...
elevation
4 # <# of triangles>, next lines <triangle #> [<vertex #>] [<neigbouring triangle #>] [attribute of region] ...Triangulation Triangles...
0 0 1 4 1 3 -1
1 1 2 4 2 0 -1 pool
2 2 3 4 3 1 -1
3 3 0 4 0 2 -1
4 # <# of segments>, next lines <segment #> <vertex #>  <vertex #> [boundary marker] ...Triangulation Segments...
0 0 1 bottom
1 1 2 right
2 2 3
3 3 0 left
0 # <# of vertices on outline>
"""


def _write(tmp_path):
    p = tmp_path / "square.tsh"
    p.write_text(SQUARE_TSH)
    return str(p)


def test_read_tsh_blocks(tmp_path):
    from anuga_cuda.io import read_tsh
    t = read_tsh(_write(tmp_path))
    assert t["vertices"].shape == (5, 2) and t["vertices"][2].tolist() == [2.0, 2.0]
    assert t["vertex_attribute_titles"] == ["elevation"]
    assert t["vertex_attributes"][:, 0].tolist() == [-1.0, -1.5, -2.0, -1.5, -1.25]
    assert t["triangles"].tolist() == [[0, 1, 4], [1, 2, 4], [2, 3, 4], [3, 0, 4]]
    assert t["triangle_neighbors"][0].tolist() == [1, 3, -1]
    assert t["triangle_tags"] == ["", "pool", "", ""]
    assert t["segments"].tolist() == [[0, 1], [1, 2], [2, 3], [3, 0]]
    assert t["segment_tags"] == ["bottom", "right", "", "left"]


def test_tsh_boundary_mapping(tmp_path):
    from anuga_cuda.io import read_tsh, tsh_to_mesh_arrays
    from anuga_cuda.mesh import Mesh
    pts, tris, bnd = tsh_to_mesh_arrays(read_tsh(_write(tmp_path)))
    # edge i of a triangle runs between its vertices i+1 and i+2: the outer
    # edge of every triangle here is edge 2 (vertices 0-1 of the row)
    assert bnd == {(0, 2): "bottom", (1, 2): "right", (3, 2): "left"}
    m = Mesh(pts, tris, bnd)
    assert sorted(m.tag_names) == ["bottom", "exterior", "left", "right"]
    assert m.number_of_boundary_elements == 4
    assert abs(m.tag_length("right") - 2.0) < 1e-15


def test_merimbula_fixture_matches_reference_file():
    from anuga_cuda.io import read_tsh, tsh_to_mesh_arrays
    g = np.load(os.path.join(HERE, "golden", "merimbula_10785.npz"))
    assert g["counts"].tolist() == [5719, 10785, 651]
    if not os.path.exists(REF_TSH):
        pytest.skip("reference mesh file not present")
    t = read_tsh(REF_TSH)
    pts, tris, bnd = tsh_to_mesh_arrays(t)
    assert np.array_equal(pts, g["points"]) and np.array_equal(tris, g["triangles"])
    names = g["tag_names"].tolist()
    assert {(int(k), int(e)): names[int(i)] for k, e, i in g["boundary"]} == bnd


def test_merimbula_mesh_builds():
    from anuga_cuda.mesh import Mesh
    g = np.load(os.path.join(HERE, "golden", "merimbula_10785.npz"))
    names = g["tag_names"].tolist()
    bnd = {(int(k), int(e)): names[int(i)] for k, e, i in g["boundary"]}
    m = Mesh(g["points"], g["triangles"], bnd)
    assert m.number_of_elements == 10785
    assert set(m.tag_names) == {"exterior", "open"}
    assert (m.areas > 0).all()
    assert m.number_of_boundary_elements == len(bnd)


@pytest.mark.parametrize("smooth", [True, False])
def test_sww_round_trip(tmp_path, smooth):
    pytest.importorskip("scipy")
    from anuga_cuda.io import SWWWriter, read_sww
    pts = np.array([[10.0, 20.0], [12.0, 20.0], [12.0, 22.0], [10.0, 22.0]])
    tris = np.array([[0, 1, 2], [0, 2, 3]])
    z = np.array([[-1.0, -2.0, -3.0], [-1.0, -3.0, -4.0]])
    path = str(tmp_path / "r.sww")
    w = SWWWriter(path, pts, tris, z, smooth=smooth, starttime=5.0)
    rng = np.random.default_rng(0)
    slices = []
    for t in (5.0, 6.5):
        q = {n: rng.standard_normal((2, 3)) for n in ("stage", "xmomentum", "ymomentum")}
        w.store_timestep(t, q)
        slices.append(q)
    r = read_sww(path)
    assert r["time"].tolist() == [5.0, 6.5]
    assert r["attributes"]["smoothing"] == (b"Yes" if smooth else b"No")
    if smooth:
        assert r["x"].tolist() == [0.0, 2.0, 2.0, 0.0] and r["volumes"].tolist() == tris.tolist()
        # node 0 and 2 are shared: averages of the two triangles' vertex values
        st = slices[1]["stage"]
        exp0 = 0.5 * (st[0, 0] + st[1, 0])
        assert abs(r["stage"][1, 0] - exp0) < 1e-6
        assert abs(r["elevation"][2] - (-3.0)) < 1e-6
    else:
        assert r["stage"].shape == (2, 6)
        assert np.allclose(r["stage"][0], slices[0]["stage"].ravel(), atol=1e-6)
        assert r["volumes"].tolist() == [[0, 1, 2], [3, 4, 5]]
    lo, hi = r["stage_range"]
    allv = np.concatenate([r["stage"].ravel()])
    assert lo <= allv.min() + 1e-6 and hi >= allv.max() - 1e-6
