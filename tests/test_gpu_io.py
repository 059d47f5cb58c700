"""Result output and real-mesh input on the GPU: SWW time slices written at
the yields of evolve, and the reference's Merimbula estuary mesh (its
tests/CUDA/merimbula/merimbula.py set-up: flat bed, a 2 m high band of
water between x = 756000 and 756500, reflective walls) against the oracle."""
import os

import numpy as np
import pytest

from helpers import gpu_from_scenario, max_rel, oracle_from_scenario

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def merimbula_scenario():
    from anuga_cuda.boundaries import Reflective_boundary
    from anuga_cuda.mesh import Mesh
    from anuga_cuda.scenarios import Scenario
    g = np.load(os.path.join(HERE, "golden", "merimbula_10785.npz"))
    names = g["tag_names"].tolist()
    bnd = {(int(k), int(e)): names[int(i)] for k, e, i in g["boundary"]}
    mesh = Mesh(g["points"], g["triangles"], bnd)
    N = mesh.number_of_elements
    xc = mesh.centroid_coordinates.reshape(-1, 2)[:, 0]
    stage = 2.0 * ((xc > 756000.0) & (xc < 756500.0)) + 1.0
    return Scenario(name="merimbula_10785", mesh=mesh, elevation_vertex=np.zeros((N, 3)),
                    stage_centroid=stage, xmom_centroid=np.zeros(N), ymom_centroid=np.zeros(N),
                    friction=np.zeros(N),
                    boundaries={t: Reflective_boundary() for t in mesh.tag_names})


def test_merimbula_matches_oracle(oracle_mod, swgpu_built):
    from anuga_cuda import DEFAULT
    sc = merimbula_scenario()
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    od.run_steps(200)
    d = gpu_from_scenario(sc, DEFAULT)
    st = d.evolve_steps(200)
    assert st.status == 0
    for name, pre in (("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom")):
        assert max_rel(d.quantities[name].centroid_values,
                       od.arrays[pre + "_centroid_values"]) <= 1e-10, name
    assert abs(d.get_water_volume() - od.mass()) <= 1e-12 * od.mass()
    m = gpu_from_scenario(sc, DEFAULT, "mixed")
    m.evolve_steps(200)
    assert max_rel(m.quantities["stage"].centroid_values,
                   d.quantities["stage"].centroid_values) < 1e-5


@pytest.mark.parametrize("smooth", [True, False])
def test_sww_written_at_yields(tmp_path, smooth, swgpu_built):
    pytest.importorskip("scipy")
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda.io import read_sww
    sc = scenarios.small_basin(10, 8, seed=3)
    d = gpu_from_scenario(sc, DEFAULT)
    d.set_name("basin")
    d.set_datadir(str(tmp_path))
    d.set_store(True)
    d.set_store_vertices_uniquely(not smooth)
    times = list(d.evolve(yieldstep=0.1, finaltime=0.3))
    r = read_sww(str(tmp_path / "basin.sww"))
    assert np.allclose(r["time"], times, rtol=0, atol=1e-12) and len(times) == 4
    wv = d.quantities["stage"].vertex_values
    tris = np.asarray(d.mesh.triangles)
    if smooth:
        cnt = np.bincount(tris.ravel(), minlength=len(d.mesh.points))
        exp = np.bincount(tris.ravel(), weights=wv.ravel(), minlength=len(d.mesh.points)) / cnt
    else:
        exp = wv.ravel()
    assert np.allclose(r["stage"][-1], exp, rtol=0, atol=1e-5)
    assert r["stage"].shape[0] == 4
    zv = d.quantities["elevation"].vertex_values
    assert np.allclose(r["elevation"].min(), zv.min(), atol=1e-5)


def test_create_domain_from_tsh_file(tmp_path, swgpu_built):
    from anuga_cuda import Reflective_boundary
    from anuga_cuda.io import create_domain_from_file
    from test_io import SQUARE_TSH
    p = tmp_path / "square.tsh"
    p.write_text(SQUARE_TSH)
    d = create_domain_from_file(str(p))
    assert sorted(d.mesh.tag_names) == ["bottom", "exterior", "left", "right"]
    z = d.quantities["elevation"].vertex_values
    assert np.isclose(z.min(), -2.0) and np.isclose(z.max(), -1.0)
    d.set_quantity("stage", -0.5)
    d.set_boundary({t: Reflective_boundary(d) for t in d.mesh.tag_names})
    v0 = d.get_water_volume()
    d.evolve_steps(20)
    assert abs(d.get_water_volume() - v0) < 1e-12 * v0


def test_clockwise_triangles_keep_caller_vertex_order(swgpu_built):
    """Vertex values set and read back in the caller's vertex order although
    the Mesh turns clockwise triangles counter-clockwise."""
    from anuga_cuda import GPU_domain
    pts = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0], [2.0, 0.5]])
    tris = np.array([[0, 2, 1], [0, 3, 2], [1, 2, 4]])   # first and last clockwise
    d = GPU_domain(pts, tris)
    z = np.array([[-1.0, -2.0, -3.0], [-4.0, -5.0, -6.0], [-7.0, -8.0, -9.0]])
    d.set_quantity("elevation", z)
    assert np.array_equal(d.quantities["elevation"].vertex_values, z)
    e = d.quantities["elevation"].edge_values
    assert np.allclose(e[:, 0], 0.5 * (z[:, 1] + z[:, 2]))
    assert np.allclose(e[:, 1], 0.5 * (z[:, 0] + z[:, 2]))
