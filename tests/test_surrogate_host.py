"""Host logic of the surrogate workflow, without a GPU: the family mesh and
its inflow segment, the Fourier tide and its delayed form, the still-water
depth under the lagged tide, the calibration of the error estimate, and the
windows the solver re-solves (sub-mesh, tags, index map, bed)."""
import numpy as np
import pytest

from anuga_cuda import surrogate as SG


@pytest.fixture(scope="module")
def fm():
    return SG.FamilyMesh(cells=32)


def test_family_mesh_tags_and_features(fm):
    m = fm.mesh
    assert set(m.tag_names) == {"bottom", "inflow", "left", "right", "top"}
    # the east-edge cells whose edge midpoints fall in [4.5, 5.5] km (the
    # hydrograph's discharge is spread over the tag's actual length)
    cell = fm.length / 32
    assert abs(m.tag_length("inflow") - 1000.0) <= cell
    assert fm.tri.shape == (fm.N, 4) and fm.tri.dtype == np.float32
    # the distance to the inflow segment is zero only on the east edge's segment
    east = fm.xy[:, 0] > fm.length - fm.length / 32
    assert fm.d_inflow.min() < fm.length / 32 and np.all(fm.d_inflow[~east] > 0)
    # the bed is the wet/dry generator's: a beach rising east through 0 at 8 km
    west, far_east = fm.xy[:, 0] < 2000.0, fm.xy[:, 0] > 9500.0
    assert fm.zc[west].max() < -50.0 and fm.zc[far_east].min() > 10.0


def test_sample_params_ranges():
    th = SG.sample_params(500, seed=1)
    lo, hi = SG.PARAM_RANGES[:, 0], SG.PARAM_RANGES[:, 1]
    assert np.all(th >= lo) and np.all(th <= hi)
    ratio = th[:, 2] / th[:, 1]
    assert np.all(ratio >= SG.DURATION_RATIO[0]) and np.all(ratio <= SG.DURATION_RATIO[1])
    assert np.array_equal(th, SG.sample_params(500, seed=1))


def test_shifted_tide_is_the_delayed_series():
    th = SG.sample_params(4, seed=2)
    t = np.linspace(0.0, 3600.0, 101)
    for p in th:
        for tau in (0.0, 250.0, 571.0):
            sh = SG.shifted_tide(p, tau)
            assert np.allclose(SG.tide(sh, t), SG.tide(p, t - tau), rtol=0, atol=1e-12)
            assert np.array_equal(sh[:5], p[:5])   # hydrograph, n and c0 untouched


def test_static_depth_under_the_lagged_tide(fm):
    th = SG.sample_params(6, seed=3)
    d = SG.static_depth(fm, th)
    assert d.shape == (6, fm.N) and np.all(d >= 0)
    # the still level never falls below the initial stage nor exceeds the
    # boundary's highest stage over the run
    w0 = th[:, 4] + th[:, 6] + th[:, 8]
    wm = SG.max_tide(th)
    sea = fm.zc < -5.0
    level = d[:, sea] + fm.zc[sea][None, :]     # d is float32: ~1e-5 m at 80 m depth
    assert np.all(level >= w0[:, None] - 1e-4)
    assert np.all(level <= wm[:, None] + 1e-4)
    # the lag grows toward the shore
    lag = SG.wave_lag(fm, 0.0)
    order = np.argsort(fm.xy[:, 0])
    assert np.all(np.diff(lag[order]) >= -1e-9) and lag.max() < 600.0


def test_calibrate_flags_the_requested_share_of_bad_blocks():
    rng = np.random.default_rng(4)
    S, N = 40, 256 * 50
    true = np.abs(rng.normal(0, 0.02, (S, N)))
    est = true * rng.uniform(0.5, 1.5, (S, N))           # an estimate that tracks the error
    k, st = SG.calibrate(est, true, tol=0.05, miss_rate=0.01)
    bmax = lambda a: a.reshape(S, -1, 256).max(axis=2)  # noqa: E731
    bad, flagged = bmax(true) > 0.05, k * bmax(est) > 0.05
    assert st["bad_blocks"] == bad.sum() > 0
    assert (bad & ~flagged).sum() <= 0.01 * bad.sum() + 1
    assert flagged.mean() < 1.0


def test_window_mesh_tags_index_map_and_bed(fm):
    xlo, ylo, yhi = 6000.0, 3000.0, 7000.0
    sub, zv, fam_idx = SG.window_mesh(fm, xlo, ylo, yhi)
    assert sub.number_of_elements == len(fam_idx) == len(set(fam_idx.tolist()))
    c = sub.centroid_coordinates.reshape(-1, 2)
    assert np.allclose(c, fm.xy[fam_idx])
    assert np.all(c[:, 0] >= xlo) and np.all((c[:, 1] >= ylo) & (c[:, 1] <= yhi))
    assert np.array_equal(zv, fm.elevation_vertex[fam_idx])
    assert {"cut_west", "exterior", "inflow", "right"} <= set(sub.tag_names)
    V = sub.vertex_coordinates.reshape(-1, 3, 2)
    for tag, test in (("cut_west", lambda mid: np.allclose(mid[:, 0], xlo, atol=200.0)),
                      ("exterior", lambda mid: np.all(mid[:, 0] > xlo - 1.0))):
        sel = sub.boundary_tag == sub.tag_names.index(tag)
        k, e = sub.boundary_cells[sel], sub.boundary_edges[sel]
        mid = 0.5 * (V[k, (e + 1) % 3] + V[k, (e + 2) % 3])
        assert sel.any() and test(mid), tag


def test_window_scenarios_cover_flagged_blocks_and_inflow(fm):
    th = SG.sample_params(3, seed=5)
    nb = (fm.N + 255) // 256
    flagged = np.zeros((3, nb), bool)
    flagged[1, nb // 2] = True                 # one block near the middle of the Morton order
    out = SG.window_scenarios(fm, th, flagged)
    assert [s for s, _, _ in out] == [1]
    _, sc, fam_idx = out[0]
    blk = SG.block_index(fm.N)
    assert np.isin(np.nonzero(blk == nb // 2)[0], fam_idx).all()
    # the inflow segment is inside every window
    assert "inflow" in sc.mesh.tag_names
    assert sc.boundaries["inflow"].peak == pytest.approx(th[1, 0])
    if "cut_west" in sc.mesh.tag_names:
        b = sc.boundaries["cut_west"]
        assert b.period == SG.TIDE_PERIOD and len(b.coefficients) == 5
