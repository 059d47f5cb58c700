"""The CPU oracle against the golden fixtures made by the reference's own
ANUGA C kernels (tests/golden/make_golden.py): bit for bit, kernel by kernel
over 40 Euler steps and over 12 RK2 and RK3 steps.  Runs everywhere (no reference sources needed)."""
import numpy as np
import pytest

from helpers import GOLDEN_CASES, bits_equal, golden_oracle, golden_params, load_golden

STEPS = 40


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_kernels_match_reference_bitwise(case, oracle_mod):
    g = load_golden(case)
    od = golden_oracle(g, oracle_mod)
    A = od.arrays
    od.protect()
    assert bits_equal(A["stage_centroid_values"], g["k/protect/stage"])
    assert bits_equal(A["xmom_centroid_values"], g["k/protect/xmom"])
    assert bits_equal(A["ymom_centroid_values"], g["k/protect/ymom"])
    od.extrapolate_second_order_sw()
    for q in ("stage", "xmom", "ymom"):
        assert bits_equal(A[q + "_vertex_values"], g[f"k/extrapolate/{q}_vertex"]), q
    od.balance_deep_and_shallow()
    for q in ("stage", "xmom", "ymom"):
        assert bits_equal(A[q + "_vertex_values"], g[f"k/balance/{q}_vertex"]), q
    od.interpolate_to_edges()
    for q in ("stage", "xmom", "ymom"):
        assert bits_equal(A[q + "_edge_values"], g[f"k/interpolate/{q}_edge"]), q
    od.update_boundary()
    ft = od.compute_fluxes()
    assert bits_equal([ft], g["k/flux/timestep"])
    for q in ("stage", "xmom", "ymom"):
        assert bits_equal(A[q + "_explicit_update"], g[f"k/flux/{q}_explicit"]), q
    od.gravity_wb()
    for q in ("xmom", "ymom"):
        assert bits_equal(A[q + "_explicit_update"], g[f"k/gravity/{q}_explicit"]), q
    od.manning_friction()
    for q in ("xmom", "ymom"):
        assert bits_equal(A[q + "_semi_implicit_update"], g[f"k/friction/{q}_semi"]), q
    assert od.update_conserved_quantities(float(g["k/update/dt"][0])) == 0
    for q in ("stage", "xmom", "ymom"):
        assert bits_equal(A[q + "_centroid_values"], g[f"k/update/{q}"]), q


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_evolve_matches_reference_bitwise(case, oracle_mod):
    g = load_golden(case)
    od = golden_oracle(g, oracle_mod)
    od.evolve_start(1.0e300)
    for s in range(STEPS):
        assert od.evolve_steps(1.0e300, None, 1) == 0
        assert od.status == 0
        assert bits_equal([od.D.timestep], g[f"run/{s}/dt"]), f"dt at step {s}"
        assert bits_equal([od.D.time], g[f"run/{s}/time"]), f"time at step {s}"
        if f"run/{s}/stage" in g:
            for q in ("stage", "xmom", "ymom"):
                assert bits_equal(od.arrays[q + "_centroid_values"], g[f"run/{s}/{q}"]), (q, s)
    for q in ("stage", "xmom", "ymom"):
        assert bits_equal(od.arrays[q + "_vertex_values"], g[f"run/final/{q}_vertex"]), q
    assert bits_equal([od.mass()], g["run/final/mass"])


RK_STEPS = 12


@pytest.mark.parametrize("method", ["rk2", "rk3"])
@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_runge_kutta_matches_reference_bitwise(case, method, oracle_mod):
    """RK2 / RK3 steps: the oracle's driver and saxpy against the golden run
    made from the reference's kernels and its _saxpy_centroid_values."""
    g = load_golden(case)
    od = golden_oracle(g, oracle_mod)
    od.set_timestepping_method(method)
    od.evolve_start(1.0e300)
    for s in range(RK_STEPS):
        assert od.evolve_steps(1.0e300, None, 1) == 0
        assert od.status == 0
        assert bits_equal([od.D.timestep], g[f"{method}/{s}/dt"]), f"dt at step {s}"
        assert bits_equal([od.D.time], g[f"{method}/{s}/time"]), f"time at step {s}"
        if f"{method}/{s}/stage" in g:
            for q in ("stage", "xmom", "ymom"):
                assert bits_equal(od.arrays[q + "_centroid_values"], g[f"{method}/{s}/{q}"]), \
                    (q, s)


def test_runge_kutta_differs_from_euler():
    """The RK fixtures are not the Euler run in disguise."""
    g = load_golden("basin_wetdry")
    assert not bits_equal(g["rk2/11/stage"], g["rk3/11/stage"])
    assert not np.array_equal(g["rk2/0/dt"], g["run/0/dt"]) or \
        not bits_equal(g["rk2/0/stage"], g["run/0/stage"])


def test_tsunami_kernels_match_reference_bitwise(oracle_mod):
    g = load_golden("basin_tsunami")
    od = golden_oracle(g, oracle_mod)
    A = od.arrays
    od.protect_swb2()
    for q in ("stage", "xmom", "ymom"):
        assert bits_equal(A[q + "_centroid_values"], g[f"k/protect_swb2/{q}"]), q
    assert od.extrapolate_second_order_edge_sw() == 0
    for q in ("stage", "xmom", "ymom"):
        assert bits_equal(A[q + "_edge_values"], g[f"k/edge_extrapolate/{q}_edge"]), q
        assert bits_equal(A[q + "_vertex_values"], g[f"k/edge_extrapolate/{q}_vertex"]), q


def test_golden_cases_cover_wet_dry_and_boundaries():
    g = load_golden("basin_wetdry")
    h = g["init/stage_centroid_values"] - g["init/bed_centroid_values"]
    assert (h <= 1e-3).any() and (h > 0.05).any(), "needs dry, shallow and wet cells"
    assert set(g["tags/type"].tolist()) >= {0, 1}, "reflective and Dirichlet boundaries"
    hs = load_golden("harbour_small")
    assert 2 in hs["tags/type"].tolist(), "time-dependent stage boundary"
    ch = load_golden("channel_vertex_limiter")
    assert set(ch["tags/type"].tolist()) >= {3, 4, 5}, "transmissive and inflow boundaries"
    assert golden_params(ch).optimised_gradient_limiter == 0, "per-quantity vertex limiter"
    assert golden_params(load_golden("basin_edge_limiter")).use_edge_limiter == 1, "edge limiter"
    assert golden_params(load_golden("basin_tsunami")).flow_algorithm == 1, "tsunami"
    nb = np.concatenate([load_golden(c)["mesh/number_of_boundaries"] for c in GOLDEN_CASES])
    assert set(nb.tolist()) == {0, 1, 2, 3}, "every number_of_boundaries branch"
    assert np.isfinite(g["run/final/mass"]).all()


def test_oracle_fourier_stage_boundary(oracle_mod):
    """The oracle's Fourier stage boundary is the five-coefficient series of
    the model time on every edge of its tag, with zero momentum."""
    from anuga_cuda import DEFAULT, Time_stage_fourier_boundary, scenarios
    from helpers import oracle_from_scenario
    sc = scenarios.channel_inflow(10, 4, seed=2)
    b = Time_stage_fourier_boundary(coefficients=(0.1, 0.04, -0.03, 0.02, -0.01), period=5.0)
    sc.boundaries = dict(sc.boundaries, right=b)
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    m = sc.mesh.boundary_tag == sc.mesh.tag_names.index("right")
    assert m.any()
    for t in (0.0, 0.7, 3.1):
        od.D.time = t
        od.distribute_to_vertices_and_edges()
        od.update_boundary()
        A = od.arrays
        assert np.allclose(A["stage_boundary_values"][m], b.evaluate(t)[0], rtol=0, atol=1e-14)
        assert not A["xmom_boundary_values"][m].any()
        assert not A["ymom_boundary_values"][m].any()
