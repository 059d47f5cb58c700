"""The remaining per-method entry points of the reference's GPU domain
against the oracle, on every golden case:

* extrapolate_second_order_sw (gpu_domain_advanced.py:1061-1161) and
  balance_deep_and_shallow (:957-995) called one after the other, as the
  reference's co-test checkpoints wrap them: vertex values bit for bit;
* manning_friction_explicit (:1330-1388): explicit momentum updates within
  1e-13 (CUDA's pow against the host libm's, one ulp);
* update_other_quantities (:2114-2151): height and velocities at centroids
  bit for bit and at boundary slots (after update_boundary) within 1e-13,
  vertex and edge values the first-order copies of the centroid values;
* the transmissive, transmissive-stage-zero-momentum and inflow-hydrograph
  boundaries of a channel: boundary values after one distribute within
  1e-13 (cbrt), and 60 Euler steps within 1e-10.
"""
import numpy as np
import pytest

from helpers import (GOLDEN_CASES, bits_equal, golden_oracle, gpu_from_golden, gpu_from_scenario,
                     load_golden, max_rel, oracle_from_scenario)

pytestmark = pytest.mark.gpu

REL_LIBM = 1e-13
REL_NSTEP = 1e-10
QUANTITIES = (("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom"))
DEFAULT_FLOW = [c for c in GOLDEN_CASES if c != "basin_tsunami"]


@pytest.mark.parametrize("case", DEFAULT_FLOW)
def test_extrapolate_then_balance_match_oracle(case, oracle_mod, swgpu_built):
    g = load_golden(case)
    od = golden_oracle(g, oracle_mod)
    d = gpu_from_golden(g)
    od.extrapolate_second_order_sw()
    d.extrapolate_second_order_sw()
    for n, p in QUANTITIES:
        assert bits_equal(d.quantities[n].vertex_values.ravel(),
                          od.arrays[p + "_vertex_values"]), ("extrapolate", n)
        # the centroid values are left as they were
        assert bits_equal(d.quantities[n].centroid_values, od.arrays[p + "_centroid_values"]), n
    od.balance_deep_and_shallow()
    d.balance_deep_and_shallow()
    for n, p in QUANTITIES:
        assert bits_equal(d.quantities[n].vertex_values.ravel(),
                          od.arrays[p + "_vertex_values"]), ("balance", n)


def test_extrapolate_refused_for_tsunami_flow(oracle_mod, swgpu_built):
    from anuga_cuda._lib import SwgpuError
    d = gpu_from_golden(load_golden("basin_tsunami"))
    with pytest.raises(SwgpuError):
        d.extrapolate_second_order_sw()


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_manning_friction_explicit_matches_oracle(case, oracle_mod, swgpu_built):
    g = load_golden(case)
    od = golden_oracle(g, oracle_mod)
    d = gpu_from_golden(g)
    od.manning_friction_explicit()
    d.manning_friction_explicit()
    for n, p in QUANTITIES[1:]:
        assert max_rel(d.quantities[n].explicit_update, od.arrays[p + "_explicit_update"]) \
            <= REL_LIBM, n
    # the semi-implicit updates are untouched
    for n, _ in QUANTITIES[1:]:
        assert not np.any(d.quantities[n].semi_implicit_update)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_update_other_quantities_matches_oracle(case, oracle_mod, swgpu_built):
    g = load_golden(case)
    od = golden_oracle(g, oracle_mod)
    d = gpu_from_golden(g)
    od.distribute_to_vertices_and_edges()
    od.update_boundary()
    d.distribute_to_vertices_and_edges()
    d.update_boundary()
    d.update_other_quantities()
    ref = od.update_other_quantities()
    for n, (c, b) in ref.items():
        q = d.quantities[n]
        got = q.centroid_values
        assert bits_equal(got, c), n
        assert bits_equal(q.vertex_values, np.repeat(got[:, None], 3, axis=1)), n
        assert bits_equal(q.edge_values, np.repeat(got[:, None], 3, axis=1)), n
        if len(b):
            assert max_rel(q.boundary_values, b, floor=1e-300) <= REL_LIBM, n


def test_update_other_quantities_mixed_follows_state(swgpu_built):
    """Mixed handles: height and velocities come from the current mixed
    state (depth h = stage - bed), not from a stale FP64 stage."""
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.small_basin(12, 10, seed=4)
    d = gpu_from_scenario(sc, DEFAULT, "mixed")
    d.evolve_steps(25)
    d.update_other_quantities()
    w = d.quantities["stage"].centroid_values
    z = d.quantities["elevation"].centroid_values
    uh = d.quantities["xmomentum"].centroid_values
    h = np.maximum(w - z, 0.0)
    assert np.allclose(d.quantities["height"].centroid_values, h, rtol=0, atol=1e-12)
    u = uh * h / (h * h + 1.0e-8)
    assert np.allclose(d.quantities["xvelocity"].centroid_values, u, rtol=1e-12, atol=1e-12)


def _channel():
    from anuga_cuda import scenarios
    sc = scenarios.channel_inflow(16, 6, seed=5, peak=0.6, rise=2.0)
    kinds = {t: type(b).__name__ for t, b in sc.boundaries.items()}
    assert kinds == {"left": "Inflow_hydrograph_boundary", "right": "Transmissive_boundary",
                     "top": "Transmissive_stage_zero_momentum_boundary",
                     "bottom": "Reflective_boundary"}, kinds
    return sc


def test_transmissive_and_inflow_boundary_values_match_oracle(oracle_mod, swgpu_built):
    from anuga_cuda import DEFAULT
    sc = _channel()
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    d = gpu_from_scenario(sc, DEFAULT)
    for t in (0.0, 1.3):  # before the hydrograph starts, and on its rise
        od.D.time = t
        d.set_time(t)
        od.distribute_to_vertices_and_edges()
        od.update_boundary()
        d.distribute_to_vertices_and_edges()
        d.update_boundary()
        for n, p in QUANTITIES:
            assert max_rel(d.quantities[n].boundary_values, od.arrays[p + "_boundary_values"],
                           floor=1e-300) <= REL_LIBM, (t, n)


def test_transmissive_and_inflow_channel_evolve_matches_oracle(oracle_mod, swgpu_built):
    from anuga_cuda import DEFAULT
    sc = _channel()
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    od.run_steps(60)
    d = gpu_from_scenario(sc, DEFAULT)
    st = d.evolve_steps(60)
    assert st.total_steps == 60 and st.status == 0
    assert abs(st.time - od.D.time) <= 1e-12 * max(od.D.time, 1.0)
    for n, p in QUANTITIES:
        assert max_rel(d.quantities[n].centroid_values,
                       od.arrays[p + "_centroid_values"]) <= REL_NSTEP, n
    assert d.get_water_volume() > 0


def _channel_with_tide():
    """The inflow channel whose downstream (right) edge is an open boundary
    with a five-coefficient Fourier stage (a tide and its first overtide)."""
    from anuga_cuda import Time_stage_fourier_boundary
    sc = _channel()
    sc.boundaries = dict(sc.boundaries)
    sc.boundaries["right"] = Time_stage_fourier_boundary(
        coefficients=(0.08, 0.03, -0.02, 0.01, 0.015), period=7.0)
    return sc


def test_fourier_stage_boundary_values_match_oracle(oracle_mod, swgpu_built):
    from anuga_cuda import DEFAULT
    sc = _channel_with_tide()
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    d = gpu_from_scenario(sc, DEFAULT)
    b = sc.boundaries["right"]
    for t in (0.0, 1.3, 4.9):
        od.D.time = t
        d.set_time(t)
        od.distribute_to_vertices_and_edges()
        od.update_boundary()
        d.distribute_to_vertices_and_edges()
        d.update_boundary()
        for n, p in QUANTITIES:
            assert max_rel(d.quantities[n].boundary_values, od.arrays[p + "_boundary_values"],
                           floor=1e-300) <= REL_LIBM, (t, n)
        # the open edge's stage is the series at t
        m = sc.mesh.boundary_tag == sc.mesh.tag_names.index("right")
        assert np.allclose(d.quantities["stage"].boundary_values[m], b.evaluate(t)[0],
                           rtol=0, atol=1e-14)


def test_fourier_stage_channel_evolve_matches_oracle(oracle_mod, swgpu_built):
    from anuga_cuda import DEFAULT
    sc = _channel_with_tide()
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    od.run_steps(60)
    d = gpu_from_scenario(sc, DEFAULT)
    st = d.evolve_steps(60)
    assert st.total_steps == 60 and st.status == 0
    assert abs(st.time - od.D.time) <= 1e-12 * max(od.D.time, 1.0)
    for n, p in QUANTITIES:
        assert max_rel(d.quantities[n].centroid_values,
                       od.arrays[p + "_centroid_values"]) <= REL_NSTEP, n
