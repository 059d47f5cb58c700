"""RK2 / RK3 timestepping on the GPU (ANUGA's evolve_one_rk2_step and
evolve_one_rk3_step over the reference's backup/saxpy methods,
gpu_domain_advanced.py:1449-1519 and :2198-2292): the fused device loop
against the oracle and against the golden runs made from the reference's own
kernels, the per-method path against the fused one, and the mixed precision
against FP64."""
import numpy as np
import pytest

from helpers import (GOLDEN_CASES, bits_equal, golden_oracle, gpu_from_golden,
                     gpu_from_scenario, load_golden, max_rel, oracle_from_scenario)

pytestmark = pytest.mark.gpu

REL_NSTEP = 1e-10   # stage / momentum after N steps (relative to max |value|)
REL_MASS = 1e-12
RK_STEPS = 12
QS = (("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom"))


@pytest.mark.parametrize("method", ["rk2", "rk3"])
@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_rk_evolve_matches_oracle_and_golden(case, method, oracle_mod, swgpu_built):
    g = load_golden(case)
    od = golden_oracle(g, oracle_mod)
    od.set_timestepping_method(method)
    od.run_steps(RK_STEPS)
    d = gpu_from_golden(g)
    d.set_timestepping_method(method)
    st = d.evolve_steps(RK_STEPS)
    assert st.total_steps == RK_STEPS and st.status == 0
    assert abs(st.time - od.D.time) <= REL_NSTEP * max(od.D.time, 1.0)
    last = RK_STEPS - 1
    assert abs(st.time - g[f"{method}/{last}/time"][0]) <= REL_NSTEP * max(st.time, 1.0)
    for name, pre in QS:
        c = d.quantities[name].centroid_values
        assert max_rel(c, od.arrays[pre + "_centroid_values"]) <= REL_NSTEP, name
        assert max_rel(c, g[f"{method}/{last}/{pre}"]) <= REL_NSTEP, name
    assert abs(d.get_water_volume() - od.mass()) <= REL_MASS * abs(od.mass())


@pytest.mark.parametrize("method", ["rk2", "rk3"])
def test_rk_long_run_with_time_boundary(method, oracle_mod, swgpu_built):
    """A tidal harbour (time-dependent stage boundary, so the stage times
    t0 + dt and t0 + dt/2 matter) for 150 steps."""
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.tidal_harbour(target_triangles=3000, seed=3)
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    od.set_timestepping_method(method)
    od.run_steps(150)
    d = gpu_from_scenario(sc, DEFAULT)
    d.set_timestepping_method(method)
    st = d.evolve_steps(150)
    assert st.status == 0
    assert abs(st.time - od.D.time) <= REL_NSTEP * max(od.D.time, 1.0)
    for name, pre in QS:
        assert max_rel(d.quantities[name].centroid_values,
                       od.arrays[pre + "_centroid_values"]) <= REL_NSTEP, name


@pytest.mark.parametrize("method", ["rk2", "rk3"])
def test_rk_per_method_matches_fused(method, swgpu_built):
    """The host-orchestrated evolve_one_rk*_step (one ABI call per method)
    against the device-resident loop."""
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.small_basin(12, 10, seed=4)
    a = gpu_from_scenario(sc, DEFAULT)
    a.set_timestepping_method(method)
    a.evolve_steps(10)
    b = gpu_from_scenario(sc, DEFAULT)
    b.evolve_steps(0)
    big = 1.0e300
    step = b.evolve_one_rk2_step if method == "rk2" else b.evolve_one_rk3_step
    for _ in range(10):
        t0 = b.get_time()
        step(big, None)
        b.set_time(t0 + b.timestep)
        b.distribute_to_vertices_and_edges()
        b.update_boundary()
    assert abs(a.get_time() - b.get_time()) <= 1e-12 * max(a.get_time(), 1.0)
    for name, _ in QS:
        assert max_rel(b.quantities[name].centroid_values,
                       a.quantities[name].centroid_values) <= REL_NSTEP, name


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rk3_graph_loop_equals_single_steps(precision, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.small_basin(14, 12, seed=5)
    a = gpu_from_scenario(sc, DEFAULT, precision)
    b = gpu_from_scenario(sc, DEFAULT, precision)
    a.set_timestepping_method("rk3")
    b.set_timestepping_method("rk3")
    a.evolve_steps(21)
    b.evolve_steps(0)
    for _ in range(21):
        b.step()
    for name, _ in QS:
        assert bits_equal(a.quantities[name].centroid_values, b.quantities[name].centroid_values)
    assert a.get_time() == b.get_time()


@pytest.mark.parametrize("method", ["rk2", "rk3"])
def test_rk_mixed_close_to_fp64(method, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.tidal_harbour(target_triangles=6000, seed=2)
    runs = {}
    for prec in ("fp64", "mixed"):
        d = gpu_from_scenario(sc, DEFAULT, prec)
        d.set_timestepping_method(method)
        st = d.evolve_steps(300)
        assert st.status == 0
        runs[prec] = d.quantities["stage"].centroid_values
    w64 = runs["fp64"]
    # measured 1.5e-7 (rk2), 1.1e-7 (rk3)
    assert np.max(np.abs(runs["mixed"] - w64)) / np.max(np.abs(w64)) < 1e-6


def test_method_switch_and_bad_method(swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.small_basin(8, 6, seed=1)
    d = gpu_from_scenario(sc, DEFAULT)
    assert d.get_timestepping_method() == "euler"
    d.evolve_steps(5)               # builds the Euler graph
    d.set_timestepping_method(2)    # ANUGA's numbering
    assert d.get_timestepping_method() == "rk2"
    st = d.evolve_steps(5)
    assert st.total_steps == 5 and st.status == 0
    with pytest.raises(ValueError):
        d.set_timestepping_method("rk4")
    from anuga_cuda._lib import lib
    assert lib().swgpu_set_timestepping_method(d._h, 7) != 0
