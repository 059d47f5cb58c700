"""The mixed path's device-resident loop: its step clock and stage commit
run as their own small kernels after the flux and the update, and a stop
takes effect after the step's distribute.  These tests check that the loop
still stops exactly where the FP64 loop stops (yields, final time, step
budgets, Runge-Kutta stages) and that a bad state halts it."""
import numpy as np
import pytest

from helpers import gpu_from_scenario

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", ["euler", "rk2", "rk3"])
def test_mixed_yields_and_steps_match_fp64(method, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.small_basin(12, 10, seed=2)
    runs = {}
    for prec in ("fp64", "mixed"):
        d = gpu_from_scenario(sc, DEFAULT, prec)
        d.set_timestepping_method(method)
        times = [t for t in d.evolve(yieldstep=0.2, finaltime=1.0)]
        runs[prec] = (times, d._state().total_steps, d.quantities["stage"].centroid_values)
    (t64, n64, w64), (tmx, nmx, wmx) = runs["fp64"], runs["mixed"]
    # the yield times are the clamped ones in both precisions, the final
    # time exactly
    assert np.allclose(t64, [0.0, 0.2, 0.4, 0.6, 0.8, 1.0], rtol=0, atol=1e-12)
    assert np.allclose(tmx, t64, rtol=0, atol=1e-12) and tmx[-1] == 1.0
    # the step counts agree to the one step per yield interval that an FP32
    # CFL bound can shift at a yield clamp
    assert abs(nmx - n64) <= 5, (nmx, n64)
    assert np.max(np.abs(wmx - w64)) <= 1e-6 * np.max(np.abs(w64))   # measured 2e-8 .. 5e-8


@pytest.mark.parametrize("method", ["euler", "rk2", "rk3"])
def test_mixed_step_budget_exact(method, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.small_basin(10, 8, seed=4)
    d = gpu_from_scenario(sc, DEFAULT, "mixed")
    d.set_timestepping_method(method)
    for k in (1, 7, 16, 17, 33):
        d.evolve_steps(k)
        assert d._state().total_steps == k   # steps of this run
    # budget runs and the same steps one run each end in the same state
    # (each evolve_steps call starts the model clock at starttime again; the
    # basin's boundaries do not depend on time)
    e = gpu_from_scenario(sc, DEFAULT, "mixed")
    e.set_timestepping_method(method)
    for _ in range(1 + 7 + 16 + 17 + 33):
        e.evolve_steps(1)
    for q in ("stage", "xmomentum", "ymomentum"):
        assert np.array_equal(d.quantities[q].centroid_values, e.quantities[q].centroid_values)


def test_mixed_nan_halts_with_status(swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda._lib import SwgpuError
    sc = scenarios.small_basin(8, 6, seed=1, wet_dry_front=False)
    sc.stage_centroid = sc.stage_centroid.copy()
    sc.stage_centroid[5] = np.nan
    d = gpu_from_scenario(sc, DEFAULT, "mixed")
    with pytest.raises(SwgpuError) as e:
        d.evolve_steps(40)
    assert e.value.status in (6, 4)   # ENONFINITE (or EDENOMINATOR from a NaN)
    # the loop stopped within a step of the bad state, not after the budget
    assert d._state().total_steps <= 2


def test_mixed_dependent_launch_off_identical(swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda.autotune import get_config, set_config
    sc = scenarios.small_basin(14, 12, seed=5)
    out = []
    for dep in (1, 0):
        d = gpu_from_scenario(sc, DEFAULT, "mixed")
        d.set_timestepping_method("rk3")
        set_config(d._h, dict(get_config(d._h), dependent_launch=dep))
        times = [t for t in d.evolve(yieldstep=0.3, finaltime=0.9)]
        out.append((times, d.quantities["xmomentum"].centroid_values.copy()))
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])


def test_timeout_status_leaves_handle_unusable(swgpu_built):
    """A kernel's SWGPU_ETIMEOUT (a bounded wait for a tile's bulk copies ran
    out) leaves the handle unusable: the status is planted in the control
    block from the host (no wait is made to run out on the GPU), and the run
    that reads it and every later call that reaches the device fail."""
    import ctypes as C
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda._lib import State_t, SwgpuError, lib
    ETIMEOUT = 11
    sc = scenarios.small_basin(8, 6, seed=1)
    d = gpu_from_scenario(sc, DEFAULT, "mixed")
    d.evolve_steps(0)
    st = d._state()
    st.status = ETIMEOUT
    d._set_state(st)
    out = State_t()
    assert lib().swgpu_evolve_run(d._h, 4, C.byref(out)) == ETIMEOUT
    assert "wait ran out" in lib().swgpu_last_error(d._h).decode()
    for call in (lambda: d.evolve_steps(2), d.distribute_to_vertices_and_edges,
                 lambda: d._set_state(st)):
        with pytest.raises(SwgpuError) as e:
            call()
        assert e.value.status == ETIMEOUT
        assert "destroy" in str(e.value)
