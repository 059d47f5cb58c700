"""Batched ensembles on the GPU: every scenario of an ensemble equals its own
single-domain run (same steps, same times, bit-identical state and water
volume), in both precisions; finished scenarios stop while others run on."""
import numpy as np
import pytest

from helpers import bits_equal, gpu_from_scenario

pytestmark = pytest.mark.gpu


def _scenarios():
    from anuga_cuda import scenarios
    return [scenarios.small_basin(10, 8, seed=1), scenarios.channel_inflow(14, 5, seed=2),
            scenarios.inflow_harbour(3000, seed=3, peak=300.0, rise=60.0),
            scenarios.small_basin(6, 5, seed=4)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_scenarios_equal_single_runs(precision, swgpu_built):
    from anuga_cuda import DEFAULT
    from anuga_cuda.ensemble import Ensemble
    scs = _scenarios()
    finals = [0.6, 1.5, 40.0, 0.2]
    ens = Ensemble(scs, DEFAULT, precision)
    states = ens.evolve(finals)
    stages = ens.centroid_values("stage")
    xmoms = ens.centroid_values("xmomentum")
    masses = ens.masses()
    for i, (sc, ft) in enumerate(zip(scs, finals)):
        d = gpu_from_scenario(sc, DEFAULT, precision)
        t = list(d.evolve(yieldstep=ft, finaltime=ft))
        st = d._state()
        assert t[-1] == ft and states[i].time == ft
        assert states[i].total_steps == st.total_steps, i
        assert states[i].status == 0
        assert bits_equal(stages[i], d.quantities["stage"].centroid_values), i
        assert bits_equal(xmoms[i], d.quantities["xmomentum"].centroid_values), i
        assert bits_equal([masses[i]], [d.get_water_volume()]), i
    # the scenarios ran different numbers of steps
    assert len({s.total_steps for s in states}) > 1


def test_step_budget_and_rk2(swgpu_built):
    from anuga_cuda import DEFAULT
    from anuga_cuda.ensemble import Ensemble
    scs = _scenarios()[:2]
    ens = Ensemble(scs, DEFAULT, "fp64")
    states = ens.evolve(1.0e6, max_steps=23)
    assert [s.total_steps for s in states] == [23, 23]
    assert all(s.stop_reason == 3 for s in states)      # step budget
    d = gpu_from_scenario(scs[1], DEFAULT)
    d.evolve_steps(23)
    assert bits_equal(ens.centroid_values("stage")[1], d.quantities["stage"].centroid_values)


def test_per_method_refused_on_ensemble(swgpu_built):
    import ctypes as C
    from anuga_cuda import DEFAULT
    from anuga_cuda._lib import lib
    from anuga_cuda.ensemble import Ensemble
    ens = Ensemble(_scenarios()[:2], DEFAULT, "fp64")
    ft = C.c_double()
    assert lib().swgpu_compute_fluxes(ens._h, C.byref(ft)) != 0
    n = C.c_int()
    assert lib().swgpu_ensemble_size(ens._h, C.byref(n)) == 0 and n.value == 2


def test_finished_scenario_costs_little_per_step(swgpu_built):
    """A scenario that has reached its finaltime while another runs on: its
    blocks read the halt flag and return without fetching their tiles.  Here
    it comes first in the launch (the deeper water sorts it first), so every
    launch still covers it; its cost per step, the ensemble's step minus the
    running scenario's own step, stays a small fraction of a live step of the
    same size (CUDA events around the graph launches)."""
    import ctypes as C
    from anuga_cuda import DEFAULT, _lib, scenarios
    from anuga_cuda._lib import check, f64p, lib
    from anuga_cuda.ensemble import Ensemble
    a = scenarios.wet_dry(m=250, seed=3)
    a.stage_centroid = a.stage_centroid + 1.0     # deeper: the smallest timestep, first
    b = scenarios.wet_dry(m=250, seed=5)

    def timed(ens, finals, warm, steps):
        ft = ens._internal(np.asarray(finals, np.float64))
        check(lib().swgpu_evolve_start(ens._h, 0.0, 1.0e6, 1.0e6), ens._h)
        check(lib().swgpu_ensemble_set_finaltimes(ens._h, f64p(ft)), ens._h)
        st, ms = _lib.State_t(), C.c_double()
        check(lib().swgpu_evolve_run_timed(ens._h, warm, C.byref(st), C.byref(ms)), ens._h)
        best = None
        for _ in range(3):
            check(lib().swgpu_evolve_run_timed(ens._h, steps, C.byref(st), C.byref(ms)), ens._h)
            best = ms.value if best is None else min(best, ms.value)
        return best / steps

    both = Ensemble([a, b], DEFAULT, "mixed")
    assert both.order == [0, 1]                  # the finishing scenario is first
    t_both = timed(both, [1.0, 1.0e6], 48, 96)
    assert both.states()[0].stop_reason == 2 and both.states()[1].stop_reason != 2
    alone = Ensemble([b], DEFAULT, "mixed")
    t_b = timed(alone, [1.0e6], 48, 96)
    halted = t_both - t_b
    print(f"running step {t_b * 1e3:.1f} us, with a finished scenario {t_both * 1e3:.1f} us")
    assert halted <= 0.15 * t_b, (t_both, t_b)
