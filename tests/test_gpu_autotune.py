"""The launch-shape autotuner: results do not depend on the shape (bit for
bit, both precisions, single domains and ensembles), bad shapes are refused,
and tuned shapes are cached."""
import json

import pytest

from helpers import bits_equal, gpu_from_scenario

pytestmark = pytest.mark.gpu

QS = ("stage", "xmomentum", "ymomentum")
ODD = {"flux_block": 64, "update_block": 512, "distribute_block": 128, "steps_per_graph": 5,
       "flux_pipelined": 1, "dependent_launch": 0}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("method", ["euler", "rk2"])
def test_results_independent_of_shape(precision, method, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda.autotune import get_config, set_config
    sc = scenarios.small_basin(14, 12, seed=5)
    a = gpu_from_scenario(sc, DEFAULT, precision)
    b = gpu_from_scenario(sc, DEFAULT, precision)
    for d in (a, b):
        d.set_timestepping_method(method)
    set_config(b._h, ODD)
    assert get_config(b._h) == ODD
    a.evolve_steps(41)
    b.evolve_steps(41)
    for q in QS:
        assert bits_equal(a.quantities[q].centroid_values, b.quantities[q].centroid_values), q
    assert a.get_time() == b.get_time()


def test_ensemble_shape_independent(swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda.autotune import set_config
    from anuga_cuda.ensemble import Ensemble
    scs = [scenarios.small_basin(9, 7, seed=1), scenarios.channel_inflow(12, 5, seed=2)]
    e1 = Ensemble(scs, DEFAULT, "mixed")
    e2 = Ensemble(scs, DEFAULT, "mixed")
    set_config(e2._h, {"flux_block": 128, "update_block": 128, "distribute_block": 256,
                       "steps_per_graph": 7, "flux_pipelined": 1})
    e1.evolve([0.5, 1.0])
    e2.evolve([0.5, 1.0])
    for a, b in zip(e1.centroid_values("stage"), e2.centroid_values("stage")):
        assert bits_equal(a, b)


def test_bad_shapes_refused(swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda._lib import SwgpuError
    from anuga_cuda.autotune import set_config
    from anuga_cuda.ensemble import Ensemble
    d = gpu_from_scenario(scenarios.small_basin(6, 5, seed=1), DEFAULT)
    with pytest.raises(SwgpuError):
        set_config(d._h, dict(ODD, update_block=1024))
    with pytest.raises(SwgpuError):
        set_config(d._h, dict(ODD, steps_per_graph=0))
    with pytest.raises(SwgpuError):
        set_config(d._h, dict(ODD, flux_block=256, flux_pipelined=1))
    e = Ensemble([scenarios.small_basin(6, 5, seed=1), scenarios.small_basin(5, 4, seed=2)],
                 DEFAULT, "fp64")
    with pytest.raises(SwgpuError):
        set_config(e._h, dict(ODD, update_block=512))


def test_tune_domain_and_cache(tmp_path, monkeypatch, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda.autotune import cache_path, tune_domain
    monkeypatch.setenv("ANUGA_CUDA_TUNE_CACHE", str(tmp_path / "tune.json"))
    sc = scenarios.small_basin(16, 12, seed=2)
    d = gpu_from_scenario(sc, DEFAULT, "mixed")
    rec = tune_domain(d, steps=4)
    assert set(rec["config"]) == {"flux_block", "update_block", "distribute_block",
                                  "steps_per_graph", "flux_pipelined", "dependent_launch"}
    assert 0 < rec["tuned_ms"] <= rec["default_ms"]
    assert json.load(open(cache_path()))
    again = tune_domain(gpu_from_scenario(sc, DEFAULT, "mixed"), steps=4)
    assert again.get("cached") and again["config"] == rec["config"]
    # the tuned domain's own state was not advanced by the tuning
    ref = gpu_from_scenario(sc, DEFAULT, "mixed")
    d.evolve_steps(30)
    ref.evolve_steps(30)
    assert bits_equal(d.quantities["stage"].centroid_values, ref.quantities["stage"].centroid_values)
