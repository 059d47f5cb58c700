"""FP64 GPU path against the CPU oracle (itself pinned bit for bit to the
reference's ANUGA C kernels).  Bar: every kernel bit-identical except where
a libm function differs from CUDA's by an ulp (pow in Manning friction, sin
in the time boundary), and after N Euler steps stage and momentum within
1e-10 relative with mass to 1e-12 relative."""
import numpy as np
import pytest

from helpers import (GOLDEN_CASES, bits_equal, golden_oracle, gpu_from_golden, gpu_from_scenario,
                     load_golden, max_rel, oracle_from_scenario)

pytestmark = pytest.mark.gpu

REL_NSTEP = 1e-10      # stage / momentum after N steps (relative to max |value|)
REL_MASS = 1e-12       # water volume
REL_LIBM = 1e-13       # one-ulp libm differences (pow, sin) after one kernel


def _q(d, name):
    q = d.quantities[name]
    return q.centroid_values, q.vertex_values.ravel(), q.edge_values.ravel()


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_methods_match_oracle(case, oracle_mod, swgpu_built):
    g = load_golden(case)
    od = golden_oracle(g, oracle_mod)
    d = gpu_from_golden(g)
    A = od.arrays
    # distribute (protect, extrapolation, balance, interpolation)
    od.distribute_to_vertices_and_edges()
    d.distribute_to_vertices_and_edges()
    for name, pre in (("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom")):
        c, v, e = _q(d, name)
        assert bits_equal(c, A[pre + "_centroid_values"]), name
        assert bits_equal(v, A[pre + "_vertex_values"]), name
        assert bits_equal(e, A[pre + "_edge_values"]), name
    # boundary values
    od.update_boundary()
    d.update_boundary()
    for name, pre in (("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom")):
        b = d.quantities[name].boundary_values
        assert max_rel(b, A[pre + "_boundary_values"][:len(b)]) <= REL_LIBM, name
    # fluxes + gravity
    ft_o = od.compute_fluxes()
    od.gravity_wb()
    ft_g = d.compute_fluxes()
    assert bits_equal([ft_g], [ft_o])
    for name, pre in (("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom")):
        assert bits_equal(d.quantities[name].explicit_update, A[pre + "_explicit_update"]), name
    # Manning friction (pow: one-ulp differences allowed)
    od.manning_friction()
    d.compute_forcing_terms()
    for name, pre in (("xmomentum", "xmom"), ("ymomentum", "ymom")):
        assert max_rel(d.quantities[name].semi_implicit_update,
                       A[pre + "_semi_implicit_update"]) <= REL_LIBM, name
    # semi-implicit update with a fixed dt
    dt = 0.5 * ft_o
    assert od.update_conserved_quantities(dt) == 0
    d.timestep = dt
    d.update_conserved_quantities()
    for name, pre in (("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom")):
        assert max_rel(d.quantities[name].centroid_values, A[pre + "_centroid_values"]) <= REL_LIBM


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_evolve_matches_oracle(case, oracle_mod, swgpu_built):
    g = load_golden(case)
    steps = 40
    od = golden_oracle(g, oracle_mod)
    od.run_steps(steps)
    d = gpu_from_golden(g)
    st = d.evolve_steps(steps)
    assert st.total_steps == steps and st.status == 0
    assert abs(st.time - od.D.time) <= REL_NSTEP * max(od.D.time, 1.0)
    for name, pre in (("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom")):
        c = d.quantities[name].centroid_values
        assert max_rel(c, od.arrays[pre + "_centroid_values"]) <= REL_NSTEP, name
    assert abs(d.get_water_volume() - od.mass()) <= REL_MASS * abs(od.mass())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_loop_equals_single_steps(precision, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.small_basin(14, 12, seed=5)
    a = gpu_from_scenario(sc, DEFAULT, precision)
    b = gpu_from_scenario(sc, DEFAULT, precision)
    a.evolve_steps(37)
    b.evolve_steps(0)
    for _ in range(37):
        b.step()
    for name in ("stage", "xmomentum", "ymomentum"):
        assert bits_equal(a.quantities[name].centroid_values, b.quantities[name].centroid_values)
        assert bits_equal(a.quantities[name].vertex_values, b.quantities[name].vertex_values)
    assert a.get_time() == b.get_time()


def test_evolve_generator_yields_like_oracle(oracle_mod, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.small_basin(12, 10, seed=2)
    d = gpu_from_scenario(sc, DEFAULT)
    times = [t for t in d.evolve(yieldstep=0.25, finaltime=1.0)]
    assert times[0] == 0.0 and times[-1] == 1.0
    assert np.allclose(times, [0.0, 0.25, 0.5, 0.75, 1.0], rtol=0, atol=1e-12)
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    od.evolve_start(0.25)
    otimes = [od.time]
    while True:
        rc = od.evolve_steps(0.25, 1.0, 10 ** 6)
        otimes.append(od.time)
        if rc == 2:
            break
        assert rc == 1
    assert np.allclose(times, otimes, rtol=0, atol=1e-12)
    for name, pre in (("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom")):
        assert max_rel(d.quantities[name].centroid_values,
                       od.arrays[pre + "_centroid_values"]) <= REL_NSTEP


def test_dam_break_long_run_matches_oracle(oracle_mod, swgpu_built):
    """The 40,000-triangle dam break (the CPU-runnable benchmark case) run
    to t = 0.5 s on both; stage and momentum to 1e-10, mass to 1e-12."""
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.dam_break()
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    od.evolve_start(1.0e300)
    rc = od.evolve_steps(1.0e300, 0.5, 10 ** 6)
    assert rc == 2
    d = gpu_from_scenario(sc, DEFAULT)
    t = list(d.evolve(yieldstep=1.0e300, finaltime=0.5))
    assert t[-1] == 0.5
    for name, pre in (("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom")):
        assert max_rel(d.quantities[name].centroid_values,
                       od.arrays[pre + "_centroid_values"]) <= REL_NSTEP, name
    assert abs(d.get_water_volume() - od.mass()) <= REL_MASS * abs(od.mass())
