"""Parity at the benchmark configurations, full length.

* Dam break, 40,000 triangles (rectangular_cross 100 x 100), FP64 to its
  stated t = 5 s: stage and momentum within 1e-10 of the oracle (relative to
  the largest value), water volume within 1e-12.
* Tidal harbour, ~45,000 triangles (Poisson-disk Delaunay, sine boundary),
  FP64 for its 2,000 steps in windows of 100 steps: each window starts both
  sides from the oracle's state and must agree to 1e-10 (volume 1e-12, model
  time to 1e-12).  A continuous 2,000-step run cannot be held to 1e-10: the
  GPU's pow (Manning friction) and sin (tide) differ from the host libm's in
  the last bit now and then, and after ~1,500 steps such a difference flips a
  wet/dry threshold somewhere.  The oracle shows the same sensitivity on its
  own: with every pow and sin result moved by one ulp
  (oracle.set_libm_ulps(1)) it differs from itself by 1e-4 in stage after
  2,000 steps.  The continuous run is held to that scale (1e-3).
* Wet/dry case, 4,000,000 triangles, FP64 for 20 steps: 1e-10.
* The mixed-precision path against the FP64 path: at 4M triangles after the
  1,000 steps the headline is quoted on, maximum stage error <= 1e-5 relative
  to the largest stage (normwise); on the harbour after 2,000 steps the depth
  of every wet triangle (h > 1 cm) within 1e-5 relative of the FP64 depth.
"""
import numpy as np
import pytest

from helpers import gpu_from_scenario, max_rel, oracle_from_scenario

pytestmark = pytest.mark.gpu

REL_NSTEP = 1e-10    # stage / momentum (relative to max |value|)
REL_MASS = 1e-12     # water volume
REL_CHAOTIC = 1e-3   # continuous runs past the wet/dry sensitivity horizon
MIXED_STAGE = 1e-5   # mixed vs FP64: stage, normwise, 4M triangles, 1,000 steps
MIXED_DEPTH = 1e-5   # mixed vs FP64: depth of wet triangles, per element
WET_FLOOR = 0.01     # metres: triangles counted as wet for the depth figure

QUANTITIES = (("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom"))


def _vs_oracle(d, od):
    return {n: max_rel(d.quantities[n].centroid_values, od.arrays[p + "_centroid_values"])
            for n, p in QUANTITIES}


def test_dam_break_to_5s_matches_oracle(oracle_mod, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.dam_break()
    assert sc.N == 40000 and sc.finaltime == 5.0
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    od.evolve_start(1.0e300)
    assert od.evolve_steps(1.0e300, 5.0, 10 ** 6) == 2
    d = gpu_from_scenario(sc, DEFAULT)
    t = list(d.evolve(yieldstep=1.0e300, finaltime=5.0))
    assert t[-1] == 5.0 == od.D.time
    for n, e in _vs_oracle(d, od).items():
        assert e <= REL_NSTEP, (n, e)
    assert abs(d.get_water_volume() - od.mass()) <= REL_MASS * abs(od.mass())


def test_harbour_2000_steps_matches_oracle_in_windows(oracle_mod, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.tidal_harbour()
    assert 40000 < sc.N < 50000 and sc.steps == 2000
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    d = gpu_from_scenario(sc, DEFAULT)
    t, window = 0.0, 100
    for w in range(sc.steps // window):
        if w:  # both sides continue from the oracle's state
            for n, p in QUANTITIES:
                v = od.arrays[p + "_vertex_values"].reshape(-1, 3)
                d._upload(n, od.arrays[p + "_centroid_values"], v, v)
        d.starttime = t
        od.evolve_start(1.0e300, t)
        assert od.evolve_steps(1.0e300, None, window) == 0
        st = d.evolve_steps(window)
        assert st.total_steps == window and st.status == 0
        assert abs(st.time - od.D.time) <= 1e-12 * od.D.time, (w, st.time, od.D.time)
        for n, e in _vs_oracle(d, od).items():
            assert e <= REL_NSTEP, (w, n, e)
        assert abs(d.get_water_volume() - od.mass()) <= REL_MASS * abs(od.mass()), w
        t = od.D.time


def test_harbour_2000_steps_continuous(oracle_mod, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.tidal_harbour()
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    od.run_steps(sc.steps)
    d = gpu_from_scenario(sc, DEFAULT)
    st = d.evolve_steps(sc.steps)
    assert st.total_steps == sc.steps and st.status == 0
    assert abs(st.time - od.D.time) <= 1e-9 * od.D.time
    for n, e in _vs_oracle(d, od).items():
        assert e <= REL_CHAOTIC, (n, e)
    # water enters and leaves through the tidal boundary: the volume follows
    # the stage there, and so drifts with it
    assert abs(d.get_water_volume() - od.mass()) <= 1e-9 * abs(od.mass())


def test_wet_dry_4M_20_steps_matches_oracle(oracle_mod, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.wet_dry(m=1000)
    assert sc.N == 4000000
    od = oracle_from_scenario(oracle_mod, sc, DEFAULT)
    od.run_steps(20)
    d = gpu_from_scenario(sc, DEFAULT)
    st = d.evolve_steps(20)
    assert st.total_steps == 20 and st.time == od.D.time
    for n, e in _vs_oracle(d, od).items():
        assert e <= REL_NSTEP, (n, e)
    assert abs(d.get_water_volume() - od.mass()) <= REL_MASS * abs(od.mass())


def mixed_errors(sc, steps, params=None):
    """Mixed against FP64 after ``steps`` steps from the same state: per
    conserved quantity the maximum and RMS difference relative to the FP64
    field's maximum and RMS, and the largest relative depth difference over
    wet triangles (FP64 depth above WET_FLOOR)."""
    from anuga_cuda import DEFAULT
    a = gpu_from_scenario(sc, params or DEFAULT, "fp64")
    b = gpu_from_scenario(sc, params or DEFAULT, "mixed")
    sa, sb = a.evolve_steps(steps), b.evolve_steps(steps)
    out = {"time": (sa.time, sb.time)}
    for n, _ in QUANTITIES:
        x, y = b.quantities[n].centroid_values, a.quantities[n].centroid_values
        dd = np.abs(x - y)
        out[n] = (float(dd.max() / np.abs(y).max()),
                  float(np.sqrt(np.mean(dd ** 2)) / np.sqrt(np.mean(y ** 2))))
    z = a.quantities["elevation"].centroid_values
    h64 = a.quantities["stage"].centroid_values - z
    hm = b.quantities["stage"].centroid_values - z
    wet = h64 > WET_FLOOR
    out["depth"] = float(np.max(np.abs(hm[wet] - h64[wet]) / h64[wet]))
    out["volume"] = (a.get_water_volume(), b.get_water_volume())
    return out


def test_mixed_wet_dry_4M_1000_steps_within_1e5(swgpu_built):
    from anuga_cuda import scenarios
    e = mixed_errors(scenarios.wet_dry(m=1000), 1000)
    print(e)
    assert e["stage"][0] <= MIXED_STAGE, e
    assert e["depth"] <= MIXED_DEPTH, e
    assert abs(e["volume"][1] - e["volume"][0]) <= 1e-12 * e["volume"][0]


def test_mixed_harbour_2000_steps_wet_depth_within_1e5(swgpu_built):
    from anuga_cuda import scenarios
    e = mixed_errors(scenarios.tidal_harbour(), 2000)
    print(e)
    assert e["depth"] <= MIXED_DEPTH, e
    assert e["stage"][0] <= REL_CHAOTIC, e
    assert abs(e["time"][1] - e["time"][0]) <= 1e-6 * e["time"][0]
    # the tide moves water across the boundary on a slightly different dt
    # sequence (FP32 CFL timestep): the volumes drift apart with it
    assert abs(e["volume"][1] - e["volume"][0]) <= 1e-8 * e["volume"][0]
