"""Known-answer and invariant tests on the GPU, both precisions:
well-balanced lake at rest (the reference's only known-answer test,
src/anuga_cuda/anuga_gpu/mytest.py:11-34, generalised to a sloping bed),
volume conservation between reflective walls, mirror symmetry of the dam
break, mixed-precision error against FP64, and clean error statuses."""
import numpy as np
import pytest

from helpers import gpu_from_scenario, max_rel

pytestmark = pytest.mark.gpu


def _lake(precision, level=0.4):
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda.boundaries import Reflective_boundary
    sc = scenarios.small_basin(10, 8, seed=0, wet_dry_front=False)
    zc = sc.elevation_vertex.mean(axis=1)
    sc.stage_centroid = np.maximum(zc, level)
    sc.xmom_centroid = np.zeros(sc.N)
    sc.ymom_centroid = np.zeros(sc.N)
    sc.boundaries = {t: Reflective_boundary() for t in sc.mesh.tag_names}
    return gpu_from_scenario(sc, DEFAULT, precision), sc


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lake_at_rest_stays_at_rest(precision, swgpu_built):
    d, sc = _lake(precision)
    w0 = d.quantities["stage"].centroid_values.copy()
    d.evolve_steps(50)
    w = d.quantities["stage"].centroid_values
    u = d.quantities["xmomentum"].centroid_values
    tol = 1e-12 if precision == "fp64" else 2e-5
    wet = sc.stage_centroid > sc.elevation_vertex.mean(axis=1) + 1e-3
    assert np.max(np.abs(w - w0)[wet]) < tol
    assert np.max(np.abs(u)) < tol


def test_four_triangle_known_answer(swgpu_built):
    """Constant stage 1 over constant bed -1: the pressure terms cancel and
    the central triangle's explicit update is zero."""
    from anuga_cuda import GPU_domain
    pts = [[0.0, 0.0], [0.0, 2.0], [2.0, 0.0], [0.0, 4.0], [2.0, 2.0], [4.0, 0.0]]
    tris = [[1, 0, 2], [1, 2, 4], [4, 2, 5], [3, 1, 4]]
    d = GPU_domain(pts, tris, reorder=False)
    d.set_quantity("elevation", -1.0)
    d.set_quantity("stage", 1.0)
    d.distribute_to_vertices_and_edges()
    d.update_boundary()
    d.compute_fluxes()
    for q in ("stage", "xmomentum", "ymomentum"):
        assert abs(d.quantities[q].explicit_update[1]) < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_volume_conserved_between_walls(precision, swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.dam_break(40, 40)
    d = gpu_from_scenario(sc, DEFAULT, precision)
    v0 = d.get_water_volume()
    d.evolve_steps(200)
    v1 = d.get_water_volume()
    assert abs(v1 - v0) <= (1e-12 if precision == "fp64" else 1e-9) * abs(v0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_dam_break_mirror_symmetry(precision, swgpu_built):
    """The rectangular_cross mesh and the dam are symmetric under y -> 100-y,
    so stage is too and y-momentum is antisymmetric."""
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.dam_break(30, 30)
    d = gpu_from_scenario(sc, DEFAULT, precision)
    d.evolve_steps(100)
    c = sc.mesh.centroid_coordinates
    key = np.round(c * 1e6).astype(np.int64)
    index = {(x, y): i for i, (x, y) in enumerate(map(tuple, key))}
    mirror = np.array([index[(x, 100_000_000 - y)] for x, y in map(tuple, key)])
    w = d.quantities["stage"].centroid_values
    vh = d.quantities["ymomentum"].centroid_values
    tol = 1e-9 if precision == "fp64" else 1e-5
    assert np.max(np.abs(w - w[mirror])) < tol
    assert np.max(np.abs(vh + vh[mirror])) < tol


def test_mixed_close_to_fp64_on_harbour(swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.tidal_harbour(target_triangles=6000, seed=4)
    a = gpu_from_scenario(sc, DEFAULT, "fp64")
    b = gpu_from_scenario(sc, DEFAULT, "mixed")
    sa = a.evolve_steps(300)
    sb = b.evolve_steps(300)
    assert abs(sa.time - sb.time) <= 1e-5 * sa.time
    err = max_rel(b.quantities["stage"].centroid_values, a.quantities["stage"].centroid_values)
    assert err < 1e-6, err   # measured 1.8e-7


def test_nan_input_reports_status(swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda._lib import SwgpuError
    sc = scenarios.small_basin(8, 6, seed=1, wet_dry_front=False)
    sc.stage_centroid = sc.stage_centroid.copy()
    sc.stage_centroid[5] = np.nan
    d = gpu_from_scenario(sc, DEFAULT, "fp64")
    with pytest.raises(SwgpuError) as e:
        d.evolve_steps(5)
    assert e.value.status in (6, 4)   # ENONFINITE (or EDENOMINATOR from a NaN)


def test_unknown_boundary_type_rejected(swgpu_built):
    from anuga_cuda import DEFAULT, GPU_domain, _lib, scenarios
    from anuga_cuda._lib import SwgpuError, check, lib
    sc = scenarios.small_basin(6, 5, seed=1)
    d = gpu_from_scenario(sc, DEFAULT, "fp64")
    arr = (_lib.BoundaryTag_t * len(sc.mesh.tag_names))()
    arr[0].type = 17
    with pytest.raises(SwgpuError):
        check(lib().swgpu_set_boundary_tags(d._h, arr, len(sc.mesh.tag_names)), d._h)
    _ = GPU_domain


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_inflow_hydrograph_volume(precision, swgpu_built):
    """Water entering through the hydrograph boundary of a channel that is
    otherwise walled: the volume gained follows the integral of Q(t) while
    the inflow cells stay shallow (critical-depth inflow)."""
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda.boundaries import Reflective_boundary
    sc = scenarios.channel_inflow(28, 10, seed=3, peak=0.4, rise=3.0)
    for t in ("right", "top"):
        sc.boundaries[t] = Reflective_boundary()
    d = gpu_from_scenario(sc, DEFAULT, precision)
    v0 = d.get_water_volume()
    times = list(d.evolve(yieldstep=1.0, finaltime=4.0))
    assert times[-1] == 4.0
    q = sc.boundaries["left"]
    ts = np.linspace(0.0, 4.0, 4001)
    qs = np.array([q.discharge(t) for t in ts])
    expect = float(np.sum(0.5 * (qs[1:] + qs[:-1]) * np.diff(ts)))
    gained = d.get_water_volume() - v0
    assert abs(gained - expect) < 0.1 * expect, (gained, expect)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_transmissive_outflow_and_mixed_close(precision, swgpu_built):
    """The channel with all its open boundaries: runs clean in both
    precisions, and the mixed precision stays within 1e-6 of FP64."""
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.channel_inflow(40, 12, seed=4, peak=1.0, rise=2.0)
    runs = {}
    for prec in ("fp64", precision):
        d = gpu_from_scenario(sc, DEFAULT, prec)
        st = d.evolve_steps(400)
        assert st.status == 0
        runs[prec] = d.quantities["stage"].centroid_values
    assert max_rel(runs[precision], runs["fp64"]) < 1e-6   # measured 9e-8


def test_limiter_variants_need_fp64(swgpu_built):
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda._lib import SwgpuError
    sc = scenarios.small_basin(8, 6, seed=1)
    for kw in ({"use_edge_limiter": 1}, {"optimised_gradient_limiter": 0},
               {"flow_algorithm": 1}):
        with pytest.raises(SwgpuError):
            gpu_from_scenario(sc, DEFAULT.replace(**kw), "mixed")
        d = gpu_from_scenario(sc, DEFAULT.replace(**kw), "fp64")
        assert d.evolve_steps(20).status == 0


def test_degenerate_timestep_protection(swgpu_built):
    """gpu_domain_advanced.py:914-951: an isolated triangle far faster than
    all others loses its momentum before the timestep is chosen."""
    from anuga_cuda import DEFAULT, scenarios
    sc = scenarios.small_basin(10, 8, seed=0, wet_dry_front=False)
    zc = sc.elevation_vertex.mean(axis=1)
    h = sc.stage_centroid - zc
    k = 0        # every edge of triangle 0 is processed by it (all neighbours are higher)
    assert h[k] > 0.1
    sc.xmom_centroid = np.zeros(sc.N)
    sc.ymom_centroid = np.zeros(sc.N)
    sc.xmom_centroid[k] = 40.0 * h[k]          # 40 m/s in one wet triangle
    d = gpu_from_scenario(sc, DEFAULT)
    d.evolve_steps(0)
    d.protect_against_isolated_degenerate_timesteps = True
    d.compute_fluxes()
    assert d.max_speed.max() > 10.0
    d.update_timestep(1.0e300, None)
    u = d.quantities["xmomentum"].centroid_values
    assert u[k] == 0.0
    with pytest.raises(NotImplementedError):
        next(iter(d.evolve(yieldstep=1.0, finaltime=1.0)))


def test_tracking_matches_stepwise(swgpu_built):
    """Maximum depth and arrival time kept on the device equal those taken
    from the state after every step (FP64, Euler and RK2)."""
    import ctypes as C
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda._lib import State_t, check, lib
    sc = scenarios.channel_inflow(14, 5, seed=2)
    zc = sc.elevation_arrays()[0]
    for method in ("euler", "rk2"):
        a = gpu_from_scenario(sc, DEFAULT)
        b = gpu_from_scenario(sc, DEFAULT)
        for d in (a, b):
            d.set_timestepping_method(method)
            d.evolve_steps(0)
        a.set_tracking(0.02)
        st = State_t()
        check(lib().swgpu_evolve_run(a._h, 60, C.byref(st)), a._h)
        hmax = np.zeros(sc.N, dtype=np.float32)
        tarr = np.full(sc.N, -1.0, dtype=np.float32)
        for _ in range(60):
            b.step()
            h = b.quantities["stage"].centroid_values - zc
            hmax = np.maximum(hmax, h.astype(np.float32))
            new = (h > 0.02) & (tarr < 0)
            tarr[new] = np.float32(b.get_time())
        hm, ta = a.get_tracking()
        assert np.array_equal(hm, hmax) and np.array_equal(ta, tarr), method
        assert (ta > 0).any() and (ta < 0).any()
