"""The timestep rule of the mixed flux kernel, checked on the CPU oracle.

ANUGA's flux loop evaluates each edge once and lowers the timestep by
radii[k] / max_speed and radii[n] / max_speed for both triangles of the edge
(src/anuga_HMPP/shallow_water_ext.c:4653-4664).  The triangle-centric GPU
kernel evaluates every interior edge twice, once from each side, and lowers
the timestep by its own triangle's radius only.  That gives the same number
because the two evaluations of an edge see the same two states with the
normal negated, so they produce bit-identical maximum speeds.  This test
checks that symmetry edge by edge, and the resulting equality of the two
minima, on the golden cases: at their initial state and after Euler steps.
The kernel's block minimum is an integer warp reduction over the timesteps'
bit patterns; the last test checks that key's order on the host."""
import numpy as np
import pytest

from helpers import GOLDEN_CASES, golden_oracle, load_golden


def _own_radius_minimum(od, ms):
    A, p = od.arrays, od.params
    r = A["radii"][:, None]
    ok = ms > p.epsilon
    t = np.full(ms.shape, np.inf)
    t[ok] = (np.broadcast_to(r, ms.shape)[ok]) / ms[ok]
    return min(float(p.evolve_max_timestep), float(t.min()))


def _check_state(od):
    A = od.arrays
    assert np.all(A["tri_full_flag"] == 1)
    ms = od.edge_speeds()
    nb = A["neighbours"].reshape(-1, 3)
    ne = A["neighbour_edges"].reshape(-1, 3)
    k, i = np.nonzero(nb >= 0)
    n, m = nb[k, i], ne[k, i]
    # the two sides of every interior edge: the same maximum speed, bit for bit
    a, b = ms[k, i], ms[n, m]
    assert np.array_equal(a.view(np.int64), b.view(np.int64))
    ft = od.compute_fluxes()
    assert _own_radius_minimum(od, ms) == ft
    return int((ms > od.params.epsilon).sum())


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_own_radius_minimum_equals_anuga_rule(case, oracle_mod):
    g = load_golden(case)
    od = golden_oracle(g, oracle_mod)
    od.distribute_to_vertices_and_edges()
    od.update_boundary()
    wet_edges = _check_state(od)
    od.evolve_start(1.0e300)
    for _ in range(10):
        assert od.evolve_one_euler_step() == 0
        od.distribute_to_vertices_and_edges()
        od.update_boundary()
        wet_edges += _check_state(od)
    assert wet_edges > 0


def _timestep_key(t):
    """The mixed flux's integer key of an FP32 timestep: the bit pattern as a
    signed integer for t >= 0 (sign bit cleared), -1 for NaN or t < 0."""
    t = np.asarray(t, np.float32)
    bits = t.view(np.int32) & np.int32(0x7FFFFFFF)
    return np.where(t >= 0, bits, np.int32(-1)).astype(np.int32)


def test_timestep_key_orders_as_the_floats():
    rng = np.random.default_rng(5)
    special = np.array([0.0, -0.0, np.inf, 3.0e38, np.finfo(np.float32).max,
                        np.finfo(np.float32).tiny, 1e-45, 1.0, 0.5], np.float32)
    for _ in range(200):
        t = np.concatenate([rng.choice(special, 8),
                            (10.0 ** rng.uniform(-40, 38, 56)).astype(np.float32)])
        rng.shuffle(t)
        k = _timestep_key(t)
        # the minimum key is the key of the minimum timestep, and maps back to it
        assert k.min() == _timestep_key(t.min())
        assert np.array_equal(np.array([k.min()], np.int32).view(np.float32), [t.min()])
        # a NaN or a negative timestep anywhere wins the minimum as -1
        for bad in (np.nan, -1.0e-3, -np.inf):
            u = t.copy()
            u[rng.integers(len(u))] = bad
            assert _timestep_key(u).min() == -1
