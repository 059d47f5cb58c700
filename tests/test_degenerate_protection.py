"""The degenerate-timestep guard of GPU_domain (host side: it runs on the
downloaded max_speed, as the reference's override does) against the
oracle's loop restatement of the reference's
apply_protection_against_isolated_degenerate_timesteps
(src/anuga_cuda/gpu_domain_advanced.py:914-951) and of ANUGA's create_bins /
histogram: the same triangles zeroed on triggering and on non-triggering
speed distributions.  No GPU: the method runs on a stand-in holding the
arrays it reads and writes."""
import types

import numpy as np
import pytest

from anuga_cuda.gpu_domain import GPU_domain
from oracle import oracle as O


def _stand_in(max_speed, xmom, ymom):
    q = {n: types.SimpleNamespace(centroid_values=np.array(a, dtype=np.float64),
                                  vertex_values=np.zeros((len(a), 3)),
                                  edge_values=np.zeros((len(a), 3)))
         for n, a in (("xmomentum", xmom), ("ymomentum", ymom))}
    d = types.SimpleNamespace(protect_against_isolated_degenerate_timesteps=True,
                              max_speed=np.array(max_speed, dtype=np.float64), quantities=q,
                              uploads=[])
    d._to_internal = lambda a: a
    d._upload = lambda name, c, v, e: d.uploads.append(name)
    return d


def _cases():
    rng = np.random.default_rng(11)
    out = []
    base = rng.uniform(0.5, 3.0, 500)
    one = base.copy()
    one[17] = 60.0                          # one isolated fast triangle: triggers
    out.append(one)
    two = base.copy()
    two[[3, 400]] = [55.0, 58.0]            # two, both above the last edge
    out.append(two)
    spread = rng.uniform(0.0, 40.0, 500)    # fast but not isolated: bins 4-8 occupied
    out.append(spread)
    slow = rng.uniform(0.0, 9.0, 500)       # below 10 m/s: nothing happens
    out.append(slow)
    flat = np.full(64, 12.0)                # all equal: a single bin
    out.append(flat)
    gap = np.concatenate([rng.uniform(0, 1, 300), rng.uniform(3.5, 4.0, 50), [30.0]])
    out.append(gap)                         # bins 1-3 occupied, 4-8 empty, one outlier
    return out


@pytest.mark.parametrize("case", range(6))
def test_guard_matches_oracle(case):
    ms = _cases()[case]
    rng = np.random.default_rng(case)
    xm, ym = rng.normal(size=len(ms)), rng.normal(size=len(ms))
    d = _stand_in(ms, xm, ym)
    GPU_domain.apply_protection_against_isolated_degenerate_timesteps(d)
    oxm, oym, _, zeroed = O.degenerate_timestep_protection(ms, xm, ym)
    assert np.array_equal(d.quantities["xmomentum"].centroid_values, oxm)
    assert np.array_equal(d.quantities["ymomentum"].centroid_values, oym)
    assert bool(d.uploads) == bool(zeroed)
    if case in (0, 1, 5):
        assert zeroed, case
    if case in (2, 3, 4):
        assert not zeroed, case


def test_guard_off_does_nothing():
    ms = _cases()[0]
    d = _stand_in(ms, np.ones(len(ms)), np.ones(len(ms)))
    d.protect_against_isolated_degenerate_timesteps = False
    GPU_domain.apply_protection_against_isolated_degenerate_timesteps(d)
    assert not d.uploads and d.quantities["xmomentum"].centroid_values.all()
