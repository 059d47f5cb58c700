"""Host-side assembly of an ensemble (no GPU): concatenated mesh arrays,
256-aligned scenario ranges, padding and boundary-slot bookkeeping."""
import numpy as np


def _assembled(scs):
    from anuga_cuda.config import DEFAULT
    from anuga_cuda.ensemble import Ensemble
    e = Ensemble.__new__(Ensemble)
    e.scenarios, e.parameters, e.precision = list(scs), DEFAULT, "mixed"
    e.order = list(range(len(scs)))
    e._build_arrays()
    return e


def test_ranges_aligned_and_topology_consistent():
    from anuga_cuda import scenarios
    scs = [scenarios.small_basin(7, 5, seed=1), scenarios.channel_inflow(9, 4, seed=2),
           scenarios.inflow_harbour(1200, seed=3)]
    e = _assembled(scs)
    A = e.arrays
    assert (e.offsets % 256 == 0).all() and e.offsets[-1] == e.N
    nbr = A["neighbours"].reshape(-1, 3)
    bc, be = A["boundary_cells"], A["boundary_edges"]
    assert len(bc) == e.Nb
    # every boundary slot m is referenced as -(m+1) by its owner edge
    assert (nbr[bc, be] == -np.arange(e.Nb) - 1).all()
    # interior neighbours stay inside the owner's scenario range
    scen = np.searchsorted(e.offsets, np.arange(e.N), side="right") - 1
    k, i = np.nonzero(nbr >= 0)
    assert (scen[nbr[k, i]] == scen[k]).all()
    ne = A["neighbour_edges"].reshape(-1, 3)
    assert (nbr[nbr[k, i], ne[k, i]] == k).all()
    # the scenarios' own triangles come first in each range, then padding
    for sc, (a, b), o1 in zip(scs, e.ranges, e.offsets[1:]):
        assert b - a == sc.N
        assert np.array_equal(A["areas"][a:b], sc.mesh.areas)
        assert (A["number_of_boundaries"][b:o1] == 3).all()
        assert (e.stage_centroid[b:o1] == 0).all() and (e.elevation_vertex[b:o1] == 0).all()
    # tag indices: every scenario tag plus one for the padding
    assert len(e.tags) == sum(len(sc.mesh.tag_names) for sc in scs) + 1
    assert A["boundary_tag"].max() == e.pad_tag


def test_ensemble_generator_distribution():
    from anuga_cuda import scenarios
    scs = scenarios.ensemble_harbours(count=6, seed=4, nmin=800, nmax=3000)
    n = np.array([sc.N for sc in scs])
    assert (n > 600).all() and (n < 3600).all()
    for sc in scs:
        q = sc.boundaries["west"]
        assert 50 <= q.peak <= 500 and 300 <= q.rise <= 1800
        assert 0.01 <= sc.friction[0] <= 0.05 and sc.finaltime == 3600.0
