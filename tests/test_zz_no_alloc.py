"""The allocation-free water-volume entry point, swgpu_water_volume_noalloc.

It exists for callers that cannot allocate device memory when they need the
volume (inside a CUDA stream capture, under a device-memory pool they do not
own, in loops that must avoid cudaMalloc's synchronisation); its scratch is a
static device array.  It sums in swgpu_mass's order, so on an FP64 handle's
own centroid arrays, in the handle's triangle order (a GPU_domain built from a
Mesh keeps the Mesh's order), it must return exactly swgpu_mass's value.
This file is collected last on purpose (a failure here leaves every other
test already run) and passes alone in a fresh process as well as after the
rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_SUBSET = 1e-12  # a sub-range against numpy's own (differently ordered) sum


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def test_noalloc_volume_matches_handle_volume_twice(swgpu_built):
    import torch
    from anuga_cuda import DEFAULT, GPU_domain, scenarios
    from anuga_cuda._lib import lib
    sc = scenarios.dam_break(60, 50)
    d = GPU_domain(mesh=sc.mesh, parameters=DEFAULT, precision="fp64")
    sc.apply_to(d)
    d.evolve_steps(25)
    expected = d.get_water_volume()
    N = sc.N
    # the caller's own device buffers (this caller can allocate; the entry
    # point does not)
    areas = _dev(torch, sc.mesh.areas)
    stage = _dev(torch, d.quantities["stage"].centroid_values)
    bed = _dev(torch, d.quantities["elevation"].centroid_values)
    out = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
    L = lib()
    for call in range(2):
        out.fill_(np.nan)
        torch.cuda.synchronize()
        rc = L.swgpu_water_volume_noalloc(areas.data_ptr(), stage.data_ptr(), bed.data_ptr(), N,
                                          out.data_ptr(), None)
        assert rc == 0, L.swgpu_last_error(None)
        torch.cuda.synchronize()
        got = float(out.item())
        assert got == expected, (call, got, expected)
    # a different size on the same (shared) scratch, then the first again
    half = N // 2
    rc = L.swgpu_water_volume_noalloc(areas.data_ptr(), stage.data_ptr(), bed.data_ptr(), half,
                                      out.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    a, w, z = sc.mesh.areas, d.quantities["stage"].centroid_values, \
        d.quantities["elevation"].centroid_values
    ref_half = float(np.sum(a[:half] * (w[:half] - z[:half])))
    assert abs(out.item() - ref_half) <= REL_SUBSET * abs(ref_half)
    # the full size again on the same scratch: the same value as before
    rc = L.swgpu_water_volume_noalloc(areas.data_ptr(), stage.data_ptr(), bed.data_ptr(), N,
                                      out.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert float(out.item()) == expected


def test_noalloc_rejects_sizes_beyond_its_scratch(swgpu_built):
    import torch
    from anuga_cuda._lib import lib
    L = lib()
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = x.data_ptr()
    assert L.swgpu_water_volume_noalloc(p, p, p, 4_194_305, p, None) == 1
    assert b"4194304" in L.swgpu_last_error(None)
    assert L.swgpu_water_volume_noalloc(p, p, p, 0, p, None) == 1
    assert L.swgpu_water_volume_noalloc(None, p, p, 4, p, None) == 1
    _ = C
