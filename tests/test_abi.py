"""The C ABI: libswgpu.so builds for sm_103a, loads, and exports exactly the
functions include/swgpu.h declares; the ctypes structs match the header's
layout.  No GPU needed (no compute call is made)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "swgpu.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(swgpu_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(swgpu_built):
    from anuga_cuda import _lib
    path = swgpu_built.library_path()
    so = ctypes.CDLL(path)
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(so, n), n
    assert sorted(_lib.EXPORTED_SYMBOLS) == names, "ctypes binding covers the header"


def test_struct_layouts_match_header():
    from anuga_cuda import _lib
    # swgpu_mesh: 2 int64 + 14 pointers; swgpu_params: 15 doubles + 10 int64
    assert ctypes.sizeof(_lib.Mesh_t) == 8 * (2 + 14)
    assert ctypes.sizeof(_lib.Params_t) == 8 * (15 + 10)
    assert ctypes.sizeof(_lib.State_t) == 8 * (7 + 6)
    assert ctypes.sizeof(_lib.BoundaryTag_t) == 8 * 9
    from anuga_cuda.config import Parameters
    import dataclasses
    assert [f.name for f in dataclasses.fields(Parameters)] == [n for n, _ in _lib.PARAM_FIELDS]


def test_missing_library_fails_loudly(tmp_path):
    from anuga_cuda import _lib
    with pytest.raises(ImportError):
        _lib.lib(str(tmp_path / "nope.so"))
