"""In-tree build of libswgpu.so for sm_103a (GB300) with nvcc.

Five translation units are compiled in parallel and linked into
``anuga_cuda/libswgpu.so`` next to this file:

* ``csrc/swgpu_fp64.cu``  -- the FP64 parity kernels, ``--fmad=false`` so that
  no multiply-add is contracted (the reference's C kernels are built the same
  way by gcc on x86-64);
* ``csrc/swgpu_mixed.cu`` -- the mixed-precision kernels (FMA allowed, FP32
  division and square root approximate, denormals flushed);
* ``csrc/swgpu_api.cu``   -- the C ABI, allocation and the evolve loop;
* ``csrc/swgpu_noalloc.cu`` -- the allocation-free water-volume entry point;
* ``csrc/swgpu_mlp.cu``   -- the BF16 tensor-core MLP surrogate.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)                     # anuga-cuda_gb300/
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG_ROOT), "include")
OBJ = os.path.join(PKG_ROOT, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE]
UNITS = {
    "swgpu_fp64.cu": ["--fmad=false"],
    "swgpu_mixed.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"],
    "swgpu_api.cu": [],
    "swgpu_noalloc.cu": ["--fmad=false"],
    "swgpu_mlp.cu": [],
}


def library_path() -> str:
    return os.path.join(HERE, "libswgpu.so")


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh"))]
    files.append(os.path.join(INCLUDE, "swgpu.h"))
    return files


def up_to_date() -> bool:
    so = library_path()
    if not os.path.exists(so):
        return False
    t = os.path.getmtime(so)
    return all(os.path.getmtime(f) <= t for f in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libswgpu.so if any source is newer; returns its path."""
    so = library_path()
    if not force and up_to_date():
        return so
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)

    def compile_one(item):
        src, extra = item
        obj = os.path.join(OBJ, src.replace(".cu", ".o"))
        cmd = [nvcc] + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS.items()))
    tmp = so + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, so)
    return so
