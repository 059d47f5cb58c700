"""Convert the reference's Merimbula mesh fixture (tests/CUDA/merimbula/
merimbula_10785.tsh, the real-estuary mesh its GPU scripts load) into a
compact fixture for tests that run where the reference is absent.

    python tests/golden/make_merimbula.py

Stores the parsed vertices, triangles and exterior boundary tags (the .tsh
reader's output, anuga_cuda.io.tsh_to_mesh_arrays) and the counts of every
block, so the reader can be checked against the file where it exists.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "anuga-cuda_gb300")]

from anuga_cuda.io import read_tsh, tsh_to_mesh_arrays  # noqa: E402

SRC = os.path.join(os.environ.get("ANUGA_CUDA_REFERENCE", "/root/reference"),
                   "tests", "CUDA", "merimbula", "merimbula_10785.tsh")
HERE = os.path.dirname(os.path.abspath(__file__))

if __name__ == "__main__":
    if not os.path.exists(SRC):
        sys.exit("reference mesh not present")
    t = read_tsh(SRC)
    pts, tris, bnd = tsh_to_mesh_arrays(t)
    keys = sorted(bnd)
    names = sorted(set(bnd.values()))
    np.savez_compressed(
        os.path.join(HERE, "merimbula_10785.npz"),
        points=pts, triangles=tris.astype(np.int32),
        boundary=np.array([(k, e, names.index(bnd[(k, e)])) for k, e in keys], dtype=np.int32),
        tag_names=np.array(names),
        counts=np.array([len(t["vertices"]), len(t["triangles"]), len(t["segments"])]),
        segment_tag_counts=np.array([t["segment_tags"].count(n) for n in names]))
    print(len(pts), len(tris), len(t["segments"]), names, len(keys))
