"""Mesh input (.tsh) and result output (.sww) on the host side of GPU_domain.

* ``read_tsh`` parses ANUGA's ASCII triangulation format (the mesh files the
  reference's Merimbula scripts load, tests/CUDA/merimbula/*.tsh, read by
  the parser of src/anuga_cuda/acc_read_triangulation/read_triangulation.py):
  the vertex, vertex-title, triangle and segment blocks; anything after the
  segment block (the outline) is ignored.
* ``create_domain_from_file`` builds a domain from such a file as ANUGA's
  function of that name does (vertex attributes become vertex quantities,
  tagged exterior segments become boundary tags, untagged exterior edges are
  tagged "exterior").
* ``SWWWriter`` writes ANUGA's SWW result format (NetCDF 3 classic, through
  scipy.io.netcdf_file): mesh, static elevation and friction, and stage and
  momenta per stored time, either smoothed onto the mesh nodes (ANUGA's
  default) or per triangle vertex.  GPU_domain stores one time slice at each
  yield of ``evolve`` when ``set_store(True)``, from vertex values copied
  back from the device (the reference's store_timestep,
  src/anuga_cuda/gpu_domain_advanced.py:2167-2172).
"""
from __future__ import annotations

import os

import numpy as np

__all__ = ["read_tsh", "tsh_to_mesh_arrays", "create_domain_from_file", "SWWWriter",
           "read_sww"]


def _counted_block_header(line):
    parts = line.split("#", 1)[0].split()
    if not parts:
        return 0, 0
    n = int(parts[0])
    m = int(parts[1]) if len(parts) > 1 else 0
    return n, m


def read_tsh(path):
    """The generated triangulation of an ANUGA .tsh file as a dict:
    vertices (P,2) float64, vertex_attributes (P,A) or None,
    vertex_attribute_titles, triangles (N,3) int64, triangle_neighbors
    (N,3), triangle_tags (N strings), segments (S,2), segment_tags."""
    with open(path, "r") as fd:
        nv, na = _counted_block_header(fd.readline())
        verts = np.zeros((nv, 2))
        attrs = np.zeros((nv, na)) if na else None
        for i in range(nv):
            f = fd.readline().split()
            verts[i] = float(f[1]), float(f[2])
            if na:
                attrs[i] = [float(x) for x in f[3:3 + na]]
        fd.readline()                       # vertex title header
        titles = [fd.readline().strip() for _ in range(na)]
        nt, _ = _counted_block_header(fd.readline())
        tris = np.zeros((nt, 3), dtype=np.int64)
        nbrs = np.zeros((nt, 3), dtype=np.int64)
        ttags = []
        for i in range(nt):
            f = fd.readline().split()
            tris[i] = int(f[1]), int(f[2]), int(f[3])
            nbrs[i] = int(f[4]), int(f[5]), int(f[6])
            ttags.append(" ".join(f[7:]))
        ns, _ = _counted_block_header(fd.readline())
        segs = np.zeros((ns, 2), dtype=np.int64)
        stags = []
        for i in range(ns):
            f = fd.readline().split()
            segs[i] = int(f[1]), int(f[2])
            stags.append(" ".join(f[3:]))
    return {"vertices": verts, "vertex_attributes": attrs, "vertex_attribute_titles": titles,
            "triangles": tris, "triangle_neighbors": nbrs, "triangle_tags": ttags,
            "segments": segs, "segment_tags": stags}


def tsh_to_mesh_arrays(tsh):
    """(points, triangles, boundary) for anuga_cuda.Mesh / GPU_domain:
    boundary maps (triangle, edge) -> tag for every tagged segment that is an
    exterior edge; other exterior edges get "exterior" from the Mesh."""
    tris = np.asarray(tsh["triangles"], dtype=np.int64)
    a = tris[:, [1, 2, 0]].ravel()
    b = tris[:, [2, 0, 1]].ravel()
    key = np.minimum(a, b) * (len(tsh["vertices"]) + 1) + np.maximum(a, b)
    uniq, counts = np.unique(key, return_counts=True)
    exterior = set(uniq[counts == 1].tolist())
    where = {}
    for e, kk in enumerate(key.tolist()):
        if kk in exterior:
            where[kk] = (e // 3, e % 3)
    boundary = {}
    nverts = len(tsh["vertices"]) + 1
    for (p, q), tag in zip(np.asarray(tsh["segments"]).tolist(), tsh["segment_tags"]):
        kk = min(p, q) * nverts + max(p, q)
        if kk in where and tag:
            boundary[where[kk]] = tag
    return np.asarray(tsh["vertices"], dtype=np.float64), tris, boundary


def create_domain_from_file(filename, DomainClass=None, **kwargs):
    """ANUGA's create_domain_from_file for .tsh files: a GPU_domain (or
    ``DomainClass``) on the file's triangulation; a vertex attribute titled
    like a quantity (e.g. "elevation") is set as that quantity's vertex
    values."""
    from .gpu_domain import GPU_domain
    cls = DomainClass or GPU_domain
    tsh = read_tsh(filename)
    pts, tris, boundary = tsh_to_mesh_arrays(tsh)
    domain = cls(pts, tris, boundary, **kwargs)
    attrs = tsh["vertex_attributes"]
    if attrs is not None:
        for j, title in enumerate(tsh["vertex_attribute_titles"]):
            if title in ("elevation", "friction", "stage"):
                domain.set_quantity(title, attrs[:, j][tris])
    return domain


class SWWWriter:
    """ANUGA SWW file (NetCDF 3 classic).  Dimensions number_of_volumes,
    number_of_vertices (3), number_of_points, number_of_timesteps
    (unlimited), numbers_in_range (2); variables x, y (float32, relative to
    the lower-left corner), volumes (int32), elevation and friction
    (static), time (float64), and stage, xmomentum, ymomentum
    (number_of_timesteps x number_of_points, float32), each with a
    *_range variable.  ``smooth`` stores values averaged onto the mesh nodes
    (ANUGA's default); otherwise every triangle vertex is its own point."""

    DYNAMIC = ("stage", "xmomentum", "ymomentum")

    def __init__(self, filename, points, triangles, elevation_vertex, friction_vertex=None,
                 smooth=True, starttime=0.0, description="anuga_cuda GPU_domain output"):
        from scipy.io import netcdf_file
        self.filename = filename
        self.smooth = bool(smooth)
        pts = np.asarray(points, dtype=np.float64)
        tris = np.asarray(triangles, dtype=np.int64)
        self.triangles = tris
        self.npoints_mesh = len(pts)
        xll, yll = float(pts[:, 0].min()), float(pts[:, 1].min())
        if self.smooth:
            P, vols = pts, tris
            self._count = np.bincount(tris.ravel(), minlength=len(pts)).astype(np.float64)
        else:
            P = pts[tris].reshape(-1, 2)
            vols = np.arange(3 * len(tris), dtype=np.int64).reshape(-1, 3)
        f = netcdf_file(filename, "w", version=1)
        f.institution = "anuga_cuda"
        f.description = description
        f.smoothing = "Yes" if self.smooth else "No"
        f.vertices_are_stored_uniquely = "False" if self.smooth else "True"
        f.order = 1
        f.starttime = float(starttime)
        f.xllcorner, f.yllcorner = xll, yll
        f.zone, f.false_easting, f.false_northing = -1, 500000, 10000000
        f.datum, f.projection, f.units = "wgs84", "UTM", "m"
        # NetCDF 3 wants the record (unlimited) dimension defined first
        f.createDimension("number_of_timesteps", None)
        f.createDimension("number_of_volumes", len(tris))
        f.createDimension("number_of_vertices", 3)
        f.createDimension("number_of_points", len(P))
        f.createDimension("numbers_in_range", 2)
        for name, col in (("x", 0), ("y", 1)):
            v = f.createVariable(name, "f", ("number_of_points",))
            v[:] = (P[:, col] - (xll if col == 0 else yll)).astype(np.float32)
        v = f.createVariable("volumes", "i", ("number_of_volumes", "number_of_vertices"))
        v[:] = vols.astype(np.int32)
        static = {"elevation": elevation_vertex}
        if friction_vertex is not None:
            static["friction"] = friction_vertex
        for name, vals in static.items():
            pv = self._to_points(vals)
            v = f.createVariable(name, "f", ("number_of_points",))
            v[:] = pv.astype(np.float32)
            r = f.createVariable(name + "_range", "f", ("numbers_in_range",))
            r[:] = np.array([pv.min(), pv.max()], dtype=np.float32)
        f.createVariable("time", "d", ("number_of_timesteps",))
        for name in self.DYNAMIC:
            f.createVariable(name, "f", ("number_of_timesteps", "number_of_points"))
            r = f.createVariable(name + "_range", "f", ("numbers_in_range",))
            r[:] = np.array([np.inf, -np.inf], dtype=np.float32)
        f.close()
        self.nsteps = 0

    def _to_points(self, vertex_values):
        vv = np.asarray(vertex_values, dtype=np.float64).reshape(-1, 3)
        if not self.smooth:
            return vv.ravel()
        acc = np.bincount(self.triangles.ravel(), weights=vv.ravel(),
                          minlength=self.npoints_mesh)
        return acc / np.maximum(self._count, 1.0)

    def store_timestep(self, time, quantities):
        """Append one time slice; ``quantities`` maps stage / xmomentum /
        ymomentum to (N, 3) vertex values."""
        from scipy.io import netcdf_file
        f = netcdf_file(self.filename, "a", version=1)
        try:
            i = self.nsteps
            f.variables["time"][i] = float(time)
            for name in self.DYNAMIC:
                pv = self._to_points(quantities[name]).astype(np.float32)
                f.variables[name][i, :] = pv
                r = f.variables[name + "_range"]
                r[:] = np.array([min(float(r[0]), float(pv.min())),
                                 max(float(r[1]), float(pv.max()))], dtype=np.float32)
            self.nsteps += 1
        finally:
            f.close()


def read_sww(filename):
    """The arrays of an SWW file as a dict of numpy arrays (copies) plus
    its global attributes under "attributes"."""
    from scipy.io import netcdf_file
    f = netcdf_file(filename, "r", mmap=False)
    try:
        out = {k: np.array(v[:]) for k, v in f.variables.items()}
        out["attributes"] = dict(f._attributes)
    finally:
        f.close()
    return out


def sww_path(datadir, name):
    return os.path.join(datadir or ".", (name or "domain") + ".sww")
