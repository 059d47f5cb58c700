"""Unstructured triangle meshes with ANUGA's neighbour structure.

ANUGA's mesh module is not part of the reference (it subclasses
``anuga.Domain``); the arrays built here are the ones the reference's GPU
domain uploads (``allocate_device_array``,
src/anuga_cuda/gpu_domain_advanced.py:582-730) and its C kernels read
(``struct domain``, src/anuga_HMPP/sw_domain.h:16-180):

* ``neighbours[k, i]``: triangle across edge ``i`` (the edge opposite vertex
  ``i``) or ``-(m+1)`` for boundary slot ``m``; boundary slots are numbered in
  sorted ``(triangle, edge)`` order.
* ``neighbour_edges[k, i]``: index of the same edge inside the neighbour.
* ``surrogate_neighbours``: neighbours with boundary entries replaced by ``k``.
* ``normals[k, 2i:2i+2]``: outward unit normal of edge ``i``;
  ``edgelengths``, ``areas``, ``centroid_coordinates``,
  ``vertex_coordinates`` (``[k, 2i:2i+2]`` = vertex ``i``).
* ``radii``: smallest centroid-to-edge-midpoint distance.

Triangles are renumbered along a Morton (Z-order) curve of their centroids,
so that a triangle's neighbours are close to it in memory and the GPU's
neighbour gathers stay within L1/L2.  Per-edge geometry is computed once per
edge and mirrored to the neighbour, so the two sides of an edge see exactly
negated normals and identical lengths, which makes the central-upwind flux
exactly antisymmetric.
"""
from __future__ import annotations

import numpy as np

__all__ = ["Mesh", "rectangular_cross", "morton_order"]


def _part1by1(v: np.ndarray) -> np.ndarray:
    """Spread the low 16 bits of v to the even bit positions."""
    v = v.astype(np.uint64) & np.uint64(0xFFFF)
    v = (v | (v << np.uint64(8))) & np.uint64(0x00FF00FF)
    v = (v | (v << np.uint64(4))) & np.uint64(0x0F0F0F0F)
    v = (v | (v << np.uint64(2))) & np.uint64(0x33333333)
    v = (v | (v << np.uint64(1))) & np.uint64(0x55555555)
    return v


def morton_order(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """Permutation sorting points along a 2x16-bit Morton curve."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    span = max(float(x.max() - x.min()), float(y.max() - y.min()), 1e-300)
    qx = np.floor((x - x.min()) / span * 65535.0).astype(np.int64)
    qy = np.floor((y - y.min()) / span * 65535.0).astype(np.int64)
    code = _part1by1(qx) | (_part1by1(qy) << np.uint64(1))
    return np.argsort(code, kind="stable")


class Mesh:
    """Triangle mesh with ANUGA's connectivity and geometry arrays.

    Parameters
    ----------
    points : (P, 2) float array
    triangles : (N, 3) int array of point indices (either orientation)
    boundary : dict ``{(triangle, edge): tag}`` for exterior edges; exterior
        edges not listed get the tag ``"exterior"`` (ANUGA's default).
    reorder : renumber triangles in Morton order of their centroids.
    """

    def __init__(self, points, triangles, boundary=None, reorder=True):
        pts = np.ascontiguousarray(points, dtype=np.float64)
        tri = np.array(triangles, dtype=np.int64, copy=True)
        if pts.ndim != 2 or pts.shape[1] != 2 or tri.ndim != 2 or tri.shape[1] != 3:
            raise ValueError("points must be (P,2) and triangles (N,3)")
        if tri.size and (tri.min() < 0 or tri.max() >= len(pts)):
            raise ValueError("triangle vertex index out of range")
        boundary = dict(boundary or {})

        # counter-clockwise orientation; a flip swaps vertices 1 and 2, which
        # swaps edges 1 and 2
        x, y = pts[tri, 0], pts[tri, 1]
        signed = (x[:, 1] - x[:, 0]) * (y[:, 2] - y[:, 0]) - (x[:, 2] - x[:, 0]) * (y[:, 1] - y[:, 0])
        if np.any(signed == 0):
            raise ValueError("degenerate (zero-area) triangle")
        cw = signed < 0
        self.flipped = cw            # caller's order: vertices 1 and 2 swapped
        if cw.any():
            tri[cw, 1], tri[cw, 2] = tri[cw, 2].copy(), tri[cw, 1].copy()
            swap = {1: 2, 2: 1, 0: 0}
            boundary = {(k, swap[e] if cw[k] else e): t for (k, e), t in boundary.items()}

        if reorder and len(tri) > 1:
            c = pts[tri].mean(axis=1)
            perm = morton_order(c[:, 0], c[:, 1])
            inv = np.empty_like(perm)
            inv[perm] = np.arange(len(perm))
            tri = tri[perm]
            boundary = {(int(inv[k]), e): t for (k, e), t in boundary.items()}
            self.permutation = perm
        else:
            self.permutation = np.arange(len(tri))

        self.points = pts
        self.triangles = tri
        self._build_topology(boundary)
        self._build_geometry()

    # ------------------------------------------------------------------
    def _build_topology(self, boundary):
        tri = self.triangles
        N = len(tri)
        a = tri[:, [1, 2, 0]]  # edge i runs from vertex i+1 to vertex i+2
        b = tri[:, [2, 0, 1]]
        lo = np.minimum(a, b).ravel()
        hi = np.maximum(a, b).ravel()
        key = lo * (len(self.points) + 1) + hi
        order = np.argsort(key, kind="stable")
        ks = key[order]
        same = ks[1:] == ks[:-1]
        if np.any(same[1:] & same[:-1]):
            raise ValueError("an edge is shared by more than two triangles")
        first = order[:-1][same]
        second = order[1:][same]
        neighbours = np.full(3 * N, -1, dtype=np.int64)
        neighbour_edges = np.full(3 * N, -1, dtype=np.int64)
        neighbours[first] = second // 3
        neighbour_edges[first] = second % 3
        neighbours[second] = first // 3
        neighbour_edges[second] = first % 3
        exterior = np.nonzero(neighbours < 0)[0]
        keys = [(int(e // 3), int(e % 3)) for e in exterior]
        keyset = set(keys)
        for kk in boundary:
            if kk not in keyset:
                raise ValueError(f"boundary edge {kk} is not an exterior edge")
        tags = {kk: boundary.get(kk, "exterior") for kk in keys}
        keys.sort()
        self.boundary = {kk: tags[kk] for kk in keys}
        self.boundary_cells = np.array([k for k, _ in keys], dtype=np.int64)
        self.boundary_edges = np.array([e for _, e in keys], dtype=np.int64)
        for m, (k, e) in enumerate(keys):
            neighbours[3 * k + e] = -m - 1
        self.neighbours = neighbours.reshape(N, 3)
        self.neighbour_edges = neighbour_edges.reshape(N, 3)
        sur = self.neighbours.copy()
        own = np.repeat(np.arange(N)[:, None], 3, axis=1)
        sur[sur < 0] = own[sur < 0]
        self.surrogate_neighbours = sur
        self.number_of_boundaries = (self.neighbours < 0).sum(axis=1).astype(np.int64)
        self.tri_full_flag = np.ones(N, dtype=np.int64)
        names = sorted(set(self.boundary.values()))
        self.tag_names = names
        index = {t: i for i, t in enumerate(names)}
        self.boundary_tag = np.array([index[self.boundary[kk]] for kk in keys], dtype=np.int64)

    def _build_geometry(self):
        tri, pts = self.triangles, self.points
        N = len(tri)
        V = pts[tri]  # (N,3,2)
        self.vertex_coordinates = np.ascontiguousarray(V.reshape(N, 6))
        self.centroid_coordinates = np.ascontiguousarray((V[:, 0] + V[:, 1] + V[:, 2]) / 3.0)
        x0, y0 = V[:, 0, 0], V[:, 0, 1]
        x1, y1 = V[:, 1, 0], V[:, 1, 1]
        x2, y2 = V[:, 2, 0], V[:, 2, 1]
        self.areas = 0.5 * ((x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0))
        # per-edge geometry, computed once on the lower-index side of each
        # interior edge and mirrored (negated normal) to the other side
        normals = np.empty((N, 3, 2))
        lengths = np.empty((N, 3))
        for i in range(3):
            pa = V[:, (i + 1) % 3]
            pb = V[:, (i + 2) % 3]
            dx = pb[:, 0] - pa[:, 0]
            dy = pb[:, 1] - pa[:, 1]
            L = np.sqrt(dx * dx + dy * dy)
            lengths[:, i] = L
            normals[:, i, 0] = dy / L
            normals[:, i, 1] = -dx / L
        nb = self.neighbours
        ne = self.neighbour_edges
        k_idx, i_idx = np.nonzero((nb >= 0) & (nb < np.arange(N)[:, None]))
        n_idx = nb[k_idx, i_idx]
        m_idx = ne[k_idx, i_idx]
        normals[k_idx, i_idx] = -normals[n_idx, m_idx]
        lengths[k_idx, i_idx] = lengths[n_idx, m_idx]
        self.normals = np.ascontiguousarray(normals.reshape(N, 6))
        self.edgelengths = np.ascontiguousarray(lengths)
        c = self.centroid_coordinates
        d = np.empty((N, 3))
        for i in range(3):
            mx = 0.5 * (V[:, (i + 1) % 3, 0] + V[:, (i + 2) % 3, 0])
            my = 0.5 * (V[:, (i + 1) % 3, 1] + V[:, (i + 2) % 3, 1])
            d[:, i] = np.sqrt((c[:, 0] - mx) ** 2 + (c[:, 1] - my) ** 2)
        self.radii = d.min(axis=1)

    # ------------------------------------------------------------------
    @property
    def number_of_elements(self) -> int:
        return len(self.triangles)

    @property
    def number_of_boundary_elements(self) -> int:
        return len(self.boundary_cells)

    def __len__(self):
        return self.number_of_elements

    def tag_length(self, tag) -> float:
        """Total length of the boundary edges carrying ``tag``."""
        t = self.tag_names.index(tag)
        sel = self.boundary_tag == t
        L = np.asarray(self.edgelengths).reshape(-1, 3)
        return float(L[self.boundary_cells[sel], self.boundary_edges[sel]].sum())

    def vertex_values(self, f):
        """Evaluate f(x, y) at the three vertices of every triangle, (N,3)."""
        V = self.vertex_coordinates.reshape(-1, 3, 2)
        return np.asarray(f(V[..., 0], V[..., 1]), dtype=np.float64) * np.ones((len(V), 3))

    def centroid_values(self, f):
        c = self.centroid_coordinates
        return np.asarray(f(c[:, 0], c[:, 1]), dtype=np.float64) * np.ones(len(c))


def rectangular_cross(m, n, len1=1.0, len2=1.0, origin=(0.0, 0.0)):
    """Points, triangles and boundary tags of an m x n grid of rectangles,
    each cut into four triangles by its centre point (ANUGA's
    rectangular_cross layout: 4*m*n triangles).  Tags: left, right, bottom,
    top."""
    m, n = int(m), int(n)
    dx, dy = len1 / m, len2 / n
    ox, oy = origin
    ii, jj = np.meshgrid(np.arange(m + 1), np.arange(n + 1), indexing="ij")
    corners = np.stack([ox + ii.ravel() * dx, oy + jj.ravel() * dy], axis=1)
    ci, cj = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    ci, cj = ci.ravel(), cj.ravel()
    centres = np.stack([ox + (ci + 0.5) * dx, oy + (cj + 0.5) * dy], axis=1)
    points = np.concatenate([corners, centres])

    def corner(i, j):
        return i * (n + 1) + j

    c = (m + 1) * (n + 1) + np.arange(m * n)
    v00, v10 = corner(ci, cj), corner(ci + 1, cj)
    v11, v01 = corner(ci + 1, cj + 1), corner(ci, cj + 1)
    # four CCW triangles per cell, edge 2 (opposite the centre) on the cell side
    bottom = np.stack([v00, v10, c], axis=1)
    right = np.stack([v10, v11, c], axis=1)
    top = np.stack([v11, v01, c], axis=1)
    left = np.stack([v01, v00, c], axis=1)
    tris = np.stack([bottom, right, top, left], axis=1).reshape(-1, 3)
    cell = np.repeat(np.arange(m * n), 4)
    side = np.tile(np.arange(4), m * n)
    boundary = {}
    I, J = ci[cell], cj[cell]
    for t in np.nonzero((side == 0) & (J == 0))[0]:
        boundary[(int(t), 2)] = "bottom"
    for t in np.nonzero((side == 1) & (I == m - 1))[0]:
        boundary[(int(t), 2)] = "right"
    for t in np.nonzero((side == 2) & (J == n - 1))[0]:
        boundary[(int(t), 2)] = "top"
    for t in np.nonzero((side == 3) & (I == 0))[0]:
        boundary[(int(t), 2)] = "left"
    return points, tris, boundary
