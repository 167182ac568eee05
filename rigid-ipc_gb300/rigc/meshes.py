"""Triangle-mesh generators for the synthetic rigid-body scenes.

Every mesh is returned as ``(V, F)`` with ``V`` an ``(n, 3)`` float64 array and
``F`` an ``(m, 3)`` int32 array of outward-oriented triangles.  Edges are derived
from the faces by :func:`edges_from_faces` (sorted, unique ``(min, max)``
pairs), which plays the role of ``igl::edges`` in the reference's scene reader
(``src/io/read_rb_scene.cpp:121-128``).  ``faces_to_edges`` follows the
reference's convention (``src/utils/mesh_selector.cpp:69-80``): entry ``(f, j)``
is the edge joining face vertices ``j`` and ``(j + 1) % 3``.
"""
from __future__ import annotations

import numpy as np


def edges_from_faces(F: np.ndarray) -> np.ndarray:
    """Unique undirected edges of a triangle mesh, sorted lexicographically."""
    F = np.asarray(F, dtype=np.int64)
    if F.size == 0:
        return np.zeros((0, 2), dtype=np.int32)
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], axis=0)
    e = np.sort(e, axis=1)
    e = np.unique(e, axis=0)
    return e.astype(np.int32)


def faces_to_edges(F: np.ndarray, E: np.ndarray) -> np.ndarray:
    """For each face, the ids of its edges (j, j+1 mod 3), j = 0, 1, 2."""
    if len(F) == 0:
        return np.zeros((0, 3), dtype=np.int32)
    nv = int(max(F.max(), E.max())) + 1
    key = E[:, 0].astype(np.int64) * nv + E[:, 1].astype(np.int64)
    order = np.argsort(key)
    skey = key[order]
    out = np.empty((len(F), 3), dtype=np.int32)
    for j in range(3):
        a = F[:, j].astype(np.int64)
        b = F[:, (j + 1) % 3].astype(np.int64)
        k = np.minimum(a, b) * nv + np.maximum(a, b)
        pos = np.searchsorted(skey, k)
        assert np.all(skey[pos] == k), "face edge missing from edge list"
        out[:, j] = order[pos]
    return out


def cube(size: float = 1.0):
    """Axis-aligned cube centred at the origin: 8 vertices, 12 triangles."""
    h = 0.5 * size
    V = np.array([[x, y, z] for x in (-h, h) for y in (-h, h) for z in (-h, h)],
                 dtype=np.float64)
    # vertex index = 4*ix + 2*iy + iz
    quads = [
        (0, 1, 3, 2),  # x = -h
        (4, 6, 7, 5),  # x = +h
        (0, 4, 5, 1),  # y = -h
        (2, 3, 7, 6),  # y = +h
        (0, 2, 6, 4),  # z = -h
        (1, 5, 7, 3),  # z = +h
    ]
    F = []
    for a, b, c, d in quads:
        F.append((a, b, c))
        F.append((a, c, d))
    F = np.array(F, dtype=np.int32)
    return V, _orient_outward(V, F)


def tessellated_box(size=(1.0, 0.2, 1.0), n=(32, 4, 32)):
    """Box centred at the origin whose faces are grids of n[a] x n[b] quads
    (two triangles each) along their two axes; vertices on the box's edges
    are shared, so the mesh is closed.  size (1, 0.2, 1) with n (32, 4, 32):
    2,562 vertices, 7,680 edges, 5,120 triangles."""
    n = [int(k) for k in n]
    ext = np.asarray(size, dtype=np.float64)
    index = {}
    V = []

    def vid(i, j, k):
        key = (i, j, k)
        if key not in index:
            index[key] = len(V)
            V.append([(i / n[0] - 0.5) * ext[0], (j / n[1] - 0.5) * ext[1],
                      (k / n[2] - 0.5) * ext[2]])
        return index[key]

    F = []
    for ax in range(3):
        a, b = [d for d in range(3) if d != ax]
        for side in (0, n[ax]):
            for u in range(n[a]):
                for w in range(n[b]):
                    q = []
                    for du, dw in ((0, 0), (1, 0), (1, 1), (0, 1)):
                        c = [0, 0, 0]
                        c[ax], c[a], c[b] = side, u + du, w + dw
                        q.append(vid(*c))
                    F.append((q[0], q[1], q[2]))
                    F.append((q[0], q[2], q[3]))
    V = np.array(V, dtype=np.float64)
    return V, _orient_outward(V, np.array(F, dtype=np.int32))


def plane(size: float = 20.0):
    """Square in the y = 0 plane, normal +y: 4 vertices, 2 triangles."""
    h = 0.5 * size
    V = np.array([[-h, 0, -h], [h, 0, -h], [h, 0, h], [-h, 0, h]], dtype=np.float64)
    F = np.array([[0, 2, 1], [0, 3, 2]], dtype=np.int32)
    return V, F


def icosphere(subdivisions: int = 3, radius: float = 1.0):
    """Subdivided icosahedron on a sphere (subdivision 3: 642 v, 1280 f)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
         (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
         (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
         (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
         (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    V = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in V]
    for _ in range(subdivisions):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                cache[key] = len(V) - 1
            return cache[key]

        nF = []
        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nF += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nF
    V = np.array(V) * radius
    F = np.array(F, dtype=np.int32)
    return V, _orient_outward(V, F)


def torus(major: float = 1.0, minor: float = 0.25, n_major: int = 48,
          n_minor: int = 24):
    """Torus around the z axis (48 x 24 segments: 1152 v, 2304 f)."""
    i = np.arange(n_major)
    j = np.arange(n_minor)
    u = 2 * np.pi * i / n_major
    v = 2 * np.pi * j / n_minor
    uu, vv = np.meshgrid(u, v, indexing="ij")
    x = (major + minor * np.cos(vv)) * np.cos(uu)
    y = (major + minor * np.cos(vv)) * np.sin(uu)
    z = minor * np.sin(vv)
    V = np.stack([x, y, z], axis=-1).reshape(-1, 3)
    F = []
    for a in range(n_major):
        for b in range(n_minor):
            p00 = a * n_minor + b
            p10 = ((a + 1) % n_major) * n_minor + b
            p01 = a * n_minor + (b + 1) % n_minor
            p11 = ((a + 1) % n_major) * n_minor + (b + 1) % n_minor
            F.append((p00, p10, p11))
            F.append((p00, p11, p01))
    F = np.array(F, dtype=np.int32)
    # outward = away from the tube centre line
    c = V[F].mean(axis=1)
    ang = np.arctan2(c[:, 1], c[:, 0])
    centre = np.stack([major * np.cos(ang), major * np.sin(ang), 0 * ang], -1)
    n = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    flip = np.einsum("ij,ij->i", n, c - centre) < 0
    F[flip] = F[flip][:, [0, 2, 1]]
    return V, F


def convex_hull(points: np.ndarray):
    """Convex hull of points in general position (all on the unit sphere)."""
    from scipy.spatial import ConvexHull

    hull = ConvexHull(points)
    used = np.unique(hull.simplices)
    remap = -np.ones(len(points), dtype=np.int64)
    remap[used] = np.arange(len(used))
    V = points[used].astype(np.float64)
    F = remap[hull.simplices].astype(np.int32)
    return V, _orient_outward(V, F)


def _orient_outward(V, F):
    """Flip faces whose normal points towards the centroid (convex meshes)."""
    F = np.array(F, dtype=np.int32)
    c = V.mean(axis=0)
    fc = V[F].mean(axis=1)
    n = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    flip = np.einsum("ij,ij->i", n, fc - c) < 0
    F[flip] = F[flip][:, [0, 2, 1]]
    return F
