"""Icosphere topology tables (host side).

The reference builds its sphere with the third-party ``meshzoo.icosa_sphere``
(util.py:17-50, call at util.py:43), which is not vendored, so its vertex
coordinates and order cannot be reproduced or checked here.  This project
generates its own icosphere on the GPU (``mesh.create_mesh``) with the
properties the reference relies on:

* ``10 k^2 + 2`` vertices and ``20 k^2`` triangles (util.py:25-28);
* the 12 icosahedron corners are vertices 0-11 (``sort_adjacency`` assumes
  it, util.py:640);
* consistent counter-clockwise winding seen from outside, so that
  ``build_adjacency`` (util.py:591-613) gives every vertex 6 distinct
  neighbours (5 at the corners);
* with even ``k`` a vertex at each pole (the reference notes this for
  meshzoo, util.py:24-26).

Layout (``k >= 1``):

* vertices 0-11: corners;
* then ``k - 1`` vertices along each of the 30 edges, edges in ascending
  ``(a, b)`` order, ``a < b``, position ``t = 1..k-1`` measured from corner
  ``a``; point = normalise((k - t) * A + t * B);
* then the ``(k-1)(k-2)/2`` interior vertices of each of the 20 faces, face
  by face, rows ``i = 1..k-2``, within a row ``j = 1..k-1-i``; point =
  normalise((k - i - j) * A + i * B + j * C) for face (A, B, C);
* triangles face by face; within a face, for ``i = 0..k-1`` and
  ``j = 0..k-1-i``: the upward triangle ``(i,j) (i+1,j) (i,j+1)`` and, if
  ``i + j < k - 1``, the downward triangle ``(i+1,j) (i+1,j+1) (i,j+1)``.

All point arithmetic is binary64 without FMA, with the sum ordered as
written, so the GPU kernel and any CPU mirror give identical bits.
"""
import numpy as np

PHI = (1.0 + np.sqrt(5.0)) / 2.0

# The standard golden-ratio icosahedron (cyclic permutations of (0, +-1, +-phi)),
# faces counter-clockwise seen from outside.
_CORNERS_RAW = (
    (-1.0, PHI, 0.0), (1.0, PHI, 0.0), (-1.0, -PHI, 0.0), (1.0, -PHI, 0.0),
    (0.0, -1.0, PHI), (0.0, 1.0, PHI), (0.0, -1.0, -PHI), (0.0, 1.0, -PHI),
    (PHI, 0.0, -1.0), (PHI, 0.0, 1.0), (-PHI, 0.0, -1.0), (-PHI, 0.0, 1.0),
)

FACES = np.array([
    [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
    [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
    [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
    [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1],
], dtype=np.int32)


def corners():
    """12 unit corner vectors, float64 (each component divided by the norm)."""
    c = np.array(_CORNERS_RAW, dtype=np.float64)
    out = np.empty_like(c)
    for i in range(12):
        x, y, z = c[i]
        r = np.sqrt((x * x + y * y) + z * z)
        out[i] = (x / r, y / r, z / r)
    return out


def edges():
    """The 30 edges as sorted (a, b) pairs, a < b, in ascending order."""
    es = set()
    for f in FACES:
        for e in range(3):
            a, b = int(f[e]), int(f[(e + 1) % 3])
            es.add((min(a, b), max(a, b)))
    return np.array(sorted(es), dtype=np.int32)


def face_edge_table():
    """Per face and per side (AB, AC, BC): [edge id, 1 if the side runs from
    the edge's lower corner to its higher one else 0], shape (20, 3, 2)."""
    eid = {tuple(e): i for i, e in enumerate(edges().tolist())}
    tab = np.zeros((20, 3, 2), dtype=np.int32)
    for f, (a, b, c) in enumerate(FACES.tolist()):
        for s, (p, q) in enumerate(((a, b), (a, c), (b, c))):
            tab[f, s, 0] = eid[(min(p, q), max(p, q))]
            tab[f, s, 1] = 1 if p < q else 0
    return tab


def counts(k):
    """(vertices, triangles) for subdivision k."""
    k = int(k)
    return 10 * k * k + 2, 20 * k * k


def interior_per_face(k):
    return (k - 1) * (k - 2) // 2


def check_divisions(k):
    k = int(k)
    if k < 1:
        raise ValueError("divisions must be a positive integer")
    if 10 * k * k + 2 > 2**31 - 1:
        raise ValueError("divisions too large: vertex ids must fit in int32")
    return k
