"""numpy mirror of the GPU icosphere generator (test helper).

Computes the same vertices (same binary64 operation order, no FMA) and the
same triangles as ``nixis_gb300.mesh.create_mesh`` so the GPU output can be
checked bit for bit on small k, and so golden fixtures can be made on a
machine without a GPU.  Layout rules are documented in
``nixis_gb300/icosphere.py``.
"""
import numpy as np

from nixis_gb300 import icosphere as ico


def _norm_rows(p):
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    r = np.sqrt((x * x + y * y) + z * z)
    return np.stack([x / r, y / r, z / r], axis=1)


def icosphere(k, with_tris=True):
    k = ico.check_divisions(k)
    C = ico.corners()
    E = ico.edges()
    FE = ico.face_edge_table()
    nv, nt = ico.counts(k)
    pts = np.empty((nv, 3), np.float64)
    pts[:12] = C
    # edge vertices
    if k > 1:
        t = np.arange(1, k, dtype=np.float64)
        for e, (a, b) in enumerate(E):
            A, B = C[a], C[b]
            p = (k - t)[:, None] * A[None, :] + t[:, None] * B[None, :]
            pts[12 + e * (k - 1): 12 + (e + 1) * (k - 1)] = _norm_rows(p)
    base_int = 12 + 30 * (k - 1)
    npf = ico.interior_per_face(k)
    for f, (a, b, c) in enumerate(ico.FACES):
        if npf == 0:
            break
        ii, jj = [], []
        for i in range(1, k - 1):
            for j in range(1, k - i):
                ii.append(i)
                jj.append(j)
        ii = np.array(ii, np.float64)
        jj = np.array(jj, np.float64)
        w0 = (k - ii - jj)
        A, B, Cc = C[a], C[b], C[c]
        p = (w0[:, None] * A[None, :] + ii[:, None] * B[None, :]) + jj[:, None] * Cc[None, :]
        pts[base_int + f * npf: base_int + (f + 1) * npf] = _norm_rows(p)
    if not with_tris:
        return pts, None

    def vid(f, i, j):
        a, b, c = ico.FACES[f]
        if i == 0 and j == 0:
            return int(a)
        if i == k and j == 0:
            return int(b)
        if i == 0 and j == k:
            return int(c)
        if j == 0:                      # side AB, position i from A
            e, fwd = FE[f, 0]
            t = i if fwd else k - i
            return 12 + int(e) * (k - 1) + t - 1
        if i == 0:                      # side AC, position j from A
            e, fwd = FE[f, 1]
            t = j if fwd else k - j
            return 12 + int(e) * (k - 1) + t - 1
        if i + j == k:                  # side BC, position j from B
            e, fwd = FE[f, 2]
            t = j if fwd else k - j
            return 12 + int(e) * (k - 1) + t - 1
        off = (i - 1) * (k - 1) - (i - 1) * i // 2 + (j - 1)
        return base_int + f * npf + off

    tris = np.empty((nt, 3), np.int32)
    n = 0
    for f in range(20):
        for i in range(k):
            for j in range(k - i):
                tris[n] = (vid(f, i, j), vid(f, i + 1, j), vid(f, i, j + 1))
                n += 1
                if i + j < k - 1:
                    tris[n] = (vid(f, i + 1, j), vid(f, i + 1, j + 1), vid(f, i, j + 1))
                    n += 1
    assert n == nt
    return pts, tris


def edge_lengths(pts, adj):
    """Per-slot neighbour distance, binary64 with erosion.py:38-40's formula,
    split into a binary32 pair (hi, lo): float32 (N, 6, 2); 0 where the slot
    is -1."""
    out = np.zeros(adj.shape + (2,), np.float32)
    valid = adj >= 0
    for k in range(6):
        j = np.where(valid[:, k], adj[:, k], 0)
        d = pts - pts[j]
        dist = np.where(valid[:, k], np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]), 0.0)
        hi = dist.astype(np.float32)
        out[:, k, 0] = hi
        out[:, k, 1] = (dist - hi.astype(np.float64)).astype(np.float32)
    return out


def tied_pixels(pts, ll):
    """Query points among whose 4 nearest vertices two are exactly as far
    (there a KD-tree's choice and order are arbitrary)."""
    q = np.asarray(ll, np.float64).reshape(-1, 3)
    d = np.sqrt(((q[:, None, 0] - pts[None, :, 0]) ** 2 + (q[:, None, 1] - pts[None, :, 1]) ** 2)
                + (q[:, None, 2] - pts[None, :, 2]) ** 2)
    s = np.sort(d, axis=1)[:, :4]
    return (s[:, 1:] == s[:, :-1]).any(axis=1).reshape(np.asarray(ll).shape[:-1])
