"""GPU icosphere, adjacency and edge lengths.

Vertices and triangles are this project's own construction (the reference's
meshzoo is not available: mesh parity is unpinned), checked bit for bit
against the numpy mirror in meshref.py.  The neighbour table is the
reference's build_adjacency + sort_adjacency of those triangles: checked
against the reference's own output (golden) and the oracle.
"""
import numpy as np
import pytest
import torch

import golden_io
import meshref
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", [1, 2, 3, 5, 8, 33])
def test_icosphere_matches_mirror_bit_exact(k):
    from nixis_gb300 import mesh
    xyz, tris = mesh.icosphere(k)
    p, t = meshref.icosphere(k)
    assert np.array_equal(xyz.cpu().numpy().view(np.uint64), p.view(np.uint64))
    assert np.array_equal(tris.cpu().numpy(), t)


@pytest.mark.parametrize("k", [1, 2, 3, 4, 6, 12])
def test_adjacency_matches_reference(k):
    from nixis_gb300 import mesh
    g = golden_io.load("mesh_erosion")
    _, tris = mesh.icosphere(k)
    adj = mesh.build_adjacency(tris)
    mesh.sort_adjacency(adj)
    assert np.array_equal(adj.cpu().numpy(), g[f"adj_k{k}"])


def test_adjacency_and_edges_large_mesh():
    from nixis_gb300 import mesh
    k = 250
    m = mesh.PlanetMesh(k)
    assert m.n == 10 * k * k + 2
    xyz, tris = mesh.icosphere(k)
    t = tris.cpu().numpy()
    adj = O.build_adjacency(t)
    O.sort_adjacency(adj)
    assert np.array_equal(m.nbr.cpu().numpy(), adj)
    p = xyz.cpu().numpy()
    assert np.abs(np.linalg.norm(p, axis=1) - 1).max() < 1e-15
    el = meshref.edge_lengths(p, adj)
    assert np.array_equal(m.edge.cpu().numpy(), el)
    assert (adj[:12, 5] == -1).all() and (adj[12:] >= 0).all()


def test_mesh_of_the_largest_config_builds():
    """divisions=2500: 62,500,002 vertices, neighbour table and edges."""
    from nixis_gb300 import mesh
    m = mesh.PlanetMesh(2500)
    assert m.n == 62_500_002
    nb = m.nbr
    assert int((nb[:12, 5] == -1).sum()) == 12
    assert int((nb[12:] < 0).sum()) == 0
    assert bool(((nb >= -1) & (nb < m.n)).all())
    e = m.edge[12:, :, 0]
    assert float(e.min()) > 0 and float(e.max()) < 1e-3
    # the poles exist for even k
    z = m.xyz[:, 2]
    assert int((z == 1.0).sum()) == 1 and int((z == -1.0).sum()) == 1
