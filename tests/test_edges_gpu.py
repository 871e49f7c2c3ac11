"""Edge cases of the drop-in functions, each against the oracle (the
reference restated): empty inputs, zero octaves, non-positive iteration
counts, the smallest meshes."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_empty_inputs_are_no_ops():
    from nixis_gb300 import terrain, erosion, climate
    v = np.zeros((0, 3))
    perm, pgi = O.init(3)
    assert terrain.sample_noise(v, perm, pgi).shape == (0,)
    assert terrain.sample_octaves(v, None, perm, pgi, 5).shape == (0,)
    e = np.zeros(0)
    assert terrain.sample_octaves(v, e, perm, pgi, 5) is e
    nb = np.zeros((0, 6), np.int32)
    h, w, s = np.zeros(0), np.zeros(0), np.zeros(0)
    erosion.erosion_iteration3(v, nb, h, w, s)
    erosion.erode_terrain3(v, nb, h, num_iter=3)
    arr = np.zeros(0, np.float32)
    climate.sample_insolation(arr, v, 1.0, 30.0, 10.0)
    assert climate.brute_daily_insolation(v, None, 1.0, 23.44).shape == (0,)
    assert climate.calc_yearly_insolation(v, None, 1.0, 23.44).shape == (0,)
    with pytest.raises(ValueError):              # the reference's np.min of an empty array
        climate.assign_surface_temp(v, np.zeros(0), 1.0, 23.44)


def test_zero_octaves_and_nonpositive_iterations():
    from nixis_gb300 import terrain, erosion, mesh
    m = mesh.PlanetMesh(6)
    pts, nbr = m.xyz.cpu().numpy(), m.nbr.cpu().numpy()
    perm, pgi = O.init(8)
    got = terrain.sample_octaves(pts, None, perm, pgi, 0)
    assert np.array_equal(got, O.sample_octaves(pts, None, perm, pgi, 0, 1.5, 0.4, 2.0, 0.5, 1.0))
    assert np.array_equal(got, np.zeros(len(pts)))
    h0 = O.rescale(O.sample_octaves(pts, None, perm, pgi, 6, 1.0, 1.0, 2.0, 0.5, 1.0), -8000.0, 8000.0)
    once = h0.copy()
    erosion.erode_terrain3(pts, nbr, once, num_iter=1)
    for n in (0, -3):
        h = h0.copy()
        erosion.erode_terrain3(pts, nbr, h, num_iter=n)       # the reference clamps to one iteration
        assert np.array_equal(h, once), n


def test_smallest_meshes_batched_plain_and_oracle():
    from nixis_gb300 import mesh, planets
    cache = mesh.MeshCache()
    reqs = [planets.PlanetRequest(seed=s, divisions=k, octaves=4, erosion_iters=it)
            for s, (k, it) in enumerate([(1, 7), (2, 5), (3, 12), (1, 0), (4, 9)])]
    b = planets.PlanetBatch(reqs, cache)
    b.run()
    torch.cuda.synchronize()
    for r, got in zip(reqs, b.results()):
        assert got.heights.shape == (r.n_vertices,)
        assert torch.equal(got.heights, planets.generate_plain(r, cache).heights), r
        assert torch.isfinite(got.heights).all()
    # k = 1 (12 vertices, every one a five-neighbour corner) against binary64
    m = cache.get(1)
    pts, nbr = m.xyz.cpu().numpy(), m.nbr.cpu().numpy()
    perm, pgi = O.init(0)
    h = O.rescale(O.sample_octaves(pts, None, perm, pgi, 4, 1.0, 1.0, 2.0, 0.5, 1.0), -8000.0, 8000.0)
    from nixis_gb300 import erosion
    hg = h.copy()
    erosion.erode_terrain3(pts, nbr, hg, num_iter=7)
    O.erode_terrain3(pts, nbr, h, num_iter=7)
    assert np.abs(hg - h).max() <= 1e-10 * np.abs(h).max()
