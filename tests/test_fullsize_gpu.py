"""The single-planet configurations at their full sizes.

C2: divisions 1000 (10,000,002 vertices), 12 octaves, seed 1, then 50
erosion iterations from water 1e-3 and sediment 0: fBm against the binary64
oracle on every vertex, erosion state against the oracle's binary64
iterations on the whole mesh (the oracle is the C restatement, OpenMP).

C3: divisions 2500 (62,500,002 vertices), 12 octaves, seed 2, 200 erosion
iterations and a year of hourly insolation: properties that do not depend on
a CPU run of the whole planet -- fBm and insolation on a random vertex sample
against the oracle, the blocked erosion equal bit for bit to the
iteration-at-a-time kernel, and sum(h + s) conserved through the run.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FBM_TOL = 1e-5        # max |error| / range of the fBm field
ERO_TOL = 1e-10       # max |error| / max |field| of h, w, s after the run
INSO_TOL = 1e-5       # max |error| / max of the annual sum


def _fbm(m, seed, octs):
    from nixis_gb300 import terrain
    perm, pgi = O.init(seed)
    sc, st = terrain._octave_args(octs, 1.0, 1.0, 2.0, 0.5, 1.0)
    out = torch.empty(m.n, dtype=torch.float64, device="cuda")
    terrain.fbm(m.xyz, perm, pgi, sc, st, 1.0, out=out)
    return out, perm, pgi


def test_c2_full_size_against_binary64():
    from nixis_gb300 import mesh, erosion
    m = mesh.PlanetMesh(1000)
    assert m.n == 10_000_002
    h, perm, pgi = _fbm(m, 1, 12)
    pts, nbr = m.xyz.cpu().numpy(), m.nbr.cpu().numpy()
    ref = O.sample_octaves(pts, None, perm, pgi, 12, 1.0, 1.0, 2.0, 0.5, 1.0)
    hg = h.cpu().numpy()
    assert np.abs(hg - ref).max() <= FBM_TOL * (ref.max() - ref.min())
    # erosion from the oracle's elevations, so both runs start from the same bits
    hm = O.rescale(ref, -8000.0, 8000.0)
    run = erosion.ErosionRun(m.xyz, m.nbr, m.edge)
    run.load(torch.from_numpy(hm).cuda(), torch.full((m.n,), 1e-3, dtype=torch.float64, device="cuda"))
    run.steps(50)
    hd = torch.empty(m.n, dtype=torch.float64, device="cuda")
    wd, sd = torch.empty_like(hd), torch.empty_like(hd)
    run.store(hd, wd, sd)
    hw, ww, sw = hm.copy(), np.full(m.n, 1e-3), np.zeros(m.n)
    for _ in range(50):
        O.erosion_iteration3(pts, nbr, hw, ww, sw)
    g = [hd.cpu().numpy(), wd.cpu().numpy(), sd.cpu().numpy()]
    for f, a, b in zip("hws", g, (hw, ww, sw)):
        assert np.abs(a - b).max() <= ERO_TOL * np.abs(b).max(), f
    # every flow choice (sign of h_n - h_i per neighbour slot) as in binary64
    jj = np.where(nbr < 0, np.arange(m.n)[:, None], nbr)
    assert int((np.sign(g[0][jj] - g[0][:, None]) != np.sign(hw[jj] - hw[:, None])).sum()) == 0


def test_c3_full_size_properties():
    from nixis_gb300 import mesh, erosion, climate, planets
    m = mesh.PlanetMesh(2500)
    assert m.n == 62_500_002
    h, perm, pgi = _fbm(m, 2, 12)
    rng = np.random.default_rng(3)
    idx = np.sort(rng.choice(m.n, 200_000, replace=False))
    pts = m.xyz[torch.from_numpy(idx).cuda()].cpu().numpy()
    ref = O.sample_octaves(pts, None, perm, pgi, 12, 1.0, 1.0, 2.0, 0.5, 1.0)
    hg = h.cpu().numpy()
    # the range of the whole field (the sample's own range is smaller)
    assert np.abs(hg[idx] - ref).max() <= FBM_TOL * (hg.max() - hg.min())
    del h
    # 200 iterations: blocked passes and one launch per iteration agree bit for bit
    req = planets.PlanetRequest(seed=2, divisions=2500, octaves=12, erosion_iters=200)
    cache = mesh.MeshCache()
    cache._m[2500] = m
    cache._order.append(2500)
    out = []
    for blocked in (True, False):
        bt = planets.PlanetBatch([req], cache, blocked=blocked)
        bt.run()
        torch.cuda.synchronize()
        res = bt.results()[0]
        out.append(res.heights.clone())
        K = res.scale_exponent
        del bt, res
    assert torch.equal(out[0], out[1])
    # binary64 metres through the planet API: finite, although the run
    # passes binary32's range (the state carries a power-of-two exponent),
    # and equal to the plain path's heights, which come from the erosion
    # state's binary64 store (nx_erosion_store, as ErosionRun.store)
    assert K > 0 and out[0].dtype == torch.float64 and torch.isfinite(out[0]).all()
    assert float(out[0].abs().max()) > 3.4e38
    plain = planets.generate_plain(req, cache)
    assert torch.equal(plain.heights, out[0])
    del out, plain
    # sum(h + s) is invariant under the update (compensated per-iteration sums)
    hm = torch.from_numpy(O.rescale(hg, -8000.0, 8000.0)).cuda()
    run = erosion.ErosionRun(m.xyz, m.nbr, m.edge)
    run.load(hm, torch.full((m.n,), 1e-3, dtype=torch.float64, device="cuda"))
    mass, _ = run.steps(200, mass=True)
    ms = mass.cpu().numpy()
    inv0, inv1 = ms[0, 0] + ms[0, 2], ms[-1, 0] + ms[-1, 2]
    assert abs(inv1 - inv0) <= 1e-12 * max(abs(ms[-1, 0]), abs(ms[-1, 2]), abs(inv0))
    hd = torch.empty(m.n, dtype=torch.float64, device="cuda")
    wd, sd = torch.empty_like(hd), torch.empty_like(hd)
    run.store(hd, wd, sd)
    assert torch.isfinite(hd).all() and torch.isfinite(wd).all() and torch.isfinite(sd).all()
    del run, hd, wd, sd
    # a year of hourly insolation on a vertex sample
    got = climate.annual_insolation(m.xyz, 1.0).cpu().numpy()[idx[:20_000]]
    want = O.annual_insolation(pts[:20_000], 1.0)
    assert np.abs(got - want).max() <= INSO_TOL * np.abs(want).max()
