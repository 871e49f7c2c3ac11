"""GPU erosion (variant 3) against the oracle and the reference's goldens.

* kernel arithmetic (height, water and sediment as binary32 pairs):
  bit-exact against the oracle's restatement, 1 and 50 iterations, with
  and without rain;
* flow choice (sign of h_n - h_i per slot): bit-exact against the binary64
  reference on the same input heights;
* trajectories against the binary64 reference: max|err| / max|field| <=
  ERO_TOL at 1, 10 and 50 iterations (stated tolerance);
* the power-of-two rescale is exact (scaling inputs by 2^100 scales
  outputs by 2^100 bit for bit) and keeps 200 iterations finite and on the
  binary64 trajectory;
* batched planets give the same bits as each planet alone.
"""
import numpy as np
import pytest
import torch

import golden_io
import meshref
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# max|err| / max|field| against binary64: state and edge lengths are
# binary32 pairs (~48 bits); measured ~4e-14 through 100 iterations
ERO_TOL = {1: 1e-10, 10: 1e-10, 30: 1e-10, 50: 1e-10, 100: 1e-10}


def golden_case(k):
    g = golden_io.load("mesh_erosion")
    pts, _ = meshref.icosphere(k, with_tris=False)
    return g, pts, g[f"adj_k{k}"]


def run_gpu(pts, adj, h, w, s, iters, rain=0.0, flow=False, mass=False):
    from nixis_gb300 import erosion
    r = erosion.ErosionRun(pts, adj)
    r.load(torch.from_numpy(np.asarray(h, np.float64)).cuda(), torch.from_numpy(np.asarray(w, np.float64)).cuda(),
           torch.from_numpy(np.asarray(s, np.float64)).cuda())
    m, f = r.steps(iters, rain=rain, flow=flow, mass=mass)
    r.check()
    hd = torch.empty(r.n, dtype=torch.float64, device="cuda")
    wd, sd = torch.empty_like(hd), torch.empty_like(hd)
    r.store(hd, wd, sd)
    return hd.cpu().numpy(), wd.cpu().numpy(), sd.cpu().numpy(), m, f, r


def test_edge_lengths_match_mirror():
    from nixis_gb300 import mesh
    for k in (6, 12):
        g, pts, adj = golden_case(k)
        el, err = mesh.edge_lengths(pts, adj)
        assert int(err.item()) == 0
        assert np.array_equal(el.cpu().numpy(), meshref.edge_lengths(pts, adj))


def flow_codes(adj, h):
    """Per slot: 1 if the neighbour is higher, 2 if lower, 0 if equal or -1
    (the reference's slope > 0 / < 0 / == 0 branches, erosion.py:238-247)."""
    out = np.zeros(len(adj), np.int64)
    for slot in range(6):
        j = adj[:, slot]
        ok = j >= 0
        d = np.where(ok, h[np.where(ok, j, 0)] - h, 0.0)
        code = np.where(~ok, 0, np.where(d > 0, 1, np.where(d < 0, 2, 0)))
        out |= code << (2 * slot)
    return out


@pytest.mark.parametrize("k", [6, 12])
@pytest.mark.parametrize("variant", ["f32", "smooth", "terraced"])
def test_kernel_arithmetic_bit_exact_and_flow_choice(k, variant):
    g, pts, adj = golden_case(k)
    h0 = g[f"ero_k{k}_{variant}_h0"]
    w0 = g[f"ero_k{k}_{variant}_w0"]
    s0 = np.zeros_like(h0)
    el = meshref.edge_lengths(pts, adj)
    st0 = O.pair_rows(h0, w0, s0)
    # one step + flow bits: state rows identical to the oracle's restatement
    _, _, _, _, flow, run = run_gpu(pts, adj, h0, w0, s0, 1, flow=True)
    assert np.array_equal(run.st.cpu().numpy(), O.erosion_iteration3_pair(el, adj, st0))
    # flow choice equals the binary64 reference's slope sign on the same heights
    f = flow.cpu().numpy().astype(np.int64) & 0xFFFF
    assert np.array_equal(f, flow_codes(adj, h0))
    # 50 steps, still bit-exact; and 20 with rain added before each step
    for iters, rain in ((50, 0.0), (20, 0.3 / 320)):
        _, _, _, _, _, run = run_gpu(pts, adj, h0, w0, s0, iters, rain=rain)
        st = st0
        for _ in range(iters):
            st = O.erosion_iteration3_pair(el, adj, st, rain)
        assert np.array_equal(run.st.cpu().numpy(), st), (iters, rain)


def rel_err(got, ref):
    return np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300)


@pytest.mark.parametrize("k", [6, 12])
@pytest.mark.parametrize("variant", ["smooth", "terraced", "f32"])
def test_trajectory_against_binary64_reference(k, variant):
    from nixis_gb300 import erosion
    g, pts, adj = golden_case(k)
    h = g[f"ero_k{k}_{variant}_h0"].copy()
    w = g[f"ero_k{k}_{variant}_w0"].copy()
    s = np.zeros_like(h)
    done = 0
    for it in g[f"ero_k{k}_{variant}_iters"]:
        for _ in range(int(it) - done):
            erosion.erosion_iteration3(pts, adj, h, w, s)      # the drop-in, float64 in place
        done = int(it)
        ref = g[f"ero_k{k}_{variant}_it{it}"]
        for f, (got, want) in enumerate(zip((h, w, s), ref)):
            e = rel_err(got, want)
            assert e <= ERO_TOL[int(it)], (k, variant, int(it), f, e)


@pytest.mark.parametrize("k", [6, 12])
def test_erode_terrain3_against_reference(k):
    from nixis_gb300 import erosion
    g, pts, adj = golden_case(k)
    h0 = g[f"ero_k{k}_smooth_h0"]
    for n_iter in (0, 3):
        h = h0.copy()
        erosion.erode_terrain3(pts, adj, h, n_iter)
        assert rel_err(h, g[f"erode3_k{k}_n{n_iter}"]) <= 1e-6


def test_rescale_is_exact_and_keeps_long_runs_finite():
    g, pts, adj = golden_case(12)
    h0 = g["ero_k12_f32_h0"]
    w0 = g["ero_k12_f32_w0"]
    s0 = np.zeros_like(h0)
    a = run_gpu(pts, adj, h0, w0, s0, 40)
    b = run_gpu(pts, adj, h0 * 2.0 ** 100, w0 * 2.0 ** 100, s0, 40)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x * 2.0 ** 100, y)
    # 200 iterations pass binary32's range (water ~1e55); the scaled state
    # stays finite and on the binary64 reference's trajectory
    hG, wG, sG, mass, _, run = run_gpu(pts, adj, h0, w0, s0, 200, mass=True)
    assert run.scale_exponent() > 0
    assert np.isfinite(hG).all() and np.isfinite(wG).all() and np.isfinite(sG).all()
    h, w, s = h0.copy(), w0.copy(), s0.copy()
    for _ in range(200):
        O.erosion_iteration3(pts, adj, h, w, s)
    assert np.abs(wG).max() > 1e40
    for got, want in ((hG, h), (wG, w), (sG, s)):
        assert rel_err(got, want) <= 1e-9
    # mass sums: sum(h + s) is invariant; the per-iteration sums match the state
    m = mass.cpu().numpy()
    assert np.allclose(m[-1], [hG.sum(), wG.sum(), sG.sum()], rtol=1e-9)
    inv = m[:, 0] + m[:, 2]
    assert np.abs(inv - inv[0]).max() <= 1e-6 * np.abs(m[:, :3]).max()


def test_hundred_iterations_on_noise_terrain_within_tolerance():
    """The single-planet erosion setting at reduced size: 12-octave fBm
    heights rescaled to +-8000 m, water 1e-3, sediment 0, 100 iterations of
    erosion_iteration3, every field against the binary64 oracle, and no
    flow choice differing from binary64's at the end."""
    from nixis_gb300 import mesh
    m = mesh.PlanetMesh(100)
    pts, adj = m.xyz.cpu().numpy(), m.nbr.cpu().numpy()
    perm, pgi = O.init(1)
    h = O.rescale(O.sample_octaves(pts, None, perm, pgi, 12, 1.0, 1.0, 2.0, 0.5, 1.0), -8000.0, 8000.0)
    w = np.full(len(pts), 1e-3)
    s = np.zeros(len(pts))
    out = {}
    hG, wG, sG, _, _, _ = run_gpu(pts, adj, h, w, s, 100)
    for _ in range(100):
        O.erosion_iteration3(pts, adj, h, w, s)
    for name, got, want in (("h", hG, h), ("w", wG, w), ("s", sG, s)):
        out[name] = rel_err(got, want)
        assert out[name] <= ERO_TOL[100], out
    assert np.array_equal(flow_codes(adj, hG), flow_codes(adj, h))


def test_steepest_descent_matches_find_lowest():
    from nixis_gb300 import erosion
    g, pts, adj = golden_case(6)
    h = g["ero_k6_terraced_h0"]
    pos, vid = erosion.steepest_descent(adj, h)
    pos = pos.cpu().numpy()
    assert np.array_equal(pos, g["find_lowest_k6"])
    vid = vid.cpu().numpy()
    for v in range(len(adj)):
        if pos[v] >= 0:
            assert vid[v] == [j for j in adj[v] if j != -1][pos[v]]
        assert erosion.find_lowest(v, adj[v], h) == (None if pos[v] < 0 else pos[v])


def test_batched_planets_equal_planets_alone():
    import ctypes
    from nixis_gb300 import _lib, _dev
    planets = []
    for k, seed, iters in ((12, 1, 37), (6, 2, 50), (9, 3, 0), (4, 4, 11), (7, 5, 36)):
        p, t = meshref.icosphere(k)
        adj = O.build_adjacency(t)
        O.sort_adjacency(adj)
        perm, pgi = O.init(seed)
        h = O.rescale(O.sample_octaves(p, None, perm, pgi, 5, 1.0, 1.0, 2.0, 0.5, 1.0), -8000, 8000)
        h = h.astype(np.float32).astype(np.float64)
        planets.append((p, adj, h, iters))
    planets.sort(key=lambda x: -x[3])
    # pack the states: each planet's rows start at a multiple of 256; its
    # neighbour ids stay local and its mesh arrays stay separate
    off, descs, meshes, hs = 0, [], [], []
    for p, adj, h, iters in planets:
        n = len(p)
        descs.append((off, n, iters))
        meshes.append((torch.from_numpy(adj).cuda(), torch.from_numpy(meshref.edge_lengths(p, adj)).cuda()))
        hs.append(np.concatenate([h, np.zeros((-n) % 256)]))
        off += n + (-n) % 256
    N = off
    hall = np.concatenate(hs).astype(np.float32)
    st = torch.zeros((N, 8), dtype=torch.float32, device="cuda")
    st_t = torch.zeros_like(st)
    for (b, n, iters) in descs:
        dst = st_t if iters & 1 else st
        dst[b:b + n, 0] = torch.from_numpy(hall[b:b + n]).cuda()
        dst[b:b + n, 2] = 1e-3
    arr = (_lib.ErosionPlanet * len(descs))(*[
        _lib.ErosionPlanet(b, n, nb.data_ptr(), el.data_ptr(), it, 0.0, 0, q)
        for q, ((b, n, it), (nb, el)) in enumerate(zip(descs, meshes))])
    pd = torch.from_numpy(np.frombuffer(bytes(arr), np.uint8).copy()).cuda()
    ws = torch.zeros(int(_lib.lib().nx_erosion_workspace_size(N, len(descs))), dtype=torch.uint8, device="cuda")
    _lib.call("nx_erosion_ctl_init", _dev.ptr(ws), ws.numel(), len(descs), _dev.stream_handle())
    _lib.call("nx_erosion_batch", _dev.ptr(pd), ctypes.cast(arr, ctypes.c_void_p), len(descs),
              _dev.ptr(st), _dev.ptr(st_t), None, _dev.ptr(ws), ws.numel(), _dev.stream_handle())
    out = st.cpu().numpy()
    for (p, adj, h, iters), (b, n, _) in zip(planets, descs):
        _, _, _, _, _, run = run_gpu(p, adj, h, np.full(len(p), np.float32(1e-3)), np.zeros(len(p)), iters)
        assert np.array_equal(out[b:b + n], run.st.cpu().numpy())


def test_bad_neighbour_id_is_reported_not_faulted():
    from nixis_gb300 import erosion
    g, pts, adj = golden_case(6)
    bad = adj.copy()
    bad[20, 3] = len(pts) + 5
    with pytest.raises(IndexError):
        erosion.erosion_iteration3(pts, bad, g["ero_k6_smooth_h0"].copy(), np.full(len(pts), 1e-3), np.zeros(len(pts)))


@pytest.mark.parametrize("tile", [40, -19, -5])
def test_tiling_covers_every_vertex_once_with_valid_rings(tile):
    """Squares of side 40 and hexagons of radius 19 and 5 (many tiles on
    face edges and around the five-neighbour corners)."""
    from nixis_gb300 import mesh
    for k in (1, 3, 17, 100):
        m = mesh.PlanetMesh(k)
        t = m.tiling(tile)
        R = t.rings
        cnt = t.counts.view(t.ntiles, R + 1).cpu().numpy()
        ids = t.ids.view(t.ntiles, t.nmax).cpu().numpy()
        members = np.concatenate([ids[i, :cnt[i, 0]] for i in range(t.ntiles)])
        assert np.array_equal(np.sort(members), np.arange(m.n))
        nbr = m.nbr.cpu().numpy()
        for i in range(0, t.ntiles, max(1, t.ntiles // 7)):
            T = cnt[i, 0]
            loc = ids[i, :cnt[i].sum()]
            assert len(set(loc.tolist())) == len(loc)
            # ring r = vertices at graph distance r from the members
            seen = set(loc[:T].tolist())
            front = set(seen)
            off = T
            for r in range(1, R + 1):
                nxt = {int(j) for v in front for j in nbr[v] if j >= 0} - seen
                assert nxt == set(loc[off:off + cnt[i, r]].tolist()), (k, i, r)
                seen |= nxt
                front = nxt
                off += cnt[i, r]


@pytest.mark.parametrize("rain", [0.0, 0.3 / 320])
def test_temporally_blocked_batch_equals_iteration_at_a_time(rain):
    from nixis_gb300 import mesh, planets, _lib
    from nixis_gb300.planets import PlanetRequest
    reqs = [PlanetRequest(seed=s, divisions=k, octaves=6, erosion_iters=it, rain=rain)
            for s, (k, it) in enumerate([(3, 9), (40, 33), (57, 1), (100, 20), (23, 7), (90, 2), (64, 0), (12, 4)])]
    cache = mesh.MeshCache()
    a = planets.PlanetBatch(reqs, cache, blocked=True)
    a.run()
    b = planets.PlanetBatch(reqs, cache, blocked=False)
    b.run()
    torch.cuda.synchronize()
    for r, x, y in zip(reqs, a.results(), b.results()):
        assert torch.equal(x.heights, y.heights), r
    # and the plain single-planet path
    for r, x in zip(reqs, a.results()):
        assert torch.equal(x.heights, planets.generate_plain(r, cache).heights), r


@pytest.mark.parametrize("rain,tile", [(0.0, None), (0.3 / 320, None), (0.3 / 320, -19), (0.0, -6)])
def test_larger_meshes_blocked_equal_iteration_at_a_time(rain, tile):
    """Meshes of divisions 160-339 (many tiles per face, tiles away from
    every face edge), pass counts with a short last pass and both parities:
    blocked == one launch per iteration, bit for bit, no error flags; with
    the default tiles and with hexagons of radius 19 and 6."""
    from dataclasses import replace
    from nixis_gb300 import autotune, mesh, planets
    from nixis_gb300.planets import PlanetRequest
    tb = autotune.DEFAULT if tile is None else replace(autotune.DEFAULT, tile_side=tile)
    reqs = [PlanetRequest(seed=s, divisions=k, octaves=7, erosion_iters=it, rain=rain)
            for s, (k, it) in enumerate([(200, 9), (250, 14), (339, 33), (160, 6), (300, 1)])]
    cache = mesh.MeshCache()
    a = planets.PlanetBatch(reqs, cache, blocked=True, tb=tb)
    a.run()
    b = planets.PlanetBatch(reqs, cache, blocked=False)
    b.run()
    torch.cuda.synchronize()
    for r, x, y in zip(reqs, a.results(), b.results()):
        assert torch.equal(x.heights, y.heights), r
    ctl = a.ws[:32 * len(reqs)].view(torch.int32).view(-1, 8)
    assert int(ctl[:, 6].abs().sum().item()) == 0


def test_temporally_blocked_long_run_rescales_like_iteration_at_a_time():
    """170 and 150 iterations: both paths rescale (at different iterations:
    per pass vs per iteration) and hold the same true values."""
    from nixis_gb300 import mesh, planets
    from nixis_gb300.planets import PlanetRequest
    reqs = [PlanetRequest(seed=1, divisions=30, octaves=5, erosion_iters=170),
            PlanetRequest(seed=2, divisions=7, octaves=5, erosion_iters=150)]
    cache = mesh.MeshCache()
    out = []
    for blocked in (True, False):
        bt = planets.PlanetBatch(reqs, cache, blocked=blocked)
        bt.run()
        torch.cuda.synchronize()
        st = bt.st.double()
        vals = []
        for i, res in enumerate(bt.results()):
            assert res.scale_exponent > 0
            b, n = bt.vbeg[i], reqs[i].n_vertices
            x = st[b:b + n]
            true = torch.stack([x[:, 0] + x[:, 1], x[:, 2] + x[:, 3], x[:, 4] + x[:, 5]]) * 2.0 ** res.scale_exponent
            assert torch.isfinite(true).all()
            vals.append(true)
        out.append(vals)
    for x, y in zip(*out):
        assert torch.equal(x, y)


def test_tiling_with_fewer_rings_than_a_pass_is_reported_not_run():
    """A batch configured for 5-iteration passes over tilings built with 4
    rings: the kernel flags err = 2 in the planet's control block and leaves
    the state alone (no out-of-range reads), and the library is usable
    afterwards."""
    from nixis_gb300 import autotune, mesh, planets
    from nixis_gb300.planets import PlanetRequest
    cache = mesh.MeshCache()
    req = PlanetRequest(seed=2, divisions=40, octaves=5, erosion_iters=10)
    bt = planets.PlanetBatch([req], cache, tb=autotune.TbConfig(40, 4, 512, 0))
    bt.tb = autotune.TbConfig(40, 5, 512, 0)       # passes of 5 over 4-ring tiles
    bt.launch()
    torch.cuda.synchronize()
    ctl = bt.ws[:32].view(torch.int32)
    assert int(ctl[6].item()) == 2
    autotune.use(autotune.DEFAULT)
    ok = planets.PlanetBatch([req], cache)
    ok.run()
    torch.cuda.synchronize()
    assert torch.equal(ok.results()[0].heights, planets.generate_plain(req, cache).heights)


def test_steps_without_mass_sums_equal_steps_with_them():
    """nx_erosion_steps with mass_dev = flow_dev = NULL (the plain path's
    call) runs the same arithmetic as with mass sums: same bits, odd and
    even iteration counts."""
    import ctypes
    from nixis_gb300 import _dev, _lib, mesh
    m = mesh.PlanetMesh(60)
    pts = m.xyz.cpu().numpy()
    perm, pgi = O.init(4)
    h = O.rescale(O.sample_octaves(pts, None, perm, pgi, 8, 1.0, 1.0, 2.0, 0.5, 1.0), -8000.0, 8000.0)
    st0 = torch.from_numpy(O.pair_rows(h, np.full(len(pts), 1e-3), np.zeros(len(pts)))).cuda()
    n = m.n
    for iters in (11, 6):
        outs = []
        for with_mass in (True, False):
            st = st0.clone()
            tmp = torch.empty_like(st)
            ws = torch.zeros(int(_lib.lib().nx_erosion_workspace_size(n, 1)), dtype=torch.uint8, device="cuda")
            pd = torch.full((ctypes.sizeof(_lib.ErosionPlanet),), 0xA5, dtype=torch.uint8, device="cuda")
            mass = torch.empty((iters, 3), dtype=torch.float64, device="cuda") if with_mass else None
            _lib.call("nx_erosion_ctl_init", _dev.ptr(ws), ws.numel(), 1, _dev.stream_handle())
            _lib.call("nx_erosion_steps", _dev.ptr(m.nbr), _dev.ptr(m.edge), n, _dev.ptr(st), _dev.ptr(tmp), iters,
                      ctypes.c_float(0.0), _dev.ptr(pd), _dev.ptr(mass) if with_mass else None, None, _dev.ptr(ws),
                      ws.numel(), _dev.stream_handle())
            torch.cuda.synchronize()
            assert int(ws[:32].view(torch.int32)[6].item()) == 0       # no error flag
            outs.append(st)
        assert torch.equal(outs[0], outs[1])
