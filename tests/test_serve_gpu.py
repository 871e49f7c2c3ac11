"""Continuous-batching server: every planet's result equals the planet
generated alone (plain per-planet path), bit for bit, including under a
memory budget that forces admission to wait for earlier planets."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def small_stream(n=14, seed=5):
    from nixis_gb300.planets import PlanetRequest
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    for i in range(n):
        t += float(rng.exponential(0.01))
        out.append((t, PlanetRequest(seed=100 + i, divisions=int(rng.integers(10, 70)),
                                     octaves=int(rng.integers(4, 13)), erosion_iters=int(rng.integers(0, 25)),
                                     insolation=bool(rng.random() < 0.5), days=10)))
    return out


def check_against_alone(tickets):
    from nixis_gb300 import planets, serve
    meshes = serve.ResidentMeshes(8 * 2**30)
    for t in tickets:
        assert t.finished is not None and t.latency > 0
        alone = planets.generate_plain(t.request, meshes)
        assert np.array_equal(t.heights, alone.heights.cpu().numpy()), t.request
        if t.request.insolation:
            assert np.array_equal(t.insolation, alone.insolation.cpu().numpy()), t.request
        else:
            assert t.insolation is None


@pytest.mark.parametrize("blocked", [True, False])
def test_served_results_equal_alone(blocked):
    """Ticks of blocked passes (default) or of single iterations."""
    from nixis_gb300 import serve
    with serve.ServeEngine(hbm_budget=4 * 2**30, arena_rows=2_000_000, slots=64, blocked=blocked) as eng:
        eng.warmup()
        assert eng.done == [] and eng.arena.used == 0
        tickets = eng.run(small_stream())
    assert eng.tick > 0
    check_against_alone(tickets)
    # the arena and slots are all returned
    assert eng.arena.used == 0 and len(eng.free_slots) == 64


def test_result_sinks_see_every_result_once():
    """result_sink (engine) and sink (plain path) receive each finished
    request's arrays -- here reduced to byte strings and dropped, as a long
    stream's caller does -- and both paths' reductions agree."""
    from nixis_gb300 import serve
    stream = small_stream(8, seed=13)
    seen = {}

    def sink(t):
        assert t.index not in seen
        seen[t.index] = (t.heights.tobytes(), None if t.insolation is None else t.insolation.tobytes())
        t.heights = t.insolation = None

    with serve.ServeEngine(hbm_budget=4 * 2**30, arena_rows=2_000_000, slots=64, result_sink=sink) as eng:
        tickets = eng.run(stream, realtime=False)
    assert sorted(seen) == list(range(len(stream)))
    assert all(t.heights is None for t in tickets)
    plain = serve.serve_plain(stream, realtime=False,
                              sink=lambda h, i: (h.numpy().tobytes(), None if i is None else i.numpy().tobytes()))
    for t, (_, _, red) in zip(tickets, plain):
        assert seen[t.index] == red, t.request


def test_admission_waits_for_memory_and_still_matches():
    from nixis_gb300 import serve
    stream = small_stream(10, seed=9)
    biggest = max(r.n_vertices for _, r in stream)
    # room for about two planets at a time: later arrivals wait for rows
    # a result arena of 1 MB: most results fall back to torch's page-locked allocator
    eng = serve.ServeEngine(hbm_budget=4 * 2**30, arena_rows=2 * biggest + 1024, slots=8, host_bytes=1 << 20)
    tickets = eng.run(stream, realtime=False)
    check_against_alone(tickets)
    waited = [t for t in tickets if t.admitted - t.arrival > 1e-4]
    assert waited, "expected some requests to wait for memory"


def test_pinned_arena_hands_out_and_takes_back_ranges():
    from nixis_gb300 import serve
    a = serve.PinnedArena(8 << 20)                 # 8 MB in 1 MB units
    b1, t1 = a.alloc(1 << 20, torch.float32)       # 4 MB
    b2, t2 = a.alloc(1 << 19, torch.float64)       # 4 MB
    assert b1.is_pinned() and b1.dtype == torch.float32 and b1.numel() == 1 << 20
    assert b2.dtype == torch.float64 and b2.numel() == 1 << 19
    assert b2.data_ptr() == b1.data_ptr() + (4 << 20)
    assert a.alloc(10, torch.float32) is None      # full
    a.release(t1)
    b3, t3 = a.alloc(100, torch.float32)
    assert b3.data_ptr() == b1.data_ptr()
    a.release(t2)
    a.release(t3)
    assert a.pages.used == 0


def test_small_and_large_planets_set_up_on_their_own_streams():
    """Planets under serve.SMALL_ROWS vertices build their meshes and run
    their noise on the higher-priority pair of streams, larger ones on the
    other; arriving interleaved (a small planet right behind a large one
    whose mesh is still being built), every result still equals the planet
    generated alone."""
    from nixis_gb300 import serve
    from nixis_gb300.planets import PlanetRequest
    ks = [470, 24, 510, 36, 16, 480, 52]
    stream = [(0.002 * i, PlanetRequest(seed=300 + i, divisions=k, octaves=6, erosion_iters=5 + 3 * i,
                                         insolation=i % 2 == 0, days=5))
              for i, k in enumerate(ks)]
    sizes = [r.n_vertices for _, r in stream]
    assert min(sizes) < serve.SMALL_ROWS <= max(sizes)
    with serve.ServeEngine(hbm_budget=16 * 2**30, arena_rows=12_000_000, slots=16) as eng:
        eng.warmup()
        tickets = eng.run(stream)
    check_against_alone(tickets)
