"""Host-side logic without a GPU: the serving arena, the request stream,
and the benchmark's multi-process (replica) timing reduction under gloo."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def test_row_arena_first_fit_and_merge():
    from nixis_gb300.serve import RowArena
    a = RowArena(256 * 10)
    x = a.alloc(300)          # 2 blocks
    y = a.alloc(256)          # 1 block
    z = a.alloc(1000)         # 4 blocks
    assert (x, y, z) == (0, 512, 768)
    assert a.alloc(1000) is None      # 3 blocks left
    a.release(y, 256)
    assert a.alloc(200) == 512        # reuses the hole
    a.release(512, 200)
    a.release(x, 300)
    a.release(z, 1000)
    assert a.free == [(0, 2560)] and a.used == 0


def test_poisson_stream_matches_its_definition():
    from nixis_gb300.serve import poisson_stream
    s = poisson_stream(2000)
    arr = np.array([a for a, _ in s])
    ks = np.array([r.divisions for _, r in s])
    assert np.all(np.diff(arr) > 0)
    assert 80 < arr[-1] < 120                     # 2000 requests at 20 / s
    assert ks.min() >= 50 and ks.max() <= 2000
    assert abs(np.mean(np.log(ks)) - 0.5 * (np.log(50) + np.log(2000))) < 0.1
    assert all(4 <= r.octaves <= 12 and 0 <= r.erosion_iters <= 100 for _, r in s)
    assert 0.45 < np.mean([r.insolation for _, r in s]) < 0.55
    assert [r.seed for _, r in s] == list(range(2000))


def _free_port():
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    v = bench.max_over_ranks(dist, 10.0 + rank)
    out[rank] = v
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_takes_the_max_over_ranks():
    port = _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    assert all(p.exitcode == 0 for p in ps)
    assert out[0] == out[1] == 11.0


def test_divisions_limits():
    # vertex ids are int32: 10 k^2 + 2 <= 2^31 - 1 holds up to k = 14654
    import pytest
    from nixis_gb300 import icosphere
    assert icosphere.check_divisions(14654) == 14654
    for bad in (0, -1, 14655):
        with pytest.raises(ValueError):
            icosphere.check_divisions(bad)


def test_mesh_eviction_prefers_meshes_no_arrived_request_needs():
    from nixis_gb300.serve import _victim
    lru = [100, 200, 300, 400]                       # least recently used first
    refs = {300: 1}                                  # in use: never evicted
    assert _victim(lru, refs) == 100                 # no queue: least recently used
    assert _victim(lru, refs, [100, 200]) == 400     # not needed by any arrived request
    assert _victim(lru, refs, [400, 100, 200]) == 200    # needed last
    assert _victim(lru, refs, [100, 200, 400]) == 400
    assert _victim([300], refs, [100]) is None
    assert _victim(lru, {}, [999]) == 100            # none needed: least recently used
