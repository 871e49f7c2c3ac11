"""The blocked-erosion autotuner: its per-device cache (CPU) and a small
tuning run whose candidates must all give the same heights (GPU)."""
import json

import pytest
import torch


def test_cache_round_trip_and_bad_entries(tmp_path):
    from nixis_gb300 import autotune as A
    p = str(tmp_path / "t.json")
    assert A.lookup("gpuX", p) is None
    A.store("gpuX", A.TbConfig(48, 3, 256, 0), {"48/3/256": 1.5}, path=p)
    A.store("gpuY", A.TbConfig(32, 5, 384, 1), path=p)
    assert A.lookup("gpuX", p) == A.TbConfig(48, 3, 256, 0)
    assert A.lookup("gpuY", p) == A.TbConfig(32, 5, 384, 1)
    assert A.parse("32/5/384p") == A.TbConfig(32, 5, 384, 1) and A.parse("32/4/384d") == A.DEFAULT
    assert A.parse("24/4/512s") == A.TbConfig(24, 4, 512, 2) and A.parse("16/3/1024o") == A.TbConfig(16, 3, 1024, 3)
    assert A.parse(A.TbConfig(48, 2, 1024, 0).label) == A.TbConfig(48, 2, 1024, 0)
    assert A.parse("24/4/256d") == A.TbConfig(24, 4, 256, 4) and A.parse("20/5/256e") == A.TbConfig(20, 5, 256, 5)
    assert A.parse("h19/4/384d") == A.TbConfig(-19, 4, 384, 4) and A.TbConfig(-19, 4, 384, 4).label == "h19/4/384d"
    assert A.parse(A.TbConfig(24, 3, 384, 4).label) == A.TbConfig(24, 3, 384, 4)
    # variants 4 / 5 fit only where their blocks per SM can reside
    assert A.fits(A.TbConfig(24, 4, 256, 4), 1024, 900) and not A.fits(A.TbConfig(40, 4, 256, 4), 2304, 2116)
    assert A.fits(A.TbConfig(20, 4, 256, 5), 784, 676) and not A.fits(A.TbConfig(24, 4, 256, 5), 1024, 900)
    with open(p) as f:
        assert json.load(f)["gpuX"]["timings_ms"] == {"48/3/256": 1.5}
    with open(p, "w") as f:
        f.write("{not json")
    assert A.lookup("gpuX", p) is None
    with open(p, "w") as f:
        json.dump({"gpuX": {"tile_side": "a"}}, f)
    assert A.lookup("gpuX", p) is None


@pytest.mark.gpu
def test_tuning_keeps_results_and_applies_the_choice():
    from nixis_gb300 import autotune as A, mesh, planets
    cands = [A.TbConfig(32, 2, 256, 0), A.TbConfig(40, 4, 512, 0), A.TbConfig(48, 3, 1024, 0), A.TbConfig(40, 4, 384, 1),
             A.TbConfig(24, 4, 512, 2), A.TbConfig(32, 3, 1024, 2), A.TbConfig(16, 4, 1024, 3),
             A.TbConfig(12, 3, 512, 3), A.TbConfig(20, 4, 256, 4), A.TbConfig(16, 3, 384, 4),
             A.TbConfig(16, 4, 256, 5), A.TbConfig(24, 3, 640, 4), A.TbConfig(20, 3, 320, 4)]
    cfg, timings = A.tune(divisions=60, iters=9, reps=1, configs=cands, save=False)
    assert cfg in cands and len(timings) == len(cands)
    assert A.current() == cfg
    # any setting gives the bits of the plain iteration-at-a-time path
    cache = mesh.MeshCache()
    req = planets.PlanetRequest(seed=4, divisions=70, octaves=7, erosion_iters=13)
    plain = planets.generate_plain(req, cache).heights
    for c in cands:
        bt = planets.PlanetBatch([req], cache, tb=c)
        bt.run()
        torch.cuda.synchronize()
        assert torch.equal(bt.results()[0].heights, plain), c
    A.use(A.DEFAULT)


def test_candidates_cover_the_default_and_fit_the_limits():
    # nx_tiling_shape is host-only: candidates need only the mesh's divisions
    from types import SimpleNamespace
    from nixis_gb300 import autotune as A
    c = A.candidates(SimpleNamespace(k=800))
    assert A.DEFAULT in c
    assert {cfg.variant for cfg in c} == set(A.DEFAULT_VARIANTS)
    for cfg in c:
        assert (cfg.tile_side in A.SIDES or -cfg.tile_side in A.HEX_RADII) and cfg.rings in A.RINGS
        assert (cfg.threads, cfg.variant) in A.THREADS
    # variants 4 and 5 only where their resident blocks' shared memory fits
    assert not A.fits(A.TbConfig(48, 4, 256, 5), (48 + 8) ** 2, (48 + 6) ** 2)
    assert A.fits(A.DEFAULT, (32 + 8) ** 2, (32 + 6) ** 2)
