"""Autotuner for the temporally blocked erosion kernel.

Four knobs set how the blocked erosion maps onto the GPU: the tile shape
and size (side x side squares of a face grid, or hexagons of the grid
points within a radius of a centre -- labelled h<radius> and stored as
tile_side = -radius; bigger tiles waste less work on halo rings but need
more shared memory per block, and a hexagon has the fewest halo vertices
for its size), the rings per pass
(iterations done in shared memory between trips to HBM; more rings mean
fewer trips but wider halos), the threads per block, and the kernel
variant: 0 reads the tile tables (neighbour indices, edge lengths) from
global memory every iteration, 1 loads the next vertex's entries ahead of
computing the current one (hides their latency, costs registers and so
resident threads), 2 copies the tile's tables to shared memory once per
pass (no per-iteration global reads, but more shared memory per block), 3
runs one vertex per thread with its table row held in registers for the
pass (small tiles only: every tile's updatable vertices must fit the block),
4 and 5 are variant 0 compiled for more resident blocks per SM (fewer
registers per thread, more warps to hide latency; they pay off only when
the tile's shared memory lets that many blocks reside).  ``tune`` times
every candidate on a synthetic planet, checks that all of them give the
same heights bit for bit (they run the same per-vertex arithmetic), keeps
the fastest and caches it per device in a JSON file
(``$NIXIS_GB300_CACHE`` or ``~/.cache/nixis_gb300/autotune.json``).
``current`` returns the cached choice for the current device, or the
defaults when this device was never tuned.
"""
import ctypes
import json
import os
from dataclasses import asdict, dataclass

import torch

from . import _dev
from ._lib import NxError, call, lib

SMEM_LIMIT = 200 * 1024          # dynamic shared memory of variants 0 and 1
SMEM_LIMIT_TABLES = 226 * 1024   # of variant 2 (the opt-in limit less static shared memory, rounded down)
ROW_SMEM = 40                    # bytes of shared memory per local vertex (two state rows + sediment)
SIDES = (16, 20, 24, 28, 32, 40, 48)
HEX_RADII = (14, 16, 17, 18, 19)   # hexagonal tiles (tile_side = -radius)
RINGS = (2, 3, 4, 5)
THREADS = ((256, 0), (512, 0), (1024, 0), (256, 1), (384, 1), (512, 2), (1024, 2), (512, 3), (1024, 3),
           (256, 4), (320, 4), (384, 4), (640, 4), (256, 5))
# resident blocks per SM that variants 4 and 5 are compiled for, by threads
MIN_BLOCKS = {(256, 4): 5, (320, 4): 4, (384, 4): 3, (640, 4): 2, (256, 5): 6}
SM_SMEM = 228 * 1024             # shared memory per SM
BLOCK_RESERVED = 1024            # shared memory the system reserves per resident block
# variants 2 and 3 measured slower on GB300 for every tile size (variant 2:
# one block per SM cannot overlap its load phase with compute; variant 3:
# tiles small enough for one vertex per thread recompute ~2x the halo):
# tried only on request
DEFAULT_VARIANTS = (0, 1, 4, 5)
SUFFIX = {0: "", 1: "p", 2: "s", 3: "o", 4: "d", 5: "e"}


@dataclass(frozen=True)
class TbConfig:
    tile_side: int = 32
    rings: int = 4
    threads: int = 384
    variant: int = 4

    @property
    def label(self):
        tile = f"h{-self.tile_side}" if self.tile_side < 0 else str(self.tile_side)
        return f"{tile}/{self.rings}/{self.threads}" + SUFFIX[self.variant]


def smem_bytes(cfg, maxnl, maxc):
    """Shared memory of a blocked launch over tiles of up to maxnl local and
    maxc updatable vertices (as the library sizes it)."""
    b = ROW_SMEM * (maxnl + (maxnl & 1))
    if cfg.variant == 2:
        b += 48 * maxc + ((12 * maxc + 15) // 16) * 16
    return b


def fits(cfg, maxnl, maxc):
    """Whether a launch over tiles of up to maxnl local and maxc updatable
    vertices is possible (variants 4 and 5: with the blocks per SM they are
    compiled for resident)."""
    if cfg.variant == 3 and maxc > cfg.threads:
        return False
    b = smem_bytes(cfg, maxnl, maxc)
    if cfg.variant in (4, 5):
        return MIN_BLOCKS[(cfg.threads, cfg.variant)] * (b + BLOCK_RESERVED) <= SM_SMEM
    return b <= (SMEM_LIMIT_TABLES if cfg.variant == 2 else SMEM_LIMIT)


DEFAULT = TbConfig()
_current = {}


def cache_path():
    d = os.environ.get("NIXIS_GB300_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "nixis_gb300")
    return os.path.join(d, "autotune.json")


def device_key(index=None):
    """Device name, SM count and library version: a tuning result is reused
    only on the same kind of GPU with the same kernels."""
    i = torch.cuda.current_device() if index is None else index
    p = torch.cuda.get_device_properties(i)
    return f"{p.name}|sm{p.multi_processor_count}|cc{p.major}.{p.minor}|lib{lib().nx_version()}"


def _load(path):
    try:
        with open(path) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def _save(path, table):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + f".{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def lookup(key, path=None):
    """The cached configuration for a device key, or None."""
    e = _load(path or cache_path()).get(key)
    if not isinstance(e, dict):
        return None
    try:
        return TbConfig(int(e["tile_side"]), int(e["rings"]), int(e["threads"]), int(e.get("variant", 0)))
    except (KeyError, TypeError, ValueError):
        return None


def store(key, cfg, timings=None, path=None):
    path = path or cache_path()
    table = _load(path)
    entry = asdict(cfg)
    if timings is not None:
        entry["timings_ms"] = timings
    table[key] = entry
    _save(path, table)


def parse(label):
    """TbConfig from its label side/rings/threads (side 'h<r>' for
    hexagons of radius r), 'p' appended for variant 1 (prefetch), 's' for
    variant 2 (tables in shared memory), 'o' for variant 3 (one vertex per
    thread), 'd' and 'e' for variants 4 and 5 (more resident blocks per
    SM)."""
    side, rings, thr = label.split("/")
    v = {"p": 1, "s": 2, "o": 3, "d": 4, "e": 5}.get(thr[-1], 0)
    tile = -int(side[1:]) if side.startswith("h") else int(side)
    return TbConfig(tile, int(rings), int(thr.rstrip("psode")), v)


def current():
    """The configuration in use on the current device (tuned, cached or default)."""
    _dev.require_cuda()
    dev = torch.cuda.current_device()
    if dev not in _current:
        _current[dev] = lookup(device_key(dev)) or DEFAULT
    return _current[dev]


def apply(cfg):
    """Make cfg the blocked kernel's setting (process wide)."""
    call("nx_erosion_tb_config", int(cfg.rings), int(cfg.threads), int(cfg.variant), 1)


def use(cfg):
    """Use cfg on the current device from now on (without tuning)."""
    _dev.require_cuda()
    _current[torch.cuda.current_device()] = cfg
    apply(cfg)


def candidates(mesh, variants=DEFAULT_VARIANTS):
    """Every (tile, rings, threads, variant) whose tiles may fit the shared
    memory (checked again against the built tiling's counts): squares of
    SIDES and hexagons of HEX_RADII."""
    out = []
    for side in SIDES + tuple(-r for r in HEX_RADII):
        for rings in RINGS:
            nt, nm, cm = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
            try:
                call("nx_tiling_shape", mesh.k, side, rings, ctypes.byref(nt), ctypes.byref(nm), ctypes.byref(cm))
            except NxError:
                continue                         # more local vertices than a tile may hold
            for threads, v in THREADS:
                if v not in variants:
                    continue
                # capacities nm / cm are about twice the real counts
                if v < 2 and nm.value * ROW_SMEM > 2 * SMEM_LIMIT:
                    continue
                out.append(TbConfig(side, rings, threads, v))
    return out


def tune(divisions=800, iters=24, reps=3, configs=None, save=True, verbose=False):
    """Time the candidates on one synthetic planet (12-octave terrain,
    `iters` erosion iterations; divisions 800 = 6.4 M vertices, ~5,000
    tiles, so that wave quantisation does not decide the choice); returns
    (best config, {config: ms}).  Every candidate must reproduce the first
    one's heights bit for bit."""
    from . import mesh as _mesh
    from . import planets as _planets
    _dev.require_cuda()
    cache = _mesh.MeshCache()
    m = cache.get(divisions)
    req = _planets.PlanetRequest(seed=12345, divisions=divisions, octaves=12, erosion_iters=iters)
    configs = list(configs) if configs is not None else candidates(m)
    timings, ref, best = {}, None, None
    configs.sort(key=lambda c: (c.tile_side, c.rings, c.threads, c.variant))
    for cfg in configs:
        m.drop_tilings(keep=(cfg.tile_side, cfg.rings))   # one tiling resident at a time
        tl = m.tiling(cfg.tile_side, cfg.rings)
        if not fits(cfg, tl.maxnl, tl.maxc):
            continue
        bt = _planets.PlanetBatch([req], cache, tb=cfg)
        bt.launch()
        torch.cuda.synchronize()
        h = bt.heights[:m.n].clone()
        if ref is None:
            ref = h
        elif not torch.equal(h, ref):
            raise RuntimeError(f"autotune: {cfg} changed the results")
        ms = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            bt.launch()
            b.record()
            b.synchronize()
            ms.append(a.elapsed_time(b))
        t = min(ms)
        timings[cfg.label] = round(t, 4)
        if verbose:
            print(f"autotune {cfg}: {t:.3f} ms", flush=True)
        if best is None or t < best[1]:
            best = (cfg, t)
        del bt
    if best is None:
        raise RuntimeError("autotune: no candidate fits")
    cfg = best[0]
    use(cfg)
    if save:
        store(device_key(), cfg, timings)
    return cfg, timings


def ensure_tuned(**kw):
    """The cached configuration for this device, tuning first if there is none."""
    _dev.require_cuda()
    cfg = lookup(device_key())
    if cfg is None:
        cfg, _ = tune(**kw)
    else:
        use(cfg)
    return cfg


__all__ = ["TbConfig", "DEFAULT", "current", "use", "apply", "tune", "ensure_tuned", "candidates", "lookup", "store",
           "device_key", "cache_path", "parse", "fits", "smem_bytes"]
