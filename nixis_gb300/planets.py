"""Whole-planet generation: fBm elevations -> metres -> erosion -> insolation.

Two execution paths over the same kernels:

* ``PlanetBatch`` -- many planets of uneven size in a handful of launches:
  one persistent fBm launch over all planets (with fused per-planet
  min/max), one launch for the rescale to metres and the initial erosion
  state, one erosion launch per pass (or iteration) over the planets still
  running, one height-extraction launch and one insolation launch per sun
  schedule.  The whole sequence can be captured once as a CUDA graph and
  replayed.
* ``generate_plain`` -- the plain per-planet GPU path: one planet at a time,
  one launch per octave and per erosion iteration, synchronised per planet.

The fBm runs in pair precision (nx_fbm_pair), the rescale to metres and
the erosion state in binary32 pairs, and heights come back in binary64:
erosion follows binary64's flow choices only from starting heights that
close to the reference's.  A planet is fully determined by its request
(seed, divisions, octaves, iterations, ...), so results are reproducible
and a planet gives the same bits alone or in any batch.
"""
import ctypes
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _dev
from . import autotune as _autotune
from . import climate as _climate
from . import mesh as _mesh
from . import opensimplex as _osx
from ._lib import ErosionPlanet, FbmPlanet, InsoPlanet, call, lib

ALIGN = 256


@dataclass(frozen=True)
class PlanetRequest:
    seed: int
    divisions: int
    octaves: int
    erosion_iters: int = 0
    insolation: bool = False
    init_roughness: float = 1.0     # base frequency
    init_strength: float = 1.0
    roughness: float = 2.0          # lacunarity
    persistence: float = 0.5
    radius: float = 1.0
    elev_lo: float = -8000.0        # util.rescale bounds (metres)
    elev_hi: float = 8000.0
    water0: float = 1e-3            # initial water (m), sediment 0
    rain: float = 0.0               # per-iteration rain (erode_terrain3 uses 0.3/320)
    axial_tilt: float = 23.44
    days: int = 365
    hours: int = 24

    @property
    def n_vertices(self):
        return 10 * self.divisions * self.divisions + 2

    def octave_args(self):
        scale, strength = [], []
        f, a = self.init_roughness, self.init_strength
        for _ in range(self.octaves):
            scale.append(f / self.radius)
            strength.append(a / self.radius)
            f *= self.roughness
            a *= self.persistence
        return scale, strength

    def schedule_key(self):
        return (self.axial_tilt, self.days, self.hours)

    def state_bytes(self):
        """Device bytes a planet needs beyond its mesh (batched path): raw
        pair sums, two state rows, binary64 heights, insolation."""
        n = self.n_vertices + ALIGN
        return n * (8 + 32 + 32 + 8 + (4 if self.insolation else 0))


def _tiling_shape(divisions, tb):
    nt, nm, cm = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    call("nx_tiling_shape", int(divisions), tb.tile_side, tb.rings, ctypes.byref(nt), ctypes.byref(nm),
         ctypes.byref(cm))
    return nt.value, nm.value, cm.value


def tile_count(divisions, tb):
    """Tiles of the temporally blocked erosion's tiling of a mesh."""
    return _tiling_shape(divisions, tb)[0]


def mesh_bytes(divisions, tb=None):
    """HBM of a resident mesh: vertices, neighbours, edge lengths and (with
    a blocked-erosion setting tb) the tiling for it."""
    n = 10 * divisions * divisions + 2
    b = n * (24 + 24 + 48)
    if tb is not None:
        nt, nm, cm = _tiling_shape(divisions, tb)
        b += nt * ((tb.rings + 1) * 4 + nm * 4 + cm * 6 * (2 + 8))
    return b


@dataclass
class PlanetResult:
    request: PlanetRequest
    heights: torch.Tensor               # float64 (N,), metres (finite for every iteration count; the
                                        # reference's erosion grows heights without bound)
    insolation: torch.Tensor = None     # float32 (N,), mean TOA W/m^2 over the schedule
    scale_exponent: int = 0


def _struct_tensor(arr):
    raw = np.frombuffer(bytes(arr), np.uint8).copy()
    return torch.from_numpy(raw).cuda()


class PlanetBatch:
    """A fixed set of planets, packed for batched execution."""

    def __init__(self, requests, meshes=None, stream=None, blocked=True, tb=None):
        _dev.require_cuda()
        if not requests:
            raise ValueError("empty batch")
        for r in requests:
            if not (0 <= r.octaves <= 32):
                raise ValueError("octaves must be in [0, 32]")
            if r.erosion_iters < 0:
                raise ValueError("erosion_iters must be >= 0")
        self.requests = list(requests)
        self.meshes = meshes if meshes is not None else _mesh.MeshCache()
        self.stream = stream
        self.blocked = blocked
        # blocked erosion setting (tile side, rings, threads): autotuned or given
        self.tb = (tb or _autotune.current()) if blocked else None
        np_ = len(requests)
        # pack in order of descending iteration count (stable)
        self.order = sorted(range(np_), key=lambda i: -requests[i].erosion_iters)
        self.vbeg = [0] * np_
        off = 0
        for i in self.order:
            self.vbeg[i] = off
            off += requests[i].n_vertices
            off = (off + ALIGN - 1) // ALIGN * ALIGN
        self.total = off
        N = off
        dev = "cuda"
        self.raw = torch.empty((N, 2), dtype=torch.float32, device=dev)     # (hi, lo) pair sums
        self.st = torch.empty((N, 8), dtype=torch.float32, device=dev)
        self.st_tmp = torch.empty((N, 8), dtype=torch.float32, device=dev)
        self.heights = torch.empty(N, dtype=torch.float64, device=dev)
        self.any_inso = any(r.insolation for r in requests)
        self.inso = torch.empty(N, dtype=torch.float32, device=dev) if self.any_inso else None
        # per-planet tables (host init, bit-exact) and min/max keys
        tabs = np.zeros((np_, 2, 256), np.int32)
        for j, i in enumerate(self.order):
            tabs[j, 0], tabs[j, 1] = _osx.init(requests[i].seed)
        self.tables = torch.from_numpy(tabs).cuda()
        mm0 = np.zeros((np_, 2), np.uint64)
        mm0[:, 0] = np.uint64(0xFFFFFFFFFFFFFFFF)
        self.minmax0 = torch.from_numpy(mm0.view(np.int64)).cuda()       # ordered 64-bit keys
        self.minmax = self.minmax0.clone()
        # descriptors (in packed order)
        chunk = int(lib().nx_fbm_chunk_size())
        fb = (FbmPlanet * np_)()
        er = (ErosionPlanet * np_)()
        c0 = 0
        self._meshes = []
        for j, i in enumerate(self.order):
            r = requests[i]
            m = self.meshes.get(r.divisions, stream=stream)
            self._meshes.append(m)
            f = fb[j]
            f.xyz = m.xyz.data_ptr()
            f.n = m.n
            f.perm = self.tables[j, 0].data_ptr()
            f.pgi = self.tables[j, 1].data_ptr()
            f.out = self.raw.data_ptr() + 8 * self.vbeg[i]
            f.minmax = self.minmax[j].data_ptr()
            f.chunk0 = c0
            c0 += (m.n + chunk - 1) // chunk
            sc, st = r.octave_args()
            sca = (ctypes.c_double * max(1, len(sc)))(*sc)
            sta = (ctypes.c_double * max(1, len(st)))(*st)
            call("nx_fbm_planet_fill", ctypes.byref(f), r.octaves, sca, sta, float(r.radius))
            e = er[j]
            e.vbeg = self.vbeg[i]
            e.n = m.n
            e.nbr = m.nbr.data_ptr()
            e.edge = m.edge.data_ptr()
            e.iters = r.erosion_iters
            e.rain = r.rain
            e.t_start = 0
            e.slot = j
            if blocked and r.erosion_iters > 0:
                tl = m.tiling(self.tb.tile_side, self.tb.rings, stream=stream)
                e.tiling = tl.dev.data_ptr()
                e.ntiles = tl.ntiles
                e.maxnl = tl.maxnl
                e.maxc = tl.maxc
        self.fb_host, self.er_host = fb, er
        self.fb_dev = _struct_tensor(fb)
        self.er_dev = _struct_tensor(er)
        rows = N
        if blocked:
            # the block map of a blocked run has one entry per tile
            nt = sum(self.meshes.get(r.divisions).tiling(self.tb.tile_side, self.tb.rings).ntiles
                     for r in requests if r.erosion_iters > 0)
            rows = max(rows, nt * ALIGN)
        self.ws = torch.zeros(int(lib().nx_erosion_workspace_size(rows, np_)), dtype=torch.uint8, device=dev)
        self.max_iters = max(r.erosion_iters for r in requests)
        # insolation groups by schedule
        self.inso_groups = []
        if self.any_inso:
            groups = {}
            for j, i in enumerate(self.order):
                if requests[i].insolation:
                    groups.setdefault(requests[i].schedule_key(), []).append(i)
            for (tilt, days, hours), members in groups.items():
                rot, tilts = _climate.annual_schedule(tilt, 365 if days == 365 else days, days, hours)
                tab, nre, pairs = _climate._plan(rot, tilts)
                ip = (InsoPlanet * len(members))()
                for q, i in enumerate(members):
                    m = self.meshes.get(requests[i].divisions)
                    ip[q].xyz = m.xyz.data_ptr()
                    ip[q].n = m.n
                    ip[q].vbeg = self.vbeg[i]
                    ip[q].radius = requests[i].radius
                self.inso_groups.append(dict(table=torch.from_numpy(tab).cuda(), nre=nre, pairs=pairs,
                                             n_tilt=len(tilts), host=ip, dev=_struct_tensor(ip), members=members,
                                             scale=_climate.SOLAR_CONSTANT / (days * hours)))
        self.graph = None

    # ------------------------------------------------------------------
    def launch(self):
        """Enqueue the whole batch on the current stream (no host sync)."""
        s = _dev.stream_handle(self.stream)
        np_ = len(self.requests)
        self.minmax.copy_(self.minmax0)
        call("nx_fbm_batch", _dev.ptr(self.fb_dev), ctypes.cast(self.fb_host, ctypes.c_void_p), np_, None, s)
        call("nx_erosion_ctl_init", _dev.ptr(self.ws), self.ws.numel(), np_, s)
        if self.blocked:
            _autotune.apply(self.tb)
        # rescale (fused into the planets' first blocked passes), erosion, heights
        call("nx_erosion_run_batch", _dev.ptr(self.er_dev), ctypes.cast(self.er_host, ctypes.c_void_p), np_,
             _dev.ptr(self.raw), _dev.ptr(self.minmax), float(self.requests[0].elev_lo),
             float(self.requests[0].elev_hi), float(self.requests[0].water0), _dev.ptr(self.st),
             _dev.ptr(self.st_tmp), _dev.ptr(self.heights), _dev.ptr(self.ws), self.ws.numel(), s)
        for g in self.inso_groups:
            call("nx_insolation_batch", _dev.ptr(g["dev"]), ctypes.cast(g["host"], ctypes.c_void_p),
                 len(g["members"]), _dev.ptr(g["table"]), g["nre"], g["pairs"], g["n_tilt"], _dev.ptr(self.inso), s)

    def capture(self):
        """Record launch() as a CUDA graph (after one eager run)."""
        self.launch()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch()
        self.graph = g
        return g

    def run(self):
        if self.graph is not None:
            self.graph.replay()
        else:
            self.launch()

    def run_to_host(self, host_out):
        """One run whose heights are copied into host_out (page-locked
        float64, at least `total` elements, packed rows as `heights`),
        pipelined for back-to-back calls: the heights alternate between two
        device buffers, the copy of a run's heights goes on a side stream
        while the next call's run proceeds, and a run waits only for the
        copy that last read the buffer it writes.  `wait_host()` blocks until
        the last copy is in host_out.  The first call captures the two CUDA
        graphs (one per buffer; an eager run and a synchronisation each)."""
        if not host_out.is_pinned() or host_out.dtype != torch.float64 or host_out.numel() < self.total:
            raise ValueError("host_out must be a page-locked float64 tensor of at least `total` elements")
        if getattr(self, "_pipe", None) is None:
            bufs = [self.heights, self.heights.clone()]      # same padding rows in both
            graphs = []
            for b in bufs:
                self.heights = b
                graphs.append(self.capture())
            self._pipe = dict(bufs=bufs, graphs=graphs, side=torch.cuda.Stream(), copied=[None, None], next=0)
        p = self._pipe
        b = p["next"]
        main = torch.cuda.current_stream()
        if p["copied"][b] is not None:
            main.wait_event(p["copied"][b])
        self.heights = p["bufs"][b]
        p["graphs"][b].replay()
        ran = torch.cuda.Event()
        ran.record(main)
        side = p["side"]
        side.wait_event(ran)
        with torch.cuda.stream(side):
            host_out[:self.total].copy_(self.heights, non_blocking=True)
            done = torch.cuda.Event()
            done.record(side)
        p["copied"][b] = done
        p["next"] = 1 - b
        self.graph = p["graphs"][b]

    def wait_host(self):
        """Block until the heights of the last run_to_host are on the host."""
        p = getattr(self, "_pipe", None)
        if p is not None and p["copied"][1 - p["next"]] is not None:
            p["copied"][1 - p["next"]].synchronize()

    def erosion_launches(self):
        """Erosion launches per run: passes of the blocked path, or iterations."""
        if any(self.er_host[j].tiling for j in range(len(self.requests))):
            return max(_tb_npass(r.erosion_iters, self.tb.rings) for r in self.requests)
        return self.max_iters

    def kernels_per_run(self):
        blocked = any(self.er_host[j].tiling for j in range(len(self.requests)))
        extra = (2 if self.max_iters > 0 else 0)       # block map + rebase
        if blocked:
            # fBm, the passes (rescale fused into the first), heights, and
            # one rescale launch for the planets without iterations
            dry = any(r.erosion_iters == 0 and r.n_vertices > 0 for r in self.requests)
            return 2 + int(dry) + self.erosion_launches() + extra + len(self.inso_groups)
        return 3 + self.erosion_launches() + extra + len(self.inso_groups)

    def fields(self, i):
        """Height, water and sediment of request i after the last run as
        binary64 true values (the reference's r_buff, wat and sed of
        erosion_iteration3, erosion.py:197-279): the erosion state's pairs
        times 2^K, exact."""
        j = self.order.index(i)
        K = int(self.ws[:32 * len(self.requests)].view(torch.int32).view(-1, 8)[j, 3].item())
        b, n = self.vbeg[i], self.requests[i].n_vertices
        rows = self.st[b:b + n].double()
        sc = 2.0 ** K
        return ((rows[:, 0] + rows[:, 1]) * sc, (rows[:, 2] + rows[:, 3]) * sc, (rows[:, 4] + rows[:, 5]) * sc)

    def results(self):
        """PlanetResult per request, in request order (views into the batch)."""
        uniform = len({(r.elev_lo, r.elev_hi, r.water0) for r in self.requests}) == 1
        if not uniform:
            raise ValueError("a batch shares elev_lo/elev_hi/water0")
        K = self.ws[:32 * len(self.requests)].view(torch.int32).view(-1, 8)[:, 3].cpu().numpy()
        out = []
        pos = {i: j for j, i in enumerate(self.order)}
        for i, r in enumerate(self.requests):
            b, n = self.vbeg[i], r.n_vertices
            ins = None
            if r.insolation:
                sc = _climate.SOLAR_CONSTANT / (r.days * r.hours)
                ins = self.inso[b:b + n] * sc
            out.append(PlanetResult(r, self.heights[b:b + n], ins, int(K[pos[i]])))
        return out


def _tb_npass(iters, R):
    """Passes of a temporally blocked run: ceil(iters/R), made = iters mod 2."""
    if iters <= 0:
        return 0
    n = (iters + R - 1) // R
    if (n ^ iters) & 1:
        n += 1
    return n


def generate_batched(requests, meshes=None):
    b = PlanetBatch(requests, meshes)
    b.run()
    return b.results()


# ----------------------------------------------------------------------
# plain per-planet path (the comparator)

class _PlainWork:
    """Reusable buffers for the plain path (grown on demand)."""

    def __init__(self):
        self.n = 0

    def ensure(self, n):
        if n > self.n:
            self.raw = torch.empty((n, 2), dtype=torch.float32, device="cuda")
            self.hm = torch.empty(n, dtype=torch.float64, device="cuda")
            self.st = torch.empty((n, 8), dtype=torch.float32, device="cuda")
            self.st_tmp = torch.empty((n, 8), dtype=torch.float32, device="cuda")
            self.ws = torch.zeros(int(lib().nx_erosion_workspace_size(n, 1)), dtype=torch.uint8, device="cuda")
            self.planet = torch.zeros(ctypes.sizeof(ErosionPlanet), dtype=torch.uint8, device="cuda")
            self.perm = torch.empty(256, dtype=torch.int32, device="cuda")
            self.pgi = torch.empty(256, dtype=torch.int32, device="cuda")
            self.n = n
        if not hasattr(self, "minmax"):
            self.minmax = torch.empty(2, dtype=torch.int64, device="cuda")
            self.init_desc = torch.zeros(ctypes.sizeof(ErosionPlanet), dtype=torch.uint8, device="cuda")


_plain = _PlainWork()

# ordered keys of the pair (0, 0): a planet with no octaves
_ZERO_KEY = (0x80000000 << 32) | 0x80000000


def generate_plain(request, meshes=None, sync=True, out=None, blocked=False):
    """One planet: a launch per octave, per erosion iteration (blocked=True:
    per temporally blocked pass of the batches' setting); synchronised.
    Same arithmetic as the batched path, so the same bits."""
    r = request
    meshes = meshes if meshes is not None else _mesh.MeshCache()
    m = meshes.get(r.divisions)
    n = m.n
    w = _plain
    w.ensure(n)
    s = _dev.stream_handle()
    perm, pgi = _osx.init(r.seed)
    w.perm.copy_(torch.from_numpy(perm))
    w.pgi.copy_(torch.from_numpy(pgi))
    scale, strength = r.octave_args()
    w.minmax.copy_(torch.tensor([-1, 0], dtype=torch.int64))          # {~0, 0}
    # the precision choice per octave follows the planet's largest amplitude, as in the batch
    amp_ref = max([abs(0.5 * a * r.radius) for a in strength], default=0.0)
    for o in range(r.octaves):
        sc = (ctypes.c_double * 1)(scale[o])
        st = (ctypes.c_double * 1)(strength[o])
        last = o == r.octaves - 1
        call("nx_fbm_pair", _dev.ptr(m.xyz), n, _dev.ptr(w.perm), _dev.ptr(w.pgi), 1, sc, st, float(r.radius),
             amp_ref, _dev.ptr(w.raw), None, 1 if o > 0 else 0, _dev.ptr(w.minmax) if last else None, None, s)
    if r.octaves == 0:
        w.raw[:n].zero_()
        k = _ZERO_KEY - (1 << 64)
        w.minmax.copy_(torch.tensor([k, k], dtype=torch.int64))
    # the rescale to metres and the initial state: the batch's kernel on one
    # planet (state in buffer 0, or in buffer iters & 1 for a blocked run)
    blocked = blocked and r.erosion_iters > 0
    d = ErosionPlanet()
    d.vbeg, d.n, d.nbr, d.edge, d.slot = 0, n, m.nbr.data_ptr(), m.edge.data_ptr(), 0
    d.iters = r.erosion_iters if blocked else 0
    d.rain = r.rain
    w.init_desc.copy_(torch.frombuffer(bytearray(bytes(d)), dtype=torch.uint8))
    call("nx_erosion_init_batch", _dev.ptr(w.init_desc), ctypes.byref(d), 1, _dev.ptr(w.raw), _dev.ptr(w.minmax),
         float(r.elev_lo), float(r.elev_hi), float(r.water0), _dev.ptr(w.st), _dev.ptr(w.st_tmp), s)
    if blocked:
        tb = _autotune.current()
        _autotune.apply(tb)
        tl = m.tiling(tb.tile_side, tb.rings)
        d.tiling, d.ntiles, d.maxnl, d.maxc = tl.dev.data_ptr(), tl.ntiles, tl.maxnl, tl.maxc
        w.init_desc.copy_(torch.frombuffer(bytearray(bytes(d)), dtype=torch.uint8))
        need = int(lib().nx_erosion_workspace_size(max(n, tl.ntiles * ALIGN), 1))
        if getattr(w, "ws_tb", None) is None or w.ws_tb.numel() < need:
            w.ws_tb = torch.zeros(need, dtype=torch.uint8, device="cuda")
        ws = w.ws_tb
        call("nx_erosion_ctl_init", _dev.ptr(ws), ws.numel(), 1, s)
        call("nx_erosion_batch", _dev.ptr(w.init_desc), ctypes.byref(d), 1, _dev.ptr(w.st), _dev.ptr(w.st_tmp), None,
             _dev.ptr(ws), ws.numel(), s)
    else:
        ws = w.ws
        call("nx_erosion_ctl_init", _dev.ptr(ws), ws.numel(), 1, s)
        call("nx_erosion_steps", _dev.ptr(m.nbr), _dev.ptr(m.edge), n, _dev.ptr(w.st), _dev.ptr(w.st_tmp),
             r.erosion_iters, ctypes.c_float(r.rain), _dev.ptr(w.planet), None, None, _dev.ptr(ws), ws.numel(), s)
    hd = w.hm[:n] if out is None else out
    call("nx_erosion_store", _dev.ptr(w.st), n, _dev.ptr(ws), _dev.ptr(hd), None, None, s)
    heights = hd.clone() if out is None else hd
    ins = None
    if r.insolation:
        rot, tilts = _climate.annual_schedule(r.axial_tilt, r.days, r.days, r.hours)
        ins = _climate.insolation_sum(m.xyz, r.radius, rot, tilts)
        ins.mul_(_climate.SOLAR_CONSTANT / (r.days * r.hours))
    if sync:
        torch.cuda.synchronize()
    return PlanetResult(r, heights, ins, 0)
