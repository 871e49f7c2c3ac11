"""Icosphere meshes on the GPU: vertices, triangles, neighbour table and
per-slot edge lengths, kept resident per subdivision.

``create_mesh`` replaces util.create_mesh (util.py:17-50, meshzoo);
``build_adjacency`` / ``sort_adjacency`` implement util.py:591-662 on the
GPU and give the reference's neighbour table for the same triangles.
"""
import ctypes
import threading

import numpy as np
import torch

from . import _dev
from . import icosphere as ico
from ._lib import call, lib

_tables_done = set()
_lock = threading.Lock()

# temporally blocked erosion: tiles are TILE_SIDE x TILE_SIDE squares of a
# face grid (a negative tile_side: hexagons of radius -tile_side) with
# TILE_RINGS halo rings (passes of up to TILE_RINGS iterations)
TILE_SIDE = 40
TILE_RINGS = 4


def _ensure_tables():
    dev = torch.cuda.current_device()
    if dev in _tables_done:
        return
    with _lock:
        if dev in _tables_done:
            return
        c = np.ascontiguousarray(ico.corners(), np.float64)
        f = np.ascontiguousarray(ico.FACES, np.int32)
        fe = np.ascontiguousarray(ico.face_edge_table(), np.int32)
        e = np.ascontiguousarray(ico.edges(), np.int32)
        vp = ctypes.c_void_p
        call("nx_icosphere_tables", c.ctypes.data_as(vp), f.ctypes.data_as(vp), fe.ctypes.data_as(vp),
             e.ctypes.data_as(vp))
        _tables_done.add(dev)


def icosphere(divisions, with_tris=True, stream=None):
    """(points float64 (N,3), cells int32 (T,3) or None) as CUDA tensors."""
    _dev.require_cuda()
    k = ico.check_divisions(divisions)
    _ensure_tables()
    nv, nt = ico.counts(k)
    xyz = torch.empty((nv, 3), dtype=torch.float64, device="cuda")
    tris = torch.empty((nt, 3), dtype=torch.int32, device="cuda") if with_tris else None
    call("nx_icosphere", k, _dev.ptr(xyz), _dev.ptr(tris), _dev.stream_handle(stream))
    return xyz, tris


def create_mesh(divisions):
    """util.create_mesh: (points float64 (10k^2+2, 3), cells int32 (20k^2, 3))
    as numpy arrays (the reference returns numpy)."""
    xyz, tris = icosphere(divisions)
    return xyz.cpu().numpy(), tris.cpu().numpy()


def _adjacency(t, stream=None):
    """Launch build_adjacency; returns (adj, error flags) without waiting."""
    if t.ndim != 2 or t.shape[1] != 3:
        raise ValueError("triangles must have shape (T, 3)")
    nt = t.shape[0]
    nv = (nt + 4) // 2
    adj = torch.empty((nv, 6), dtype=torch.int32, device="cuda")
    ws = torch.empty(int(lib().nx_adjacency_workspace_size(nv)), dtype=torch.uint8, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    call("nx_build_adjacency", _dev.ptr(t), nt, nv, _dev.ptr(adj), _dev.ptr(ws), ws.numel(), _dev.ptr(err),
         _dev.stream_handle(stream))
    return adj, err


def _check_adjacency(e):
    if e & 1:
        raise ValueError("build_adjacency: a triangle references a vertex id outside [0, (T+4)/2)")
    if e & 2:
        raise ValueError("build_adjacency: a vertex has more than 6 neighbours")


def build_adjacency(triangles, stream=None):
    """util.build_adjacency: (N,6) int32 neighbour rows in triangle order,
    -1 padded (CUDA tensor; numpy in -> numpy out)."""
    host = _dev.is_host(triangles)
    t = _dev.to_device(triangles, np.int32, name="triangles")
    adj, err = _adjacency(t, stream)
    _check_adjacency(int(err.item()))
    return adj.cpu().numpy() if host else adj


def sort_adjacency(adj, stream=None):
    """util.sort_adjacency, in place (numpy or CUDA tensor)."""
    host = _dev.is_host(adj)
    a = _dev.to_device(adj, np.int32, name="adj")
    out = torch.empty_like(a)
    call("nx_sort_adjacency", _dev.ptr(a), _dev.ptr(out), a.shape[0], _dev.stream_handle(stream))
    if host:
        adj[...] = out.cpu().numpy()
    else:
        adj.copy_(out)
    return adj


def edge_lengths(xyz, nbr, stream=None):
    """float32 (N,6,2) per-slot neighbour distances (binary64, split into
    (hi, lo) pairs)."""
    x = _dev.to_device(xyz, np.float64, name="verts")
    nb = _dev.to_device(nbr, np.int32, name="neighbors")
    n = x.shape[0]
    if nb.shape != (n, 6):
        raise ValueError("neighbors must have shape (N, 6)")
    el = torch.empty((n, 6, 2), dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    call("nx_edge_lengths", _dev.ptr(x), _dev.ptr(nb), n, _dev.ptr(el), _dev.ptr(err), _dev.stream_handle(stream))
    return el, err


class PlanetMesh:
    """A subdivision's resident mesh: xyz float64 (N,3), nbr int32 (N,6),
    edge float32 (N,6,2) pairs; triangles are dropped after the adjacency is
    built.  With defer_checks the build only enqueues work on the stream
    (no host wait); check() reads the error flags later."""

    def __init__(self, divisions, stream=None, defer_checks=False):
        self.k = ico.check_divisions(divisions)
        self.n = ico.counts(self.k)[0]
        s = stream if stream is not None else torch.cuda.current_stream()
        xyz, tris = icosphere(self.k, stream=stream)
        # the vertices alone are ready here (work that needs only them, like
        # the noise, can start on another stream while the rest is built)
        self.xyz_ready = torch.cuda.Event()
        self.xyz_ready.record(s)
        adj, aerr = _adjacency(tris, stream)
        del tris
        nbr = torch.empty_like(adj)
        call("nx_sort_adjacency", _dev.ptr(adj), _dev.ptr(nbr), self.n, _dev.stream_handle(stream))
        del adj
        self.xyz = xyz
        self.nbr = nbr
        self.edge, eerr = edge_lengths(xyz, nbr, stream=stream)
        # the whole mesh is ready here (an event of its own, so a later user
        # need not wait for whatever else its stream has queued since)
        self.built = torch.cuda.Event()
        self.built.record(s)
        self._errs = (aerr, eerr)
        self._tilings = {}
        if not defer_checks:
            self.check()

    def check(self):
        """Raise if the adjacency or edge-length kernels flagged an error."""
        if self._errs is None:
            return
        aerr, eerr = (int(e.item()) for e in self._errs)
        self._errs = None
        _check_adjacency(aerr)
        if eerr:
            raise RuntimeError("mesh adjacency produced an invalid neighbour id")

    def tiling(self, tile_side=TILE_SIDE, rings=TILE_RINGS, stream=None):
        """The mesh's tiling for temporally blocked erosion (built once)."""
        key = (tile_side, rings)
        if key not in self._tilings:
            self._tilings[key] = MeshTiling(self, tile_side, rings, stream)
            self._nbytes = None
        return self._tilings[key]

    def drop_tilings(self, keep=None):
        """Free every tiling but the one keyed (tile_side, rings) = keep."""
        for key in [k for k in self._tilings if k != keep]:
            del self._tilings[key]
        self._nbytes = None

    @property
    def nbytes(self):
        if getattr(self, "_nbytes", None) is None:
            self._nbytes = (self.xyz.numel() * 8 + self.nbr.numel() * 4 + self.edge.numel() * 4 +
                            sum(t.nbytes for t in self._tilings.values()))
        return self._nbytes


class MeshTiling:
    """Tiles of a mesh with their halo rings (nx_tiling), resident in HBM."""

    def __init__(self, mesh, tile_side=TILE_SIDE, rings=TILE_RINGS, stream=None):
        nt, nm, cm = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        call("nx_tiling_shape", mesh.k, tile_side, rings, ctypes.byref(nt), ctypes.byref(nm), ctypes.byref(cm))
        self.ntiles, self.nmax, self.cmax, self.rings = nt.value, nm.value, cm.value, rings
        dev = "cuda"
        self.counts = torch.zeros(self.ntiles * (rings + 1), dtype=torch.int32, device=dev)
        self.ids = torch.empty(self.ntiles * self.nmax, dtype=torch.int32, device=dev)
        # (+8: the shared-table kernel copies whole 16-byte units past a tile's last row)
        self.lnbr = torch.empty(self.ntiles * self.cmax * 6 + 8, dtype=torch.int16, device=dev)
        self.ledge = torch.empty(self.ntiles * self.cmax * 12, dtype=torch.float32, device=dev)
        err = torch.zeros(3, dtype=torch.int32, device=dev)
        call("nx_tiling_build", mesh.k, tile_side, rings, _dev.ptr(mesh.nbr), _dev.ptr(mesh.edge), _dev.ptr(self.counts),
             _dev.ptr(self.ids), _dev.ptr(self.lnbr), _dev.ptr(self.ledge), _dev.ptr(err), _dev.stream_handle(stream))
        from ._lib import Tiling
        t = Tiling(self.ntiles, rings, self.nmax, self.cmax, self.counts.data_ptr(), self.ids.data_ptr(),
                   self.lnbr.data_ptr(), self.ledge.data_ptr())
        # the counts come back and the descriptor goes up without a host wait;
        # maxnl / maxc wait for them only when first read
        s = stream if stream is not None else torch.cuda.current_stream()
        with torch.cuda.stream(s):
            self._err_host = torch.empty(3, dtype=torch.int32, pin_memory=True)
            self._err_host.copy_(err, non_blocking=True)
            self._dev_host = torch.empty(ctypes.sizeof(t), dtype=torch.uint8, pin_memory=True)
            self._dev_host.numpy()[:] = np.frombuffer(bytes(t), np.uint8)
            self.dev = self._dev_host.to("cuda", non_blocking=True)
            self._ready = torch.cuda.Event()
            self._ready.record(s)
        self._err = err
        self._counts = None
        self.k = mesh.k

    def _resolve(self):
        if self._counts is None:
            self._ready.synchronize()
            e = self._err_host.numpy()
            if e[0]:
                raise RuntimeError(f"tiling of divisions {self.k} failed (flags {int(e[0])})")
            self._counts = (int(e[1]), int(e[2]))
        return self._counts

    def ready(self):
        """True once the build's counts are on the host (no wait)."""
        return self._counts is not None or self._ready.query()

    @property
    def maxnl(self):
        return self._resolve()[0]

    @property
    def maxc(self):
        return self._resolve()[1]

    @property
    def nbytes(self):
        return self.counts.numel() * 4 + self.ids.numel() * 4 + self.lnbr.numel() * 2 + self.ledge.numel() * 4


class MeshCache:
    """Meshes kept resident in HBM, keyed by divisions, LRU-evicted past a
    byte budget."""

    def __init__(self, budget_bytes=None):
        self.budget = budget_bytes
        self._m = {}
        self._order = []

    def get(self, divisions, stream=None):
        k = int(divisions)
        if k in self._m:
            self._order.remove(k)
            self._order.append(k)
            return self._m[k]
        m = PlanetMesh(k, stream=stream)
        self._m[k] = m
        self._order.append(k)
        self._evict()
        return m

    def _evict(self):
        if self.budget is None:
            return
        while len(self._order) > 1 and self.nbytes > self.budget:
            k = self._order.pop(0)
            del self._m[k]

    @property
    def nbytes(self):
        return sum(m.nbytes for m in self._m.values())

    def __contains__(self, k):
        return int(k) in self._m
