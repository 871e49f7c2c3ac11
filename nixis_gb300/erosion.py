"""Drop-in for the reference's erosion module, variant 3 (the one nixis.py
calls, nixis.py:410), plus the steepest-descent rule of find_lowest.

State on the GPU is binary32 pairs (hi + lo) with a per-planet power-of-two
scale (exact, see csrc/nx_erosion.cu); results are returned in the reference's float64
arrays, updated in place like the reference.
"""
import ctypes

import numpy as np
import torch

from . import _dev
from . import mesh as _mesh
from ._lib import ErosionPlanet, call, lib

RAIN = 0.3 / 320            # erosion.py:182
EVAPORATION = 0.1 / 320     # erosion.py:205
SOLUBILITY = 0.01 / 320     # erosion.py:206
CAPACITY = 0.2 / 320        # erosion.py:207


class ErosionRun:
    """Resident erosion state of one planet (binary32 pairs).

    verts float64 (N,3) and neighbors int32 (N,6) as CUDA tensors (or
    numpy); fields are loaded from float64 heights / water / sediment."""

    def __init__(self, verts, neighbors, edge=None, stream=None):
        self.stream = stream
        self.xyz = _dev.to_device(verts, np.float64, name="verts")
        _dev.check_vertices(self.xyz)
        self.n = self.xyz.shape[0]
        self.nbr = _dev.to_device(neighbors, np.int32, (self.n, 6), "neighbors")
        if edge is None:
            edge, err = _mesh.edge_lengths(self.xyz, self.nbr, stream=stream)
            if int(err.item()):
                raise IndexError("neighbors holds an id outside [-1, N)")
        self.edge = edge
        n = self.n
        self.st = torch.empty((n, 8), dtype=torch.float32, device="cuda")    # (h, w, s as hi/lo pairs, 0, 0)
        self.st_tmp = torch.empty_like(self.st)
        self.ws = torch.zeros(int(lib().nx_erosion_workspace_size(n, 1)), dtype=torch.uint8, device="cuda")
        self.planet = torch.zeros(ctypes.sizeof(ErosionPlanet), dtype=torch.uint8, device="cuda")  # one descriptor
        self.iters_done = 0

    def load(self, heights, water=None, sediment=None):
        h = _dev.to_device(heights, np.float64, (self.n,), "heights")
        w = None if water is None else _dev.to_device(water, np.float64, (self.n,), "water")
        s = None if sediment is None else _dev.to_device(sediment, np.float64, (self.n,), "sediment")
        call("nx_erosion_load", _dev.ptr(h), _dev.ptr(w), _dev.ptr(s), self.n, _dev.ptr(self.st),
             _dev.ptr(self.ws), self.ws.numel(), _dev.stream_handle(self.stream))
        self.iters_done = 0
        return self

    def steps(self, iters, rain=0.0, mass=False, flow=False):
        """Run `iters` iterations; returns (mass float64 (iters,3) or None,
        flow uint16 (N,) of the last iteration or None)."""
        iters = int(iters)
        m = torch.empty((max(iters, 1), 3), dtype=torch.float64, device="cuda") if mass else None
        f = torch.zeros(self.n, dtype=torch.int16, device="cuda") if flow else None
        call("nx_erosion_steps", _dev.ptr(self.nbr), _dev.ptr(self.edge), self.n, _dev.ptr(self.st),
             _dev.ptr(self.st_tmp), iters, float(rain), _dev.ptr(self.planet), _dev.ptr(m), _dev.ptr(f),
             _dev.ptr(self.ws), self.ws.numel(), _dev.stream_handle(self.stream))
        self.iters_done += iters
        return (m[:iters] if mass else None), f

    def store(self, heights, water=None, sediment=None):
        """Write the state as float64 true values into the given CUDA tensors."""
        call("nx_erosion_store", _dev.ptr(self.st), self.n, _dev.ptr(self.ws),
             _dev.ptr(heights), _dev.ptr(water), _dev.ptr(sediment), _dev.stream_handle(self.stream))

    def scale_exponent(self):
        return int(self.ws[:32].view(torch.int32)[3].item())

    def check(self):
        err = int(self.ws[:32].view(torch.int32)[6].item())
        if err:
            raise IndexError("neighbors holds an id outside [-1, N)")


def erosion_iteration3(verts, neighbors, r_buff, wat, sed):
    """erosion.erosion_iteration3 (erosion.py:197-279): one Jacobi step;
    r_buff (heights), wat and sed are updated in place."""
    _run_inplace(verts, neighbors, r_buff, wat, sed, 1, 0.0, with_fields=True)


def erode_terrain3(nodes, neighbors, heights, num_iter=1, snapshot=False):
    """erosion.erode_terrain3 (erosion.py:172-192): num_iter <= 0 runs once;
    water and sediment start at zero and 0.3/320 of rain is added before
    each iteration; heights are updated in place.  Per-iteration PNG
    snapshots (image export) are not part of this library."""
    if snapshot:
        raise NotImplementedError("erosion snapshots (PNG export) are not provided by nixis_gb300")
    if num_iter <= 0:
        num_iter = 1
    _run_inplace(nodes, neighbors, heights, None, None, int(num_iter), RAIN, with_fields=False)


def _run_inplace(verts, neighbors, h, w, s, iters, rain, with_fields):
    host = _dev.is_host(h)
    for a in (h, w, s):
        if a is None:
            continue
        if host and (not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous):
            raise ValueError("fields must be C-contiguous float64 arrays")
    if len(verts) == 0:
        # the reference's loop over vertices runs zero times
        for a, name in ((h, "heights"), (w, "water"), (s, "sediment")):
            if a is not None and tuple(a.shape) != (0,):
                raise ValueError(f"{name}: expected shape (0,), got {tuple(a.shape)}")
        return
    run = ErosionRun(verts, neighbors)
    hd = _dev.to_device(h, np.float64, (run.n,), "heights")
    wd = _dev.to_device(w, np.float64, (run.n,), "water") if w is not None else None
    sd = _dev.to_device(s, np.float64, (run.n,), "sediment") if s is not None else None
    run.load(hd, wd, sd)
    run.steps(iters, rain=rain)
    run.check()
    if with_fields:
        run.store(hd, wd, sd)
    else:
        run.store(hd)
    if host:
        h[...] = hd.cpu().numpy()
        if w is not None:
            w[...] = wd.cpu().numpy()
            s[...] = sd.cpu().numpy()
    else:
        for dst, src in ((h, hd), (w, wd), (s, sd)):
            if dst is not None and dst.data_ptr() != src.data_ptr():
                dst.copy_(src)


def find_lowest(vert, nbr, height):
    """erosion.find_lowest (erosion.py:398-406) for one vertex (host rule)."""
    alts = [height[i] for i in nbr if i != -1]
    lowest = min(alts)
    if lowest < height[vert]:
        return alts.index(lowest)
    return None


def steepest_descent(neighbors, heights, stream=None):
    """find_lowest for every vertex on the GPU: (pos int32 (N,), vid int32
    (N,)); pos is the reference's return value (-1 for None), vid the
    neighbour id it designates."""
    nb = _dev.to_device(neighbors, np.int32, name="neighbors")
    h = _dev.to_device(heights, np.float64, name="heights")
    n = nb.shape[0]
    pos = torch.empty(n, dtype=torch.int32, device="cuda")
    vid = torch.empty(n, dtype=torch.int32, device="cuda")
    call("nx_steepest_descent", _dev.ptr(nb), _dev.ptr(h), n, _dev.ptr(pos), _dev.ptr(vid), _dev.stream_handle(stream))
    return pos, vid


__all__ = ["erosion_iteration3", "erode_terrain3", "find_lowest", "steepest_descent", "ErosionRun",
           "ErosionPlanet", "RAIN", "EVAPORATION", "SOLUBILITY", "CAPACITY"]
