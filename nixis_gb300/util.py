"""The reference util functions on the hot path's edges (util.py).

Coordinate helpers are scalar host math like the reference's; mesh and
adjacency builders run on the GPU (see mesh.py); ``rescale`` is the plain
min/max normalisation used to map elevations to metres.
"""
import math

import numpy as np
import torch

from . import mesh as _mesh
from . import _dev

create_mesh = _mesh.create_mesh
build_adjacency = _mesh.build_adjacency
sort_adjacency = _mesh.sort_adjacency


def xyz2latlon(x, y, z, r):
    """util.xyz2latlon (util.py:59-75), degrees, asin argument clamped."""
    lat = math.degrees(math.asin(min(max(z / r, -1), 1)))
    lon = math.degrees(math.atan2(y, x))
    return lat, lon


def latlon2xyz(lat, lon, r):
    """util.latlon2xyz (util.py:79-88)."""
    x = r * math.cos(lat * (math.pi / 180)) * math.cos(lon * (math.pi / 180))
    y = r * math.cos(lat * (math.pi / 180)) * math.sin(lon * (math.pi / 180))
    z = r * math.sin(lat * (math.pi / 180))
    return x, y, z


def rescale(x, lower, upper):
    """util.rescale (util.py:110-140, mode=None, mid=None): min/max
    normalise to [lower, upper].  numpy in -> numpy out (host), CUDA tensor
    in -> CUDA tensor out."""
    if _dev.is_host(x):
        x = np.asarray(x, np.float64)
        mn, mx = x.min(), x.max()
        return ((x - mn) / (mx - mn)) * (upper - lower) + lower
    mn, mx = torch.aminmax(x)
    return ((x - mn) / (mx - mn)) * (upper - lower) + lower
