"""The reference util functions on the hot path's edges (util.py).

Coordinate helpers are scalar host math like the reference's; mesh and
adjacency builders run on the GPU (see mesh.py); the height shaping of
nixis.py:332-364 (rescale, find_percent_val, power_rescale, the elevation
mask) runs on the GPU in binary64 (csrc/nx_shape.cu).
"""
import math

import numpy as np
import torch

from . import mesh as _mesh
from . import _dev
from ._lib import call, lib

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


_FORMS = {None: 0, "lower": 2, "upper": 3}


def _ws(n):
    return torch.empty(int(lib().nx_shape_workspace_size(n)), dtype=torch.uint8, device="cuda")


def _f64(x):
    host = _dev.is_host(x)
    xd = _dev.to_device(x, np.float64, name="x").reshape(-1)
    if xd.numel() == 0:
        raise ValueError("zero-size array has no minimum or maximum")
    return host, xd


def rescale(x, lower, upper, mid=None, mode=None, u_min=None, u_max=None, stream=None):
    """util.rescale (util.py:110-176) on the GPU, binary64, every form:
    plain min/max normalisation to [lower, upper]; with `mid`, each side of
    mid mapped separately; mode 'lower' / 'upper' rescale only that side;
    u_min / u_max widen the input range.  numpy in -> numpy out, CUDA tensor
    in -> CUDA tensor out.  As in the reference, a mode without mid returns
    x unchanged and an unknown mode returns None."""
    if mode is not None and mode not in ("lower", "upper"):
        return None
    if mode is not None and mid is None:
        return x
    form = 1 if (mode is None and mid is not None) else _FORMS[mode]
    host, xd = _f64(x)
    n = xd.numel()
    out = torch.empty_like(xd)
    ws = _ws(n)
    call("nx_rescale", _dev.ptr(xd), n, float(lower), float(upper), float(mid if mid is not None else 0.0), form,
         float(u_min if u_min is not None else 0.0), int(u_min is not None),
         float(u_max if u_max is not None else 0.0), int(u_max is not None), _dev.ptr(out), _dev.ptr(ws), ws.numel(),
         _dev.stream_handle(stream))
    return out.cpu().numpy() if host else out


def power_rescale(x, mask=None, mode=None, power=1.0, stream=None):
    """util.power_rescale (util.py:179-250) on the GPU: the values selected
    by mode (1: mask true, 0: mask false) are mapped to [0, 1] over their
    range, raised to `power` and mapped back; the range is the reference's
    running min/max update (a new running minimum is not compared with the
    maximum).  Other modes return a copy."""
    host, xd = _f64(x)
    n = xd.numel()
    m = -1 if mode not in (0, 1) else int(mode)
    md = None
    if m >= 0:
        if mask is None:
            raise ValueError("power_rescale: mode 0 or 1 needs a mask")
        md = _dev.to_device(np.asarray(mask, dtype=np.uint8) if _dev.is_host(mask) else mask.to(torch.uint8),
                            np.uint8, (n,), "mask")
    out = torch.empty_like(xd)
    ws = _ws(n)
    call("nx_power_rescale", _dev.ptr(xd), n, _dev.ptr(md), m, float(power), _dev.ptr(out), _dev.ptr(ws), ws.numel(),
         _dev.stream_handle(stream))
    return out.cpu().numpy() if host else out


def find_percent_val(minval, maxval, percent):
    """util.find_percent_val (util.py:556-566): percents outside (0, 100)
    become 50 (the reference prints a warning)."""
    if not 0.0 < percent < 100.0:
        percent = 50.0
    return minval + ((maxval - minval) * percent / 100.0)


def make_bool_elevation_mask(height, mask_elevation, stream=None):
    """terrain.make_bool_elevation_mask (terrain.py:61-72): height <=
    mask_elevation, as a bool array (numpy) or bool CUDA tensor."""
    host = _dev.is_host(height)
    hd = _dev.to_device(height, np.float64, name="height").reshape(-1)
    n = hd.numel()
    m = torch.empty(n, dtype=torch.uint8, device="cuda")
    call("nx_elevation_mask", _dev.ptr(hd), n, float(mask_elevation), _dev.ptr(m), _dev.stream_handle(stream))
    return m.cpu().numpy().astype(bool) if host else m.bool()


def shape_heights(height, min_alt=-4000.0, max_alt=8850.0, ocean_percent=55.0, stream=None):
    """The post-noise shaping of nixis.py:332-364 in one device-side
    sequence (no host round trip): rescale to [min_alt, max_alt], ocean
    level at ocean_percent of the range, ocean mask, power_rescale of the
    ocean (0.5) and of the land (2.0), shift by the level, rescale about 0.
    Returns (heights, ocean mask, ocean level) -- numpy/float for numpy
    input, CUDA tensors for a CUDA tensor."""
    host, hd = _f64(height)
    n = hd.numel()
    out, tmp = torch.empty_like(hd), torch.empty_like(hd)
    mask = torch.empty(n, dtype=torch.uint8, device="cuda")
    level = torch.empty(1, dtype=torch.float64, device="cuda")
    ws = _ws(n)
    call("nx_shape_heights", _dev.ptr(hd), n, float(min_alt), float(max_alt), float(ocean_percent), _dev.ptr(out),
         _dev.ptr(tmp), _dev.ptr(mask), _dev.ptr(level), _dev.ptr(ws), ws.numel(), _dev.stream_handle(stream))
    if host:
        return out.cpu().numpy(), mask.cpu().numpy().astype(bool), float(level.item())
    return out, mask.bool(), level
