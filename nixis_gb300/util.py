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


# ---------------------------------------------------------------------------
# Equirectangular maps (util.py:290-366, nixis.py:270-302).  The reference
# finds each pixel's 3 nearest vertices with a scipy KD-tree; here they come
# from point location in the icosphere's face grid (exact nearest three;
# ties in distance go to the lower vertex id, where the KD-tree's order is
# arbitrary).

def make_ll_arr(width, height, radius, device=False, stream=None):
    """util.make_ll_arr (util.py:290-310): (height, width, 3) float64 xyz of
    every pixel's latitude/longitude (numpy, or a CUDA tensor with device)."""
    _dev.require_cuda()
    out = torch.empty((int(height), int(width), 3), dtype=torch.float64, device="cuda")
    call("nx_make_ll", int(width), int(height), float(radius), _dev.ptr(out), _dev.stream_handle(stream))
    return out if device else out.cpu().numpy()


def query_nearest3(verts, neighbors, divisions, queries, stream=None):
    """The 3 nearest vertices of each query point, as the reference's
    KDTree(points).query(queries, k=3): (distances, indices), each of shape
    queries.shape[:-1] + (3,), ascending.  verts / neighbors: an icosphere
    of `divisions` made by this library (any radius)."""
    from . import mesh as _m
    host = _dev.is_host(queries)
    _m._ensure_tables()
    xyz = _dev.to_device(verts, np.float64, name="verts")
    nb = _dev.to_device(neighbors, np.int32, name="neighbors")
    q = _dev.to_device(queries, np.float64, name="queries")
    shape = tuple(q.shape[:-1]) + (3,)
    q = q.reshape(-1, 3)
    d = torch.empty((q.shape[0], 3), dtype=torch.float64, device="cuda")
    i = torch.empty((q.shape[0], 3), dtype=torch.int64, device="cuda")
    call("nx_nearest3", int(divisions), _dev.ptr(xyz), _dev.ptr(nb), xyz.shape[0], _dev.ptr(q), q.shape[0],
         _dev.ptr(d), _dev.ptr(i), _dev.stream_handle(stream))
    d, i = d.reshape(shape), i.reshape(shape)
    return (d.cpu().numpy(), i.cpu().numpy()) if host else (d, i)


def _sample(dists, nbrs, colors, stream=None):
    cd = _dev.to_device(colors, np.float64, name="colors").reshape(-1)
    d = _dev.to_device(dists, np.float64, name="dists").reshape(-1, 3)
    i = _dev.to_device(nbrs, np.int64, name="nbrs").reshape(-1, 3)
    out = torch.empty(d.shape[0], dtype=torch.float64, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    call("nx_sample_gray", _dev.ptr(d), _dev.ptr(i), d.shape[0], _dev.ptr(cd), cd.numel(), _dev.ptr(out), _dev.ptr(err),
         _dev.stream_handle(stream))
    if int(err.item()):
        raise IndexError("nbrs holds an index outside the colours")
    return out


def _as_dtype(values, like):
    dt = like.dtype if isinstance(like, np.ndarray) else np.dtype(str(like.dtype).replace("torch.", ""))
    return values.astype(dt)


def make_gray_array(width, height, dists, nbrs, colors):
    """util.make_gray_array (util.py:342-366): per pixel the inverse-distance
    weighting of its 3 neighbours' colours, truncated to an integer and
    returned in the colours' dtype, shape (height, width)."""
    v = _sample(dists, nbrs, colors).cpu().numpy().reshape(int(height), int(width))
    return _as_dtype(v, colors)


def make_rgb_array(width, height, dists, nbrs, colors):
    """util.make_rgb_array (util.py:312-340): the same value in 3 channels,
    shape (height, width, 3)."""
    g = make_gray_array(width, height, dists, nbrs, colors)
    return np.repeat(g[:, :, None], 3, axis=2)


def equirect_map(verts, neighbors, divisions, colors, width, height, radius, stream=None):
    """A whole map on the GPU: pixel positions, nearest three vertices, and
    the gray weighting of `colors` (the reference's make_ll_arr + KD-tree
    query + make_gray_array); returns (height, width) in the colours' dtype."""
    ll = make_ll_arr(width, height, radius, device=True, stream=stream)
    d, i = query_nearest3(verts, neighbors, divisions, ll, stream=stream)
    v = _sample(d, i, colors, stream=stream).cpu().numpy().reshape(int(height), int(width))
    return _as_dtype(v, colors)
