"""Drop-in for the insolation part of the reference's climate module
(climate.py:167-201, 415-597) and the fused annual accumulation.

``sample_insolation`` keeps the reference's in-place float32 ``arr +=``;
``insolation_sum`` evaluates any (tilt x rotation) schedule in one kernel;
``annual_insolation`` is the year of days x hourly sun positions.  The
latitude-table path (``calc_insolation_slice``, ``interpolate_insolation``,
``calc_daily_insolation``, ``calc_yearly_insolation``) builds its tables and
interpolates on the GPU; tables are cached per (radius, tilts).
"""
import ctypes
import math

import numpy as np
import torch

from . import _dev
from ._lib import call

SOLAR_CONSTANT = 1361.0  # W/m^2


def day2deg(year_length, day):
    """climate.day2deg (climate.py:167-171)."""
    return (day / year_length) * 360.0


def calculate_seasonal_tilt(axial_tilt, degrees):
    """climate.calculate_seasonal_tilt (climate.py:192-201)."""
    return math.sin(degrees * math.pi / 180) * axial_tilt


def _plan(rot_deg, tilt_deg):
    rot = np.ascontiguousarray(rot_deg, np.float64)
    tilt = np.ascontiguousarray(tilt_deg, np.float64)
    tab = np.zeros(2 * (len(rot) + len(tilt)), np.float32)
    nre = ctypes.c_int(0)
    pairs = ctypes.c_int(0)
    vp = ctypes.c_void_p
    call("nx_insolation_plan", rot.ctypes.data_as(vp), len(rot), tilt.ctypes.data_as(vp), len(tilt),
         tab.ctypes.data_as(vp), ctypes.byref(nre), ctypes.byref(pairs))
    used = 2 * (nre.value + len(tilt))
    return tab[:used], nre.value, pairs.value


def insolation_sum(verts, radius, rotations, tilts, out=None, accumulate=False, stream=None):
    """Sum over every (tilt, rotation) of sample_insolation's term.

    verts float64 (N,3) (CUDA tensor or numpy); rotations/tilts in degrees.
    Returns a float32 CUDA tensor (N,) (or adds into `out`)."""
    xyz = _dev.to_device(verts, np.float64, name="verts")
    _dev.check_vertices(xyz)
    n = xyz.shape[0]
    tab, nre, pairs = _plan(rotations, tilts)
    tdev = _dev.to_device(tab, np.float32, name="table")
    if out is None:
        out = torch.empty(n, dtype=torch.float32, device="cuda")
        accumulate = False
    if out.dtype != torch.float32 or out.shape != (n,) or not out.is_cuda:
        raise ValueError("out must be a float32 CUDA tensor of shape (N,)")
    call("nx_insolation", _dev.ptr(xyz), n, float(radius), _dev.ptr(tdev), nre, pairs, len(tilts), _dev.ptr(out),
         1 if accumulate else 0, _dev.stream_handle(stream))
    return out


def sample_insolation(arr, verts, radius, rotation, tilt):
    """climate.sample_insolation (climate.py:415-444): arr += the insolation
    term for one sun position, in place (numpy float32 like the reference,
    or a float32 CUDA tensor)."""
    if _dev.is_host(arr):
        if arr.dtype != np.float32 or not arr.flags.c_contiguous:
            raise ValueError("arr must be a C-contiguous float32 array")
        dev = _dev.to_device(arr, np.float32)
        insolation_sum(verts, radius, [float(rotation)], [float(tilt)], out=dev, accumulate=True)
        arr[...] = dev.cpu().numpy()
        return
    insolation_sum(verts, radius, [float(rotation)], [float(tilt)], out=arr, accumulate=True)


def brute_daily_insolation(verts, altitudes, radius, tilt, snapshot=False):
    """climate.brute_daily_insolation (climate.py:450-489): 360 rotations of
    one degree from -180, one tilt; a new float32 array."""
    if snapshot:
        raise NotImplementedError("insolation snapshots (PNG export) are not provided by nixis_gb300")
    host = _dev.is_host(verts)
    rot = [-180.0 + i * 1.0 for i in range(360)]
    out = insolation_sum(verts, radius, rot, [float(tilt)])
    return out.cpu().numpy() if host else out


def calc_instant_insolation(verts, altitudes, radius, rotation, tilt):
    """climate.calc_instant_insolation (climate.py:492-500)."""
    host = _dev.is_host(verts)
    out = insolation_sum(verts, radius, [float(rotation)], [float(tilt)])
    return out.cpu().numpy() if host else out


def annual_schedule(axial_tilt=23.44, year_length=365, days=365, hours=24):
    """Sun positions of a circular orbit: hourly rotations -180 + (360/hours) h
    and daily tilts calculate_seasonal_tilt(axial_tilt, day2deg(year_length, d))."""
    rot_amt = 360.0 / hours
    rot = []
    r = -180.0
    for _ in range(hours):
        rot.append(r)
        r += rot_amt
    tilts = [calculate_seasonal_tilt(axial_tilt, day2deg(year_length, d)) for d in range(days)]
    return rot, tilts


def annual_insolation(verts, radius, axial_tilt=23.44, year_length=365, days=365, hours=24, mean_wm2=False,
                      out=None, stream=None):
    """Sum of sample_insolation terms over `days` x `hours` sun positions
    (float32 CUDA tensor).  With mean_wm2, converted to the mean top-of-
    atmosphere flux: SOLAR_CONSTANT * sum / (days * hours)."""
    rot, tilts = annual_schedule(axial_tilt, year_length, days, hours)
    s = insolation_sum(verts, radius, rot, tilts, out=out, stream=stream)
    if mean_wm2:
        s.mul_(SOLAR_CONSTANT / (days * hours))
    return s


_tables = {}


def _slice_tables(radius, tilts):
    """Device float32 (len(tilts), 181) latitude tables (cached)."""
    key = (float(radius), tuple(float(t) for t in tilts))
    t = _tables.get(key)
    if t is None:
        _dev.require_cuda()
        td = torch.tensor(list(key[1]), dtype=torch.float64, device="cuda")
        t = torch.empty((len(tilts), 181), dtype=torch.float32, device="cuda")
        call("nx_insolation_slices", _dev.ptr(td), len(tilts), float(radius), _dev.ptr(t), _dev.stream_handle())
        if len(_tables) > 64:
            _tables.clear()
        _tables[key] = t
    return t


def calc_insolation_slice(radius, tilt):
    """climate.calc_insolation_slice (climate.py:503-533): float32 (181,),
    entry i the summed insolation of latitude i (i <= 90) or i - 181, over
    360 rotations of one degree."""
    return _slice_tables(radius, [tilt])[0].cpu().numpy()


def interpolate_insolation(verts, lookup_table, insolation, radius):
    """climate.interpolate_insolation (climate.py:551-577): insolation[v] =
    the table interpolated at the vertex's latitude, in place (numpy float32
    or a float32 CUDA tensor)."""
    xyz = _dev.to_device(verts, np.float64, name="verts")
    _dev.check_vertices(xyz)
    n = xyz.shape[0]
    tab = _dev.to_device(lookup_table, np.float32, (181,), "lookup_table")
    host = _dev.is_host(insolation)
    out = torch.empty(n, dtype=torch.float32, device="cuda") if host else insolation
    if not host and (out.dtype != torch.float32 or out.shape != (n,)):
        raise ValueError("insolation must be a float32 array of shape (N,)")
    call("nx_interpolate_insolation", _dev.ptr(xyz), n, float(radius), _dev.ptr(tab), 1, _dev.ptr(out), 0,
         _dev.stream_handle())
    if host:
        insolation[...] = out.cpu().numpy()


def calc_daily_insolation(verts, altitudes, radius, tilt):
    """climate.calc_daily_insolation (climate.py:536-548): a new float32
    array (altitudes do not enter the result, as in the reference)."""
    host = _dev.is_host(verts)
    xyz = _dev.to_device(verts, np.float64, name="verts")
    _dev.check_vertices(xyz)
    out = torch.empty(xyz.shape[0], dtype=torch.float32, device="cuda")
    tab = _slice_tables(radius, [tilt])
    call("nx_interpolate_insolation", _dev.ptr(xyz), xyz.shape[0], float(radius), _dev.ptr(tab), 1, _dev.ptr(out), 0,
         _dev.stream_handle())
    return out.cpu().numpy() if host else out


def calc_yearly_insolation(points, height, radius, axial_tilt, snapshot=False):
    """climate.calc_yearly_insolation (climate.py:579-597): the daily tables
    of 360 orbital degrees (tilt calculate_seasonal_tilt(axial_tilt, x)),
    interpolated at every vertex and summed in binary32; a new float32 array."""
    if snapshot:
        raise NotImplementedError("insolation snapshots (PNG export) are not provided by nixis_gb300")
    host = _dev.is_host(points)
    xyz = _dev.to_device(points, np.float64, name="points")
    _dev.check_vertices(xyz)
    n = xyz.shape[0]
    tab = _slice_tables(radius, [calculate_seasonal_tilt(axial_tilt, x) for x in range(360)])
    out = torch.empty(n, dtype=torch.float32, device="cuda")
    call("nx_interpolate_insolation", _dev.ptr(xyz), n, float(radius), _dev.ptr(tab), 360, _dev.ptr(out), 0,
         _dev.stream_handle())
    return out.cpu().numpy() if host else out


def assign_surface_temp(verts, altitudes, radius, tilt):
    """climate.assign_surface_temp (climate.py:345-411): a new float32 array,
    vertex v's max(cos(|lat - tilt| * pi / 180), 0) with lat from
    util.xyz2latlon.  The reference rescales the altitudes to [0, 0]
    (alt_intensity = 0), which gives 0 at every vertex (NaN for a constant
    field), so its altitude branch (h2 > 0) is never taken; altitudes must
    still give one value per vertex, and an empty mesh raises as the
    reference's np.min does."""
    host = _dev.is_host(verts)
    xyz = _dev.to_device(verts, np.float64, name="verts")
    _dev.check_vertices(xyz)
    n = xyz.shape[0]
    if altitudes is None or len(altitudes) != n:
        raise ValueError("altitudes must hold one value per vertex")
    if n == 0:
        raise ValueError("zero-size array to reduction operation minimum which has no identity")
    out = torch.empty(n, dtype=torch.float32, device="cuda")
    call("nx_surface_temp", _dev.ptr(xyz), n, float(radius), float(tilt), _dev.ptr(out), _dev.stream_handle())
    return out.cpu().numpy() if host else out
