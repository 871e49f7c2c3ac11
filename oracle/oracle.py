"""ctypes front end for the CPU oracle (nx_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``, always as the checker or the
timed CPU baseline, never as part of the product path.

Each wrapper takes and returns numpy arrays and mirrors one reference function
(see the citations in nx_oracle.c).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libnx_oracle.so")
_lib = None

_d = ctypes.c_double
_i64 = ctypes.c_int64
_i32 = ctypes.c_int
_p = ctypes.c_void_p


def build(force=False):
    """Compile nx_oracle.c with the committed Makefile."""
    src = os.path.join(_HERE, "nx_oracle.c")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        sig = {
            "nxo_perm_init": (_i32, [_i64, _p, _p]),
            "nxo_noise3d": (_d, [_d, _d, _d, _p, _p]),
            "nxo_noise3d_trace": (_d, [_d, _d, _d, _p, _p, _p, _p]),
            "nxo_noise3d_batch": (None, [_p, _i64, _p, _p, _p, _p, _p]),
            "nxo_sample_noise": (None, [_p, _i64, _p, _p, _d, _d, _d, _p]),
            "nxo_sample_octaves": (None, [_p, _i64, _p, _p, _p, _i32, _d, _d, _d, _d, _d]),
            "nxo_make_bool_elevation_mask": (None, [_p, _i64, _d, _p]),
            "nxo_erosion_iteration3": (_i32, [_p, _p, _i64, _p, _p, _p]),
            "nxo_erode_terrain3": (_i32, [_p, _p, _i64, _p, _i32]),
            "nxo_erosion_iteration3_pair": (None, [_p, _p, _i64, _p, ctypes.c_float, _p]),
            "nxo_find_lowest": (_i32, [_i64, _p, _p]),
            "nxo_day2deg": (_d, [_d, _d]),
            "nxo_calculate_seasonal_tilt": (_d, [_d, _d]),
            "nxo_sample_insolation": (None, [_p, _p, _i64, _d, _d, _d]),
            "nxo_sample_insolation_f64": (None, [_p, _p, _i64, _d, _d, _d]),
            "nxo_annual_insolation": (None, [_p, _i64, _d, _d, _i32, _i32, _i32, _p, _p]),
            "nxo_build_adjacency": (_i32, [_p, _i64, _p]),
            "nxo_sort_adjacency": (_i32, [_p, _i64]),
            "nxo_rescale": (None, [_p, _i64, _d, _d, _p]),
            "nxo_rescale_full": (None, [_p, _i64, _d, _d, _d, ctypes.c_int, _d, ctypes.c_int, _d, ctypes.c_int, _p]),
            "nxo_find_percent_val": (_d, [_d, _d, _d]),
            "nxo_power_rescale": (None, [_p, _i64, _p, ctypes.c_int, _d, _p]),
            "nxo_shape_heights": (_d, [_p, _i64, _d, _d, _d, _p, _p, _p]),
            "nxo_calc_insolation_slice": (None, [_d, _d, _p]),
            "nxo_interpolate_insolation": (None, [_p, _i64, _p, _p, _d]),
            "nxo_calc_yearly_insolation": (None, [_p, _i64, _d, _d, _p]),
            "nxo_assign_surface_temp": (None, [_p, _i64, _d, _d, _p]),
            "nxo_make_ll": (None, [ctypes.c_int, ctypes.c_int, _d, _p]),
            "nxo_nearest3": (None, [_p, _i64, _p, _i64, _p, _p]),
            "nxo_make_gray": (None, [_p, _p, _i64, _p, _p]),
            "nxo_num_threads": (_i32, []),
            "nxo_icosphere": (_i32, [_i32, _p, _p, _p, _p, _p, _p]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def num_threads():
    return lib().nxo_num_threads()


def init(seed=0):
    """opensimplex.init -> (perm int32[256], perm_grad_index_3D int32[256])"""
    perm = np.zeros(256, np.int32)
    pgi = np.zeros(256, np.int32)
    lib().nxo_perm_init(int(seed), _ptr(perm), _ptr(pgi))
    return perm, pgi


def noise3d(x, y, z, perm, pgi):
    perm = _c(perm, np.int32)
    pgi = _c(pgi, np.int32)
    return lib().nxo_noise3d(float(x), float(y), float(z), _ptr(perm), _ptr(pgi))


def noise3d_batch(xyz, perm, pgi, trace=False):
    """noise3d at each row of xyz.  With trace=True also returns the (N,10)
    lattice decisions [xsb, ysb, zsb, region, ext0 xyz, ext1 xyz] and the
    (N,25) hashed lattice points [count, x0, y0, z0, ...] in call order."""
    xyz = _c(xyz, np.float64)
    perm = _c(perm, np.int32)
    pgi = _c(pgi, np.int32)
    n = xyz.shape[0]
    out = np.zeros(n, np.float64)
    tr = np.zeros((n, 10), np.int32) if trace else None
    calls = np.zeros((n, 25), np.int32) if trace else None
    lib().nxo_noise3d_batch(_ptr(xyz), n, _ptr(perm), _ptr(pgi), _ptr(out),
                            _ptr(tr) if trace else None, _ptr(calls) if trace else None)
    return (out, tr, calls) if trace else out


def sample_noise(verts, perm, pgi, n_roughness=1, n_strength=0.2, radius=1):
    verts = _c(verts, np.float64)
    out = np.zeros(len(verts), np.float64)
    lib().nxo_sample_noise(_ptr(verts), len(verts), _ptr(_c(perm, np.int32)), _ptr(_c(pgi, np.int32)),
                           float(n_roughness), float(n_strength), float(radius), _ptr(out))
    return out


def sample_octaves(verts, elevations, perm, pgi, n_octaves=1, n_init_roughness=1.5,
                   n_init_strength=0.4, n_roughness=2.0, n_persistence=0.5, world_radius=1.0):
    verts = _c(verts, np.float64)
    if elevations is None:
        elev = np.zeros(len(verts), np.float64)
    else:
        elev = _c(elevations, np.float64).copy()
    lib().nxo_sample_octaves(_ptr(verts), len(verts), _ptr(elev), _ptr(_c(perm, np.int32)),
                             _ptr(_c(pgi, np.int32)), int(n_octaves), float(n_init_roughness),
                             float(n_init_strength), float(n_roughness), float(n_persistence),
                             float(world_radius))
    return elev


def erosion_iteration3(verts, neighbors, r_buff, wat, sed):
    """In place on r_buff, wat, sed (float64, C-contiguous), like the reference."""
    verts = _c(verts, np.float64)
    nbr = _c(neighbors, np.int32)
    for a in (r_buff, wat, sed):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    rc = lib().nxo_erosion_iteration3(_ptr(verts), _ptr(nbr), len(nbr), _ptr(r_buff), _ptr(wat), _ptr(sed))
    if rc:
        raise MemoryError("oracle erosion_iteration3: allocation failed")


def erode_terrain3(nodes, neighbors, heights, num_iter=1):
    nodes = _c(nodes, np.float64)
    nbr = _c(neighbors, np.int32)
    assert heights.dtype == np.float64 and heights.flags.c_contiguous
    rc = lib().nxo_erode_terrain3(_ptr(nodes), _ptr(nbr), len(nbr), _ptr(heights), int(num_iter))
    if rc:
        raise MemoryError("oracle erode_terrain3: allocation failed")


def erosion_iteration3_pair(edge_len, neighbors, st, rain=0.0):
    """The update with the GPU kernel's arithmetic on rows (h_hi, h_lo,
    w_hi, w_lo, s_hi, s_lo, 0, 0) (float32 (N,8)) with edge lengths as
    (hi, lo) pairs (float32 (N,6,2)); returns the new rows."""
    el = _c(edge_len, np.float32)
    nbr = _c(neighbors, np.int32)
    st = _c(st, np.float32)
    out = np.empty_like(st)
    lib().nxo_erosion_iteration3_pair(_ptr(el), _ptr(nbr), len(nbr), _ptr(st), float(np.float32(rain)), _ptr(out))
    return out


def pair_rows(h, w, s):
    """float64 fields -> (N,8) float32 state rows (each field split into a
    binary32 pair, as the GPU loads them)."""
    st = np.zeros((len(h), 8), np.float32)
    for c, v in ((0, h), (2, w), (4, s)):
        v = np.asarray(v, np.float64)
        st[:, c] = v.astype(np.float32)
        st[:, c + 1] = (v - st[:, c].astype(np.float64)).astype(np.float32)
    return st


def split_heights(h):
    """float64 heights -> (h_hi, h_lo) float32 pairs, as the GPU loads them."""
    h = np.asarray(h, np.float64)
    hi = h.astype(np.float32)
    lo = (h - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


def find_lowest(vert, nbr6, height):
    nbr6 = _c(nbr6, np.int32)
    h = _c(height, np.float64)
    r = lib().nxo_find_lowest(int(vert), _ptr(nbr6), _ptr(h))
    return None if r < 0 else r


def day2deg(year_length, day):
    return lib().nxo_day2deg(float(year_length), float(day))


def calculate_seasonal_tilt(axial_tilt, degrees):
    return lib().nxo_calculate_seasonal_tilt(float(axial_tilt), float(degrees))


def sample_insolation(arr, verts, radius, rotation, tilt):
    """In place on arr (float32 like the reference, or float64 for the exact sum)."""
    verts = _c(verts, np.float64)
    assert arr.flags.c_contiguous
    if arr.dtype == np.float32:
        lib().nxo_sample_insolation(_ptr(arr), _ptr(verts), len(verts), float(radius), float(rotation), float(tilt))
    elif arr.dtype == np.float64:
        lib().nxo_sample_insolation_f64(_ptr(arr), _ptr(verts), len(verts), float(radius), float(rotation), float(tilt))
    else:
        raise TypeError("arr must be float32 or float64")


def annual_insolation(verts, radius, axial_tilt=23.44, year_length=365, days=365, hours=24,
                      with_f32=False):
    """Sum over days x hours sun positions; float64 sum (and the float32
    running sum the reference would keep, if with_f32)."""
    verts = _c(verts, np.float64)
    acc = np.zeros(len(verts), np.float64)
    acc32 = np.zeros(len(verts), np.float32) if with_f32 else None
    lib().nxo_annual_insolation(_ptr(verts), len(verts), float(radius), float(axial_tilt),
                                int(year_length), int(days), int(hours), _ptr(acc),
                                _ptr(acc32) if with_f32 else None)
    return (acc, acc32) if with_f32 else acc


def build_adjacency(triangles):
    tris = _c(triangles, np.int32)
    nv = (len(tris) + 4) // 2
    adj = np.full((nv, 6), -1, np.int32)
    if lib().nxo_build_adjacency(_ptr(tris), len(tris), _ptr(adj)):
        raise ValueError("build_adjacency: a vertex has more than 6 neighbours")
    return adj


def sort_adjacency(adj):
    """In place, like the reference."""
    assert adj.dtype == np.int32 and adj.flags.c_contiguous
    if lib().nxo_sort_adjacency(_ptr(adj), len(adj)):
        raise MemoryError("sort_adjacency: allocation failed")


def rescale(x, lower, upper):
    x = _c(x, np.float64)
    out = np.empty_like(x)
    lib().nxo_rescale(_ptr(x), len(x), float(lower), float(upper), _ptr(out))
    return out


_FORMS = {None: 0, "lower": 2, "upper": 3}


def rescale_full(x, lower, upper, mid=None, mode=None, u_min=None, u_max=None):
    """util.rescale (util.py:110-176) in every form; returns a new array, or
    x itself when a mode is given without mid (as the reference does)."""
    x = _c(x, np.float64)
    if mode is not None and mid is None:
        return x
    form = 1 if (mode is None and mid is not None) else _FORMS[mode]
    out = np.empty_like(x)
    lib().nxo_rescale_full(_ptr(x), len(x), float(lower), float(upper), float(mid or 0.0), form,
                           float(u_min or 0.0), int(u_min is not None), float(u_max or 0.0), int(u_max is not None),
                           _ptr(out))
    return out


def find_percent_val(minval, maxval, percent):
    return lib().nxo_find_percent_val(float(minval), float(maxval), float(percent))


def power_rescale(x, mask=None, mode=None, power=1.0):
    x = _c(x, np.float64)
    m = _c(np.zeros(len(x), np.uint8) if mask is None else np.asarray(mask).astype(np.uint8), np.uint8)
    out = np.empty_like(x)
    lib().nxo_power_rescale(_ptr(x), len(x), _ptr(m), -1 if mode is None else int(mode), float(power), _ptr(out))
    return out


def shape_heights(h, min_alt=-4000.0, max_alt=8850.0, ocean_percent=55.0):
    """nixis.py:332-364 -> (heights, ocean mask, ocean level)."""
    h = _c(h, np.float64)
    out, tmp = np.empty_like(h), np.empty_like(h)
    mask = np.empty(len(h), np.uint8)
    level = lib().nxo_shape_heights(_ptr(h), len(h), float(min_alt), float(max_alt), float(ocean_percent), _ptr(out),
                                    _ptr(tmp), _ptr(mask))
    return out, mask, level


def calc_insolation_slice(radius, tilt):
    out = np.empty(181, np.float32)
    lib().nxo_calc_insolation_slice(float(radius), float(tilt), _ptr(out))
    return out


def interpolate_insolation(verts, table, radius):
    v = _c(verts, np.float64)
    t = _c(table, np.float32)
    out = np.empty(len(v), np.float32)
    lib().nxo_interpolate_insolation(_ptr(v), len(v), _ptr(t), _ptr(out), float(radius))
    return out


def assign_surface_temp(verts, radius, tilt):
    v = _c(verts, np.float64)
    out = np.empty(len(v), np.float32)
    lib().nxo_assign_surface_temp(_ptr(v), len(v), float(radius), float(tilt), _ptr(out))
    return out


def calc_yearly_insolation(verts, radius, axial_tilt):
    v = _c(verts, np.float64)
    out = np.empty(len(v), np.float32)
    lib().nxo_calc_yearly_insolation(_ptr(v), len(v), float(radius), float(axial_tilt), _ptr(out))
    return out


def make_ll_arr(width, height, radius):
    out = np.empty((height, width, 3), np.float64)
    lib().nxo_make_ll(int(width), int(height), float(radius), _ptr(out))
    return out


def nearest3(verts, queries):
    """(dists (..., 3), indices (..., 3)) of the 3 nearest vertices, exact."""
    v = _c(verts, np.float64)
    q = _c(np.asarray(queries, np.float64).reshape(-1, 3), np.float64)
    d = np.empty((len(q), 3), np.float64)
    i = np.empty((len(q), 3), np.int64)
    lib().nxo_nearest3(_ptr(v), len(v), _ptr(q), len(q), _ptr(d), _ptr(i))
    shape = np.asarray(queries).shape[:-1] + (3,)
    return d.reshape(shape), i.reshape(shape)


def make_gray_array(width, height, dists, nbrs, colors):
    d = _c(np.asarray(dists, np.float64).reshape(-1, 3), np.float64)
    n = _c(np.asarray(nbrs, np.int64).reshape(-1, 3), np.int64)
    c = _c(colors, np.float64)
    out = np.empty(len(d), np.float64)
    lib().nxo_make_gray(_ptr(d), _ptr(n), len(d), _ptr(c), _ptr(out))
    return out.reshape(height, width)


def icosphere(k, with_tris=True):
    """CPU icosphere with the GPU generator's layout (vertices, triangles)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "_ico_tables", os.path.join(os.path.dirname(_HERE), "nixis_gb300", "icosphere.py"))
    ico = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ico)
    k = int(k)
    nv, nt = ico.counts(k)
    c = _c(ico.corners(), np.float64)
    f = _c(ico.FACES, np.int32)
    fe = _c(ico.face_edge_table(), np.int32)
    e = _c(ico.edges(), np.int32)
    xyz = np.empty((nv, 3), np.float64)
    tris = np.empty((nt, 3), np.int32) if with_tris else None
    if lib().nxo_icosphere(k, _ptr(c), _ptr(f), _ptr(fe), _ptr(e), _ptr(xyz), _ptr(tris) if with_tris else None):
        raise ValueError("bad divisions")
    return xyz, tris


def planet_mesh(k):
    """(vertices, neighbour table) for divisions k, all on the CPU."""
    xyz, tris = icosphere(k)
    adj = build_adjacency(tris)
    sort_adjacency(adj)
    return xyz, adj
