"""ctypes binding of libnixis_gb300.so (the C ABI in include/nixis_gb300.h).

The library is the only compute path: if it cannot be built or loaded, every
entry point raises.  There is no CPU fallback.
"""
import ctypes
import os
import threading

from . import build as _build

_p = ctypes.c_void_p
_i32 = ctypes.c_int
_i64 = ctypes.c_int64
_d = ctypes.c_double
_u64 = ctypes.c_ulonglong

# name -> (restype, argtypes); every symbol declared in include/nixis_gb300.h
SIGNATURES = {
    "nx_last_error": (ctypes.c_char_p, []),
    "nx_version": (_i32, []),
    "nx_launch_count": (_u64, []),
    "nx_perm_init": (_i32, [_i64, _p, _p]),
    "nx_fbm": (_i32, [_p, _i64, _p, _p, _i32, _p, _p, _d, _p, _p, _i32, _p, _p]),
    "nx_sample_octaves": (_i32, [_p, _i64, _p, _p, _i32, _d, _d, _d, _d, _d, _p, _p, _i32, _p]),
    "nx_noise3d_trace": (_i32, [_p, _i64, _p, _p, _d, _p, _p, _p, _p, _p]),
    "nx_icosphere_tables": (_i32, [_p, _p, _p, _p]),
    "nx_icosphere": (_i32, [_i32, _p, _p, _p]),
    "nx_adjacency_workspace_size": (ctypes.c_size_t, [_i64]),
    "nx_build_adjacency": (_i32, [_p, _i64, _i64, _p, _p, ctypes.c_size_t, _p, _p]),
    "nx_sort_adjacency": (_i32, [_p, _p, _i64, _p]),
    "nx_edge_lengths": (_i32, [_p, _p, _i64, _p, _p, _p]),
    "nx_erosion_workspace_size": (ctypes.c_size_t, [_i64, _i32]),
    "nx_erosion_ctl_init": (_i32, [_p, ctypes.c_size_t, _i32, _p]),
    "nx_erosion_load": (_i32, [_p, _p, _p, _i64, _p, _p, ctypes.c_size_t, _p]),
    "nx_erosion_steps": (_i32, [_p, _p, _i64, _p, _p, _i32, ctypes.c_float, _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "nx_erosion_batch": (_i32, [_p, _p, _i32, _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "nx_erosion_store": (_i32, [_p, _i64, _p, _p, _p, _p, _p]),
    "nx_steepest_descent": (_i32, [_p, _p, _i64, _p, _p, _p]),
    "nx_insolation_plan": (_i32, [_p, _i32, _p, _i32, _p, _p, _p]),
    "nx_insolation": (_i32, [_p, _i64, _d, _p, _i32, _i32, _i32, _p, _i32, _p]),
    "nx_insolation_batch": (_i32, [_p, _p, _i32, _p, _i32, _i32, _i32, _p, _p]),
    "nx_fbm_planet_fill": (_i32, [_p, _i32, _p, _p, _d]),
    "nx_fbm_chunk_size": (_i32, []),
    "nx_fbm_batch": (_i32, [_p, _p, _i32, _p, _p]),
    "nx_fbm_pair": (_i32, [_p, _i64, _p, _p, _i32, _p, _p, _d, _d, _p, _p, _i32, _p, _p, _p]),
    "nx_erosion_init_batch": (_i32, [_p, _p, _i32, _p, _p, _d, _d, _d, _p, _p, _p]),
    "nx_erosion_heights_batch": (_i32, [_p, _p, _i32, _p, _p, _p, _p]),
    "nx_erosion_run_batch": (_i32, [_p, _p, _i32, _p, _p, _d, _d, _d, _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "nx_erosion_steps_noalloc": (_i32, [_p, _p, _i64, _p, _i32, ctypes.c_float, _p, _p, _p]),
    "nx_erosion_tick": (_i32, [_p, _p, _i32, _i32, _p, _p, _p, ctypes.c_size_t, _i32, _i32, _p]),
    "nx_erosion_finish": (_i32, [_p, _i32, _p, _p]),
    "nx_erosion_finish_passes": (_i32, [_p, _i32, _p, _p]),
    "nx_erosion_ticks": (_i32, [_p, _p, _i32, _i32, _i32, _p, _p, _p, ctypes.c_size_t, _i32, _i32, _p]),
    "nx_erosion_passes": (_i32, [_p, _p, _i32, _i32, _i32, _p, _p, _p, ctypes.c_size_t, _i32, _i32, _p]),
    "nx_erosion_npass": (_i32, [_i32]),
    "nx_shape_workspace_size": (ctypes.c_size_t, [_i64]),
    "nx_insolation_slices": (_i32, [_p, _i32, _d, _p, _p]),
    "nx_make_ll": (_i32, [_i32, _i32, _d, _p, _p]),
    "nx_nearest3": (_i32, [_i32, _p, _p, _i64, _p, _i64, _p, _p, _p]),
    "nx_sample_gray": (_i32, [_p, _p, _i64, _p, _i64, _p, _p, _p]),
    "nx_interpolate_insolation": (_i32, [_p, _i64, _d, _p, _i32, _p, _i32, _p]),
    "nx_surface_temp": (_i32, [_p, _i64, _d, _d, _p, _p]),
    "nx_rescale": (_i32, [_p, _i64, _d, _d, _d, _i32, _d, _i32, _d, _i32, _p, _p, ctypes.c_size_t, _p]),
    "nx_power_rescale": (_i32, [_p, _i64, _p, _i32, _d, _p, _p, ctypes.c_size_t, _p]),
    "nx_elevation_mask": (_i32, [_p, _i64, _d, _p, _p]),
    "nx_shape_heights": (_i32, [_p, _i64, _d, _d, _d, _p, _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "nx_tiling_shape": (_i32, [_i32, _i32, _i32, _p, _p, _p]),
    "nx_erosion_tb_config": (_i32, [_i32, _i32, _i32, _i32]),
    "nx_tiling_build": (_i32, [_i32, _i32, _i32, _p, _p, _p, _p, _p, _p, _p, _p]),
}

NX_MAX_OCTAVES = 32


class FbmPlanet(ctypes.Structure):
    """nx_fbm_planet (include/nixis_gb300.h)."""
    _fields_ = [("xyz", ctypes.c_void_p), ("n", ctypes.c_int64), ("perm", ctypes.c_void_p),
                ("pgi", ctypes.c_void_p), ("out", ctypes.c_void_p), ("minmax", ctypes.c_void_p),
                ("n_octaves", ctypes.c_int32), ("chunk0", ctypes.c_int32), ("pow2", ctypes.c_int32),
                ("norm_mask", ctypes.c_uint32),
                ("s1", ctypes.c_float * NX_MAX_OCTAVES), ("s2", ctypes.c_float * NX_MAX_OCTAVES),
                ("s3", ctypes.c_float * NX_MAX_OCTAVES), ("amp_hi", ctypes.c_float * NX_MAX_OCTAVES),
                ("amp_lo", ctypes.c_float * NX_MAX_OCTAVES), ("s", ctypes.c_double * NX_MAX_OCTAVES)]


class InsoPlanet(ctypes.Structure):
    """nx_inso_planet (include/nixis_gb300.h)."""
    _fields_ = [("xyz", ctypes.c_void_p), ("n", ctypes.c_int64), ("vbeg", ctypes.c_int64),
                ("radius", ctypes.c_double)]


class ErosionPlanet(ctypes.Structure):
    """nx_erosion_planet (include/nixis_gb300.h)."""
    _fields_ = [("vbeg", ctypes.c_int64), ("n", ctypes.c_int64), ("nbr", ctypes.c_void_p),
                ("edge", ctypes.c_void_p), ("iters", ctypes.c_int32), ("rain", ctypes.c_float),
                ("t_start", ctypes.c_int32), ("slot", ctypes.c_int32), ("tiling", ctypes.c_void_p),
                ("ntiles", ctypes.c_int32), ("maxnl", ctypes.c_int32), ("maxc", ctypes.c_int32),
                ("pad", ctypes.c_int32)]


class Tiling(ctypes.Structure):
    """nx_tiling (include/nixis_gb300.h)."""
    _fields_ = [("ntiles", ctypes.c_int32), ("rings", ctypes.c_int32), ("nmax", ctypes.c_int32),
                ("cmax", ctypes.c_int32), ("counts", ctypes.c_void_p), ("ids", ctypes.c_void_p),
                ("lnbr", ctypes.c_void_p), ("ledge", ctypes.c_void_p)]

_lock = threading.Lock()
_LIB = None


class NxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"nixis_gb300 error {code}: {msg}")
        self.code = code


def lib():
    """Load (building first if needed) the CUDA library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    with _lock:
        if _LIB is None:
            if os.environ.get("NIXIS_GB300_NO_BUILD") != "1":
                _build.build()
            if not os.path.exists(_build.LIB):
                raise RuntimeError(f"{_build.LIB} is missing; build it with python -m nixis_gb300.build")
            L = ctypes.CDLL(_build.LIB)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _LIB = L
    return _LIB


def check(rc):
    if rc != 0:
        raise NxError(rc, lib().nx_last_error().decode(errors="replace"))


def call(name, *args):
    check(getattr(lib(), name)(*args))


def launch_count():
    return int(lib().nx_launch_count())
