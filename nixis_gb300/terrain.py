"""Drop-in for the reference's terrain module (terrain.py:12-72).

Arrays may be numpy (copied to the GPU and back, like-for-like with the
reference) or CUDA tensors (used in place).  The fBm is one fused kernel over
all octaves.  Float64 results (the reference's dtype) come from the
pair-precision kernel (nx_fbm_pair: within ~1e-13 of the binary64 sums,
close enough that erosion run on them keeps the reference's flow choices);
float32 results from the binary32 kernel (nx_fbm, ~1e-6 of the range).
"""
import ctypes

import numpy as np
import torch

from . import _dev
from ._lib import call, NxError  # noqa: F401


def _octave_args(n_octaves, n_init_roughness, n_init_strength, n_roughness, n_persistence, world_radius):
    # terrain.py:35-46: per-octave scale f/R and strength a/R in binary64
    scale, strength = [], []
    f, a = n_init_roughness, n_init_strength
    for _ in range(int(n_octaves)):
        scale.append(f / world_radius)
        strength.append(a / world_radius)
        f *= n_roughness
        a *= n_persistence
    return scale, strength


def fbm(verts, perm, pgi, scale, strength, radius, out=None, accumulate=False, out_dtype=torch.float64,
        stream=None, count_fallbacks=False):
    """Sum over octaves o of (noise3d(v * scale[o]) + 1) * 0.5 * strength[o] * radius,
    in pair precision for a float64 `out` (the default) and in binary32 for a
    float32 one.

    verts: float64 (N,3) CUDA tensor (or numpy).  `out`, if given, is a CUDA
    tensor (float64 or float32) written (or added to, with accumulate=True).
    Returns (out, n_fallback) where n_fallback counts vertex-octaves decided
    on the binary64 path (only when count_fallbacks)."""
    xyz = _dev.to_device(verts, np.float64, name="verts")
    _dev.check_vertices(xyz)
    n = xyz.shape[0]
    p = _dev.to_device(perm, np.int32, (256,), "perm")
    g = _dev.to_device(pgi, np.int32, (256,), "pgi")
    if out is None:
        out = torch.zeros(n, dtype=out_dtype, device="cuda")
        accumulate = False
    if out.shape != (n,) or not out.is_cuda or not out.is_contiguous():
        raise ValueError("out must be a contiguous CUDA tensor of shape (N,)")
    no = len(scale)
    sc = (ctypes.c_double * max(no, 1))(*scale)
    st = (ctypes.c_double * max(no, 1))(*strength)
    nfb = torch.zeros(1, dtype=torch.int64, device="cuda") if count_fallbacks else None
    if out.dtype == torch.float64:
        # pair precision; the octaves' amplitudes set its per-octave form (amp_ref 0)
        call("nx_fbm_pair", _dev.ptr(xyz), n, _dev.ptr(p), _dev.ptr(g), no, sc, st, float(radius), 0.0, None,
             _dev.ptr(out), 1 if accumulate else 0, None, _dev.ptr(nfb), _dev.stream_handle(stream))
    elif out.dtype == torch.float32:
        call("nx_fbm", _dev.ptr(xyz), n, _dev.ptr(p), _dev.ptr(g), no, sc, st, float(radius), None,
             _dev.ptr(out), 1 if accumulate else 0, _dev.ptr(nfb), _dev.stream_handle(stream))
    else:
        raise ValueError("out must be float64 or float32")
    return out, (int(nfb.item()) if count_fallbacks else None)


def sample_noise(verts, perm, pgi, n_roughness=1, n_strength=0.2, radius=1):
    """terrain.sample_noise (terrain.py:12-28): a new float64 array of
    (noise3d(v * n_roughness) + 1) * 0.5 * n_strength * radius."""
    host = _dev.is_host(verts)
    out, _ = fbm(verts, perm, pgi, [float(n_roughness)], [float(n_strength)], float(radius))
    return out.cpu().numpy() if host else out


def sample_octaves(verts, elevations, perm, pgi, n_octaves=1, n_init_roughness=1.5, n_init_strength=0.4,
                   n_roughness=2.0, n_persistence=0.5, world_radius=1.0):
    """terrain.sample_octaves (terrain.py:32-59).  With `elevations` None a new
    float64 array is returned; otherwise the octaves are added to it in place
    and it is returned (numpy arrays are updated in place too)."""
    scale, strength = _octave_args(n_octaves, n_init_roughness, n_init_strength, n_roughness,
                                   n_persistence, world_radius)
    host = _dev.is_host(verts) if elevations is None else _dev.is_host(elevations)
    if elevations is None:
        out, _ = fbm(verts, perm, pgi, scale, strength, world_radius)
        return out.cpu().numpy() if host else out
    if host:
        if elevations.dtype != np.float64 or not elevations.flags.c_contiguous:
            raise ValueError("elevations must be a C-contiguous float64 array")
        dev = _dev.to_device(elevations, np.float64)
        fbm(verts, perm, pgi, scale, strength, world_radius, out=dev, accumulate=True)
        elevations[...] = dev.cpu().numpy()
        return elevations
    fbm(verts, perm, pgi, scale, strength, world_radius, out=elevations, accumulate=True)
    return elevations


def make_bool_elevation_mask(height, mask_elevation):
    """terrain.make_bool_elevation_mask (terrain.py:61-72): height <=
    mask_elevation, on the GPU (see util.make_bool_elevation_mask)."""
    from .util import make_bool_elevation_mask as _mask
    return _mask(height, mask_elevation)
