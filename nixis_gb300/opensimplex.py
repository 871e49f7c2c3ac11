"""Drop-in for the reference's opensimplex module (3-D path).

``init`` (opensimplex.py:90-107) runs on the host through the C ABI and is
bit-exact.  ``noise3d`` / ``noisearr3d`` (opensimplex.py:257-759) evaluate on
the GPU; values are binary32 with the lattice decisions equal to binary64's.
The 2-D and 4-D generators of the reference are not part of this path.
"""
import ctypes

import numpy as np
import torch

from . import _dev
from ._lib import call

DEFAULT_SEED = 0
STRETCH_CONSTANT_3D = -1.0 / 6
SQUISH_CONSTANT_3D = 1.0 / 3
NORM_CONSTANT_3D = 103

# opensimplex.py:51-60
GRADIENTS_3D = (
    -11, 4, 4, -4, 11, 4, -4, 4, 11,
    11, 4, 4, 4, 11, 4, 4, 4, 11,
    -11, -4, 4, -4, -11, 4, -4, -4, 11,
    11, -4, 4, 4, -11, 4, 4, -4, 11,
    -11, 4, -4, -4, 11, -4, -4, 4, -11,
    11, 4, -4, 4, 11, -4, 4, 4, -11,
    -11, -4, -4, -4, -11, -4, -4, -4, -11,
    11, -4, -4, 4, -11, -4, 4, -4, -11,
)


def init(seed=DEFAULT_SEED):
    """opensimplex.init: (perm, perm_grad_index_3D), two int32[256] arrays."""
    perm = np.zeros(256, np.int32)
    pgi = np.zeros(256, np.int32)
    call("nx_perm_init", int(seed), perm.ctypes.data_as(ctypes.c_void_p), pgi.ctypes.data_as(ctypes.c_void_p))
    return perm, pgi


def _tables_dev(perm, pgi):
    return _dev.to_device(perm, np.int32, (256,), "perm"), _dev.to_device(pgi, np.int32, (256,), "pgi")


def noise3d_trace(points, perm, pgi, scale=1.0, stream=None):
    """noise3d at each row of `points` (float64 (N,3), numpy or CUDA tensor)
    with its integer decisions.  Returns CUDA tensors (value float32 (N,),
    trace int32 (N,10), slots int32 (N,9,5)) and the number of points whose
    decisions took the binary64 path."""
    xyz = _dev.to_device(points, np.float64, name="points")
    _dev.check_vertices(xyz, "points")
    n = xyz.shape[0]
    p, g = _tables_dev(perm, pgi)
    val = torch.empty(n, dtype=torch.float32, device="cuda")
    tr = torch.empty((n, 10), dtype=torch.int32, device="cuda")
    sl = torch.empty((n, 9, 5), dtype=torch.int32, device="cuda")
    nfb = torch.zeros(1, dtype=torch.int64, device="cuda")
    call("nx_noise3d_trace", _dev.ptr(xyz), n, _dev.ptr(p), _dev.ptr(g), float(scale), _dev.ptr(val),
         _dev.ptr(tr), _dev.ptr(sl), _dev.ptr(nfb), _dev.stream_handle(stream))
    return val, tr, sl, int(nfb.item())


def noisearr3d(x, y, z, perm, perm_grad_index_3D):
    """opensimplex.noisearr3d: noise3d over arrays x, y, z (float64 result)."""
    pts = np.stack([np.asarray(x, np.float64).ravel(), np.asarray(y, np.float64).ravel(),
                    np.asarray(z, np.float64).ravel()], axis=1)
    val, _, _, _ = noise3d_trace(pts, perm, perm_grad_index_3D)
    return val.double().cpu().numpy()


def noise3d(x, y, z, perm, perm_grad_index_3D):
    """opensimplex.noise3d at one point (a GPU launch per call; use
    noisearr3d or terrain.sample_noise for arrays)."""
    return float(noisearr3d([x], [y], [z], perm, perm_grad_index_3D)[0])
