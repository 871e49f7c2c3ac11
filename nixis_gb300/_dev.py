"""Device-buffer plumbing: numpy arrays are staged through pinned host memory
to CUDA tensors and back; CUDA tensors are used in place (zero copy)."""
import numpy as np
import torch

_NP2T = {np.float64: torch.float64, np.float32: torch.float32, np.int32: torch.int32,
         np.int64: torch.int64, np.uint8: torch.uint8}


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("nixis_gb300 needs a CUDA GPU (sm_103a); none is available")


def stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes_void(s.cuda_stream)


def ctypes_void(v):
    import ctypes
    return ctypes.c_void_p(int(v))


def ptr(t):
    import ctypes
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def is_host(a):
    return isinstance(a, np.ndarray)


def to_device(a, dtype, shape=None, name="array"):
    """Return a contiguous CUDA tensor of `dtype` holding `a` (numpy or torch)."""
    require_cuda()
    tdt = _NP2T[np.dtype(dtype).type]
    if isinstance(a, torch.Tensor):
        t = a
        if t.device.type != "cuda":
            t = t.to("cuda", non_blocking=False)
        if t.dtype != tdt:
            t = t.to(tdt)
        t = t.contiguous()
    else:
        arr = np.ascontiguousarray(a, dtype=dtype)
        t = torch.from_numpy(arr).pin_memory().to("cuda", non_blocking=True)
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name}: expected shape {tuple(shape)}, got {tuple(t.shape)}")
    return t


def check_vertices(v, name="verts"):
    if v.ndim != 2 or v.shape[1] != 3:
        raise ValueError(f"{name}: expected shape (N, 3), got {tuple(v.shape)}")


def check_tables(perm, pgi):
    p = np.asarray(perm.cpu() if isinstance(perm, torch.Tensor) else perm)
    g = np.asarray(pgi.cpu() if isinstance(pgi, torch.Tensor) else pgi)
    if p.shape != (256,) or g.shape != (256,):
        raise ValueError("perm and perm_grad_index_3D must have 256 entries")
    if p.min() < 0 or p.max() > 255 or g.min() < 0 or g.max() > 69 or np.any(g % 3):
        raise ValueError("perm / perm_grad_index_3D are not tables made by init()")
