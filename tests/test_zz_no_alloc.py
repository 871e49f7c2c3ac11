"""The no-allocation erosion entry point against the allocating one.

nx_erosion_steps_noalloc serves callers that cannot allocate device memory
(inside another application's memory pool, or in loops where the device
synchronisation of cudaMalloc/cudaFree is not acceptable): it keeps its
scratch in a fixed array inside the library.  This file is collected last so
a run that stops at its first failure has run every other test before it.
Both calls go through the C ABI; the second call runs on different inputs
after the first one left its contents in the shared scratch.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _state(pts, seed, octaves):
    perm, pgi = O.init(seed)
    h = O.rescale(O.sample_octaves(pts, None, perm, pgi, octaves, 1.0, 1.0, 2.0, 0.5, 1.0), -8000.0, 8000.0)
    st = O.pair_rows(h, np.full(len(pts), 1e-3), np.zeros(len(pts)))
    return torch.from_numpy(st).cuda()


def _allocating(m, st, iters, rain, with_mass=True):
    from nixis_gb300 import _dev, _lib
    n = m.n
    st = st.clone()
    tmp = torch.empty_like(st)
    ws = torch.zeros(int(_lib.lib().nx_erosion_workspace_size(n, 1)), dtype=torch.uint8, device="cuda")
    pd = torch.zeros(ctypes.sizeof(_lib.ErosionPlanet), dtype=torch.uint8, device="cuda")
    mass = torch.empty((max(iters, 1), 3), dtype=torch.float64, device="cuda") if with_mass else None
    _lib.call("nx_erosion_ctl_init", _dev.ptr(ws), ws.numel(), 1, _dev.stream_handle())
    _lib.call("nx_erosion_steps", _dev.ptr(m.nbr), _dev.ptr(m.edge), n, _dev.ptr(st), _dev.ptr(tmp), iters,
              ctypes.c_float(rain), _dev.ptr(pd), _dev.ptr(mass) if with_mass else None, None, _dev.ptr(ws),
              ws.numel(), _dev.stream_handle())
    K = int(ws[:32].view(torch.int32)[3].item())
    return st, (mass[:iters] if with_mass else None), K


def _noalloc(m, st, iters, rain, with_mass=True, with_status=True):
    from nixis_gb300 import _dev, _lib
    st = st.clone()
    mass = torch.empty((max(iters, 1), 3), dtype=torch.float64, device="cuda") if with_mass else None
    status = torch.full((2,), -7, dtype=torch.int32, device="cuda") if with_status else None
    _lib.call("nx_erosion_steps_noalloc", _dev.ptr(m.nbr), _dev.ptr(m.edge), m.n, _dev.ptr(st), iters,
              ctypes.c_float(rain), _dev.ptr(mass) if with_mass else None,
              _dev.ptr(status) if with_status else None, _dev.stream_handle())
    return st, (mass[:iters] if with_mass else None), (status.cpu().numpy() if with_status else None)


def test_noalloc_matches_allocating_entry_point_twice():
    from nixis_gb300 import mesh
    m = mesh.PlanetMesh(100)                 # 100,002 vertices
    cases = [(_state(m.xyz.cpu().numpy(), 3, 10), 37, 0.0),
             (_state(m.xyz.cpu().numpy(), 8, 6), 20, 0.3 / 320)]
    for st, iters, rain in cases:            # two calls in a row
        a, ma, Ka = _allocating(m, st, iters, rain)
        b, mb, status = _noalloc(m, st, iters, rain)
        torch.cuda.synchronize()
        # same kernels and arithmetic: the tolerance (1e-10 of max|field|) is met bit for bit
        assert torch.equal(a, b)
        assert torch.equal(ma, mb)
        assert status[0] == Ka and status[1] == 0


def test_noalloc_without_mass_sums_or_status_matches_allocating_entry_point():
    """mass_dev and status_dev are optional: without them the run takes the
    same per-iteration kernel and gives the same bits as the allocating
    entry point called without mass sums, and as a call with them."""
    from nixis_gb300 import mesh
    m = mesh.PlanetMesh(100)
    st = _state(m.xyz.cpu().numpy(), 5, 9)
    for iters in (13, 8):                   # two calls in a row, odd and even counts
        a, _, _ = _allocating(m, st, iters, 0.0, with_mass=False)
        b, _, _ = _noalloc(m, st, iters, 0.0, with_mass=False, with_status=False)
        c, _, _ = _noalloc(m, st, iters, 0.0)
        torch.cuda.synchronize()
        assert torch.equal(a, b)
        assert torch.equal(b, c)


def test_noalloc_rejects_meshes_above_its_fixed_scratch():
    from nixis_gb300 import _lib
    L = _lib.lib()
    rc = L.nx_erosion_steps_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), 262145, ctypes.c_void_p(16), 1,
                                    ctypes.c_float(0.0), None, None, None)
    assert rc == 1
    assert b"exceed the fixed scratch" in L.nx_last_error()
