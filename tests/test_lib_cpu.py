"""Host-side checks that need no GPU: the C-ABI library builds, loads and
exports every function include/*.h declares; host-only entry points
(nx_perm_init) match the reference's golden tables."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import golden_io

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*[\s\*]+(nx_[A-Za-z0-9_]+)\s*\(", src, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    from nixis_gb300 import _lib
    L = _lib.lib()
    names = declared_functions()
    assert len(names) >= 5
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_perm_init_matches_reference_tables():
    from nixis_gb300 import opensimplex as osx
    g = golden_io.load("perm")
    for s, p, q in zip(g["seeds"], g["perm"], g["pgi"]):
        perm, pgi = osx.init(int(s))
        assert np.array_equal(perm, p), s
        assert np.array_equal(pgi, q), s


def test_error_reporting_without_gpu_work():
    from nixis_gb300 import _lib
    L = _lib.lib()
    rc = L.nx_perm_init(0, None, None)
    assert rc == 1
    assert b"null" in L.nx_last_error()
    assert L.nx_version() >= 10000


def test_descriptor_layouts_match_the_header():
    """The ctypes mirrors of the C structs have the header's sizes (the C
    side asserts the same sizes at compile time)."""
    from nixis_gb300 import _lib
    assert ctypes.sizeof(_lib.ErosionPlanet) == 72
    assert ctypes.sizeof(_lib.Tiling) == 48
    assert _lib.ErosionPlanet.maxc.offset == 64


def test_host_only_entry_points_reject_bad_arguments():
    """Argument checks of the host-only functions: status codes and
    messages, no exceptions, nothing launched."""
    from nixis_gb300 import _lib
    L = _lib.lib()
    i32 = ctypes.c_int32
    nt, nm, cm = i32(), i32(), i32()
    ok = L.nx_tiling_shape(800, 32, 4, ctypes.byref(nt), ctypes.byref(nm), ctypes.byref(cm))
    assert ok == 0 and nm.value >= (32 + 8) ** 2 and cm.value >= (32 + 6) ** 2 and cm.value <= nm.value
    assert cm.value % 4 == 0
    assert L.nx_tiling_shape(800, 32, 9, ctypes.byref(nt), ctypes.byref(nm), ctypes.byref(cm)) == 1   # rings
    assert L.nx_tiling_shape(800, 1, 4, ctypes.byref(nt), ctypes.byref(nm), ctypes.byref(cm)) == 1    # side
    assert L.nx_tiling_shape(4000, 200, 4, ctypes.byref(nt), ctypes.byref(nm), ctypes.byref(cm)) == 1  # too large
    assert b"too large" in L.nx_last_error()
    # blocked-kernel settings: threads must go with the variant
    assert L.nx_erosion_tb_config(4, 384, 4, 1) == 0
    assert L.nx_erosion_tb_config(4, 384, 0, 1) == 1
    assert b"do not go with" in L.nx_last_error()
    assert L.nx_erosion_tb_config(0, 512, 0, 1) == 1
    assert L.nx_erosion_tb_config(4, 384, 4, 1) == 0
    # passes of a blocked run: ceil(iters / 4) made to the parity of iters
    for it, want in ((0, 0), (1, 1), (4, 2), (5, 3), (8, 2), (9, 3), (100, 26), (101, 27)):
        assert L.nx_erosion_npass(it) == want, it


def _hex_tiles_of_face(k, rho):
    """Restatement of the hexagonal tiling's assignment: every grid point
    (i, j) of a face triangle to the centre m a + n b (a = (2 rho + 1,
    -rho), b = (rho, rho + 1)) within graph distance rho, searched among the
    four lattice points at the floors of its lattice coordinates."""
    N = 3 * rho * rho + 3 * rho + 1
    I, J = np.meshgrid(np.arange(k + 1), np.arange(k + 1), indexing="ij")
    keep = I + J <= k
    I, J = I[keep], J[keep]
    m0 = np.floor_divide((rho + 1) * I - rho * J, N)
    n0 = np.floor_divide(rho * I + (2 * rho + 1) * J, N)
    hits = np.zeros(len(I), int)
    tile = np.zeros((len(I), 2), int)
    for dm in (0, 1):
        for dn in (0, 1):
            m, n = m0 + dm, n0 + dn
            di, dj = I - (m * (2 * rho + 1) + n * rho), J - (-m * rho + n * (rho + 1))
            ok = np.maximum(np.maximum(abs(di), abs(dj)), abs(di + dj)) <= rho
            hits += ok
            tile[ok] = np.stack([m[ok], n[ok]], 1)
    return hits, tile


@pytest.mark.parametrize("rho", [2, 5, 14, 19, 22])
def test_hexagonal_tiles_cover_each_face_point_once_and_are_all_used(rho):
    """Hexagons of radius rho tile the face grid: each point has exactly one
    centre among the four candidates the tiling kernel tries, and
    nx_tiling_shape counts exactly the hexagons that receive points of the
    face triangle (every tile is a block of the erosion launches; the one
    or two per face that hold only points of an edge whose home is the
    other face stay empty)."""
    import ctypes
    from nixis_gb300 import _lib
    L = _lib.lib()
    for k in (1, 2, 7, 40, 100, 333):
        hits, tile = _hex_tiles_of_face(k, rho)
        assert hits.min() == 1 and hits.max() == 1, (k, rho)
        used = len({(int(a), int(b)) for a, b in tile})
        nt, nm, cm = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        assert L.nx_tiling_shape(k, -rho, 4, ctypes.byref(nt), ctypes.byref(nm), ctypes.byref(cm)) == 0
        assert nt.value == 20 * used, (k, rho)
        R = 4
        assert nm.value >= 3 * (rho + R) ** 2 + 3 * (rho + R) + 1 and cm.value % 4 == 0
    for bad in (-1, -65, 0, 1):
        assert L.nx_tiling_shape(100, bad, 4, ctypes.byref(nt), ctypes.byref(nm), ctypes.byref(cm)) != 0
