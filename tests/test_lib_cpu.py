"""Host-side checks that need no GPU: the C-ABI library builds, loads and
exports every function include/*.h declares; host-only entry points
(nx_perm_init) match the reference's golden tables."""
import ctypes
import glob
import os
import re

import numpy as np

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
