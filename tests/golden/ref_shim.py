"""Import the reference Nixis modules as plain Python, for generating golden vectors.

Test infrastructure only: nothing in the package, the benchmark or the GPU
tests imports this module.  It runs only where the reference sources are
present (the build container), and is used by ``make_golden.py`` to produce
the committed fixtures under ``tests/golden/``.

The reference JIT-compiles its hot loops with numba, which is not installed
here.  The shim registers stand-in modules before importing the reference:

* ``numba.njit`` becomes an identity decorator.  ``opensimplex.over`` is
  declared ``@njit(["int32(int32)"])`` (opensimplex.py:110-112), so under numba
  its argument is truncated to a signed 32-bit integer; the stand-in keeps that
  by returning ``low 32 bits, sign-extended`` for that signature.
* ``numba.prange`` becomes ``range``.
* ``meshzoo``, ``meshio`` and ``PIL`` (imported at util.py:6-8 but not used by
  the hot path) become empty modules.
* ``erosion.calc_distance`` (erosion.py:38-40) squares with ``** 2``.  numba
  lowers a float raised to an integer literal to repeated multiplication
  (``x * x``, correctly rounded), while numpy's float64 scalar ``** 2`` goes
  through ``pow`` and is off by one ulp for some inputs.  The shim rebinds
  ``calc_distance`` to the same expression with ``x * x`` so the fixtures
  follow the numba build.

Python floats and numpy float64 scalars are IEEE binary64 without FMA
contraction, which is also numba's default (no fastmath), so the floating-point
results equal the numba build's for the same permutation tables.
"""
import os
import sys
import types

# The reference's source directory (the nixis checkout); required, no default.
REFERENCE_DIR = os.environ.get("NIXIS_REFERENCE_DIR", "")


def _int32_wrap(x):
    return ((int(x) + 2**31) % 2**32) - 2**31


def _njit(*args, **kwargs):
    # @njit used bare: @njit def f(...)
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    sigs = args[0] if args else kwargs.get("signature_or_function")

    def deco(fn):
        if isinstance(sigs, (list, tuple)) and any("int32(int32)" in str(s) for s in sigs):
            def wrapped(x):
                return _int32_wrap(fn(_int32_wrap(x)))
            wrapped.__name__ = fn.__name__
            return wrapped
        return fn
    return deco


def _install_stubs():
    numba = types.ModuleType("numba")
    numba.njit = _njit
    numba.jit = _njit
    numba.prange = range
    sys.modules["numba"] = numba
    for name in ("meshzoo", "meshio"):
        sys.modules[name] = types.ModuleType(name)
    pil = types.ModuleType("PIL")
    pil.Image = None
    sys.modules["PIL"] = pil


_loaded = None


def load():
    """Return a namespace with the reference modules opensimplex, terrain,
    erosion, climate and util, imported unchanged through the stubs."""
    global _loaded
    if _loaded is not None:
        return _loaded
    if not REFERENCE_DIR:
        raise RuntimeError("set NIXIS_REFERENCE_DIR to the nixis source directory")
    if not os.path.isdir(REFERENCE_DIR):
        raise RuntimeError(f"reference sources not found at {REFERENCE_DIR}")
    _install_stubs()
    sys.path.insert(0, REFERENCE_DIR)
    sys.dont_write_bytecode = True
    import opensimplex, terrain, erosion, climate, util  # noqa: E401
    import numpy as np

    def calc_distance(v0, v1):
        dx = v0[0] - v1[0]
        dy = v0[1] - v1[1]
        dz = v0[2] - v1[2]
        return np.sqrt(dx * dx + dy * dy + dz * dz)

    erosion.calc_distance = calc_distance
    _loaded = types.SimpleNamespace(opensimplex=opensimplex, terrain=terrain,
                                    erosion=erosion, climate=climate, util=util)
    return _loaded
