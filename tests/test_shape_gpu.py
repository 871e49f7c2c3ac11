"""Height shaping on the GPU (nixis.py:332-364): util.rescale in every
form, power_rescale, the elevation mask and the whole sequence, against the
reference's golden vectors and the oracle.

Bars: rescale and the mask are bit-exact (the same binary64 operations);
the masked range of power_rescale (the reference's running min/max update)
is exact: with power 1 the outputs are bit-exact, including at 10 M values
on inputs built to exercise the chunked scan (descending runs, the masked
maximum first, runs across chunk boundaries).  The power itself: the
reference raises with libm's pow, which is not correctly rounded (it
differs from the correctly rounded square root and product in ~0.1 % of
values, by 1 ulp); the GPU uses the correctly rounded square root and
product for powers 0.5 and 2 and CUDA's pow otherwise: 1 ulp (0.5, 2) and
a few ulp (other powers) of the reference at the [0, 1] step, held to 4 and
16 ulp of the field's largest magnitude once mapped back (values near zero
are not compared in ulps of themselves).
"""
import numpy as np
import pytest
import torch

import golden_io
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_rescale_forms_and_mask_match_golden():
    from nixis_gb300 import util, terrain
    g = golden_io.load("shaping")
    x = g["x"]
    assert np.array_equal(util.rescale(x, -10, 20, mid=0.5), g["rescale_mid"])
    assert np.array_equal(util.rescale(x, -10, 20, mid=0.5, mode="lower"), g["rescale_lower"])
    assert np.array_equal(util.rescale(x, -10, 20, mid=0.5, mode="upper"), g["rescale_upper"])
    assert np.array_equal(util.rescale(x, 0, 1, u_min=-100, u_max=100), g["rescale_umin_umax"])
    assert np.array_equal(util.rescale(x, 0, 1, u_min=0, u_max=1), g["rescale_umin_inside"])
    assert util.rescale(x, 0, 1, mode="lower") is x            # a mode without mid: unchanged
    assert util.rescale(x, 0, 1, mid=0.0, mode="sideways") is None
    h1 = g["h1"]
    assert np.array_equal(util.rescale(g["noise"], -4000.0, 8850.0), h1)
    assert np.array_equal(terrain.make_bool_elevation_mask(h1, g["ocean_level"][0]), g["ocean"].astype(bool))
    # CUDA tensors in, CUDA tensors out
    xt = torch.from_numpy(x).cuda()
    assert torch.equal(util.rescale(xt, -10, 20, mid=0.5).cpu(), torch.from_numpy(g["rescale_mid"]))


def ulps(a, b):
    """Largest difference in ulps of the reference's largest magnitude."""
    a, b = np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()
    return float(np.abs(a - b).max() / np.spacing(np.abs(b).max()))


def test_power_rescale_matches_golden():
    from nixis_gb300 import util
    g = golden_io.load("shaping")
    x, m = g["x"], g["pmask"].astype(bool)
    for mode, p, tol in ((1, 0.5, 4), (0, 2.0, 4), (1, 3.0, 16), (0, 0.25, 16)):
        got, want = util.power_rescale(x, m, mode, p), g[f"power_m{mode}_p{p}"]
        assert np.array_equal(got[m != mode], want[m != mode])     # unselected values untouched
        assert ulps(got, want) <= tol, (mode, p)
    assert ulps(util.power_rescale(g["y"], m, 1, 0.5), g["power_first_is_max"]) <= 4
    assert np.array_equal(util.power_rescale(x, m, None, 2.0), x)
    # power 1: the same operations as the oracle, so the masked range is checked bit for bit
    assert np.array_equal(util.power_rescale(g["y"], m, 1, 1.0), O.power_rescale(g["y"], m.astype(np.uint8), 1, 1.0))


def test_shape_heights_matches_golden():
    from nixis_gb300 import util
    g = golden_io.load("shaping")
    h, mask, level = util.shape_heights(g["noise"])
    assert level == g["ocean_level"][0]
    assert np.array_equal(mask, g["ocean"].astype(bool))
    assert ulps(h, g["h5"]) <= 4


def scan_cases(n, rng):
    """Inputs for the masked-range scan at n values."""
    x = rng.normal(0.0, 1.0, n)
    m = rng.random(n) < 0.5
    yield "random", x, m
    d = np.linspace(5.0, -5.0, n)                 # every masked value a new running minimum
    yield "descending", d, m
    y = x.copy()
    first = int(np.argmax(m))
    y[first] = y[m].max() + 3.0                   # the masked maximum comes first
    yield "first_is_max", y, m
    z = np.repeat(rng.normal(0.0, 1.0, n // 4096 + 1), 4096)[:n] - np.arange(n) * 1e-9
    yield "chunk_runs", z, rng.random(n) < 0.9


def test_power_rescale_large_equals_oracle():
    from nixis_gb300 import util
    rng = np.random.default_rng(3)
    n = 10_000_000 + 123
    for name, x, m in scan_cases(n, rng):
        for mode in (0, 1):
            got = util.power_rescale(x, m, mode, 1.0)
            want = O.power_rescale(x, m.astype(np.uint8), mode, 1.0)
            assert np.array_equal(got, want), (name, mode)
    got = util.power_rescale(x, m, 1, 2.0)
    assert ulps(got, O.power_rescale(x, m.astype(np.uint8), 1, 2.0)) <= 4
    x = rng.normal(0.0, 1.0, n)
    assert np.array_equal(util.rescale(x, -4000.0, 8850.0), O.rescale_full(x, -4000.0, 8850.0))
    assert np.array_equal(util.rescale(x, -4000.0, 8850.0, mid=0.1), O.rescale_full(x, -4000.0, 8850.0, mid=0.1))


def test_shape_heights_on_device_equals_oracle():
    from nixis_gb300 import mesh, terrain, util
    m = mesh.PlanetMesh(300)
    perm, pgi = O.init(9)
    h = terrain.sample_octaves(m.xyz, None, perm, pgi, 8, 1.0, 1.0, 2.0, 0.5, 1.0)
    out, mask, level = util.shape_heights(h)
    want, wmask, wlevel = O.shape_heights(h.cpu().numpy())
    assert float(level.item()) == wlevel
    assert np.array_equal(mask.cpu().numpy(), wmask.astype(bool))
    assert ulps(out.cpu().numpy(), want) <= 4
