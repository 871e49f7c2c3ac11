"""GPU insolation against the reference's goldens and the binary64 oracle sum.

Tolerance (stated): per-vertex |err| <= 1e-5 * max|sum| against the binary64
sum of the reference's terms; single-position calls against the reference's
own float32 results to 2e-6 absolute (terms are <= 1).
"""
import numpy as np
import pytest
import torch

import golden_io
import meshref
from oracle import oracle as O

pytestmark = pytest.mark.gpu

INSO_TOL = 1e-5


def test_single_positions_match_reference():
    from nixis_gb300 import climate
    g = golden_io.load("insolation")
    pts, _ = meshref.icosphere(4, with_tris=False)
    for a, r in enumerate(g["rots"]):
        for b, t in enumerate(g["tilts"]):
            arr = np.zeros(len(pts), np.float32)
            climate.sample_insolation(arr, pts, 1.0, r, t)
            np.testing.assert_allclose(arr, g["single"][a, b], rtol=0, atol=2e-6)
    arr = np.zeros(len(pts), np.float32)
    for r in g["rots"]:
        climate.sample_insolation(arr, pts, 1.0, r, 23.44)
    np.testing.assert_allclose(arr, g["cumulative"], rtol=0, atol=1e-5)
    np.testing.assert_allclose([climate.calculate_seasonal_tilt(23.44, climate.day2deg(365, d)) for d in range(365)],
                               g["seasonal_tilt"], rtol=0, atol=1e-12)


def test_brute_daily_matches_reference():
    from nixis_gb300 import climate
    g = golden_io.load("insolation")
    p3, _ = meshref.icosphere(3, with_tris=False)
    got = climate.brute_daily_insolation(p3, None, 1.0, 23.44)
    ref64 = O.annual_insolation(p3, 1.0, axial_tilt=0.0, days=1, hours=360)  # tilt 0 schedule, checked below
    ref = g["daily_unit"]
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()
    got = climate.brute_daily_insolation(p3 * 6378100.0, None, 6378100.0, 10.0)
    ref = g["daily_earth"]
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()
    assert ref64.shape == (len(p3),)


def annual_ref(pts, radius, days, hours, tilt=23.44):
    return O.annual_insolation(pts, radius, axial_tilt=tilt, days=days, hours=hours)


@pytest.mark.parametrize("k", [4, 16])
def test_annual_sum_against_binary64(k):
    from nixis_gb300 import climate
    pts, _ = meshref.icosphere(k, with_tris=False)
    got = climate.annual_insolation(pts, 1.0).cpu().numpy().astype(np.float64)
    ref = annual_ref(pts, 1.0, 365, 24)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err <= INSO_TOL, err
    # the reference's own float32 running sum is farther from the exact sum
    _, ref32 = O.annual_insolation(pts, 1.0, axial_tilt=23.44, days=365, hours=24, with_f32=True)
    assert err <= np.abs(ref32 - ref).max() / np.abs(ref).max() + 1e-7


def test_annual_sum_random_vertices_and_schedules():
    from nixis_gb300 import climate
    rng = np.random.default_rng(9)
    u = rng.normal(size=(100000, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    got = climate.annual_insolation(u, 1.0).cpu().numpy()
    ref = annual_ref(u, 1.0, 365, 24)
    assert np.abs(got - ref).max() / np.abs(ref).max() <= INSO_TOL
    # odd rotation counts (no 180-degree pairs) and an earth-radius sphere
    got = climate.annual_insolation(u[:20000] * 6378100.0, 6378100.0, days=30, hours=7).cpu().numpy()
    ref = annual_ref(u[:20000] * 6378100.0, 6378100.0, 30, 7)
    assert np.abs(got - ref).max() / np.abs(ref).max() <= INSO_TOL


def test_schedule_with_vertical_tilts_takes_the_direct_form():
    """Days with |cos tilt| < 2^-20 (tilt +-90) leave the factored per-day
    sum for the direct form; mixed with ordinary days (a full group of 8
    days and a remainder), against the binary64 sum of the reference's
    terms."""
    from nixis_gb300 import climate
    rng = np.random.default_rng(11)
    u = rng.normal(size=(20000, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    rot, _ = climate.annual_schedule(23.44, 365, 1, 24)
    tilts = [23.44, 90.0, 10.0, -90.0, 0.0, 45.0, 89.99, -23.44, 90.0, 5.0, -60.0]
    got = climate.insolation_sum(u, 1.0, rot, tilts).cpu().numpy()
    ref = np.zeros(len(u), np.float64)
    for t in tilts:
        for r in rot:
            O.sample_insolation(ref, u, 1.0, r, t)
    assert np.abs(got - ref).max() / np.abs(ref).max() <= INSO_TOL


@pytest.mark.parametrize("days", [1, 512, 513, 700])
def test_schedule_lengths_on_both_staged_paths(days):
    """Schedules of up to 512 days are summed by breakpoints (days sorted by
    |tan tilt|, per-vertex bucket lookups), longer ones day by day in groups
    of 8; a year of 700 days, one of 513 and one of 512 (with ties of
    |tan tilt| between days of opposite tilt) and a single day, against the
    binary64 sum of the reference's terms."""
    from nixis_gb300 import climate
    rng = np.random.default_rng(days)
    u = rng.normal(size=(20000, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    u[:50, 2] = 0.0                     # on the equator: every threshold |z| |tan| is 0
    u[:50] /= np.linalg.norm(u[:50], axis=1)[:, None]
    got = climate.annual_insolation(u, 1.0, days=days, year_length=days, hours=24).cpu().numpy()
    ref = O.annual_insolation(u, 1.0, axial_tilt=23.44, year_length=days, days=days, hours=24)
    assert np.abs(got - ref).max() / np.abs(ref).max() <= INSO_TOL


def test_zero_tilt_schedule_by_breakpoints():
    """Every tilt 0 (all thresholds 0, an empty bucket range): the breakpoint
    sum against the binary64 sum."""
    from nixis_gb300 import climate
    rng = np.random.default_rng(12)
    u = rng.normal(size=(20000, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    rot, _ = climate.annual_schedule(23.44, 365, 1, 24)
    tilts = [0.0] * 40
    got = climate.insolation_sum(u, 1.0, rot, tilts).cpu().numpy()
    ref = np.zeros(len(u), np.float64)
    for t in tilts:
        for r in rot:
            O.sample_insolation(ref, u, 1.0, r, t)
    assert np.abs(got - ref).max() / np.abs(ref).max() <= INSO_TOL


def test_vertices_off_the_sphere_use_the_general_formula():
    from nixis_gb300 import climate
    rng = np.random.default_rng(10)
    u = rng.normal(size=(20000, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    v = u * rng.uniform(0.9, 1.1, size=(len(u), 1))
    got = climate.annual_insolation(v, 1.0, days=20, hours=24).cpu().numpy()
    ref = annual_ref(v, 1.0, 20, 24)
    assert np.abs(got - ref).max() / np.abs(ref).max() <= INSO_TOL


# ---------------------------------------------------------------------------
# latitude-table path (climate.py:503-597).  The tables sum 360 binary64
# terms in binary32 as the reference does; CUDA's and libm's asin/atan2/cos
# differ in the last bits of a term, which can move a binary32 rounding by
# one ulp: tables and interpolations are held to 2 ulp of their maximum,
# the 360-table year to 1e-6 of its maximum.

def test_lut_tables_and_interpolation_match_reference():
    import golden_io
    from nixis_gb300 import climate
    g = golden_io.load("lut_insolation")
    for i, (r, t) in enumerate(g["slice_cases"]):
        got, want = climate.calc_insolation_slice(r, t), g[f"slice_{i}"]
        assert np.abs(got - want).max() <= 2 * np.spacing(np.float32(want.max())), i
    p8, _ = meshref.icosphere(8)
    d = climate.calc_daily_insolation(p8, np.zeros(len(p8)), 1.0, 23.44)
    assert np.abs(d - g["daily_k8_t23"]).max() <= 2 * np.spacing(np.float32(g["daily_k8_t23"].max()))
    ins = np.zeros(len(p8), np.float32)
    climate.interpolate_insolation(p8 * 6378100.0, g["slice_2"], ins, 6378100.0)
    # the table is given: only the latitude (one asin) can differ
    assert np.abs(ins - g["interp_k8_earth"]).max() <= 2 * np.spacing(np.float32(g["interp_k8_earth"].max()))
    p4, _ = meshref.icosphere(4)
    y = climate.calc_yearly_insolation(p4, np.zeros(len(p4)), 1.0, 23.44)
    assert np.abs(y - g["yearly_k4_t23"]).max() <= 1e-6 * g["yearly_k4_t23"].max()


def test_lut_interpolation_is_bit_exact_on_random_tables():
    # tables of random binary32 values (full mantissas, mixed magnitudes):
    # the interpolation (binary32 pairs, binary64 near rounding boundaries)
    # must give the reference's binary32 result.  Only a latitude whose asin
    # rounds differently on the GPU and in libm can move a result, by 1 ulp.
    from nixis_gb300 import climate
    rng = np.random.default_rng(21)
    n = 1 << 20
    p = rng.normal(size=(n, 3))
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    p *= 6378100.0
    for scale in (1.0, 1e-3, 3e4):
        tab = (rng.random(181) * scale).astype(np.float32)
        tab[rng.random(181) < 0.05] = 0.0
        got = np.zeros(n, np.float32)
        climate.interpolate_insolation(p, tab, got, 6378100.0)
        want = O.interpolate_insolation(p, tab, 6378100.0)
        diff = got.view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64)
        assert np.abs(diff).max() <= 1, scale
        assert np.count_nonzero(diff) <= 8, (scale, np.count_nonzero(diff))


def test_surface_temp_matches_reference():
    # assign_surface_temp (climate.py:345-411): one asin and one cos per
    # vertex in binary64, stored as binary32; CUDA's and libm's last bits
    # can move a binary32 rounding by one ulp
    import golden_io
    from nixis_gb300 import climate, mesh
    g = golden_io.load("surface_temp")
    p8, _ = meshref.icosphere(8)
    for i, (r, t) in enumerate(g["cases"]):
        got = climate.assign_surface_temp(p8 * r, g["altitudes"], r, t)
        want = g[f"temp_{i}"]
        assert got.dtype == np.float32 and got.shape == want.shape
        diff = got.view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64)
        assert np.abs(diff).max() <= 1, i
    m = mesh.PlanetMesh(300)
    y = climate.assign_surface_temp(m.xyz, torch.zeros(m.n, dtype=torch.float64, device="cuda"), 1.0, 23.44)
    want = O.assign_surface_temp(m.xyz.cpu().numpy(), 1.0, 23.44)
    diff = y.cpu().numpy().view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64)
    assert np.abs(diff).max() <= 1 and np.count_nonzero(diff) <= m.n // 1000
    with pytest.raises(ValueError):
        climate.assign_surface_temp(p8, np.zeros(3), 1.0, 0.0)


def test_lut_yearly_on_a_large_sphere_matches_oracle():
    from nixis_gb300 import climate, mesh
    m = mesh.PlanetMesh(300)
    y = climate.calc_yearly_insolation(m.xyz, None, 1.0, 23.44).cpu().numpy()
    rng = np.random.default_rng(5)
    idx = rng.choice(m.n, 20000, replace=False)
    want = O.calc_yearly_insolation(m.xyz.cpu().numpy()[idx], 1.0, 23.44)
    assert np.abs(y[idx] - want).max() <= 1e-6 * want.max()
    assert np.isfinite(y).all() and y.min() > 0       # with a tilt even the poles see the sun
