"""The CPU oracle against the golden vectors made by executing the reference.

Bit-exact for the permutation tables, noise3d (value and hashed lattice
points), sample_noise, sample_octaves, rescale, adjacency, find_lowest and
erosion (pure +,-,*,/,sqrt arithmetic in both).  Insolation uses libm vs
numpy transcendental functions, so it is compared to 1 binary32 ulp-level
tolerance.
"""
import numpy as np
import pytest

import golden_io
import meshref
from oracle import oracle as O


def test_perm_tables_bit_exact():
    g = golden_io.load("perm")
    for s, p, q in zip(g["seeds"], g["perm"], g["pgi"]):
        perm, pgi = O.init(int(s))
        assert np.array_equal(perm, p), s
        assert np.array_equal(pgi, q), s
        assert sorted(perm.tolist()) == list(range(256))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_noise3d_bit_exact_with_hashed_points(seed):
    g = golden_io.load("noise3d")
    perm, pgi = O.init(seed)
    vals, trace, calls = O.noise3d_batch(g["points"], perm, pgi, trace=True)
    ref = g[f"value_{seed}"]
    assert np.array_equal(vals.view(np.uint64), ref.view(np.uint64))
    assert np.array_equal(calls, g[f"calls_{seed}"])


def test_sample_octaves_and_sample_noise_bit_exact():
    g = golden_io.load("octaves")
    for ci in range(int(g["ncases"])):
        k, seed, n_oct, f0, a0, lac, pers, radius, with_elev = g[f"case{ci}_params"]
        pts, _ = meshref.icosphere(int(k))
        verts = pts * radius if radius != 1.0 else pts
        perm, pgi = O.init(int(seed))
        e_in = g[f"case{ci}_elev_in"] if with_elev else None
        e = O.sample_octaves(verts, e_in, perm, pgi, int(n_oct), f0, a0, lac, pers, radius)
        assert np.array_equal(e, g[f"case{ci}_out"]), ci
        sn = O.sample_noise(verts, perm, pgi, 1.7 / radius, 0.3 / radius, radius)
        assert np.array_equal(sn, g[f"case{ci}_sample_noise"]), ci
    assert np.array_equal(O.rescale(g["rescale_in"], -8000.0, 8000.0), g["rescale_out"])


@pytest.mark.parametrize("k", [1, 2, 3, 4, 6, 12])
def test_adjacency_matches_reference(k):
    g = golden_io.load("mesh_erosion")
    pts, tris = meshref.icosphere(k)
    adj = O.build_adjacency(tris)
    O.sort_adjacency(adj)
    assert np.array_equal(adj, g[f"adj_k{k}"])


@pytest.mark.parametrize("k", [6, 12])
@pytest.mark.parametrize("variant", ["smooth", "terraced", "f32"])
def test_erosion_iteration3_bit_exact(k, variant):
    g = golden_io.load("mesh_erosion")
    pts, _ = meshref.icosphere(k)
    adj = g[f"adj_k{k}"]
    h = g[f"ero_k{k}_{variant}_h0"].copy()
    w = g[f"ero_k{k}_{variant}_w0"].copy()
    s = np.zeros_like(h)
    done = 0
    for it in g[f"ero_k{k}_{variant}_iters"]:
        for _ in range(int(it) - done):
            O.erosion_iteration3(pts, adj, h, w, s)
        done = int(it)
        ref = g[f"ero_k{k}_{variant}_it{it}"]
        assert np.array_equal(np.stack([h, w, s]), ref), (k, variant, it)


@pytest.mark.parametrize("k", [6, 12])
@pytest.mark.parametrize("variant", ["smooth", "terraced", "f32"])
def test_pair_restatement_tracks_golden_trajectories(k, variant):
    """The GPU kernel's arithmetic (state and edge lengths as binary32
    pairs), restated on the CPU, stays within 1e-10 of max|field| of the
    reference's binary64 trajectory at every golden checkpoint (measured
    4e-14), and makes the same flow choice (sign of h_n - h_i) at every
    slot."""
    g = golden_io.load("mesh_erosion")
    pts, _ = meshref.icosphere(k)
    adj = g[f"adj_k{k}"]
    el = meshref.edge_lengths(pts, adj)
    h0 = g[f"ero_k{k}_{variant}_h0"]
    st = O.pair_rows(h0, g[f"ero_k{k}_{variant}_w0"], np.zeros_like(h0))
    done = 0
    for it in g[f"ero_k{k}_{variant}_iters"]:
        for _ in range(int(it) - done):
            st = O.erosion_iteration3_pair(el, adj, st)
        done = int(it)
        ref = g[f"ero_k{k}_{variant}_it{it}"]
        got = [st[:, c].astype(np.float64) + st[:, c + 1] for c in (0, 2, 4)]
        for f, (a, b) in enumerate(zip(got, ref)):
            assert np.abs(a - b).max() <= 1e-10 * np.abs(b).max(), (k, variant, int(it), f)
        j = np.where(adj < 0, np.arange(len(adj))[:, None], adj)
        assert np.array_equal(np.sign(got[0][j] - got[0][:, None]), np.sign(ref[0][j] - ref[0][:, None]))


@pytest.mark.parametrize("k", [6, 12])
def test_erode_terrain3_bit_exact(k):
    g = golden_io.load("mesh_erosion")
    pts, _ = meshref.icosphere(k)
    adj = g[f"adj_k{k}"]
    h0 = g[f"ero_k{k}_smooth_h0"]
    for n_iter in (0, 3):
        h = h0.copy()
        O.erode_terrain3(pts, adj, h, n_iter)
        assert np.array_equal(h, g[f"erode3_k{k}_n{n_iter}"])


def test_shaping_bit_exact():
    """util.rescale in every form, find_percent_val, power_rescale (including
    the running-maximum quirk) and the whole nixis.py:332-364 sequence."""
    g = golden_io.load("shaping")
    x, m = g["x"], g["pmask"]
    assert np.array_equal(O.rescale_full(x, -10, 20, mid=0.5), g["rescale_mid"])
    assert np.array_equal(O.rescale_full(x, -10, 20, mid=0.5, mode="lower"), g["rescale_lower"])
    assert np.array_equal(O.rescale_full(x, -10, 20, mid=0.5, mode="upper"), g["rescale_upper"])
    assert np.array_equal(O.rescale_full(x, 0, 1, u_min=-100, u_max=100), g["rescale_umin_umax"])
    assert np.array_equal(O.rescale_full(x, 0, 1, u_min=0, u_max=1), g["rescale_umin_inside"])
    for mode, p in ((1, 0.5), (0, 2.0), (1, 3.0), (0, 0.25)):
        assert np.array_equal(O.power_rescale(x, m, mode, p), g[f"power_m{mode}_p{p}"]), (mode, p)
    assert np.array_equal(O.power_rescale(g["y"], m, 1, 0.5), g["power_first_is_max"])
    h, mask, level = O.shape_heights(g["noise"])
    assert np.array_equal(h, g["h5"]) and np.array_equal(mask, g["ocean"]) and level == g["ocean_level"][0]
    assert [O.find_percent_val(-4000, 8850, p) for p in (55.0, 0.0, 100.0, 12.5)] == list(g["percent_vals"])


def test_lut_insolation_bit_exact():
    """calc_insolation_slice, interpolate_insolation, calc_daily_insolation
    (climate.py:503-577) and a full calc_yearly_insolation (579-597)."""
    g = golden_io.load("lut_insolation")
    for i, (r, t) in enumerate(g["slice_cases"]):
        assert np.array_equal(O.calc_insolation_slice(r, t), g[f"slice_{i}"]), i
    p8, _ = meshref.icosphere(8)
    assert np.array_equal(O.interpolate_insolation(p8, O.calc_insolation_slice(1.0, 23.44), 1.0), g["daily_k8_t23"])
    assert np.array_equal(O.interpolate_insolation(p8 * 6378100.0, g["slice_2"], 6378100.0), g["interp_k8_earth"])
    p4, _ = meshref.icosphere(4)
    assert np.array_equal(O.calc_yearly_insolation(p4, 1.0, 23.44), g["yearly_k4_t23"])


def test_surface_temp_bit_exact():
    """assign_surface_temp (climate.py:345-411) for four radii and tilts."""
    g = golden_io.load("surface_temp")
    p8, _ = meshref.icosphere(8)
    for i, (r, t) in enumerate(g["cases"]):
        assert np.array_equal(O.assign_surface_temp(p8 * r, r, t), g[f"temp_{i}"]), i


def test_image_sampling_matches_reference():
    """make_ll_arr, the 3 nearest vertices (equal to scipy's KD-tree except
    where two candidates are exactly as far: the KD-tree's order among ties
    is arbitrary) and make_gray_array (util.py:290-366)."""
    g = golden_io.load("image")
    (W, H), r = g["wh"], g["radius"][0]
    assert np.array_equal(O.make_ll_arr(W, H, r), g["ll"])
    pts, _ = meshref.icosphere(16)
    d, i = O.nearest3(pts * r, g["ll"])
    assert np.array_equal(d, g["dists"])
    tie = tied_pixels(pts * r, g["ll"])
    assert np.array_equal(i[~tie], g["nbrs"][~tie])
    assert np.array_equal(O.make_gray_array(W, H, g["dists"], g["nbrs"], g["colors"]), g["gray"])


def tied_pixels(pts, ll):
    return meshref.tied_pixels(pts, ll)


def test_find_lowest_matches_reference():
    g = golden_io.load("mesh_erosion")
    adj = g["adj_k6"]
    h = g["ero_k6_terraced_h0"]
    got = np.array([(-1 if (r := O.find_lowest(v, adj[v], h)) is None else r) for v in range(len(adj))])
    assert np.array_equal(got, g["find_lowest_k6"])


def test_insolation_matches_reference():
    g = golden_io.load("insolation")
    pts, _ = meshref.icosphere(4)
    for a, r in enumerate(g["rots"]):
        for b, t in enumerate(g["tilts"]):
            arr = np.zeros(len(pts), np.float32)
            O.sample_insolation(arr, pts, 1.0, r, t)
            np.testing.assert_allclose(arr, g["single"][a, b], rtol=0, atol=2e-7)
    arr = np.zeros(len(pts), np.float32)
    for r in g["rots"]:
        O.sample_insolation(arr, pts, 1.0, r, 23.44)
    np.testing.assert_allclose(arr, g["cumulative"], rtol=0, atol=1e-6)
    np.testing.assert_allclose([O.calculate_seasonal_tilt(23.44, O.day2deg(365, d)) for d in range(365)],
                               g["seasonal_tilt"], rtol=0, atol=1e-13)
    assert np.array_equal([O.day2deg(365, d) for d in range(365)], g["day2deg"])


def test_brute_daily_insolation_matches_reference():
    g = golden_io.load("insolation")
    p3, _ = meshref.icosphere(3)
    for key, radius, tilt in (("daily_unit", 1.0, 23.44), ("daily_earth", 6378100.0, 10.0)):
        verts = p3 * radius if radius != 1.0 else p3
        # brute_daily_insolation: 360 steps of 1 degree starting at -180, float32 accumulation
        arr = np.zeros(len(p3), np.float32)
        rot = -180.0
        for _ in range(360):
            O.sample_insolation(arr, verts, radius, rot, tilt)
            rot += 1.0
        np.testing.assert_allclose(arr, g[key], rtol=2e-6, atol=2e-5)
        # the exact (binary64) sum agrees with the reference's binary32 sum to its rounding
        _, acc32 = O.annual_insolation(verts, radius, axial_tilt=0.0, days=1, hours=360, with_f32=True)
