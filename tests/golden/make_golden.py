"""Generate the golden vectors in tests/golden/ by executing the reference.

Run where the reference sources are, naming their directory:

    NIXIS_REFERENCE_DIR=<nixis checkout> python tests/golden/make_golden.py

Every expected value in the output comes from the reference's own Python
functions (opensimplex.init / noise3d, terrain.sample_noise / sample_octaves,
erosion.erosion_iteration3 / erode_terrain3 / find_lowest,
climate.sample_insolation / brute_daily_insolation / calculate_seasonal_tilt /
day2deg, util.build_adjacency / sort_adjacency / rescale / power_rescale /
find_percent_val, terrain.make_bool_elevation_mask, climate.calc_insolation_slice /
interpolate_insolation / calc_daily_insolation / calc_yearly_insolation /
assign_surface_temp, util.make_ll_arr / make_gray_array with scipy's KDTree query) imported through
ref_shim.  `python tests/golden/make_golden.py shaping` regenerates one set.  Inputs are seeded; meshes come from tests/meshref.py (the same
construction as the GPU generator).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import ref_shim  # noqa: E402
import meshref  # noqa: E402


def quiet(fn, *a, **k):
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def gen_perm(R):
    seeds = list(range(64)) + [-1, -123456, 2**31 - 1, 2**31, 2**40 + 7, 999999, 123456789]
    perms, pgis = [], []
    for s in seeds:
        p, g = R.opensimplex.init(s)
        perms.append(np.asarray(p, np.int32))
        pgis.append(np.asarray(g, np.int32))
    np.savez_compressed(os.path.join(HERE, "perm.npz"), seeds=np.array(seeds, np.int64),
                        perm=np.stack(perms), pgi=np.stack(pgis))


def boundary_points(rng, n):
    """Points whose skewed coordinates sit on or within ~1e-12 of the
    lattice-cell and region boundaries of noise3d."""
    pts = []
    eps_list = [0.0, 1e-15, -1e-15, 1e-12, -1e-12, 3e-9, -3e-9]
    for _ in range(n):
        base = rng.integers(-300, 300, size=3).astype(np.float64)
        kind = rng.integers(0, 8)
        e = eps_list[rng.integers(0, len(eps_list))]
        f = rng.random(3)
        if kind == 0:           # on a cell face: xins ~ 0
            f[0] = e if e >= 0 else 1 + e
        elif kind == 1:         # in_sum ~ 1
            f[2] = 1 + e - f[0] - f[1]
        elif kind == 2:         # in_sum ~ 2
            f = 0.5 + 0.5 * f
            f[2] = 2 + e - f[0] - f[1]
        elif kind == 3:         # ties between scores
            f[1] = f[0] + e
        elif kind == 4:         # octahedron p1 = xins + yins ~ 1
            f[1] = 1 + e - f[0]
            f[2] = 0.3 + 0.4 * f[2]
        elif kind == 5:         # all equal
            f[:] = f[0]
        elif kind == 6:         # wins ~ a_score in the tetrahedra
            f[0] = (1 - f[1] - f[2]) / 2 + e
        else:                   # lattice point exactly
            f[:] = 0
        xs = base + f
        s = xs.sum()
        pts.append(xs + s / 3.0)      # inverse of the skew x + (x+y+z)(-1/6)
    return np.array(pts, np.float64)


def gen_noise(R):
    osi = R.opensimplex
    rng = np.random.default_rng(1234)
    pts = [rng.uniform(-40, 40, size=(1500, 3))]
    u = rng.normal(size=(1500, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    for i in range(12):
        pts.append(u[i * 125:(i + 1) * 125] * 2.0**i)
    pts.append(boundary_points(rng, 1500))
    pts.append(np.array([[0.0, 0.0, 0.0], [-0.0, 0.0, -0.0], [1.0, 1.0, 1.0], [1e5, -3e4, 7e3],
                         [-2.5, -2.5, -2.5], [0.5, 0.5, 0.5]], np.float64))
    pts = np.concatenate(pts)
    out = {}
    orig = osi.extrapolate3d
    for seed in (0, 1, 2):
        perm, pgi = osi.init(seed)
        vals = np.empty(len(pts))
        calls = np.zeros((len(pts), 25), np.int32)
        rec = []

        def wrapper(xsb, ysb, zsb, dx, dy, dz, p, g):
            rec.append((xsb, ysb, zsb))
            return orig(xsb, ysb, zsb, dx, dy, dz, p, g)

        osi.extrapolate3d = wrapper
        try:
            for i, (x, y, z) in enumerate(pts):
                rec.clear()
                vals[i] = osi.noise3d(float(x), float(y), float(z), perm, pgi)
                calls[i, 0] = len(rec)
                for c, t in enumerate(rec):
                    calls[i, 1 + 3 * c: 4 + 3 * c] = t
        finally:
            osi.extrapolate3d = orig
        out[f"value_{seed}"] = vals
        out[f"calls_{seed}"] = calls
    np.savez_compressed(os.path.join(HERE, "noise3d.npz"), points=pts, **out)


def gen_octaves(R):
    ter = R.terrain
    osi = R.opensimplex
    cases = []
    # (k, seed, n_oct, init_rough, init_strength, rough, persist, radius, with_elev)
    cases.append((5, 0, 8, 1.0, 1.0, 2.0, 0.5, 1.0, False))        # the 8-octave plain method
    cases.append((16, 1, 12, 1.0, 1.0, 2.0, 0.5, 1.0, False))      # 12 octaves
    cases.append((8, 5, 7, 1.5, 0.4, 2.5, 0.5, 6378100.0, False))  # nixis.py's defaults, nixis.py:312-320
    cases.append((4, 9, 3, 1.0, 0.2, 2.0, 0.5, 1.0, True))         # accumulate into given elevations
    out = {}
    for ci, (k, seed, n_oct, f0, a0, lac, pers, radius, with_elev) in enumerate(cases):
        pts, tris = meshref.icosphere(k)
        verts = pts * radius if radius != 1.0 else pts.copy()
        perm, pgi = osi.init(seed)
        elev0 = np.linspace(-1.0, 1.0, len(verts)) if with_elev else None
        e_in = None if elev0 is None else elev0.copy()
        e = quiet(ter.sample_octaves, verts, e_in, perm, pgi, n_oct, f0, a0, lac, pers, radius)
        out[f"case{ci}_params"] = np.array([k, seed, n_oct, f0, a0, lac, pers, radius, with_elev], np.float64)
        out[f"case{ci}_elev_in"] = elev0 if elev0 is not None else np.zeros(0)
        out[f"case{ci}_out"] = np.asarray(e, np.float64)
        sn = ter.sample_noise(verts, perm, pgi, 1.7 / radius, 0.3 / radius, radius)
        out[f"case{ci}_sample_noise"] = np.asarray(sn, np.float64)
    # rescale (util.py:110-140) of the first case to +-8000 m
    out["rescale_in"] = out["case0_out"]
    out["rescale_out"] = np.asarray(R.util.rescale(out["case0_out"], -8000.0, 8000.0), np.float64)
    np.savez_compressed(os.path.join(HERE, "octaves.npz"), ncases=len(cases), **out)


def gen_mesh_erosion(R):
    util = R.util
    ero = R.erosion
    osi = R.opensimplex
    ter = R.terrain
    out = {}
    for k in (1, 2, 3, 4, 6, 12):
        pts, tris = meshref.icosphere(k)
        adj = util.build_adjacency(tris)
        util.sort_adjacency(adj)
        out[f"adj_k{k}"] = np.asarray(adj, np.int32)
    for k, seed, iters in ((6, 3, (1, 10, 50)), (12, 4, (1, 10, 30))):
        pts, tris = meshref.icosphere(k)
        adj = out[f"adj_k{k}"].copy()
        perm, pgi = osi.init(seed)
        h = quiet(ter.sample_octaves, pts, None, perm, pgi, 6, 1.0, 1.0, 2.0, 0.5, 1.0)
        h = np.asarray(util.rescale(h, -8000.0, 8000.0), np.float64)
        for variant in ("smooth", "terraced", "f32"):
            hv = h.copy()
            if variant == "terraced":       # many exactly equal neighbours: slope == 0 branch
                hv = np.round(hv / 500.0) * 500.0
            if variant == "f32":            # binary32-representable inputs
                hv = hv.astype(np.float32).astype(np.float64)
            w = np.full(len(pts), 1e-3)
            if variant == "f32":
                w = w.astype(np.float32).astype(np.float64)
            s = np.zeros(len(pts))
            out[f"ero_k{k}_{variant}_h0"] = hv.copy()
            out[f"ero_k{k}_{variant}_w0"] = w.copy()
            done = 0
            for it in iters:
                for _ in range(it - done):
                    ero.erosion_iteration3(pts, adj, hv, w, s)
                done = it
                out[f"ero_k{k}_{variant}_it{it}"] = np.stack([hv, w, s]).copy()
            out[f"ero_k{k}_{variant}_iters"] = np.array(iters, np.int32)
        # erode_terrain3: rain before each pass, num_iter <= 0 runs once
        for n_iter in (0, 3):
            hv = h.copy()
            quiet(ero.erode_terrain3, pts, adj, hv, n_iter)
            out[f"erode3_k{k}_n{n_iter}"] = hv.copy()
        out[f"ero_k{k}_seed"] = np.array([seed], np.int32)
    # find_lowest (erosion.py:398-406) on terraced heights (ties)
    pts, tris = meshref.icosphere(6)
    adj = out["adj_k6"]
    hv = out["ero_k6_terraced_h0"]
    fl = np.array([(-1 if (r := ero.find_lowest(v, adj[v], hv)) is None else r) for v in range(len(pts))],
                  np.int32)
    out["find_lowest_k6"] = fl
    np.savez_compressed(os.path.join(HERE, "mesh_erosion.npz"), **out)


def gen_insolation(R):
    cli = R.climate
    out = {}
    pts, _ = meshref.icosphere(4)
    rots = [-180.0, -97.5, 0.0, 33.0, 179.0]
    tilts = [-23.44, 0.0, 10.0, 23.44, 90.0]
    single = np.zeros((len(rots), len(tilts), len(pts)), np.float32)
    for a, r in enumerate(rots):
        for b, t in enumerate(tilts):
            arr = np.zeros(len(pts), np.float32)
            cli.sample_insolation(arr, pts, 1.0, r, t)
            single[a, b] = arr
    out["single"] = single
    out["rots"] = np.array(rots)
    out["tilts"] = np.array(tilts)
    # cumulative float32 accumulation over several calls
    arr = np.zeros(len(pts), np.float32)
    for r in rots:
        cli.sample_insolation(arr, pts, 1.0, r, 23.44)
    out["cumulative"] = arr
    # brute_daily_insolation (360 one-degree steps), unit and earth radius
    p3, _ = meshref.icosphere(3)
    out["daily_unit"] = np.asarray(cli.brute_daily_insolation(p3, np.zeros(len(p3)), 1.0, 23.44), np.float32)
    out["daily_earth"] = np.asarray(cli.brute_daily_insolation(p3 * 6378100.0, np.zeros(len(p3)), 6378100.0, 10.0),
                                    np.float32)
    out["seasonal_tilt"] = np.array([cli.calculate_seasonal_tilt(23.44, cli.day2deg(365, d)) for d in range(365)])
    out["day2deg"] = np.array([cli.day2deg(365, d) for d in range(365)])
    np.savez_compressed(os.path.join(HERE, "insolation.npz"), **out)


def gen_shaping(R):
    """The post-noise shaping of nixis.py:330-364 (rescale to [min_alt,
    max_alt], ocean level at a percent of the range, elevation mask, masked
    power rescales, shift, two-sided rescale about 0) on 12-octave terrain,
    plus rescale's mid/mode/u_min/u_max forms and power_rescale on arrays
    that exercise its running min/max update (a masked value that is the
    running minimum is not considered for the maximum)."""
    util, ter, osi = R.util, R.terrain, R.opensimplex
    out = {}
    pts, _ = meshref.icosphere(24)
    perm, pgi = osi.init(5)
    h = np.asarray(quiet(ter.sample_octaves, pts, None, perm, pgi, 12, 1.0, 1.0, 2.0, 0.5, 1.0), np.float64)
    out["noise"] = h.copy()
    min_alt, max_alt, ocean_percent = -4000.0, 8850.0, 55.0       # nixis.py:312-315
    h1 = np.asarray(util.rescale(h, min_alt, max_alt), np.float64)
    ocean_level = util.find_percent_val(np.amin(h1), np.amax(h1), ocean_percent)
    ocean = np.asarray(ter.make_bool_elevation_mask(h1, ocean_level))
    h2 = np.asarray(quiet(util.power_rescale, h1, mask=ocean, mode=1, power=0.5), np.float64)
    h3 = np.asarray(quiet(util.power_rescale, h2, mask=ocean, mode=0, power=2.0), np.float64)
    h4 = h3 - ocean_level
    h5 = np.asarray(util.rescale(h4, min_alt, max_alt, mid=0), np.float64)
    out.update(h1=h1, ocean_level=np.array([ocean_level]), ocean=ocean.astype(np.uint8), h2=h2, h3=h3, h5=h5)
    rng = np.random.default_rng(17)
    x = rng.normal(0.0, 3.0, 2000)
    out["x"] = x
    out["rescale_mid"] = np.asarray(util.rescale(x, -10.0, 20.0, mid=0.5), np.float64)
    out["rescale_lower"] = np.asarray(util.rescale(x, -10.0, 20.0, mid=0.5, mode="lower"), np.float64)
    out["rescale_upper"] = np.asarray(util.rescale(x, -10.0, 20.0, mid=0.5, mode="upper"), np.float64)
    out["rescale_umin_umax"] = np.asarray(util.rescale(x, 0.0, 1.0, u_min=-100.0, u_max=100.0), np.float64)
    out["rescale_umin_inside"] = np.asarray(util.rescale(x, 0.0, 1.0, u_min=0.0, u_max=1.0), np.float64)
    m = rng.random(2000) < 0.4
    out["pmask"] = m.astype(np.uint8)
    for mode, power in ((1, 0.5), (0, 2.0), (1, 3.0), (0, 0.25)):
        out[f"power_m{mode}_p{power}"] = np.asarray(quiet(util.power_rescale, x, mask=m, mode=mode, power=power),
                                                    np.float64)
    # the first masked value is the largest masked value: the running
    # update never records it as the maximum
    y = x.copy()
    first = int(np.argmax(m))
    y[first] = np.max(y[m]) + 1.0
    out["y"] = y
    out["power_first_is_max"] = np.asarray(quiet(util.power_rescale, y, mask=m, mode=1, power=0.5), np.float64)
    out["percent_vals"] = np.array([util.find_percent_val(-4000.0, 8850.0, p) for p in (55.0, 0.0, 100.0, 12.5)])
    np.savez_compressed(os.path.join(HERE, "shaping.npz"), **out)


def gen_lut_insolation(R):
    """The latitude-table insolation path (climate.py:503-597):
    calc_insolation_slice for a few tilts and radii, calc_daily_insolation
    and interpolate_insolation on icosphere vertices, and a full
    calc_yearly_insolation (360 daily tables) on a small sphere."""
    cl = R.climate
    out = {}
    cases = [(1.0, 23.44), (1.0, 0.0), (1.0, -17.3), (6378100.0, 10.0)]
    out["slice_cases"] = np.array(cases)
    for i, (r, t) in enumerate(cases):
        out[f"slice_{i}"] = np.asarray(cl.calc_insolation_slice(r, t), np.float32)
    p8, _ = meshref.icosphere(8)
    h8 = np.linspace(-1.0, 1.0, len(p8))
    out["daily_k8_t23"] = np.asarray(quiet(cl.calc_daily_insolation, p8, h8, 1.0, 23.44), np.float32)
    tab = out["slice_2"]
    ins = np.zeros(len(p8), np.float32)
    pe = p8 * 6378100.0
    cl.interpolate_insolation(pe, tab, ins, 6378100.0)
    out["interp_k8_earth"] = ins
    p4, _ = meshref.icosphere(4)
    out["yearly_k4_t23"] = np.asarray(quiet(cl.calc_yearly_insolation, p4, np.zeros(len(p4)), 1.0, 23.44),
                                      np.float32)
    np.savez_compressed(os.path.join(HERE, "lut_insolation.npz"), **out)


def gen_surface_temp(R):
    """climate.assign_surface_temp (climate.py:345-411) on icosphere
    vertices for a few radii and tilts, with varying altitudes."""
    cl = R.climate
    out = {}
    p8, _ = meshref.icosphere(8)
    rng = np.random.default_rng(31)
    h8 = rng.normal(size=len(p8))
    cases = [(1.0, 23.44), (1.0, 0.0), (6378100.0, -17.3), (2.5, 90.0)]
    out["cases"] = np.array(cases)
    out["altitudes"] = h8
    for i, (r, t) in enumerate(cases):
        out[f"temp_{i}"] = np.asarray(cl.assign_surface_temp(p8 * r, h8, r, t), np.float32)
    np.savez_compressed(os.path.join(HERE, "surface_temp.npz"), **out)


def gen_image(R):
    """Equirectangular map sampling (util.py:290-367, nixis.py:270-302):
    make_ll_arr's pixel positions, the 3 nearest vertices of each pixel from
    scipy's KD-tree (as build_KDTree + query(k=3)), and make_gray_array's
    inverse-distance weighting of rescaled heights."""
    from scipy.spatial import KDTree
    util, ter, osi = R.util, R.terrain, R.opensimplex
    out = {}
    pts, _ = meshref.icosphere(16)
    radius = 2.5
    pts = pts * radius
    perm, pgi = osi.init(21)
    h = np.asarray(quiet(ter.sample_octaves, pts / radius, None, perm, pgi, 6, 1.0, 1.0, 2.0, 0.5, 1.0), np.float64)
    colors = np.asarray(util.rescale(h, 0, 255), np.float64)
    W, H = 64, 32
    ll = np.asarray(util.make_ll_arr(W, H, radius), np.float64)
    dists, nbrs = KDTree(pts, leafsize=10).query(ll, k=3)
    gray = np.asarray(util.make_gray_array(W, H, dists, nbrs, colors))
    out.update(radius=np.array([radius]), heights=h, colors=colors, ll=ll, dists=np.asarray(dists),
               nbrs=np.asarray(nbrs, np.int64), gray=gray, wh=np.array([W, H]))
    np.savez_compressed(os.path.join(HERE, "image.npz"), **out)


GENERATORS = {"perm": gen_perm, "noise": gen_noise, "octaves": gen_octaves, "mesh_erosion": gen_mesh_erosion,
              "insolation": gen_insolation, "shaping": gen_shaping,
              "lut_insolation": gen_lut_insolation, "image": gen_image, "surface_temp": gen_surface_temp}


def main():
    R = ref_shim.load()
    names = sys.argv[1:] or list(GENERATORS)
    for name in names:
        GENERATORS[name](R)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
