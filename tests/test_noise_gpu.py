"""GPU fBm / noise3d against the oracle and the reference's golden vectors.

Bit-exact: lattice cell, region, both extra lattice points, the set of
lattice points hashed, and the gradient fetched for each of them.  Values:
binary32 against the binary64 reference, |err| <= 2e-6 per noise3d value and
<= 1e-5 of the elevation range for sample_octaves (the stated elevation
tolerance).
"""
import numpy as np
import pytest
import torch

import golden_io
import meshref
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GRAD3 = np.array([
    -11, 4, 4, -4, 11, 4, -4, 4, 11, 11, 4, 4, 4, 11, 4, 4, 4, 11,
    -11, -4, 4, -4, -11, 4, -4, -4, 11, 11, -4, 4, 4, -11, 4, 4, -4, 11,
    -11, 4, -4, -4, 11, -4, -4, 4, -11, 11, 4, -4, 4, 11, -4, 4, 4, -11,
    -11, -4, -4, -4, -11, -4, -4, -4, -11, 11, -4, -4, 4, -11, -4, 4, -4, -11], np.int64)

ELEV_TOL = 1e-5     # max |err| / (max - min) of the elevations


def cpu_hash(perm, pgi, x, y, z):
    """opensimplex.py:124 on int arrays: perm_grad_index_3D of a lattice point."""
    p = perm.astype(np.int64)
    return pgi[(p[(p[x & 255] + y) & 255] + z) & 255]


def check_points(pts, seed, scale=1.0, check_sets=True):
    from nixis_gb300 import opensimplex as osx
    perm, pgi = O.init(seed)
    val, tr, sl, nfb = osx.noise3d_trace(pts, perm, pgi, scale=scale)
    val, tr, sl = val.cpu().numpy(), tr.cpu().numpy(), sl.cpu().numpy()
    sp = pts * scale
    ref_val, ref_tr, ref_calls = O.noise3d_batch(sp, perm, pgi, trace=True)
    # lattice cell, region, extra points: identical
    bad = np.argwhere((tr != ref_tr).any(1)).ravel()
    assert bad.size == 0, (bad[:5], tr[bad[:3]], ref_tr[bad[:3]], sp[bad[:3]])
    # every evaluated slot fetched the gradient of its lattice point
    x, y, z = (sl[..., c].astype(np.int64) for c in range(3))
    gi = cpu_hash(perm, pgi, x, y, z)
    want = (GRAD3[gi] + 16) | ((GRAD3[gi + 1] + 16) << 8) | ((GRAD3[gi + 2] + 16) << 16)
    assert np.array_equal(sl[..., 3], want)
    if check_sets:
        # the used slots with positive binary64 attenuation are exactly the
        # lattice points the reference hashed (its extrapolate3d calls)
        L = sl[..., :3].astype(np.float64)
        real = L + (L.sum(-1, keepdims=True) * (1.0 / 3))
        d = sp[:, None, :] - real
        attn = 2.0 - (d * d).sum(-1)
        used = sl[..., 4] == 1
        for i in range(len(sp)):
            ref = sorted(tuple(ref_calls[i, 1 + 3 * c: 4 + 3 * c]) for c in range(ref_calls[i, 0]))
            got = sorted(tuple(sl[i, k, :3]) for k in range(9) if used[i, k] and attn[i, k] > 0)
            if ref != got:
                amb = [k for k in range(9) if used[i, k] and abs(attn[i, k]) < 1e-9]
                assert amb, (i, ref, got)
    np.testing.assert_allclose(val, ref_val, rtol=0, atol=2e-6)
    return nfb


def test_noise3d_golden_points_bit_exact_decisions():
    g = golden_io.load("noise3d")
    pts = g["points"]
    total_fb = 0
    for seed in (0, 1, 2):
        perm, pgi = O.init(seed)
        # the oracle is pinned to the reference's own values
        assert np.array_equal(O.noise3d_batch(pts, perm, pgi), g[f"value_{seed}"])
        total_fb += check_points(pts, seed)
    # the near-boundary points made the binary64 decision path run
    assert total_fb > 0


@pytest.mark.parametrize("octave", [0, 5, 11, 15])
def test_noise3d_sphere_points_at_octave_scales(octave):
    rng = np.random.default_rng(100 + octave)
    u = rng.normal(size=(200000, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    check_points(u, seed=octave, scale=2.0 ** octave, check_sets=False)


def test_noise3d_general_scale_and_large_radius():
    # the reference driver's setting: vertices scaled by 6378100 m, scale f/R
    rng = np.random.default_rng(5)
    u = rng.normal(size=(100000, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    R = 6378100.0
    for f in (1.5, 1.5 * 2.5 ** 3, 1.5 * 2.5 ** 6):
        check_points(u * R, seed=7, scale=f / R, check_sets=False)


def test_sample_octaves_golden():
    from nixis_gb300 import terrain
    g = golden_io.load("octaves")
    for ci in range(int(g["ncases"])):
        k, seed, n_oct, f0, a0, lac, pers, radius, with_elev = g[f"case{ci}_params"]
        pts, _ = meshref.icosphere(int(k), with_tris=False)
        verts = pts * radius if radius != 1.0 else pts
        perm, pgi = O.init(int(seed))
        ref = g[f"case{ci}_out"]
        e_in = g[f"case{ci}_elev_in"].copy() if with_elev else None
        got = terrain.sample_octaves(verts, e_in, perm, pgi, int(n_oct), f0, a0, lac, pers, radius)
        if with_elev:
            assert got is e_in          # updated in place, like the reference
        rng_ = ref.max() - ref.min()
        assert np.abs(got - ref).max() <= ELEV_TOL * rng_, ci
        sn = terrain.sample_noise(verts, perm, pgi, 1.7 / radius, 0.3 / radius, radius)
        refn = g[f"case{ci}_sample_noise"]
        assert np.abs(sn - refn).max() <= ELEV_TOL * max(refn.max() - refn.min(), 1e-300), ci


def test_fbm_plain_method_full_size():
    """divisions=250 (625,002 vertices), 8 octaves, base frequency 1,
    lacunarity 2, persistence 0.5, seed 0, scaled to +-8000 m: every vertex
    against the oracle, and the decisions of every vertex-octave."""
    from nixis_gb300 import terrain
    pts, _ = meshref.icosphere(250, with_tris=False)
    perm, pgi = O.init(0)
    ref = O.sample_octaves(pts, None, perm, pgi, 8, 1.0, 1.0, 2.0, 0.5, 1.0)
    got = terrain.sample_octaves(torch.from_numpy(pts).cuda(), None, perm, pgi, 8, 1.0, 1.0, 2.0, 0.5, 1.0)
    got = got.cpu().numpy()
    r = ref.max() - ref.min()
    err = np.abs(got - ref)
    assert err.max() <= ELEV_TOL * r, err.max() / r
    # after the reference's rescale to +-8000 m (util.py:110-140)
    m_ref = O.rescale(ref, -8000.0, 8000.0)
    m_got = O.rescale(got, -8000.0, 8000.0)
    assert np.abs(m_got - m_ref).max() <= ELEV_TOL * 16000.0
    for o in range(8):
        check_points(pts, seed=0, scale=2.0 ** o, check_sets=False)


def test_fbm_float32_output_and_accumulate():
    from nixis_gb300 import terrain
    rng = np.random.default_rng(3)
    u = rng.normal(size=(50000, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    perm, pgi = O.init(11)
    scale, strength = terrain._octave_args(6, 1.0, 1.0, 2.0, 0.5, 1.0)
    base = torch.linspace(-1, 1, len(u), dtype=torch.float32, device="cuda")
    out32 = base.clone()
    terrain.fbm(u, perm, pgi, scale, strength, 1.0, out=out32, accumulate=True)
    ref = O.sample_octaves(u, base.double().cpu().numpy(), perm, pgi, 6, 1.0, 1.0, 2.0, 0.5, 1.0)
    assert np.abs(out32.double().cpu().numpy() - ref).max() <= 2e-6 * (ref.max() - ref.min())


# Pair-precision fBm (the planet paths): |err| of the raw sum against the
# binary64 reference, relative to the field's range.  Measured ~1e-14; the
# erosion needs starting heights within ~1e-11 of binary64's to keep its
# flow choices (random raw errors of 1e-10 flipped some on 900,002 vertices).
PAIR_TOL = 2e-13


def _fbm_pair(pts, perm, pgi, scale, strength, radius, per_octave=False, f64=False):
    import ctypes
    from nixis_gb300 import _dev, _lib
    xyz = torch.from_numpy(np.ascontiguousarray(pts, np.float64)).cuda()
    n = len(pts)
    p = torch.from_numpy(perm).cuda()
    g = torch.from_numpy(pgi).cuda()
    pair = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    mm = torch.tensor([-1, 0], dtype=torch.int64, device="cuda")
    out64 = torch.zeros(n, dtype=torch.float64, device="cuda") if f64 else None
    groups = [[o] for o in range(len(scale))] if per_octave else [list(range(len(scale)))]
    for q, grp in enumerate(groups):
        sc = (ctypes.c_double * len(grp))(*[scale[o] for o in grp])
        st = (ctypes.c_double * len(grp))(*[strength[o] for o in grp])
        last = q == len(groups) - 1
        _lib.call("nx_fbm_pair", _dev.ptr(xyz), n, _dev.ptr(p), _dev.ptr(g), len(grp), sc, st, float(radius),
                  max(abs(0.5 * a * radius) for a in strength), _dev.ptr(pair), _dev.ptr(out64) if (f64 and last) else None, 1 if q > 0 else 0,
                  _dev.ptr(mm) if last else None, None, _dev.stream_handle())
    torch.cuda.synchronize()
    return pair.cpu().numpy(), mm.cpu().numpy().view(np.uint64), (out64.cpu().numpy() if f64 else None)


def _unkey(k):
    k = np.uint32(k)
    b = (k ^ np.uint32(0x80000000)) if (k & np.uint32(0x80000000)) else ~k
    return np.array([b], np.uint32).view(np.float32)[0]


@pytest.mark.parametrize("case", ["unit_pow2", "driver_radius"])
def test_fbm_pair_against_binary64(case):
    """The planet paths' fBm: within PAIR_TOL of the reference's binary64
    sums on a 12-octave field (power-of-two scales: base frequency 1,
    lacunarity 2, radius 1; and the reference driver's 1.5/6378100-style
    scales, which take the general coordinate product); one launch over all
    octaves equals one launch per octave bit for bit; the binary64 output is
    hi + lo; min/max keys are those of the extreme pair sums."""
    from nixis_gb300 import terrain
    rng = np.random.default_rng(5)
    u = rng.normal(size=(300_000, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    if case == "unit_pow2":
        R, args = 1.0, (12, 1.0, 1.0, 2.0, 0.5, 1.0)
        pts = u
    else:
        R = 6378100.0
        args = (12, 1.5, 0.4, 2.0, 0.5, R)
        pts = u * R
    perm, pgi = O.init(17)
    scale, strength = terrain._octave_args(*args)
    ref = O.sample_octaves(pts, None, perm, pgi, *args)
    one, mm, o64 = _fbm_pair(pts, perm, pgi, scale, strength, R, f64=True)
    each, _, _ = _fbm_pair(pts, perm, pgi, scale, strength, R, per_octave=True)
    assert np.array_equal(one, each)
    got = one[:, 0].astype(np.float64) + one[:, 1].astype(np.float64)
    assert np.array_equal(o64, got)
    err = np.abs(got - ref).max() / (ref.max() - ref.min())
    assert err <= PAIR_TOL, err
    lo = float(_unkey(mm[0] >> np.uint64(32))) + float(_unkey(mm[0] & np.uint64(0xFFFFFFFF)))
    hi = float(_unkey(mm[1] >> np.uint64(32))) + float(_unkey(mm[1] & np.uint64(0xFFFFFFFF)))
    assert lo == got.min() and hi == got.max()
