/*
 * nx_oracle.c -- CPU restatement of the Nixis per-vertex terrain hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it to produce the
 * expected results.  Nothing in the shipped library links or calls it.
 *
 * Every function restates one reference function in binary64 with the
 * reference's own operation order, so that (built with -ffp-contract=off and
 * without fast-math) its results equal the reference's bit for bit wherever
 * the reference uses only +,-,*,/ and sqrt.  Where the reference calls
 * transcendental functions (insolation), libm's results may differ from
 * numpy's by an ulp; those outputs are compared with a tolerance.
 *
 * Pinning: tests/golden/ holds vectors produced by executing the reference's
 * own Python functions (through tests/golden/ref_shim.py); the CPU test suite
 * checks this file against every one of them.
 *
 * Reference files (paths within the MightyBOBcnc/nixis project):
 *   opensimplex.py  init, over, fastfloor, extrapolate3d, noise3d
 *   terrain.py      sample_noise, sample_octaves, make_bool_elevation_mask
 *   erosion.py      calc_slope, calc_distance, erosion_iteration3,
 *                   erode_terrain3, find_lowest
 *   climate.py      day2deg, calculate_seasonal_tilt, sample_insolation,
 *                   brute_daily_insolation
 *   util.py         xyz2latlon, rescale, find_first, build_adjacency,
 *                   next_vert, sort_adjacency
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define NXO_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------------ */
/* OpenSimplex 3-D                                                           */
/* ------------------------------------------------------------------------ */

/* opensimplex.py:26-27 */
static const double STRETCH_3D = -1.0 / 6;
static const double SQUISH_3D = 1.0 / 3;
/* opensimplex.py:32 */
static const double NORM_3D = 103;

/* opensimplex.py:51-60: 24 gradient vectors (72 ints), directions to the
 * vertices of a rhombicuboctahedron.  A data table: it has to be identical. */
static const int GRAD3[72] = {
    -11, 4, 4, -4, 11, 4, -4, 4, 11,
    11, 4, 4, 4, 11, 4, 4, 4, 11,
    -11, -4, 4, -4, -11, 4, -4, -4, 11,
    11, -4, 4, 4, -11, 4, 4, -4, 11,
    -11, 4, -4, -4, 11, -4, -4, 4, -11,
    11, 4, -4, 4, 11, -4, 4, 4, -11,
    -11, -4, -4, -4, -11, -4, -4, -4, -11,
    11, -4, -4, 4, -11, -4, 4, -4, -11,
};

/* opensimplex.py:110-112: `over` has the numba signature int32(int32), so
 * its argument is truncated to the low 32 bits and sign-extended. */
static int64_t trunc_i32(uint64_t v) { return (int64_t)(int32_t)(uint32_t)v; }

/* opensimplex.py:90-107.  The 64-bit LCG step wraps (numba int64), then the
 * state is truncated to int32; `r` is Python/numba floor-mod. */
NXO_API int nxo_perm_init(int64_t seed, int32_t *perm, int32_t *pgi)
{
    const uint64_t MUL = 6364136223846793005ULL, ADD = 1442695040888963407ULL;
    int64_t source[256];
    for (int i = 0; i < 256; ++i) source[i] = i;
    int64_t s = seed;
    for (int k = 0; k < 3; ++k) s = trunc_i32((uint64_t)s * MUL + ADD);
    for (int i = 255; i >= 0; --i) {
        s = trunc_i32((uint64_t)s * MUL + ADD);
        int64_t m = i + 1;
        int64_t r = (s + 31) % m;
        if (r < 0) r += m;               /* floor-mod */
        perm[i] = (int32_t)source[r];
        /* int((perm[i] % 24.0) * 3) */
        pgi[i] = (int32_t)(fmod((double)perm[i], 24.0) * 3.0);
        source[r] = source[i];
    }
    return 0;
}

/* opensimplex.py:18-21 */
static int64_t fastfloor(double x)
{
    int64_t xi = (int64_t)x;
    return x < (double)xi ? xi - 1 : xi;
}

/* opensimplex.py:123-131 */
static double extrapolate3d(int64_t xsb, int64_t ysb, int64_t zsb, double dx, double dy,
                            double dz, const int32_t *perm, const int32_t *pgi)
{
    int64_t idx = pgi[(perm[(perm[xsb & 0xFF] + ysb) & 0xFF] + zsb) & 0xFF];
    return (double)GRAD3[idx] * dx + (double)GRAD3[idx + 1] * dy + (double)GRAD3[idx + 2] * dz;
}

/*
 * opensimplex.py:266-759.  `trace`, when not NULL, receives the integer
 * decisions: [xsb, ysb, zsb, region (0: tetra at 0, 1: tetra at 1,
 * 2: octahedron), ext0 (x,y,z), ext1 (x,y,z)].
 *
 * The contributions are added to `value` in the reference's order, each one
 * only when its attenuation 2 - |d|^2 is positive (ADDC).
 */
#define ADDC(xv, yv, zv, dx, dy, dz)                                          \
    do {                                                                      \
        double _a = 2 - (dx) * (dx) - (dy) * (dy) - (dz) * (dz);              \
        if (_a > 0) {                                                         \
            _a *= _a;                                                         \
            value += _a * _a * extrapolate3d(xv, yv, zv, dx, dy, dz, perm, pgi); \
            if (calls && calls[0] < 8) {                                      \
                int32_t *_c = calls + 1 + 3 * calls[0];                       \
                _c[0] = (int32_t)(xv); _c[1] = (int32_t)(yv); _c[2] = (int32_t)(zv); \
                calls[0] += 1;                                                \
            }                                                                 \
        }                                                                     \
    } while (0)

/* `calls`, when not NULL, receives the lattice points that were hashed
 * (extrapolate3d calls), in call order: [count, x0, y0, z0, x1, ...], 25 ints. */
NXO_API double nxo_noise3d_trace(double x, double y, double z, const int32_t *perm,
                                 const int32_t *pgi, int32_t *trace, int32_t *calls)
{
    if (calls) memset(calls, 0, 25 * sizeof(int32_t));
    double stretch = (x + y + z) * STRETCH_3D;
    double xs = x + stretch, ys = y + stretch, zs = z + stretch;
    int64_t xsb = fastfloor(xs), ysb = fastfloor(ys), zsb = fastfloor(zs);
    double squish = (double)(xsb + ysb + zsb) * SQUISH_3D;
    double xb = (double)xsb + squish, yb = (double)ysb + squish, zb = (double)zsb + squish;
    double xins = xs - (double)xsb, yins = ys - (double)ysb, zins = zs - (double)zsb;
    double in_sum = xins + yins + zins;
    double dx0 = x - xb, dy0 = y - yb, dz0 = z - zb;

    int64_t xe0, ye0, ze0, xe1, ye1, ze1;
    double dxe0, dye0, dze0, dxe1, dye1, dze1;
    double value = 0;
    int region;

    if (in_sum <= 1) {
        region = 0;
        /* which two of (0,0,1), (0,1,0), (1,0,0) are closest */
        int ap = 0x01, bp = 0x02;
        double as = xins, bs = yins;
        if (as >= bs && zins > bs) { bs = zins; bp = 0x04; }
        else if (as < bs && zins > as) { as = zins; ap = 0x04; }
        double wins = 1 - in_sum;
        if (wins > as || wins > bs) {
            int c = (bs > as) ? bp : ap;
            if ((c & 0x01) == 0) { xe0 = xsb - 1; xe1 = xsb; dxe0 = dx0 + 1; dxe1 = dx0; }
            else { xe0 = xe1 = xsb + 1; dxe0 = dxe1 = dx0 - 1; }
            if ((c & 0x02) == 0) {
                ye0 = ye1 = ysb; dye0 = dye1 = dy0;
                if ((c & 0x01) == 0) { ye1 -= 1; dye1 += 1; }
                else { ye0 -= 1; dye0 += 1; }
            } else { ye0 = ye1 = ysb + 1; dye0 = dye1 = dy0 - 1; }
            if ((c & 0x04) == 0) { ze0 = zsb; ze1 = zsb - 1; dze0 = dz0; dze1 = dz0 + 1; }
            else { ze0 = ze1 = zsb + 1; dze0 = dze1 = dz0 - 1; }
        } else {
            int c = ap | bp;
            if ((c & 0x01) == 0) { xe0 = xsb; xe1 = xsb - 1; dxe0 = dx0 - 2 * SQUISH_3D; dxe1 = dx0 + 1 - SQUISH_3D; }
            else { xe0 = xe1 = xsb + 1; dxe0 = dx0 - 1 - 2 * SQUISH_3D; dxe1 = dx0 - 1 - SQUISH_3D; }
            if ((c & 0x02) == 0) { ye0 = ysb; ye1 = ysb - 1; dye0 = dy0 - 2 * SQUISH_3D; dye1 = dy0 + 1 - SQUISH_3D; }
            else { ye0 = ye1 = ysb + 1; dye0 = dy0 - 1 - 2 * SQUISH_3D; dye1 = dy0 - 1 - SQUISH_3D; }
            if ((c & 0x04) == 0) { ze0 = zsb; ze1 = zsb - 1; dze0 = dz0 - 2 * SQUISH_3D; dze1 = dz0 + 1 - SQUISH_3D; }
            else { ze0 = ze1 = zsb + 1; dze0 = dz0 - 1 - 2 * SQUISH_3D; dze1 = dz0 - 1 - SQUISH_3D; }
        }
        ADDC(xsb, ysb, zsb, dx0, dy0, dz0);
        double dx1 = dx0 - 1 - SQUISH_3D, dy1 = dy0 - 0 - SQUISH_3D, dz1 = dz0 - 0 - SQUISH_3D;
        ADDC(xsb + 1, ysb, zsb, dx1, dy1, dz1);
        double dx2 = dx0 - 0 - SQUISH_3D, dy2 = dy0 - 1 - SQUISH_3D, dz2 = dz1;
        ADDC(xsb, ysb + 1, zsb, dx2, dy2, dz2);
        double dx3 = dx2, dy3 = dy1, dz3 = dz0 - 1 - SQUISH_3D;
        ADDC(xsb, ysb, zsb + 1, dx3, dy3, dz3);
    } else if (in_sum >= 2) {
        region = 1;
        /* which two of (1,1,0), (1,0,1), (0,1,1) are closest */
        int ap = 0x06, bp = 0x05;
        double as = xins, bs = yins;
        if (as <= bs && zins < bs) { bs = zins; bp = 0x03; }
        else if (as > bs && zins < as) { as = zins; ap = 0x03; }
        double wins = 3 - in_sum;
        if (wins < as || wins < bs) {
            int c = (bs < as) ? bp : ap;
            if ((c & 0x01) != 0) { xe0 = xsb + 2; xe1 = xsb + 1; dxe0 = dx0 - 2 - 3 * SQUISH_3D; dxe1 = dx0 - 1 - 3 * SQUISH_3D; }
            else { xe0 = xe1 = xsb; dxe0 = dxe1 = dx0 - 3 * SQUISH_3D; }
            if ((c & 0x02) != 0) {
                ye0 = ye1 = ysb + 1; dye0 = dye1 = dy0 - 1 - 3 * SQUISH_3D;
                if ((c & 0x01) != 0) { ye1 += 1; dye1 -= 1; }
                else { ye0 += 1; dye0 -= 1; }
            } else { ye0 = ye1 = ysb; dye0 = dye1 = dy0 - 3 * SQUISH_3D; }
            if ((c & 0x04) != 0) { ze0 = zsb + 1; ze1 = zsb + 2; dze0 = dz0 - 1 - 3 * SQUISH_3D; dze1 = dz0 - 2 - 3 * SQUISH_3D; }
            else { ze0 = ze1 = zsb; dze0 = dze1 = dz0 - 3 * SQUISH_3D; }
        } else {
            int c = ap & bp;
            if ((c & 0x01) != 0) { xe0 = xsb + 1; xe1 = xsb + 2; dxe0 = dx0 - 1 - SQUISH_3D; dxe1 = dx0 - 2 - 2 * SQUISH_3D; }
            else { xe0 = xe1 = xsb; dxe0 = dx0 - SQUISH_3D; dxe1 = dx0 - 2 * SQUISH_3D; }
            if ((c & 0x02) != 0) { ye0 = ysb + 1; ye1 = ysb + 2; dye0 = dy0 - 1 - SQUISH_3D; dye1 = dy0 - 2 - 2 * SQUISH_3D; }
            else { ye0 = ye1 = ysb; dye0 = dy0 - SQUISH_3D; dye1 = dy0 - 2 * SQUISH_3D; }
            if ((c & 0x04) != 0) { ze0 = zsb + 1; ze1 = zsb + 2; dze0 = dz0 - 1 - SQUISH_3D; dze1 = dz0 - 2 - 2 * SQUISH_3D; }
            else { ze0 = ze1 = zsb; dze0 = dz0 - SQUISH_3D; dze1 = dz0 - 2 * SQUISH_3D; }
        }
        double dx3 = dx0 - 1 - 2 * SQUISH_3D, dy3 = dy0 - 1 - 2 * SQUISH_3D, dz3 = dz0 - 0 - 2 * SQUISH_3D;
        ADDC(xsb + 1, ysb + 1, zsb, dx3, dy3, dz3);
        double dx2 = dx3, dy2 = dy0 - 0 - 2 * SQUISH_3D, dz2 = dz0 - 1 - 2 * SQUISH_3D;
        ADDC(xsb + 1, ysb, zsb + 1, dx2, dy2, dz2);
        double dx1 = dx0 - 0 - 2 * SQUISH_3D, dy1 = dy3, dz1 = dz2;
        ADDC(xsb, ysb + 1, zsb + 1, dx1, dy1, dz1);
        double dxa = dx0 - 1 - 3 * SQUISH_3D, dya = dy0 - 1 - 3 * SQUISH_3D, dza = dz0 - 1 - 3 * SQUISH_3D;
        ADDC(xsb + 1, ysb + 1, zsb + 1, dxa, dya, dza);
    } else {
        region = 2;
        /* octahedron: (0,0,1) vs (1,1,0) */
        double as, bs;
        int ap, bp, a_far, b_far;
        double p1 = xins + yins;
        if (p1 > 1) { as = p1 - 1; ap = 0x03; a_far = 1; }
        else { as = 1 - p1; ap = 0x04; a_far = 0; }
        /* (0,1,0) vs (1,0,1) */
        double p2 = xins + zins;
        if (p2 > 1) { bs = p2 - 1; bp = 0x05; b_far = 1; }
        else { bs = 1 - p2; bp = 0x02; b_far = 0; }
        /* (1,0,0) vs (0,1,1) replaces the further of the two if closer */
        double p3 = yins + zins;
        if (p3 > 1) {
            double score = p3 - 1;
            if (as <= bs && as < score) { ap = 0x06; a_far = 1; }
            else if (as > bs && bs < score) { bp = 0x06; b_far = 1; }
        } else {
            double score = 1 - p3;
            if (as <= bs && as < score) { ap = 0x01; a_far = 0; }
            else if (as > bs && bs < score) { bp = 0x01; b_far = 0; }
        }
        if (a_far == b_far) {
            if (a_far) {
                dxe0 = dx0 - 1 - 3 * SQUISH_3D; dye0 = dy0 - 1 - 3 * SQUISH_3D; dze0 = dz0 - 1 - 3 * SQUISH_3D;
                xe0 = xsb + 1; ye0 = ysb + 1; ze0 = zsb + 1;
                int c = ap & bp;
                if ((c & 0x01) != 0) {
                    dxe1 = dx0 - 2 - 2 * SQUISH_3D; dye1 = dy0 - 2 * SQUISH_3D; dze1 = dz0 - 2 * SQUISH_3D;
                    xe1 = xsb + 2; ye1 = ysb; ze1 = zsb;
                } else if ((c & 0x02) != 0) {
                    dxe1 = dx0 - 2 * SQUISH_3D; dye1 = dy0 - 2 - 2 * SQUISH_3D; dze1 = dz0 - 2 * SQUISH_3D;
                    xe1 = xsb; ye1 = ysb + 2; ze1 = zsb;
                } else {
                    dxe1 = dx0 - 2 * SQUISH_3D; dye1 = dy0 - 2 * SQUISH_3D; dze1 = dz0 - 2 - 2 * SQUISH_3D;
                    xe1 = xsb; ye1 = ysb; ze1 = zsb + 2;
                }
            } else {
                dxe0 = dx0; dye0 = dy0; dze0 = dz0;
                xe0 = xsb; ye0 = ysb; ze0 = zsb;
                int c = ap | bp;
                if ((c & 0x01) == 0) {
                    dxe1 = dx0 + 1 - SQUISH_3D; dye1 = dy0 - 1 - SQUISH_3D; dze1 = dz0 - 1 - SQUISH_3D;
                    xe1 = xsb - 1; ye1 = ysb + 1; ze1 = zsb + 1;
                } else if ((c & 0x02) == 0) {
                    dxe1 = dx0 - 1 - SQUISH_3D; dye1 = dy0 + 1 - SQUISH_3D; dze1 = dz0 - 1 - SQUISH_3D;
                    xe1 = xsb + 1; ye1 = ysb - 1; ze1 = zsb + 1;
                } else {
                    dxe1 = dx0 - 1 - SQUISH_3D; dye1 = dy0 - 1 - SQUISH_3D; dze1 = dz0 + 1 - SQUISH_3D;
                    xe1 = xsb + 1; ye1 = ysb + 1; ze1 = zsb - 1;
                }
            }
        } else {
            int c1 = a_far ? ap : bp;
            int c2 = a_far ? bp : ap;
            if ((c1 & 0x01) == 0) {
                dxe0 = dx0 + 1 - SQUISH_3D; dye0 = dy0 - 1 - SQUISH_3D; dze0 = dz0 - 1 - SQUISH_3D;
                xe0 = xsb - 1; ye0 = ysb + 1; ze0 = zsb + 1;
            } else if ((c1 & 0x02) == 0) {
                dxe0 = dx0 - 1 - SQUISH_3D; dye0 = dy0 + 1 - SQUISH_3D; dze0 = dz0 - 1 - SQUISH_3D;
                xe0 = xsb + 1; ye0 = ysb - 1; ze0 = zsb + 1;
            } else {
                dxe0 = dx0 - 1 - SQUISH_3D; dye0 = dy0 - 1 - SQUISH_3D; dze0 = dz0 + 1 - SQUISH_3D;
                xe0 = xsb + 1; ye0 = ysb + 1; ze0 = zsb - 1;
            }
            dxe1 = dx0 - 2 * SQUISH_3D; dye1 = dy0 - 2 * SQUISH_3D; dze1 = dz0 - 2 * SQUISH_3D;
            xe1 = xsb; ye1 = ysb; ze1 = zsb;
            if ((c2 & 0x01) != 0) { dxe1 -= 2; xe1 += 2; }
            else if ((c2 & 0x02) != 0) { dye1 -= 2; ye1 += 2; }
            else { dze1 -= 2; ze1 += 2; }
        }
        double dx1 = dx0 - 1 - SQUISH_3D, dy1 = dy0 - 0 - SQUISH_3D, dz1 = dz0 - 0 - SQUISH_3D;
        ADDC(xsb + 1, ysb, zsb, dx1, dy1, dz1);
        double dx2 = dx0 - 0 - SQUISH_3D, dy2 = dy0 - 1 - SQUISH_3D, dz2 = dz1;
        ADDC(xsb, ysb + 1, zsb, dx2, dy2, dz2);
        double dx3 = dx2, dy3 = dy1, dz3 = dz0 - 1 - SQUISH_3D;
        ADDC(xsb, ysb, zsb + 1, dx3, dy3, dz3);
        double dx4 = dx0 - 1 - 2 * SQUISH_3D, dy4 = dy0 - 1 - 2 * SQUISH_3D, dz4 = dz0 - 0 - 2 * SQUISH_3D;
        ADDC(xsb + 1, ysb + 1, zsb, dx4, dy4, dz4);
        double dx5 = dx4, dy5 = dy0 - 0 - 2 * SQUISH_3D, dz5 = dz0 - 1 - 2 * SQUISH_3D;
        ADDC(xsb + 1, ysb, zsb + 1, dx5, dy5, dz5);
        double dx6 = dx0 - 0 - 2 * SQUISH_3D, dy6 = dy4, dz6 = dz5;
        ADDC(xsb, ysb + 1, zsb + 1, dx6, dy6, dz6);
    }
    ADDC(xe0, ye0, ze0, dxe0, dye0, dze0);
    ADDC(xe1, ye1, ze1, dxe1, dye1, dze1);

    if (trace) {
        trace[0] = (int32_t)xsb; trace[1] = (int32_t)ysb; trace[2] = (int32_t)zsb;
        trace[3] = region;
        trace[4] = (int32_t)xe0; trace[5] = (int32_t)ye0; trace[6] = (int32_t)ze0;
        trace[7] = (int32_t)xe1; trace[8] = (int32_t)ye1; trace[9] = (int32_t)ze1;
    }
    return value / NORM_3D;
}

NXO_API double nxo_noise3d(double x, double y, double z, const int32_t *perm, const int32_t *pgi)
{
    return nxo_noise3d_trace(x, y, z, perm, pgi, NULL, NULL);
}

/* Batch form of noise3d with the lattice trace (10 ints per point) and the
 * hashed lattice points (25 ints per point). */
NXO_API void nxo_noise3d_batch(const double *xyz, int64_t n, const int32_t *perm,
                               const int32_t *pgi, double *out, int32_t *trace, int32_t *calls)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
        out[i] = nxo_noise3d_trace(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], perm, pgi,
                                   trace ? trace + 10 * i : NULL, calls ? calls + 25 * i : NULL);
}

/* terrain.py:12-28: noise3d(v * roughness), then (e + 1) * 0.5 * strength * radius */
NXO_API void nxo_sample_noise(const double *xyz, int64_t n, const int32_t *perm,
                              const int32_t *pgi, double roughness, double strength,
                              double radius, double *out)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double e = nxo_noise3d(xyz[3 * i] * roughness, xyz[3 * i + 1] * roughness,
                               xyz[3 * i + 2] * roughness, perm, pgi);
        out[i] = (e + 1) * 0.5 * strength * radius;
    }
}

/* terrain.py:32-59: elevations += sample_noise(verts, f / R, a / R, R) per
 * octave; f *= roughness, a *= persistence.  `elev` is accumulated in place
 * (the caller passes zeros for `elevations=None`). */
NXO_API void nxo_sample_octaves(const double *xyz, int64_t n, double *elev, const int32_t *perm,
                                const int32_t *pgi, int n_octaves, double init_roughness,
                                double init_strength, double roughness, double persistence,
                                double world_radius)
{
    double f0[64], a0[64];
    if (n_octaves > 64) n_octaves = 64;
    double f = init_roughness, a = init_strength;
    for (int o = 0; o < n_octaves; ++o) {
        f0[o] = f / world_radius;
        a0[o] = a / world_radius;
        f *= roughness;
        a *= persistence;
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double acc = elev[i];
        for (int o = 0; o < n_octaves; ++o) {
            double e = nxo_noise3d(xyz[3 * i] * f0[o], xyz[3 * i + 1] * f0[o],
                                   xyz[3 * i + 2] * f0[o], perm, pgi);
            acc += (e + 1) * 0.5 * a0[o] * world_radius;
        }
        elev[i] = acc;
    }
}

/* terrain.py:61-72 */
NXO_API void nxo_make_bool_elevation_mask(const double *h, int64_t n, double level, uint8_t *mask)
{
    for (int64_t i = 0; i < n; ++i) mask[i] = h[i] <= level ? 1 : 0;
}

/* ------------------------------------------------------------------------ */
/* Erosion (variant 3)                                                       */
/* ------------------------------------------------------------------------ */

/* erosion.py:38-40; `**2` is a correctly rounded square. */
static double calc_distance(const double *a, const double *b)
{
    double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return sqrt(dx * dx + dy * dy + dz * dz);
}

/* erosion.py:205-207 */
#define EVAPORATION (0.1 / 320)
#define SOLUBILITY (0.01 / 320)
#define CAPACITY (0.2 / 320)

/* erosion.py:197-279: Jacobi update.  All reads come from the input arrays,
 * writes go to copies that replace the inputs at the end. */
NXO_API int nxo_erosion_iteration3(const double *xyz, const int32_t *nbr, int64_t n, double *h,
                                   double *w, double *s)
{
    double *hb = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    double *wb = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    double *sb = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (!hb || !wb || !sb) { free(hb); free(wb); free(sb); return -1; }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double self = h[i];
        double sed_amt = s[i], wat_amt = w[i];
        for (int k = 0; k < 6; ++k) {
            int32_t j = nbr[6 * i + k];
            if (j == -1) continue;
            double d = calc_distance(xyz + 3 * i, xyz + 3 * (int64_t)j);
            double slope = (h[j] - self) / (d + 0.00001);       /* erosion.py:34-36 */
            if (slope > 0) { sed_amt += SOLUBILITY * w[j]; wat_amt += w[j] * d; }
            else if (slope < 0) { sed_amt -= SOLUBILITY * w[j]; wat_amt -= w[j] * d; }
        }
        double hn = h[i] - sed_amt;
        double sn = s[i] + sed_amt;
        double wn = w[i] + (wat_amt - wat_amt * EVAPORATION);
        if (sn > CAPACITY * wn) {
            hn += sn - CAPACITY * wn;
            sn -= sn - CAPACITY * wn;
        }
        hb[i] = hn; sb[i] = sn; wb[i] = wn;
    }
    memcpy(h, hb, sizeof(double) * (size_t)n);
    memcpy(w, wb, sizeof(double) * (size_t)n);
    memcpy(s, sb, sizeof(double) * (size_t)n);
    free(hb); free(wb); free(sb);
    return 0;
}

/* erosion.py:172-192 (without snapshots): num_iter <= 0 runs once; water and
 * sediment start at zero; rain 0.3/320 is added before each iteration. */
NXO_API int nxo_erode_terrain3(const double *xyz, const int32_t *nbr, int64_t n, double *h,
                               int num_iter)
{
    if (num_iter <= 0) num_iter = 1;
    double *w = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    double *s = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    if (!w || !s) { free(w); free(s); return -1; }
    const double rain = 0.3 / 320;
    for (int it = 0; it < num_iter; ++it) {
        for (int64_t i = 0; i < n; ++i) w[i] += rain;
        if (nxo_erosion_iteration3(xyz, nbr, n, h, w, s)) { free(w); free(s); return -1; }
    }
    free(w); free(s);
    return 0;
}

/*
 * The same update evaluated with the GPU kernel's arithmetic, operation for
 * operation, so the kernel can be checked bit for bit.  Height, water and
 * sediment are unevaluated pairs hi + lo of binary32s (about 48 significant
 * bits); edge lengths are supplied per neighbour slot as pairs too
 * (edge_len[12*i+2k] + edge_len[12*i+2k+1], computed once in binary64).  State rows are 8
 * floats: (h_hi, h_lo, w_hi, w_lo, s_hi, s_lo, 0, 0).  `rain` (binary32) is
 * added to every vertex's water before the update, as erode_terrain3 does
 * (erosion.py:182-184).
 *
 * Per neighbour j in slot order the flow sign g (+1, -1, 0) is the sign of
 * (hj_hi - hi_hi) + (hj_lo - hi_lo); the update accumulates S = sum g*w_j
 * and W = w_i + sum g*w_j*d_j (erosion.py:238-247) in pairs, then
 * sed_amt = s_i + sol*S, h -= sed_amt, s += sed_amt,
 * w = w_i + W*(1 - evap), and the capacity test moves s - cap*w to h
 * (erosion.py:261-267).  sol, 1 - evap and cap are binary64 constants
 * split into pairs.
 */
typedef struct { float h, l; } nxo_pair;

/* Knuth's two-sum: s + e == a + b exactly. */
static void two_sum(float a, float b, float *s, float *e)
{
    float x = a + b;
    float bb = x - a;
    *e = (a - (x - bb)) + (b - bb);
    *s = x;
}

/* pair + pair, renormalised */
static nxo_pair padd(nxo_pair a, nxo_pair b)
{
    float s, e;
    two_sum(a.h, b.h, &s, &e);
    e = e + (a.l + b.l);
    nxo_pair r;
    r.h = s + e;
    r.l = e - (r.h - s);
    return r;
}

/* pair * (ch + cl), not renormalised */
static nxo_pair pmul(nxo_pair a, float ch, float cl)
{
    nxo_pair r;
    r.h = a.h * ch;
    float e = fmaf(a.h, ch, -r.h);
    e = fmaf(a.h, cl, e);
    r.l = fmaf(a.l, ch, e);
    return r;
}

/* (wh + wl) + r with r binary32, not renormalised */
static nxo_pair prain(float wh, float wl, float r)
{
    float s, e;
    two_sum(wh, r, &s, &e);
    nxo_pair x = {s, wl + e};
    return x;
}

static void split_const(double c, float *h, float *l)
{
    *h = (float)c;
    *l = (float)(c - (double)*h);
}

NXO_API void nxo_erosion_iteration3_pair(const float *edge_len, const int32_t *nbr, int64_t n, const float *st,
                                         float rain, float *out)
{
    float sol_h, sol_l, oe_h, oe_l, cap_h, cap_l;
    split_const(SOLUBILITY, &sol_h, &sol_l);
    split_const(1.0 - EVAPORATION, &oe_h, &oe_l);
    split_const(CAPACITY, &cap_h, &cap_l);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const float *me = st + 8 * i;
        const nxo_pair hi = {me[0], me[1]}, si = {me[4], me[5]};
        const nxo_pair wi = prain(me[2], me[3], rain);
        float Sh = 0.0f, Sl = 0.0f, Wh = wi.h, Wl = wi.l;
        for (int k = 0; k < 6; ++k) {
            int32_t j = nbr[6 * i + k];
            if (j == -1) continue;
            const float dh = edge_len[12 * i + 2 * k], dl = edge_len[12 * i + 2 * k + 1];
            const float *o = st + 8 * (int64_t)j;
            const float diff = (o[0] - hi.h) + (o[1] - hi.l);
            const float g = diff > 0 ? 1.0f : (diff < 0 ? -1.0f : 0.0f);
            const nxo_pair wj = prain(o[2], o[3], rain);
            const float xh = g * wj.h, xl = g * wj.l;
            const float p = xh * dh;
            float pe = fmaf(xh, dh, -p);
            pe = fmaf(xh, dl, pe);
            pe = fmaf(xl, dh, pe);
            float s, e;
            two_sum(Sh, xh, &s, &e);
            Sl = Sl + (e + xl);
            Sh = s;
            two_sum(Wh, p, &s, &e);
            Wl = Wl + (e + pe);
            Wh = s;
        }
        const nxo_pair S = {Sh, Sl}, W = {Wh, Wl};
        const nxo_pair sed = padd(si, pmul(S, sol_h, sol_l));
        const nxo_pair nsed = {-sed.h, -sed.l};
        nxo_pair hn = padd(hi, nsed);
        nxo_pair sn = padd(si, sed);
        const nxo_pair wn = padd(wi, pmul(W, oe_h, oe_l));
        const nxo_pair c = pmul(wn, cap_h, cap_l);
        nxo_pair cw;
        cw.h = c.h + c.l;
        cw.l = c.l - (cw.h - c.h);
        if ((sn.h - cw.h) + (sn.l - cw.l) > 0) {
            const nxo_pair ncw = {-cw.h, -cw.l};
            const nxo_pair ex = padd(sn, ncw);
            hn = padd(hn, ex);
            sn = cw;
        }
        float *q = out + 8 * i;
        q[0] = hn.h; q[1] = hn.l; q[2] = wn.h; q[3] = wn.l; q[4] = sn.h; q[5] = sn.l; q[6] = 0.0f; q[7] = 0.0f;
    }
}

/* erosion.py:398-406 with util.py:580-587: among the neighbours that are not
 * -1, the position (in that filtered list) of the first minimum, if it is
 * strictly lower than the vertex itself; -1 otherwise (the reference returns
 * None). */
NXO_API int nxo_find_lowest(int64_t vert, const int32_t *nbr6, const double *h)
{
    double alts[6];
    int m = 0;
    for (int k = 0; k < 6; ++k)
        if (nbr6[k] != -1) alts[m++] = h[nbr6[k]];
    if (m == 0) return -1;
    double lowest = alts[0];
    for (int k = 1; k < m; ++k)
        if (alts[k] < lowest) lowest = alts[k];
    if (lowest < h[vert]) {
        for (int k = 0; k < m; ++k)
            if (alts[k] == lowest) return k;
    }
    return -1;
}

/* ------------------------------------------------------------------------ */
/* Insolation                                                                */
/* ------------------------------------------------------------------------ */

static const double PI = 3.141592653589793;

/* climate.py:167-171 */
NXO_API double nxo_day2deg(double year_length, double day) { return (day / year_length) * 360.0; }

/* climate.py:192-201 */
NXO_API double nxo_calculate_seasonal_tilt(double axial_tilt, double degrees)
{
    return sin(degrees * PI / 180) * axial_tilt;
}

/* climate.py:415-444 with util.py:59-75 (xyz2latlon): one insolation term. */
static double insolation_term(double x, double y, double z, double radius, double cr, double sr,
                              double ct, double st)
{
    double rx = x * cr - y * sr;
    double ry = x * sr + y * cr;
    double rz = z;
    double tx = rx * ct + rz * st;
    double ty = ry;
    double tz = rz * ct - rx * st;
    double q = tz / radius;
    if (q < -1) q = -1;
    if (q > 1) q = 1;
    double lat = asin(q) * (180.0 / PI);
    double lon = atan2(ty, tx) * (180.0 / PI);
    double a = cos(fabs(lat) * PI / 180);
    double b = cos(lon * PI / 180);
    if (a < 0) a = 0;
    if (b < 0) b = 0;
    return a * b;
}

/* climate.py:415-444: arr (float32) += term, rounded to binary32 each call. */
NXO_API void nxo_sample_insolation(float *arr, const double *xyz, int64_t n, double radius,
                                   double rotation, double tilt)
{
    double cr = cos(rotation * PI / 180), sr = sin(rotation * PI / 180);
    double ct = cos(tilt * PI / 180), st = sin(tilt * PI / 180);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
        arr[i] = (float)((double)arr[i] +
                         insolation_term(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], radius, cr, sr, ct, st));
}

/* Same terms accumulated in binary64 (the exact-sum comparator). */
NXO_API void nxo_sample_insolation_f64(double *arr, const double *xyz, int64_t n, double radius,
                                       double rotation, double tilt)
{
    double cr = cos(rotation * PI / 180), sr = sin(rotation * PI / 180);
    double ct = cos(tilt * PI / 180), st = sin(tilt * PI / 180);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
        arr[i] += insolation_term(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], radius, cr, sr, ct, st);
}

/*
 * Sum of sample_insolation over `days` x `hours` sun positions:
 * rotation = -180 + (360/hours) * h, tilt = calculate_seasonal_tilt(axial_tilt,
 * day2deg(year_length, d)).  This is the brute_daily_insolation loop
 * (climate.py:450-489) run once per day of a year.  Accumulated in binary64
 * into acc (per vertex); acc32, when not NULL, receives the reference's
 * binary32 running sum.
 */
NXO_API void nxo_annual_insolation(const double *xyz, int64_t n, double radius, double axial_tilt,
                                   int year_length, int days, int hours, double *acc, float *acc32)
{
    double rot_amt = 360.0 / hours;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double s = 0;
        float s32 = 0.0f;
        for (int d = 0; d < days; ++d) {
            double tilt = nxo_calculate_seasonal_tilt(axial_tilt, nxo_day2deg((double)year_length, (double)d));
            double ct = cos(tilt * PI / 180), st = sin(tilt * PI / 180);
            double rotation = -180.0;
            for (int h = 0; h < hours; ++h) {
                double cr = cos(rotation * PI / 180), sr = sin(rotation * PI / 180);
                double t = insolation_term(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], radius, cr, sr, ct, st);
                s += t;
                s32 = (float)((double)s32 + t);
                rotation += rot_amt;
            }
        }
        acc[i] += s;
        if (acc32) acc32[i] = s32;
    }
}

/* util.py:79-88 */
static void latlon2xyz(double lat, double lon, double r, double *o)
{
    o[0] = r * cos(lat * (PI / 180)) * cos(lon * (PI / 180));
    o[1] = r * cos(lat * (PI / 180)) * sin(lon * (PI / 180));
    o[2] = r * sin(lat * (PI / 180));
}

/* climate.py:503-533: 181 entries, entry i holding latitude i for i <= 90
 * and i - 181 above (the reference's negative indexing), each the binary32
 * sum of sample_insolation over 360 rotations of 1 degree from -180. */
NXO_API void nxo_calc_insolation_slice(double radius, double tilt, float *out)
{
    double v[181 * 3];
    for (int i = -90; i <= 90; ++i) latlon2xyz((double)i, 0.0, radius, v + 3 * ((i + 181) % 181));
    for (int i = 0; i < 181; ++i) out[i] = 0.0f;
    double rotation = -180.0;
    for (int x = 0; x < 360; ++x) {
        double cr = cos(rotation * PI / 180), sr = sin(rotation * PI / 180);
        double ct = cos(tilt * PI / 180), st = sin(tilt * PI / 180);
        for (int i = 0; i < 181; ++i)
            out[i] = (float)((double)out[i] + insolation_term(v[3 * i], v[3 * i + 1], v[3 * i + 2], radius, cr, sr, ct, st));
        rotation += 1.0;
    }
}

/* climate.py:551-577: linear interpolation between the table entries of
 * floor(lat) and ceil(lat) (the latitude depends on z only); the difference of the two binary32 entries is
 * taken in binary32, the rest in binary64, the result rounded to binary32. */
static float interp_one(const float *table, double z, double radius)
{
    double q = z / radius;
    if (q < -1) q = -1;
    if (q > 1) q = 1;
    const double lat = asin(q) * (180.0 / PI);
    const long lower = (long)floor(lat), upper = (long)ceil(lat);
    const float tl = table[(lower + 181) % 181], tu = table[(upper + 181) % 181];
    if (lower == upper) return tl;
    const float dt = tu - tl;
    return (float)((double)tl + (lat - (double)lower) * ((double)dt / (double)(upper - lower)));
}

NXO_API void nxo_interpolate_insolation(const double *xyz, int64_t n, const float *table, float *out, double radius)
{
    for (int64_t i = 0; i < n; ++i) out[i] = interp_one(table, xyz[3 * i + 2], radius);
}

/* climate.py:345-411 (assign_surface_temp) per vertex: max(cos(|lat - tilt|
 * * pi / 180), 0) as binary32, lat as util.xyz2latlon (util.py:59-75).  The
 * altitude term rescale(altitudes, 0, 0) is 0 or NaN everywhere, never > 0,
 * so the reference's altitude branch does not contribute. */
NXO_API void nxo_assign_surface_temp(const double *xyz, int64_t n, double radius, double tilt, float *out)
{
    for (int64_t i = 0; i < n; ++i) {
        double q = xyz[3 * i + 2] / radius;
        if (q < -1) q = -1;
        if (q > 1) q = 1;
        const double lat = asin(q) * (180.0 / PI);
        const double c = cos(fabs(lat - tilt) * PI / 180);
        out[i] = (float)(0.0 > c ? 0.0 : c);     /* Python max(c, 0): c unless 0 > c */
    }
}

/* climate.py:579-597 (no snapshots): 360 daily tables at the seasonal tilt
 * of each orbital degree, interpolated and summed in binary32. */
NXO_API void nxo_calc_yearly_insolation(const double *xyz, int64_t n, double radius, double axial_tilt, float *out)
{
    float *tab = (float *)malloc(sizeof(float) * 181 * 360);
    if (!tab) return;
    for (int d = 0; d < 360; ++d) nxo_calc_insolation_slice(radius, nxo_calculate_seasonal_tilt(axial_tilt, (double)d),
                                                             tab + 181 * d);
    for (int64_t i = 0; i < n; ++i) {
        float acc = 0.0f;
        for (int d = 0; d < 360; ++d)
            acc = acc + interp_one(tab + 181 * d, xyz[3 * i + 2], radius);
        out[i] = acc;
    }
    free(tab);
}

/* util.py:290-310 (make_ll_arr): pixel (h, w) of a width x height map at
 * latitude max(90 - h*180/(height-1), -90), longitude max(-180 + w*360/width,
 * -180), as xyz on the sphere of the radius. */
NXO_API void nxo_make_ll(int width, int height, double radius, double *out)
{
    const double latpercent = 180.0 / (double)(height - 1), lonpercent = 360.0 / (double)width;
    for (int h = 0; h < height; ++h)
        for (int w = 0; w < width; ++w) {
            double lat = 90.0 - ((double)h * latpercent), lon = -180.0 + ((double)w * lonpercent);
            if (lat < -90.0) lat = -90.0;
            if (lon < -180.0) lon = -180.0;
            latlon2xyz(lat, lon, radius, out + 3 * ((int64_t)h * width + w));
        }
}

/* The 3 nearest vertices of each query point, by brute force (the exact
 * answer the reference's KD-tree query(k=3) gives, nixis.py:278-283):
 * distances sqrt((dx*dx + dy*dy) + dz*dz) ascending, ties by index. */
NXO_API void nxo_nearest3(const double *xyz, int64_t nv, const double *q, int64_t nq, double *dist, int64_t *idx)
{
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < nq; ++p) {
        double bd[3] = {INFINITY, INFINITY, INFINITY};
        int64_t bi[3] = {-1, -1, -1};
        for (int64_t v = 0; v < nv; ++v) {
            const double dx = q[3 * p] - xyz[3 * v], dy = q[3 * p + 1] - xyz[3 * v + 1], dz = q[3 * p + 2] - xyz[3 * v + 2];
            const double d = sqrt((dx * dx + dy * dy) + dz * dz);
            int k = 3;
            while (k > 0 && (d < bd[k - 1] || (d == bd[k - 1] && v < bi[k - 1]))) --k;
            if (k < 3) {
                for (int m = 2; m > k; --m) { bd[m] = bd[m - 1]; bi[m] = bi[m - 1]; }
                bd[k] = d;
                bi[k] = v;
            }
        }
        for (int k = 0; k < 3; ++k) { dist[3 * p + k] = bd[k]; idx[3 * p + k] = bi[k]; }
    }
}

/* util.py:342-366 (make_gray_array) per pixel: weights 1 / ((d + 1e-5) / sum d),
 * normalised, the weighted sum of the 3 colours truncated toward zero. */
NXO_API void nxo_make_gray(const double *dist, const int64_t *idx, int64_t npix, const double *colors, double *out)
{
    for (int64_t p = 0; p < npix; ++p) {
        const double *d = dist + 3 * p;
        const double sd = (d[0] + d[1]) + d[2];
        double ws[3];
        for (int k = 0; k < 3; ++k) ws[k] = 1 / ((d[k] + 0.00001) / sd);
        const double t = (ws[0] + ws[1]) + ws[2];
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) acc += colors[idx[3 * p + k]] * (ws[k] / t);
        out[p] = trunc(acc);
    }
}

/* ------------------------------------------------------------------------ */
/* Mesh adjacency and scalar helpers                                          */
/* ------------------------------------------------------------------------ */

/* util.py:591-613: for each triangle (in order) append t1 to adj[t0], t2 to
 * adj[t1], t0 to adj[t2], each into the first -1 slot.  Vertex count is
 * (ntri + 4) / 2. */
NXO_API int nxo_build_adjacency(const int32_t *tris, int64_t ntri, int32_t *adj)
{
    int64_t nv = (ntri + 4) / 2;
    for (int64_t i = 0; i < 6 * nv; ++i) adj[i] = -1;
    for (int64_t t = 0; t < ntri; ++t) {
        for (int e = 0; e < 3; ++e) {
            int32_t a = tris[3 * t + e], b = tris[3 * t + (e + 1) % 3];
            int32_t *row = adj + 6 * (int64_t)a;
            int k = 0;
            while (k < 6 && row[k] != -1) ++k;
            if (k == 6) return -1;        /* the reference would write row[-1] */
            row[k] = b;
        }
    }
    return 0;
}

static int contains(const int32_t *row, int32_t v)
{
    for (int k = 0; k < 6; ++k) if (row[k] == v) return 1;
    return 0;
}

/* util.py:623-629 */
static int32_t next_vert(int32_t v, const int32_t *arr1, const int32_t *arr2)
{
    for (int k = 0; k < 6; ++k) {
        int32_t i = arr1[k];
        if (contains(arr2, i) && i != v) return i;
    }
    return -1;
}

/* util.py:638-662: walk each vertex's neighbours into a ring, starting from
 * slot 0; vertices 0-11 have 5 neighbours (slot 5 = -1).  The walk only tests
 * membership in neighbour rows, which does not depend on their order, so the
 * rows are read from an unsorted copy and every vertex is independent. */
NXO_API int nxo_sort_adjacency(int32_t *adj, int64_t nv)
{
    int32_t *src = (int32_t *)malloc(sizeof(int32_t) * 6 * (size_t)(nv > 0 ? nv : 1));
    if (!src) return -1;
    memcpy(src, adj, sizeof(int32_t) * 6 * (size_t)nv);
#pragma omp parallel for schedule(static)
    for (int64_t idx = 0; idx < nv; ++idx) {
        int deg = idx < 12 ? 5 : 6;
        int32_t visited[6] = {-1, -1, -1, -1, -1, -1};
        const int32_t *row = src + 6 * idx;
        int32_t pv = (int32_t)idx, nvx = row[0];
        for (int i = 0; i < deg - 1; ++i) {
            visited[i] = nvx;
            nvx = nvx >= 0 ? next_vert(pv, row, src + 6 * (int64_t)nvx) : -1;
            pv = visited[i];
        }
        visited[deg - 1] = nvx;
        memcpy(adj + 6 * idx, visited, sizeof(visited));
    }
    free(src);
    return 0;
}

/*
 * Icosphere inputs on the CPU (this project's construction, documented in
 * nixis_gb300/icosphere.py; the reference's meshzoo is unavailable).  Tables:
 * corners float64[36], faces int32[60], face sides int32[120], edges
 * int32[60].  Same binary64 operation order as the GPU generator.
 */
static void nrm3(double *p)
{
    double r = sqrt((p[0] * p[0] + p[1] * p[1]) + p[2] * p[2]);
    p[0] = p[0] / r; p[1] = p[1] / r; p[2] = p[2] / r;
}

static int32_t face_vid(const int32_t *faces, const int32_t *fe, int f, int64_t i, int64_t j, int64_t k)
{
    const int32_t *F = faces + 3 * f;
    if (i == 0 && j == 0) return F[0];
    if (i == k && j == 0) return F[1];
    if (i == 0 && j == k) return F[2];
    int side; int64_t pos;
    if (j == 0) { side = 0; pos = i; }
    else if (i == 0) { side = 1; pos = j; }
    else if (i + j == k) { side = 2; pos = j; }
    else {
        int64_t npf = (k - 1) * (k - 2) / 2;
        int64_t off = (i - 1) * (k - 1) - (i - 1) * i / 2 + (j - 1);
        return (int32_t)(12 + 30 * (k - 1) + f * npf + off);
    }
    int e = fe[6 * f + 2 * side];
    int64_t t = fe[6 * f + 2 * side + 1] ? pos : k - pos;
    return (int32_t)(12 + e * (k - 1) + t - 1);
}

NXO_API int nxo_icosphere(int k, const double *corners, const int32_t *faces, const int32_t *fe,
                          const int32_t *edges, double *xyz, int32_t *tris)
{
    if (k < 1) return -1;
    int64_t K = k;
    for (int c = 0; c < 36; ++c) xyz[c] = corners[c];
    for (int e = 0; e < 30; ++e) {
        const double *A = corners + 3 * edges[2 * e], *B = corners + 3 * edges[2 * e + 1];
        for (int64_t t = 1; t < K; ++t) {
            double *p = xyz + 3 * (12 + e * (K - 1) + t - 1);
            for (int c = 0; c < 3; ++c) p[c] = (double)(K - t) * A[c] + (double)t * B[c];
            nrm3(p);
        }
    }
    int64_t npf = (K - 1) * (K - 2) / 2, base = 12 + 30 * (K - 1);
    for (int f = 0; f < 20; ++f) {
        const double *A = corners + 3 * faces[3 * f], *B = corners + 3 * faces[3 * f + 1], *C = corners + 3 * faces[3 * f + 2];
        int64_t q = 0;
        for (int64_t i = 1; i < K - 1; ++i)
            for (int64_t j = 1; j < K - i; ++j, ++q) {
                double *p = xyz + 3 * (base + f * npf + q);
                for (int c = 0; c < 3; ++c) p[c] = ((double)(K - i - j) * A[c] + (double)i * B[c]) + (double)j * C[c];
                nrm3(p);
            }
    }
    if (tris) {
        int64_t n = 0;
        for (int f = 0; f < 20; ++f)
            for (int64_t i = 0; i < K; ++i)
                for (int64_t j = 0; j < K - i; ++j) {
                    int32_t *t = tris + 3 * n++;
                    t[0] = face_vid(faces, fe, f, i, j, K); t[1] = face_vid(faces, fe, f, i + 1, j, K);
                    t[2] = face_vid(faces, fe, f, i, j + 1, K);
                    if (i + j < K - 1) {
                        t = tris + 3 * n++;
                        t[0] = face_vid(faces, fe, f, i + 1, j, K); t[1] = face_vid(faces, fe, f, i + 1, j + 1, K);
                        t[2] = face_vid(faces, fe, f, i, j + 1, K);
                    }
                }
    }
    return 0;
}

/* util.py:110-140 (mode=None, mid=None): min/max normalise to [lower, upper]. */
NXO_API void nxo_rescale(const double *x, int64_t n, double lower, double upper, double *out)
{
    if (n <= 0) return;
    double mn = x[0], mx = x[0];
    for (int64_t i = 1; i < n; ++i) {
        if (x[i] < mn) mn = x[i];
        if (x[i] > mx) mx = x[i];
    }
    double xr = mx - mn, nr = upper - lower;
    for (int64_t i = 0; i < n; ++i) out[i] = ((x[i] - mn) / xr) * nr + lower;
}

/* util.py:110-176, every form.  form: 0 plain, 1 with mid (each side of mid
 * mapped separately), 2 mode 'lower' (only x <= mid), 3 mode 'upper' (only
 * x >= mid).  u_min / u_max widen the input range (util.py:128-131). */
NXO_API void nxo_rescale_full(const double *x, int64_t n, double lower, double upper, double mid, int form,
                              double u_min, int has_umin, double u_max, int has_umax, double *out)
{
    if (n <= 0) return;
    double x_min = x[0], x_max = x[0];
    for (int64_t i = 1; i < n; ++i) {
        if (x[i] < x_min) x_min = x[i];
        if (x[i] > x_max) x_max = x[i];
    }
    if (has_umin && u_min < x_min) x_min = u_min;
    if (has_umax && u_max > x_max) x_max = u_max;
    for (int64_t i = 0; i < n; ++i) {
        const double v = x[i];
        double r = v;
        if (form == 0) {
            r = ((v - x_min) / (x_max - x_min)) * (upper - lower) + lower;
        } else if (form == 1) {
            if (v <= mid) r = ((v - x_min) / (mid - x_min)) * (mid - lower) + lower;
            else r = ((v - mid) / (x_max - mid)) * (upper - mid) + mid;
        } else if (form == 2) {
            if (v <= mid) r = ((v - x_min) / (mid - x_min)) * (mid - lower) + lower;
        } else {
            if (v >= mid) r = ((v - mid) / (x_max - mid)) * (upper - mid) + mid;
        }
        out[i] = r;
    }
}

/* util.py:556-566 */
NXO_API double nxo_find_percent_val(double minval, double maxval, double percent)
{
    if (!(0.0 < percent && percent < 100.0)) percent = 50.0;
    return minval + ((maxval - minval) * percent / 100.0);
}

/* util.py:179-250.  mode: -1 (None), 0 (rescale where mask is false), 1
 * (where mask is true).  The masked range comes from the reference's
 * running update (a new running minimum is not compared with the maximum). */
NXO_API void nxo_power_rescale(const double *x, int64_t n, const uint8_t *mask, int mode, double power, double *out)
{
    if (n <= 0) return;
    const double temp_upper = 1.0, temp_lower = 0.0, temp_range = temp_upper - temp_lower;
    double x_min = x[0], x_max = x[0];
    for (int64_t i = 1; i < n; ++i) {
        if (x[i] < x_min) x_min = x[i];
        if (x[i] > x_max) x_max = x[i];
    }
    double lo = x_max, hi = x_min;
    for (int64_t i = 0; i < n; ++i) {
        const int sel = mode == 1 ? mask[i] != 0 : (mode == 0 ? mask[i] == 0 : 0);
        if (sel && x[i] < lo) lo = x[i];
        else if (sel && x[i] > hi) hi = x[i];
    }
    const double range = hi - lo;
    for (int64_t i = 0; i < n; ++i) {
        const int sel = mode == 1 ? mask[i] != 0 : (mode == 0 ? mask[i] == 0 : 0);
        double v = x[i];
        if (sel) {
            v = ((v - lo) / range) * temp_range + temp_lower;
            v = pow(v, power);
            v = ((v - temp_lower) / temp_range) * range + lo;
        }
        out[i] = v;
    }
}

/* nixis.py:332-364: rescale to [min_alt, max_alt], ocean level, mask, the
 * two masked power rescales, shift, rescale about 0.  tmp: n doubles. */
NXO_API double nxo_shape_heights(const double *h, int64_t n, double min_alt, double max_alt, double ocean_percent,
                                 double *out, double *tmp, uint8_t *mask)
{
    nxo_rescale_full(h, n, min_alt, max_alt, 0.0, 0, 0.0, 0, 0.0, 0, out);
    double mn = out[0], mx = out[0];
    for (int64_t i = 1; i < n; ++i) {
        if (out[i] < mn) mn = out[i];
        if (out[i] > mx) mx = out[i];
    }
    const double level = nxo_find_percent_val(mn, mx, ocean_percent);
    nxo_make_bool_elevation_mask(out, n, level, mask);
    nxo_power_rescale(out, n, mask, 1, 0.5, tmp);
    nxo_power_rescale(tmp, n, mask, 0, 2.0, out);
    for (int64_t i = 0; i < n; ++i) tmp[i] = out[i] - level;
    nxo_rescale_full(tmp, n, min_alt, max_alt, 0.0, 1, 0.0, 0, 0.0, 0, out);
    return level;
}

NXO_API int nxo_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
