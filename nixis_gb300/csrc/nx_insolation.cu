// nx_insolation.cu -- per-vertex insolation accumulated over sun positions.
//
// Replaces the loop of climate.sample_insolation calls (climate.py:415-444;
// driven over rotations as in brute_daily_insolation, climate.py:450-489).
// For one sun position (rotation theta about z, tilt tau about y) the
// reference adds, per vertex,
//   max(cos|lat|, 0) * max(cos lon, 0)
// with lat, lon of the rotated and tilted point (util.xyz2latlon,
// util.py:59-75).  For a vertex on the sphere of the given radius r this
// equals max(t, 0) / r with
//   t = A cos(theta) + B sin(theta) + C,  A = x cos(tau), B = -y cos(tau),
//   C = z sin(tau)
// (cos lat = sqrt(tx^2+ty^2)/r, cos lon = tx/sqrt(tx^2+ty^2)).  When the
// rotations come in pairs theta, theta + 180 degrees (every even uniform
// schedule, e.g. 24 hours of 15 degrees), the pair contributes
//   max(C+u, 0) + max(C-u, 0) = C + max(|C|, |u|),  u = A cos + B sin,
// i.e. two operations per sun position.  Vertices off that sphere
// (| |v|^2 - r^2 | > 1e-12 r^2) take the reference's general formula.
//
// With u = cos(tau) U(theta), U = x cos(theta) - y sin(theta) the same on
// every day, a day's pairs sum to n C + |cos tau| sum_h max(c, |U_h|),
// c = |z| |tan tau|.  Schedules of up to SORT_MAX days are then summed by
// breakpoints: each max picks one side, so over the year the sum is
// sum_h [ |U_h| (sum of |cos| over days with c < |U_h|) + |z| (sum of
// |cos| |tan| over the other days) ], both inner sums read from prefix /
// suffix sums over the days sorted by |tan tau| (built once per block), at
// a count found through a bucket index: twelve lookups per vertex for a
// year of hourly positions.  Longer schedules sum day by day (paired lanes,
// groups of 8 days, Kahan across groups), so the result tracks the binary64
// sum either way.
#include "nx_common.cuh"

namespace nx {
void note_launch(int k);
}

namespace {

struct InsoArgs {
    const double *xyz;
    int64_t n;
    double r;
    float inv_r;
    const float2 *tilt;    // (cos tau, sin tau) per tilt
    int n_tilt;
    const float2 *rot;     // (cos theta, sin theta): all rotations, or the first half in pair mode
    int n_rot;             // number of entries in rot
    int pairs;             // 1: each rot entry stands for theta and theta + 180
    float *out;
    int accumulate;
};

// climate.py:419-442 for a vertex off the sphere of radius r (binary32).
__device__ __forceinline__ float general_term(float x, float y, float z, float inv_r, float ct, float st, float cr, float sr)
{
    float rx = x * cr - y * sr;
    float ry = x * sr + y * cr;
    float tx = rx * ct + z * st;
    float ty = ry;
    float tz = z * ct - rx * st;
    float q = fminf(fmaxf(tz * inv_r, -1.0f), 1.0f);
    float clat = sqrtf(fmaxf(1.0f - q * q, 0.0f));
    float h2 = tx * tx + ty * ty;
    float clon = h2 > 0.0f ? tx * rsqrtf(h2) : 1.0f;    // atan2(0, 0) = 0 -> cos = 1
    return clat * fmaxf(clon, 0.0f);
}

// Sum over the schedule for one vertex.
// Tilts whose per-day constants a block stages in shared memory (16 B each).
constexpr int TILT_STAGE_MAX = 2048;

// Per-day constants of the factored pair sum, (|cos tau|, |sin tau| / |cos
// tau|, HP sin tau, 0); days with |cos tau| < 2^-20 (the direct form) get
// zeros, which add nothing to the factored sum, and are listed after the
// days (day indices as ints, their count in entry n_tilt.y); entry n_tilt.x
// holds the sum of HP sin tau over the factored days (day order, binary64,
// rounded once), so a vertex adds its days' C terms as one product.
// Shared memory: tilt_smem(a).
template <int HP>
__device__ __forceinline__ void stage_tilts(const InsoArgs &a, float4 *tt)
{
    for (int d = threadIdx.x; d < a.n_tilt; d += blockDim.x) {
        const float2 t = a.tilt[d];
        const float ak = fabsf(t.x);
        tt[d] = ak >= 0x1p-20f ? make_float4(ak, __fdiv_rn(fabsf(t.y), ak), (float)HP * t.y, 0.0f)
                               : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int *direct = reinterpret_cast<int *>(tt + a.n_tilt + 1);
        double sc = 0.0;
        int nd = 0;
        for (int d = 0; d < a.n_tilt; ++d) {
            const float4 k = tt[d];
            if (k.x > 0.0f) sc += (double)k.z;
            else direct[nd++] = d;
        }
        tt[a.n_tilt] = make_float4((float)sc, __int_as_float(nd), 0.0f, 0.0f);
    }
    __syncthreads();
}

// Days per group of the staged sum: a group's days accumulate in paired
// lanes (one FFMA2 per day), the groups are added with compensation.
constexpr int DAY_GROUP = 8;

// Schedules of up to SORT_MAX days are also summed by breakpoints.  With
// c_d = |z| tan_d (tan_d = |tan tau_d|, cos_d = |cos tau_d|) and a_h = |U_h|,
// the factored days' part of the year is
//   sum_d cos_d sum_h max(c_d, a_h)
//     = sum_h [ a_h sum_{d: c_d < a_h} cos_d + |z| sum_{d: c_d >= a_h} cos_d tan_d ],
// exactly (each max picks one side).  With the days sorted by tan_d, both
// inner sums are a prefix sum P0 and a suffix sum Q1 of the sorted days,
// read at the count B_h of days with tan_d < a_h / |z|; a vertex then needs
// twelve searches instead of a max and an add per pair and day.
// Shared memory after the staged constants (floats): T[SP] the sorted tan_d
// padded with +inf to a power of two SP > factored days (at least one +inf
// sentinel), P0[nf + 1] and Q1[nf + 1] (binary64 sums rounded once), the
// cos_d in sorted order, and a bucket index of SP + 1 ints: with tmax the
// largest tan_d and NB = SP buckets of width tmax / NB, F[b] = the count of
// days with tan_d < b tmax / NB (F[NB] = nf).  A search for t > tmax is nf;
// otherwise it starts at F[b] for b = floor(t NB / tmax) and steps down
// while the day below is not below t and up while the next day is below t
// (a step or two: the buckets hold under one day on average), which ends
// at the exact count whatever the rounding of b.
constexpr int SORT_MAX = 512;

__host__ __device__ __forceinline__ int sort_pad(int n)
{
    int p = 1;
    while (p < n) p <<= 1;
    return p;
}

// Builds T, P0, Q1 from the staged constants (after stage_tilts); returns
// the number of factored days.  Called by the whole block.
__device__ __forceinline__ int stage_breakpoints(const InsoArgs &a, const float4 *tt, float *T, float *P0, float *Q1,
                                                 float *CS, int *F, float &scale, float &tmax)
{
    const int nd = __float_as_int(tt[a.n_tilt].y);
    const int nf = a.n_tilt - nd;
    const int sp = sort_pad(nf + 1);
    // rank sort of the factored days by (tan, day): position = how many
    // factored days come before
    for (int d = threadIdx.x; d < a.n_tilt; d += blockDim.x) {
        const float4 k = tt[d];
        if (!(k.x > 0.0f)) continue;
        int rank = 0;
        for (int e = 0; e < a.n_tilt; ++e) {
            const float4 o = tt[e];
            rank += (o.x > 0.0f && (o.y < k.y || (o.y == k.y && e < d))) ? 1 : 0;
        }
        T[rank] = k.y;
        CS[rank] = k.x;
    }
    for (int j = nf + threadIdx.x; j < sp; j += blockDim.x) T[j] = __int_as_float(0x7F800000);
    __syncthreads();
    // prefix sums of cos and suffix sums of cos * tan, binary64, one warp:
    // a lane sums its run of days, the runs are scanned across the warp
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const int per = (nf + 31) / 32;
        const int j0 = min(nf, lane * per), j1 = min(nf, j0 + per);
        double s0 = 0.0, s1 = 0.0;
        for (int j = j0; j < j1; ++j) {
            s0 += (double)CS[j];
            s1 += (double)CS[j] * (double)T[j];
        }
        double e0 = s0, e1 = s1;                  // inclusive scan over the lanes
        for (int o = 1; o < 32; o <<= 1) {
            const double u0 = __shfl_up_sync(0xFFFFFFFFu, e0, o), u1 = __shfl_up_sync(0xFFFFFFFFu, e1, o);
            if (lane >= o) { e0 += u0; e1 += u1; }
        }
        const double tot1 = __shfl_sync(0xFFFFFFFFu, e1, 31);
        const double tot0 = __shfl_sync(0xFFFFFFFFu, e0, 31);
        e0 -= s0;                                 // exclusive
        e1 -= s1;
        for (int j = j0; j < j1; ++j) {
            P0[j] = (float)e0;
            Q1[j] = (float)(tot1 - e1);
            e0 += (double)CS[j];
            e1 += (double)CS[j] * (double)T[j];
        }
        if (lane == 0) {
            P0[nf] = (float)tot0;
            Q1[nf] = 0.0f;
        }
    }
    // the bucket index: F[b] by a binary search per bucket
    tmax = nf > 0 ? T[nf - 1] : 0.0f;
    scale = tmax > 0.0f ? (float)sp / tmax : 0.0f;
    const float width = tmax / (float)sp;
    for (int b = threadIdx.x; b <= sp; b += blockDim.x) {
        if (b == sp) { F[b] = nf; continue; }
        const float edge = (float)b * width;
        int c = 0;
        for (int step = sp >> 1; step > 0; step >>= 1) c += T[c + step - 1] < edge ? step : 0;
        F[b] = c;
    }
    __syncthreads();
    return nf;
}

// Breakpoint tables of a block (stage_breakpoints), or nf < 0 for none.
struct Breaks {
    const float *T = nullptr, *P0 = nullptr, *Q1 = nullptr;
    const int *F = nullptr;
    int nf = -1, sp = 0;       // factored days, buckets
    float scale = 0.0f, tmax = 0.0f;
};

template <int HP>
__device__ __forceinline__ float inso_vertex(const InsoArgs &a, double X, double Y, double Z, double r, float inv_r,
                                             const float4 *tt = nullptr, const Breaks &bk = Breaks())
{
    const double rho2 = X * X + Y * Y + Z * Z;
    const double r2 = r * r;
    const bool on_sphere = fabs(rho2 - r2) <= 1e-12 * r2;
    const float x = (float)X, y = (float)Y, z = (float)Z;
    float tot = 0.0f, comp = 0.0f;          // Kahan over tilts
    const int nr = HP > 0 ? HP : a.n_rot;
    if (on_sphere && HP > 0 && (HP & 1) == 0 && a.pairs) {
        // u = A cos(theta) + B sin(theta) = k U(theta) with k = cos(tau) and
        // U = x cos(theta) - y sin(theta) the same for every day, so per day
        //   sum_h max(|C|, |u_h|) = |k| sum_h max(|C| / |k|, |U_h|)
        // (exact in real arithmetic): |U_h| is formed once per vertex and a
        // day costs a max and an add per rotation pair.  Days with |k| near 0
        // take the direct form.
        float au[HP > 0 ? HP : 2];
#pragma unroll
        for (int h = 0; h < (HP > 0 ? HP : 2); ++h) {
            const float2 q = a.rot[h];
            au[h] = fabsf(fmaf(x, q.x, -(y * q.y)));
        }
        if (tt) {
            // constants staged by the block: per day a shared load, one
            // multiply for the threshold, the max / add of each pair and one
            // paired multiply-add into the group's lanes; the days' C terms
            // come in at the end as z times their staged sum, the (rare)
            // direct-form days after the others
            const float az = fabsf(z);
            auto add = [&](float s) {
                const float yk = s - comp;
                const float tk = tot + yk;
                comp = (tk - tot) - yk;
                tot = tk;
            };
            if (bk.nf >= 0) {
                // B_h = number of sorted days with tan_d < a_h / |z|
                // (|z| = 0: every day for a_h > 0, none for a_h = 0)
                const float iz = 1.0f / az;
                float th[HP > 0 ? HP : 2];
                int B[HP > 0 ? HP : 2];
#pragma unroll
                for (int h = 0; h < (HP > 0 ? HP : 2); ++h) {
                    th[h] = au[h] > 0.0f ? au[h] * iz : 0.0f;
                    B[h] = 0;
                }
#pragma unroll
                for (int h = 0; h < (HP > 0 ? HP : 2); ++h) {
                    if (th[h] > bk.tmax) {
                        B[h] = bk.nf;
                    } else {
                        const int b = min((int)(th[h] * bk.scale), bk.sp - 1);
                        int c = bk.F[b];
                        while (c > 0 && !(bk.T[c - 1] < th[h])) --c;
                        while (c < bk.nf && bk.T[c] < th[h]) ++c;
                        B[h] = c;
                    }
                }
                float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
                for (int h = 0; h < (HP > 0 ? HP : 2); h += 2) {
                    const int b0 = min(B[h], bk.nf), b1 = min(B[h + 1], bk.nf);
                    s0 = fmaf(au[h], bk.P0[b0], fmaf(az, bk.Q1[b0], s0));
                    s1 = fmaf(au[h + 1], bk.P0[b1], fmaf(az, bk.Q1[b1], s1));
                }
                tot = s0 + s1;
            } else {
            auto day = [&](int d, float2 g) {
                const float4 k = tt[d];
                const float c = az * k.y;
                float2 acc = make_float2(fmaxf(c, au[0]), fmaxf(c, au[1]));
#pragma unroll
                for (int h = 2; h < (HP > 0 ? HP : 2); h += 2)
                    acc = __fadd2_rn(acc, make_float2(fmaxf(c, au[h]), fmaxf(c, au[h + 1])));
                return __ffma2_rn(make_float2(k.x, k.x), acc, g);
            };
            const int full = a.n_tilt - a.n_tilt % DAY_GROUP;
            for (int d0 = 0; d0 < full; d0 += DAY_GROUP) {
                float2 g = make_float2(0.0f, 0.0f);
#pragma unroll
                for (int j = 0; j < DAY_GROUP; ++j) g = day(d0 + j, g);
                add(g.x + g.y);
            }
            if (full < a.n_tilt) {
                float2 g = make_float2(0.0f, 0.0f);
                for (int d = full; d < a.n_tilt; ++d) g = day(d, g);
                add(g.x + g.y);
            }
            }   // days one by one
            const float4 e = tt[a.n_tilt];
            const int nd = __float_as_int(e.y);
            const int *direct = reinterpret_cast<const int *>(tt + a.n_tilt + 1);
            for (int i = 0; i < nd; ++i) {
                const float2 t = a.tilt[direct[i]];
                const float A = x * t.x, B = -(y * t.x), C = z * t.y, aC = fabsf(C);
                float s = 0.0f;
#pragma unroll
                for (int h = 0; h < (HP > 0 ? HP : 2); ++h) {
                    const float2 q = a.rot[h];
                    s += fmaxf(aC, fabsf(fmaf(A, q.x, B * q.y)));
                }
                add(fmaf((float)HP, C, s));
            }
            add(z * e.x);
            return tot * inv_r;
        }
        for (int d = 0; d < a.n_tilt; ++d) {
            const float2 t = a.tilt[d];
            const float C = z * t.y, aC = fabsf(C), ak = fabsf(t.x);
            float s;
            if (ak >= 0x1p-20f) {
                const float c = __fdividef(aC, ak);
                float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
                for (int h = 0; h < (HP > 0 ? HP : 2); h += 2)
                    acc = __fadd2_rn(acc, make_float2(fmaxf(c, au[h]), fmaxf(c, au[h + 1])));
                s = fmaf(ak, acc.x + acc.y, (float)HP * C);
            } else {
                const float A = x * t.x, B = -(y * t.x);
                s = 0.0f;
#pragma unroll
                for (int h = 0; h < (HP > 0 ? HP : 2); ++h) {
                    const float2 q = a.rot[h];
                    s += fmaxf(aC, fabsf(fmaf(A, q.x, B * q.y)));
                }
                s = fmaf((float)HP, C, s);
            }
            float yk = s - comp;
            float tk = tot + yk;
            comp = (tk - tot) - yk;
            tot = tk;
        }
        return tot * inv_r;
    }
    if (on_sphere) {
        float2 rt[HP > 0 ? HP : 1];
        if (HP > 0) {
#pragma unroll
            for (int h = 0; h < (HP > 0 ? HP : 1); ++h) rt[h] = a.rot[h];
        }
        for (int d = 0; d < a.n_tilt; ++d) {
            const float2 t = a.tilt[d];
            const float A = x * t.x, B = -(y * t.x), C = z * t.y;
            float s = 0.0f;
            if (a.pairs) {
                const float aC = fabsf(C);
                if (HP > 0) {
#pragma unroll
                    for (int h = 0; h < (HP > 0 ? HP : 1); ++h) {
                        float u = fmaf(A, rt[h].x, B * rt[h].y);
                        s += fmaxf(aC, fabsf(u));
                    }
                } else {
                    for (int h = 0; h < nr; ++h) {
                        float2 q = a.rot[h];
                        float u = fmaf(A, q.x, B * q.y);
                        s += fmaxf(aC, fabsf(u));
                    }
                }
                s = fmaf((float)nr, C, s);
            } else {
                for (int h = 0; h < nr; ++h) {
                    float2 q = a.rot[h];
                    s += fmaxf(fmaf(A, q.x, fmaf(B, q.y, C)), 0.0f);
                }
            }
            float yk = s - comp;
            float tk = tot + yk;
            comp = (tk - tot) - yk;
            tot = tk;
        }
        return tot * inv_r;
    }
    for (int d = 0; d < a.n_tilt; ++d) {
        const float2 t = a.tilt[d];
        float s = 0.0f;
        for (int h = 0; h < nr; ++h) {
            float2 q = a.rot[h];
            s += general_term(x, y, z, inv_r, t.x, t.y, q.x, q.y);
            if (a.pairs) s += general_term(x, y, z, inv_r, t.x, t.y, -q.x, -q.y);
        }
        float yk = s - comp;
        float tk = tot + yk;
        comp = (tk - tot) - yk;
        tot = tk;
    }
    return tot;
}

// The block's breakpoint tables after the staged constants (see SORT_MAX).
template <int HP>
__device__ __forceinline__ Breaks stage_all(const InsoArgs &a, float4 *s_tilt)
{
    Breaks bk;
    stage_tilts<HP>(a, s_tilt);
    if (a.n_tilt <= SORT_MAX) {
        float *base = reinterpret_cast<float *>(reinterpret_cast<int *>(s_tilt + a.n_tilt + 1) + a.n_tilt);
        const int sp = sort_pad(a.n_tilt + 1);
        float *T = base, *P0 = T + sp, *Q1 = P0 + a.n_tilt + 1, *CS = Q1 + a.n_tilt + 1;
        int *F = reinterpret_cast<int *>(CS + a.n_tilt + 1);
        bk.nf = stage_breakpoints(a, s_tilt, T, P0, Q1, CS, F, bk.scale, bk.tmax);
        bk.sp = sort_pad(bk.nf + 1);
        bk.F = F;
        bk.T = T;
        bk.P0 = P0;
        bk.Q1 = Q1;
    }
    return bk;
}

template <int HP>
__global__ void __launch_bounds__(256, 3) insolation_kernel(InsoArgs a)
{
    extern __shared__ float4 s_tilt[];
    const bool staged = HP > 0 && a.pairs && a.n_tilt <= TILT_STAGE_MAX;
    Breaks bk;
    if (staged) bk = stage_all<HP>(a, s_tilt);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        float tot = inso_vertex<HP>(a, a.xyz[3 * i], a.xyz[3 * i + 1], a.xyz[3 * i + 2], a.r, a.inv_r,
                                    staged ? s_tilt : nullptr, bk);
        a.out[i] = a.accumulate ? a.out[i] + tot : tot;
    }
}

// Many planets: planet p's vertices fill packed rows [vbeg, vbeg + n)
// (vbeg a multiple of 256); one block covers 256 rows of one planet.
template <int HP>
__global__ void __launch_bounds__(256, 3) insolation_batch_kernel(InsoArgs a, const nx_inso_planet *__restrict__ P, int np,
                                                               int64_t total_rows)
{
    extern __shared__ float4 s_tilt[];
    const bool staged = HP > 0 && a.pairs && a.n_tilt <= TILT_STAGE_MAX;
    Breaks bk;
    if (staged) bk = stage_all<HP>(a, s_tilt);
    for (int64_t blk = blockIdx.x; blk * 256 < total_rows; blk += gridDim.x) {
        const int64_t row = blk * 256 + threadIdx.x;
        int lo = 0, hi = np - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (P[mid].vbeg <= blk * 256) lo = mid; else hi = mid - 1;
        }
        const nx_inso_planet &pl = P[lo];
        const int64_t i = row - pl.vbeg;
        if (i < 0 || i >= pl.n) continue;
        const double r = pl.radius;
        float tot = inso_vertex<HP>(a, pl.xyz[3 * i], pl.xyz[3 * i + 1], pl.xyz[3 * i + 2], r, (float)(1.0 / r),
                                    staged ? s_tilt : nullptr, bk);
        a.out[row] = tot;
    }
}

// ---------------------------------------------------------------------------
// Latitude-table path (climate.py:503-597): per tilt, a table of 181
// latitudes (entry i = latitude i for i <= 90, i - 181 above), each the
// binary32 running sum over 360 rotations of 1 degree from -180 of the
// reference's binary64 term at (lat, lon 0) (calc_insolation_slice with
// sample_insolation's formula); then per vertex a linear
// interpolation between floor(lat) and ceil(lat), summed in binary32 over
// the tables (calc_yearly_insolation adds 360 daily tables).

constexpr double DEG = 3.141592653589793 / 180;

// One block per table, one thread per latitude entry.  The table's points
// lie on the sphere of the given radius at longitude 0 (y = 0), so the
// reference's term equals max(tx, 0) / radius with tx = x cos(theta)
// cos(tau) + z sin(tau) (the identity at the top of this file); it is
// evaluated in binary64 and summed in binary32 over the 360 rotations
// (-180, -179, ..., 179 degrees: the running sum of 1.0 steps is exact) as
// the reference sums its binary64 terms.  The rotations' cosines are
// computed once per block into shared memory.
__global__ void __launch_bounds__(192) slice_kernel(const double *__restrict__ tilts, int n_tilts, double radius,
                                                    float *__restrict__ tables)
{
    __shared__ double rc[360];
    const int d = blockIdx.x, i = threadIdx.x;
    for (int j = i; j < 360; j += blockDim.x) rc[j] = cos((-180.0 + (double)j) * 3.141592653589793 / 180);
    __syncthreads();
    if (d >= n_tilts || i >= 181) return;
    const double lat = (double)(i <= 90 ? i : i - 181);
    // util.latlon2xyz (util.py:79-88) at lon 0
    const double x = radius * cos(lat * DEG) * cos(0.0 * DEG);
    const double z = radius * sin(lat * DEG);
    const double tilt = tilts[d];
    const double ct = cos(tilt * 3.141592653589793 / 180), st = sin(tilt * 3.141592653589793 / 180);
    const double xc = x * ct, zs = z * st, inv_r = 1.0 / radius;
    float acc = 0.0f;
    for (int j = 0; j < 360; ++j) {
        const double tx = __fma_rn(xc, rc[j], zs);
        acc = __double2float_rn(__dadd_rn((double)acc, __dmul_rn(fmax(tx, 0.0), inv_r)));
    }
    tables[181 * d + i] = acc;
}

// One interpolation of climate.py:575, round32(tl + frac * (tu - tl)) with
// tu - tl rounded to binary32 and the product and sum rounded to binary64,
// computed in binary32 pairs.  frac = fh + fl (+ a remainder below 2^-48
// frac); with M = max(|tl|, |tu|) the pair value v' = sh + t is within
// 2^-45 M of the exact tl + frac (tu - tl), and the reference's binary64
// value within 2^-52 M of it.  When v' lies more than 2^-43 M from every
// binary32 rounding boundary both round to the same binary32 value r;
// otherwise (about one evaluation in 2^19) the binary64 formula is used.
__device__ __forceinline__ float interp_one(float tl, float tu, float fh, float fl, double frac)
{
    const float dd = __fsub_rn(tu, tl);
    const float ph = __fmul_rn(fh, dd);
    const float pl = __fmaf_rn(fl, dd, __fmaf_rn(fh, dd, -ph));   // fh*dd = ph + (fh*dd - ph) exactly
    // two-sum tl + ph = sh + se
    const float sh = __fadd_rn(tl, ph);
    const float bb = __fsub_rn(sh, tl);
    const float se = __fadd_rn(__fsub_rn(tl, __fsub_rn(sh, bb)), __fsub_rn(ph, bb));
    const float t = __fadd_rn(se, pl);
    // two-sum sh + t = r + e: v' - r = e exactly
    const float r = __fadd_rn(sh, t);
    const float b2 = __fsub_rn(r, sh);
    const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(r, b2)), __fsub_rn(t, b2));
    const float M = fmaxf(fabsf(tl), fabsf(tu));
    const uint32_t rb = __float_as_uint(r) & 0x7FFFFFFFu;
    const uint32_t ex = rb >> 23;
    if (ex > 24 && ex < 255) {
        // half an ulp of |r| away from zero, and toward zero (a quarter ulp
        // below a power of two)
        const float hu = __uint_as_float((ex - 24) << 23);
        const float hd = (rb & 0x7FFFFFu) ? hu : 0.5f * hu;
        const float ea = __float_as_uint(r) >> 31 ? -e : e;     // e measured away from zero
        const float dist = ea >= 0.0f ? __fsub_rn(hu, ea) : __fadd_rn(hd, ea);
        if (dist > 0x1p-43f * M) return r;
    } else if (M == 0.0f) {
        return r;                                                // tl = tu = 0
    }
    return __double2float_rn(__dadd_rn((double)tl, __dmul_rn(frac, (double)dd)));
}

// climate.py:551-577 per vertex and table, summed in binary32 over tables.
// The reference divides the table difference by upper - lower, which is
// exactly 1.0 whenever lower != upper, so no division is issued.
__global__ void __launch_bounds__(256) interp_kernel(const double *__restrict__ xyz, int64_t n, double radius,
                                                     const float *__restrict__ tables, int n_tables,
                                                     float *__restrict__ out, int accumulate)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const double q = fmin(fmax(xyz[3 * v + 2] / radius, -1.0), 1.0);
        const double lat = asin(q) * (180.0 / 3.141592653589793);
        const double fl = floor(lat), cl = ceil(lat);
        const int lower = (int)fl, upper = (int)cl;
        const int il = (lower + 181) % 181, iu = (upper + 181) % 181;
        const double frac = lat - fl;
        const float fh = __double2float_rn(frac);
        const float fr = __double2float_rn(__dsub_rn(frac, (double)fh));
        float acc = accumulate ? out[v] : 0.0f;
        for (int d = 0; d < n_tables; ++d) {
            const float tl = __ldg(tables + 181 * d + il), tu = __ldg(tables + 181 * d + iu);
            const float val = lower != upper ? interp_one(tl, tu, fh, fr, frac) : tl;
            acc = (n_tables == 1 && !accumulate) ? val : __fadd_rn(acc, val);
        }
        out[v] = acc;
    }
}

// climate.assign_surface_temp (climate.py:345-411) per vertex: latitude as
// util.xyz2latlon (util.py:59-75), then max(cos(|lat - tilt| * pi / 180), 0)
// in binary64 with the reference's operation order, stored as binary32.
// The reference's altitude term h2 = rescale(altitudes, 0, 0) is 0 (NaN for
// a constant field) at every vertex, so its h2 > 0 branch is never taken.
__global__ void __launch_bounds__(256) surface_temp_kernel(const double *__restrict__ xyz, int64_t n, double radius,
                                                           double tilt, float *__restrict__ out)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const double q = fmin(fmax(__ddiv_rn(xyz[3 * v + 2], radius), -1.0), 1.0);
        const double lat = __dmul_rn(asin(q), 180.0 / 3.141592653589793);
        const double a = __ddiv_rn(__dmul_rn(fabs(__dsub_rn(lat, tilt)), 3.141592653589793), 180.0);
        const double c = cos(a);
        out[v] = __double2float_rn(0.0 > c ? 0.0 : c);     // Python max(c, 0): c unless 0 > c
    }
}

// Dynamic shared memory of the 12-pair kernels: the staged tilt constants.
size_t tilt_smem(const InsoArgs &a)
{
    if (!a.pairs || a.n_tilt > TILT_STAGE_MAX) return 0;
    size_t b = sizeof(float4) * ((size_t)a.n_tilt + 1) + sizeof(int) * (size_t)a.n_tilt;
    if (a.n_tilt <= SORT_MAX)      // T (padded), P0, Q1, the sorted cosines, the bucket index
        b += sizeof(float) * ((size_t)sort_pad(a.n_tilt + 1) + 3 * ((size_t)a.n_tilt + 1)) +
             sizeof(int) * ((size_t)sort_pad(a.n_tilt + 1) + 1);
    return b;
}

int grid_for(int64_t n, int per_sm = 8)
{
    int64_t g = (n + 255) / 256;
    int64_t cap = (int64_t)nx::sm_count() * per_sm;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

// Blocks of a 12-pair launch: a block that sums by breakpoints sorts the
// schedule first, so the grid is the resident blocks (3 per SM) and each
// block takes many vertices.
int grid_staged(int64_t n, const InsoArgs &a)
{
    return grid_for(n, a.pairs && a.n_tilt <= SORT_MAX ? 3 : 8);
}

}  // namespace

// Degrees -> (cos, sin) as the reference computes them (climate.py:423-436:
// cos(angle * pi / 180) in binary64), rounded to binary32.
static void trig_table(const double *deg, int n, float *out)
{
    const double PI = 3.141592653589793;
    for (int i = 0; i < n; ++i) {
        double a = deg[i] * PI / 180;
        out[2 * i] = (float)cos(a);
        out[2 * i + 1] = (float)sin(a);
    }
}

NX_EXPORT int nx_insolation_plan(const double *rot_deg, int n_rot, const double *tilt_deg, int n_tilt,
                                 float *table_host, int *n_rot_entries, int *pairs)
{
    if (n_rot < 0 || n_tilt < 0 || !table_host || !n_rot_entries || !pairs || (n_rot && !rot_deg) ||
        (n_tilt && !tilt_deg))
        return nx::fail(NX_EINVAL, "nx_insolation_plan: bad arguments");
    // pair mode: rotation h + n/2 is rotation h + 180 degrees exactly
    int pr = 0;
    if (n_rot > 0 && n_rot % 2 == 0) {
        pr = 1;
        for (int h = 0; h < n_rot / 2; ++h)
            if (rot_deg[h + n_rot / 2] != rot_deg[h] + 180.0) { pr = 0; break; }
    }
    int nr = pr ? n_rot / 2 : n_rot;
    trig_table(rot_deg, nr, table_host);
    trig_table(tilt_deg, n_tilt, table_host + 2 * nr);
    *n_rot_entries = nr;
    *pairs = pr;
    return NX_OK;
}

NX_EXPORT int nx_insolation(const double *xyz_dev, int64_t n, double radius, const float *table_dev, int n_rot_entries,
                            int pairs, int n_tilt, float *out_dev, int accumulate, void *stream)
{
    if (n < 0 || n_rot_entries < 0 || n_tilt < 0) return nx::fail(NX_EINVAL, "nx_insolation: negative size");
    if (n == 0) return NX_OK;
    if (!xyz_dev || !out_dev || ((n_rot_entries || n_tilt) && !table_dev))
        return nx::fail(NX_EINVAL, "nx_insolation: null pointer");
    if (!(radius > 0.0)) return nx::fail(NX_EINVAL, "nx_insolation: radius must be > 0");
    cudaStream_t s = (cudaStream_t)stream;
    if (n_rot_entries == 0 || n_tilt == 0) {
        if (!accumulate) NX_CHECK_CUDA(cudaMemsetAsync(out_dev, 0, sizeof(float) * (size_t)n, s));
        return NX_OK;
    }
    InsoArgs a;
    a.xyz = xyz_dev;
    a.n = n;
    a.r = radius;
    a.inv_r = (float)(1.0 / radius);
    a.rot = (const float2 *)table_dev;
    a.n_rot = n_rot_entries;
    a.pairs = pairs ? 1 : 0;
    a.tilt = (const float2 *)table_dev + n_rot_entries;
    a.n_tilt = n_tilt;
    a.out = out_dev;
    a.accumulate = accumulate;
    if (a.pairs && n_rot_entries == 12)
        insolation_kernel<12><<<grid_staged(n, a), 256, tilt_smem(a), s>>>(a);
    else
        insolation_kernel<0><<<grid_for(n), 256, 0, s>>>(a);
    NX_CHECK_LAUNCH("insolation_kernel");
    nx::note_launch(1);
    return NX_OK;
}

NX_EXPORT int nx_insolation_batch(const nx_inso_planet *planets_dev, const nx_inso_planet *planets_host, int nplanets,
                                  const float *table_dev, int n_rot_entries, int pairs, int n_tilt, float *out_dev,
                                  void *stream)
{
    if (nplanets <= 0) return NX_OK;
    if (!planets_dev || !planets_host || !out_dev || !table_dev || n_rot_entries <= 0 || n_tilt <= 0)
        return nx::fail(NX_EINVAL, "nx_insolation_batch: bad arguments");
    int64_t total = 0;
    for (int p = 0; p < nplanets; ++p) {
        const nx_inso_planet &P = planets_host[p];
        if (P.vbeg % 256 || P.n < 0 || (P.n > 0 && !P.xyz) || !(P.radius > 0) || P.vbeg < total)
            return nx::fail(NX_EINVAL, "nx_insolation_batch: planet %d: rows must be packed, 256-aligned", p);
        total = P.vbeg + P.n;
    }
    InsoArgs a;
    a.xyz = nullptr;
    a.n = 0;
    a.r = 1.0;
    a.inv_r = 1.0f;
    a.rot = (const float2 *)table_dev;
    a.n_rot = n_rot_entries;
    a.pairs = pairs ? 1 : 0;
    a.tilt = (const float2 *)table_dev + n_rot_entries;
    a.n_tilt = n_tilt;
    a.out = out_dev;
    a.accumulate = 0;
    cudaStream_t s = (cudaStream_t)stream;
    int grid = a.pairs && n_rot_entries == 12 ? grid_staged(total, a) : grid_for(total);
    if (a.pairs && n_rot_entries == 12)
        insolation_batch_kernel<12><<<grid, 256, tilt_smem(a), s>>>(a, planets_dev, nplanets, total);
    else
        insolation_batch_kernel<0><<<grid, 256, 0, s>>>(a, planets_dev, nplanets, total);
    NX_CHECK_LAUNCH("insolation_batch_kernel");
    nx::note_launch(1);
    return NX_OK;
}

// Daily latitude tables for n_tilts tilts (degrees, device array):
// tables_dev float[n_tilts * 181].
NX_EXPORT int nx_insolation_slices(const double *tilts_dev, int n_tilts, double radius, float *tables_dev,
                                   void *stream)
{
    if (n_tilts <= 0 || !tilts_dev || !tables_dev || !(radius > 0.0))
        return nx::fail(NX_EINVAL, "nx_insolation_slices: bad arguments");
    slice_kernel<<<n_tilts, 192, 0, (cudaStream_t)stream>>>(tilts_dev, n_tilts, radius, tables_dev);
    NX_CHECK_LAUNCH("slice_kernel");
    nx::note_launch(1);
    return NX_OK;
}

// Interpolated insolation of every vertex from n_tables tables, summed in
// binary32 in table order (accumulate = 1 adds to out_dev; with one table
// and accumulate = 0 the value is written as interpolate_insolation does).
NX_EXPORT int nx_interpolate_insolation(const double *xyz_dev, int64_t n, double radius, const float *tables_dev,
                                        int n_tables, float *out_dev, int accumulate, void *stream)
{
    if (n < 0 || n_tables <= 0 || (n > 0 && (!xyz_dev || !tables_dev || !out_dev)) || !(radius > 0.0))
        return nx::fail(NX_EINVAL, "nx_interpolate_insolation: bad arguments");
    if (n == 0) return NX_OK;
    interp_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(xyz_dev, n, radius, tables_dev, n_tables, out_dev,
                                                                 accumulate);
    NX_CHECK_LAUNCH("interp_kernel");
    nx::note_launch(1);
    return NX_OK;
}

// climate.assign_surface_temp: out_dev float[n] for the vertices xyz_dev.
NX_EXPORT int nx_surface_temp(const double *xyz_dev, int64_t n, double radius, double tilt, float *out_dev,
                              void *stream)
{
    if (n < 0 || (n > 0 && (!xyz_dev || !out_dev)) || !(radius > 0.0))
        return nx::fail(NX_EINVAL, "nx_surface_temp: bad arguments");
    if (n == 0) return NX_OK;
    surface_temp_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(xyz_dev, n, radius, tilt, out_dev);
    NX_CHECK_LAUNCH("surface_temp_kernel");
    nx::note_launch(1);
    return NX_OK;
}
