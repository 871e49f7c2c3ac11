// nx_noise.cu -- fused fractal OpenSimplex-3D noise (fBm) for sm_103a.
//
// Replaces terrain.sample_octaves / terrain.sample_noise (terrain.py:12-59)
// over opensimplex.noise3d (opensimplex.py:266-759).
//
// Design
//  * One thread per vertex, all octaves in registers; persistent grid of
//    (#SM x resident CTAs) walking the vertex range.
//  * The seeded tables live in shared memory as one packed word per entry
//    [bits 0-6: gz+16 | bits 7-14: perm | bits 16-23: gx+16 | 24-31: gy+16],
//    replicated 32 times (entry k of lane l at word 32*k + l) so the three
//    dependent hash loads of a warp never conflict on a bank.
//  * Arithmetic is binary32.  The lattice cell, the region and the two extra
//    lattice points must equal what binary64 decides.  The large-magnitude
//    part of the skew is removed exactly: x*scale is formed as a float pair,
//    split into an integer A and a fraction a in [-1/2, 1/2], and with
//    T = Ax+Ay+Az = 6q + r the skewed coordinate becomes
//    xs = (Ax - q) + (a_x - (r + a_x + a_y + a_z)/6), whose second term is
//    O(1) and carries an absolute error of at most 2.2e-7 for
//    |x*scale| < 2^16 (the bound is worked through at decide_f32).  Every
//    comparison that decides the cell or region records its margin; the
//    compared quantities combine up to three such terms with a few more
//    roundings (errors below 1.3e-6), and when the smallest margin is below
//    TAU = 4e-6 (> 3x that), or |x*scale| >= 2^16, that lane recomputes the
//    decisions in binary64 with the reference's operation order
//    (decide_f64), so the decisions always equal the reference's.
//  * The 6 or 8 contributions are evaluated branch-free as 9 slots: the
//    corner (0,0,0)|(1,1,1), the six mixed corners, and the two extra points,
//    with masks per region; hash prefixes of the fixed slots are shared.
#include "nx_common.cuh"

#include <vector>

#include <cmath>

namespace {

constexpr float MAGIC = 12582912.0f;   // 1.5 * 2^23: v + MAGIC rounds v to an integer, |v| < 2^22
constexpr int MAGIC_BITS = 0x4B400000;
constexpr float TAU = 4.0e-6f;         // decision margin below which binary64 decides
constexpr float PMAX = 65536.0f;       // |x*scale| bound of the binary32 decision path
constexpr float THIRD = 1.0f / 3.0f;
constexpr float SIXTH = 1.0f / 6.0f;
constexpr float GBIAS = 8388624.0f;    // 2^23 + 16: removes the byte bias of a packed gradient

// opensimplex.py:51-60 (GRADIENTS_3D), used only to build the packed table.
__constant__ int c_grad3[72] = {
    -11, 4, 4, -4, 11, 4, -4, 4, 11,
    11, 4, 4, 4, 11, 4, 4, 4, 11,
    -11, -4, 4, -4, -11, 4, -4, -4, 11,
    11, -4, 4, 4, -11, 4, 4, -4, 11,
    -11, 4, -4, -4, 11, -4, -4, 4, -11,
    11, 4, -4, 4, 11, -4, 4, 4, -11,
    -11, -4, -4, -4, -11, -4, -4, -4, -11,
    11, -4, -4, 4, -11, -4, 4, -4, -11,
};

struct FbmParams {
    int n_oct;
    float s_hi[NX_MAX_OCTAVES];   // scale[o] as a binary32 pair
    float s_lo[NX_MAX_OCTAVES];
    float amp[NX_MAX_OCTAVES];    // 0.5 * strength[o] * radius
    double s[NX_MAX_OCTAVES];     // scale[o] (binary64 decision path)
};

static_assert(sizeof(nx_fbm_planet) == 960, "fBm planet descriptor layout");

constexpr int TABLE_WORDS = 256 * 32;
constexpr int TABLE_BYTES = TABLE_WORDS * 4;

__device__ __forceinline__ void build_table(uint32_t *T, const int32_t *__restrict__ perm,
                                            const int32_t *__restrict__ pgi)
{
    for (int i = threadIdx.x; i < TABLE_WORDS; i += blockDim.x) {
        int k = i >> 5;
        uint32_t p = (uint32_t)perm[k] & 255u;
        int g = pgi[k];
        g = g < 0 ? 0 : (g > 69 ? 69 : g);
        uint32_t w = ((uint32_t)(c_grad3[g + 2] + 16) & 0x7Fu) | (p << 7) |
                     ((uint32_t)(c_grad3[g] + 16) << 16) | ((uint32_t)(c_grad3[g + 1] + 16) << 24);
        T[i] = w;
    }
}

// The pair path's table: the same layout with the gradient's index (0-23,
// perm_grad_index_3D / 3) in bits 0-4 instead of the gradient bytes; the
// gradients themselves come as binary32 from s_grad.
__device__ __forceinline__ void build_table_pair(uint32_t *T, const int32_t *__restrict__ perm,
                                                 const int32_t *__restrict__ pgi)
{
    for (int i = threadIdx.x; i < TABLE_WORDS; i += blockDim.x) {
        int k = i >> 5;
        uint32_t p = (uint32_t)perm[k] & 255u;
        int g = pgi[k];
        g = g < 0 ? 0 : (g > 69 ? 69 : g);
        T[i] = (uint32_t)(g / 3) | (p << 7);
    }
}

// GRADIENTS_3D as binary32 (x, y, z, 0), and as sign masks (bit 31 of each
// component) with the axis of the +-11 component (every gradient has one
// +-11 and two +-4 components), filled per block.
__shared__ float4 s_grad[24];
__shared__ uint4 s_gsign[24];

__device__ __forceinline__ void init_grad_table()
{
    for (int i = threadIdx.x; i < 24; i += blockDim.x) {
        const int gx = c_grad3[3 * i], gy = c_grad3[3 * i + 1], gz = c_grad3[3 * i + 2];
        s_grad[i] = make_float4((float)gx, (float)gy, (float)gz, 0.0f);
        const uint32_t a = (gx == 11 || gx == -11) ? 0u : ((gy == 11 || gy == -11) ? 1u : 2u);
        s_gsign[i] = make_uint4(gx < 0 ? 0x80000000u : 0u, gy < 0 ? 0x80000000u : 0u, gz < 0 ? 0x80000000u : 0u, a);
    }
}

// Hash table load: bits 7-14 of a select the entry; lb = this lane's byte
// offset of replica 0 in shared memory.
__device__ __forceinline__ uint32_t lk(uint32_t lb, int a)
{
    uint32_t v;
    uint32_t addr = lb + ((uint32_t)a & 0x7F80u);
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(addr));
    return v;
}

// Split a binary64 into hi + lo binary32 with integer operations (no FP64
// unit): hi = value truncated to 24 significant bits, lo = the next 23 bits.
// |x - (hi+lo)| <= 2^-47 |x|.  Magnitudes outside [2^-74, 2^127] give lo = 0
// (and hi = +-0 or +-inf); such lanes take the binary64 path anyway.
__device__ __forceinline__ void split_f64(double v, float &hi, float &lo)
{
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    uint32_t hw = (uint32_t)(b >> 32), lw = (uint32_t)b;
    int e = (int)((hw >> 20) & 0x7FF) - 1023;
    uint32_t sign = hw & 0x80000000u;
    if (e < -126) { hi = __uint_as_float(sign); lo = 0.0f; return; }
    if (e > 127) { hi = __uint_as_float(sign | 0x7F800000u); lo = 0.0f; return; }
    uint32_t top = ((hw & 0xFFFFFu) << 3) | (lw >> 29);
    hi = __uint_as_float(sign | ((uint32_t)(e + 127) << 23) | top);
    if (e < -74 + 6) { lo = 0.0f; return; }
    // remainder bits 28..6 of the low word, as 23-bit integer times 2^(e-46)
    uint32_t rem = (lw & 0x1FFFFFFFu) >> 6;
    float r = __uint_as_float(0x4B000000u | rem) - 8388608.0f;    // exact
    float sc = __uint_as_float((uint32_t)(e - 46 + 127) << 23);
    lo = __uint_as_float(__float_as_uint(r * sc) | sign);
}

// Decisions of noise3d (opensimplex.py:302-700) in either precision.  For
// float, `m` tracks the smallest |a-b| over the comparisons on the taken
// path; for double it is unused.  Extra-point offsets are relative to the
// cell origin (components in {-1,0,1,2}).
struct Decision {
    int region;
    float e0x, e0y, e0z, e1x, e1y, e1z;   // decide() only
    uint32_t w;                           // the offsets + 1, two bits each (e0x, e0y, e0z, e1x, e1y, e1z)
    float E[6];                           // displacement offsets e + (ex + ey + ez) / 3 of both points
};

template <typename T, bool TRACK>
struct Cmp {
    float m;
    __device__ __forceinline__ void note(T a, T b)
    {
        if (TRACK) m = fminf(m, fabsf((float)(a - b)));
    }
    __device__ __forceinline__ bool gt(T a, T b) { note(a, b); return a > b; }
    __device__ __forceinline__ bool ge(T a, T b) { note(a, b); return a >= b; }
    __device__ __forceinline__ bool lt(T a, T b) { note(a, b); return a < b; }
    __device__ __forceinline__ bool le(T a, T b) { note(a, b); return a <= b; }
};

template <typename T, bool TRACK>
__device__ __forceinline__ void decide(T xins, T yins, T zins, T in_sum, Cmp<T, TRACK> &C,
                                       Decision &D)
{
    const T one = (T)1, two = (T)2, three = (T)3;
    if (C.le(in_sum, one)) {
        // tetrahedron at (0,0,0): closest two of (1,0,0), (0,1,0), (0,0,1)
        D.region = 0;
        int ap = 1, bp = 2;
        T as = xins, bs = yins;
        if (C.ge(as, bs)) {
            if (C.gt(zins, bs)) { bs = zins; bp = 4; }
        } else {
            if (C.gt(zins, as)) { as = zins; ap = 4; }
        }
        T wins = one - in_sum;
        bool near0 = C.gt(wins, as);
        if (!near0) near0 = C.gt(wins, bs);
        if (near0) {
            int c = C.gt(bs, as) ? bp : ap;
            if ((c & 1) == 0) { D.e0x = -1.f; D.e1x = 0.f; } else { D.e0x = 1.f; D.e1x = 1.f; }
            if ((c & 2) == 0) {
                D.e0y = 0.f; D.e1y = 0.f;
                if ((c & 1) == 0) D.e1y = -1.f; else D.e0y = -1.f;
            } else { D.e0y = 1.f; D.e1y = 1.f; }
            if ((c & 4) == 0) { D.e0z = 0.f; D.e1z = -1.f; } else { D.e0z = 1.f; D.e1z = 1.f; }
        } else {
            int c = ap | bp;
            if ((c & 1) == 0) { D.e0x = 0.f; D.e1x = -1.f; } else { D.e0x = 1.f; D.e1x = 1.f; }
            if ((c & 2) == 0) { D.e0y = 0.f; D.e1y = -1.f; } else { D.e0y = 1.f; D.e1y = 1.f; }
            if ((c & 4) == 0) { D.e0z = 0.f; D.e1z = -1.f; } else { D.e0z = 1.f; D.e1z = 1.f; }
        }
    } else if (C.ge(in_sum, two)) {
        // tetrahedron at (1,1,1): closest two of (1,1,0), (1,0,1), (0,1,1)
        D.region = 1;
        int ap = 6, bp = 5;
        T as = xins, bs = yins;
        if (C.le(as, bs)) {
            if (C.lt(zins, bs)) { bs = zins; bp = 3; }
        } else {
            if (C.lt(zins, as)) { as = zins; ap = 3; }
        }
        T wins = three - in_sum;
        bool near1 = C.lt(wins, as);
        if (!near1) near1 = C.lt(wins, bs);
        if (near1) {
            int c = C.lt(bs, as) ? bp : ap;
            if ((c & 1) != 0) { D.e0x = 2.f; D.e1x = 1.f; } else { D.e0x = 0.f; D.e1x = 0.f; }
            if ((c & 2) != 0) {
                D.e0y = 1.f; D.e1y = 1.f;
                if ((c & 1) != 0) D.e1y = 2.f; else D.e0y = 2.f;
            } else { D.e0y = 0.f; D.e1y = 0.f; }
            if ((c & 4) != 0) { D.e0z = 1.f; D.e1z = 2.f; } else { D.e0z = 0.f; D.e1z = 0.f; }
        } else {
            int c = ap & bp;
            if ((c & 1) != 0) { D.e0x = 1.f; D.e1x = 2.f; } else { D.e0x = 0.f; D.e1x = 0.f; }
            if ((c & 2) != 0) { D.e0y = 1.f; D.e1y = 2.f; } else { D.e0y = 0.f; D.e1y = 0.f; }
            if ((c & 4) != 0) { D.e0z = 1.f; D.e1z = 2.f; } else { D.e0z = 0.f; D.e1z = 0.f; }
        }
    } else {
        // octahedron between them
        D.region = 2;
        T as, bs, score;
        int ap, bp;
        bool af, bf;
        T p1 = xins + yins;
        if (C.gt(p1, one)) { as = p1 - one; ap = 3; af = true; }
        else { as = one - p1; ap = 4; af = false; }
        T p2 = xins + zins;
        if (C.gt(p2, one)) { bs = p2 - one; bp = 5; bf = true; }
        else { bs = one - p2; bp = 2; bf = false; }
        T p3 = yins + zins;
        bool t3 = C.gt(p3, one);
        score = t3 ? p3 - one : one - p3;
        if (C.le(as, bs)) {
            if (C.lt(as, score)) { ap = t3 ? 6 : 1; af = t3; }
        } else {
            if (C.lt(bs, score)) { bp = t3 ? 6 : 1; bf = t3; }
        }
        if (af == bf) {
            if (af) {
                D.e0x = 1.f; D.e0y = 1.f; D.e0z = 1.f;
                int c = ap & bp;
                if (c & 1) { D.e1x = 2.f; D.e1y = 0.f; D.e1z = 0.f; }
                else if (c & 2) { D.e1x = 0.f; D.e1y = 2.f; D.e1z = 0.f; }
                else { D.e1x = 0.f; D.e1y = 0.f; D.e1z = 2.f; }
            } else {
                D.e0x = 0.f; D.e0y = 0.f; D.e0z = 0.f;
                int c = ap | bp;
                if ((c & 1) == 0) { D.e1x = -1.f; D.e1y = 1.f; D.e1z = 1.f; }
                else if ((c & 2) == 0) { D.e1x = 1.f; D.e1y = -1.f; D.e1z = 1.f; }
                else { D.e1x = 1.f; D.e1y = 1.f; D.e1z = -1.f; }
            }
        } else {
            int c1 = af ? ap : bp;
            int c2 = af ? bp : ap;
            if ((c1 & 1) == 0) { D.e0x = -1.f; D.e0y = 1.f; D.e0z = 1.f; }
            else if ((c1 & 2) == 0) { D.e0x = 1.f; D.e0y = -1.f; D.e0z = 1.f; }
            else { D.e0x = 1.f; D.e0y = 1.f; D.e0z = -1.f; }
            D.e1x = 0.f; D.e1y = 0.f; D.e1z = 0.f;
            if (c2 & 1) D.e1x = 2.f;
            else if (c2 & 2) D.e1y = 2.f;
            else D.e1z = 2.f;
        }
    }
}


// Octahedron extra points (opensimplex.py:535-700) from the six comparison
// outcomes g1 = p1 > 1, g2 = p2 > 1, t3 = p3 > 1, ale = |p1-1| <= |p2-1|,
// a_lt = |p1-1| < |p3-1|, b_lt = |p2-1| < |p3-1| (bit k of b).  Offsets are
// in {-1, 0, 1, 2}; a block tabulates all 64 cases once (s_extra) and the
// per-lane decision looks its case up.
__device__ __forceinline__ uint32_t octa_case(int b)
{
    const bool g1 = b & 1, g2 = b & 2, t3 = b & 4, ale = b & 8, a_lt = b & 16, b_lt = b & 32;
    const bool swa = ale && a_lt, swb = !ale && b_lt;
    const int oap = swa ? (t3 ? 6 : 1) : (g1 ? 3 : 4);
    const int obp = swb ? (t3 ? 6 : 1) : (g2 ? 5 : 2);
    const bool af = swa ? t3 : g1, bf = swb ? t3 : g2;
    float o0x, o0y, o0z, o1x, o1y, o1z;
    if (af == bf) {
        const int c = af ? (oap & obp) : (oap | obp);
        const float b = af ? 1.f : 0.f;
        o0x = b; o0y = b; o0z = b;
        // af: the single bit of c picks the axis that gets 2; otherwise the
        // first axis whose bit is clear gets -1 and the others 1
        const bool c1 = (c & 1) != 0, c2 = (c & 2) != 0;
        const bool ax = af ? c1 : !c1, ay = af ? (!c1 && c2) : (c1 && !c2);
        const bool az = !ax && !ay;
        const float hit = af ? 2.f : -1.f, miss = af ? 0.f : 1.f;
        o1x = ax ? hit : miss; o1y = ay ? hit : miss; o1z = az ? hit : miss;
    } else {
        const int c1 = af ? oap : obp, c2 = af ? obp : oap;
        const bool bx = (c1 & 1) == 0, by = !bx && (c1 & 2) == 0;
        const bool bz = !bx && !by;
        o0x = bx ? -1.f : 1.f; o0y = by ? -1.f : 1.f; o0z = bz ? -1.f : 1.f;
        const bool qx = (c2 & 1) != 0, qy = !qx && (c2 & 2) != 0;
        const bool qz = !qx && !qy;
        o1x = qx ? 2.f : 0.f; o1y = qy ? 2.f : 0.f; o1z = qz ? 2.f : 0.f;
    }
    const float o[6] = {o0x, o0y, o0z, o1x, o1y, o1z};
    uint32_t w = 0;
#pragma unroll
    for (int k = 0; k < 6; ++k) w |= (uint32_t)((int)o[k] + 1) << (2 * k);
    return w;
}

// Tetrahedron extra points (opensimplex.py:302-533) from the comparison
// outcomes, in the mirrored form the binary32 decision uses (region 1's
// comparisons are region 0's with both sides negated): bit 0 x >= y, 1
// z > y, 2 z > x, 3 wins > as, 4 wins > bs, 5 bs > as (as, bs the scores
// the first three select), 6 region 1 (offsets t become 1 - t).
__device__ __forceinline__ uint32_t tetra_case(int b)
{
    const bool xy = b & 1, zb = b & 2, za = b & 4, n1 = b & 8, n2 = b & 16, cnb = b & 32, r1 = b & 64;
    const bool repb = xy && zb, repa = !xy && za;
    const int ap = repa ? 4 : 1, bp = repb ? 4 : 2;
    const bool near = n1 || n2;
    const int cn = cnb ? bp : ap;
    const int cf = ap | bp;
    const bool cn1 = (cn & 1) != 0, cn2 = (cn & 2) != 0, cn4 = (cn & 4) != 0;
    float t[6];
    t[0] = near ? (cn1 ? 1.f : -1.f) : ((cf & 1) ? 1.f : 0.f);
    t[3] = near ? (cn1 ? 1.f : 0.f) : ((cf & 1) ? 1.f : -1.f);
    t[1] = near ? (cn2 ? 1.f : (cn1 ? -1.f : 0.f)) : ((cf & 2) ? 1.f : 0.f);
    t[4] = near ? (cn2 ? 1.f : (cn1 ? 0.f : -1.f)) : ((cf & 2) ? 1.f : -1.f);
    t[2] = near ? (cn4 ? 1.f : 0.f) : ((cf & 4) ? 1.f : 0.f);
    t[5] = near ? (cn4 ? 1.f : -1.f) : ((cf & 4) ? 1.f : -1.f);
    uint32_t w = 0;
#pragma unroll
    for (int k = 0; k < 6; ++k) w |= (uint32_t)((int)(r1 ? 1.f - t[k] : t[k]) + 1) << (2 * k);
    return w;
}

// Offset k of a case word: ((w >> 2k) & 3) - 1.
__device__ __forceinline__ int word_offset(uint32_t w, int k)
{
    return (int)((w >> (2 * k)) & 3u) - 1;
}

// The displacement offsets of an extra point o: o + (ox + oy + oz) / 3
// per component (the point's skewed position relative to the cell
// origin's), rounded step by step.
__device__ __forceinline__ void extra_disp(float ox, float oy, float oz, float *E)
{
    const float s = __fmul_rn(__fadd_rn(__fadd_rn(ox, oy), oz), THIRD);
    E[0] = __fadd_rn(ox, s);
    E[1] = __fadd_rn(oy, s);
    E[2] = __fadd_rn(oz, s);
}

// Case word and displacement offsets of a decision from its six offsets
// (the binary64 path).
__device__ __forceinline__ void pack_extra(Decision &D)
{
    const float o[6] = {D.e0x, D.e0y, D.e0z, D.e1x, D.e1y, D.e1z};
    uint32_t w = 0;
#pragma unroll
    for (int k = 0; k < 6; ++k) w |= (uint32_t)((int)o[k] + 1) << (2 * k);
    D.w = w;
    extra_disp(o[0], o[1], o[2], D.E);
    extra_disp(o[3], o[4], o[5], D.E + 3);
}

// Extra-point table of a block: [0, 64) octahedron cases, [64, 192)
// tetrahedron cases.  Entry i is two float4s: the six displacement offsets
// (E0x, E0y, E0z, E1x), (E1y, E1z, case word as bits, 0).
__shared__ float4 s_extra[2 * 192];

// Fill s_extra (the caller synchronises the block before use).
__device__ __forceinline__ void init_extra_table()
{
    for (int i = threadIdx.x; i < 192; i += blockDim.x) {
        const uint32_t w = i < 64 ? octa_case(i) : tetra_case(i - 64);
        float E[6];
        extra_disp((float)word_offset(w, 0), (float)word_offset(w, 1), (float)word_offset(w, 2), E);
        extra_disp((float)word_offset(w, 3), (float)word_offset(w, 4), (float)word_offset(w, 5), E + 3);
        s_extra[2 * i] = make_float4(E[0], E[1], E[2], E[3]);
        s_extra[2 * i + 1] = make_float4(E[4], E[5], __uint_as_float(w), 0.0f);
    }
}

// (offset k of a case word + 1) * 128: the offset's step in a hash address.
__device__ __forceinline__ int word_step(uint32_t w, int k)
{
    return (int)((k < 4 ? w << (7 - 2 * k) : w >> (2 * k - 7)) & 0x180u);
}

// The same decision for the binary32 path without data-dependent branches
// (lanes of a warp sit in different regions at high octaves).  Regions 0
// and 1 are mirror images: region 1's comparisons are region 0's with both
// sides negated (exact), its lattice-point codes are 7 - region 0's and its
// offsets are 1 - region 0's; both tetrahedra and the octahedron are
// evaluated and the region selects.  Every comparison evaluated records its
// margin (a superset of those the branching form records), so a lane keeps
// its binary32 decision only when all of them clear the margin.
__device__ __forceinline__ int decide_sel(float x, float y, float z, float in_sum, Cmp<float, true> &C, int &region)
{
    const bool r0 = C.le(in_sum, 1.0f);
    const bool r1 = !r0 && C.ge(in_sum, 2.0f);
    // tetrahedron (region 0 form; s = -1 mirrors the comparisons for region 1)
    const float s = r1 ? -1.0f : 1.0f;
    const bool xy = C.ge(s * x, s * y);
    const bool zb = C.gt(s * z, s * y);
    const bool za = C.gt(s * z, s * x);
    const bool repb = xy && zb, repa = !xy && za;
    const float as = repa ? z : x, bs = repb ? z : y;
    const float wins = (r1 ? 3.0f : 1.0f) - in_sum;
    const bool n1 = C.gt(s * wins, s * as);
    const bool n2 = C.gt(s * wins, s * bs);
    const bool cnb = C.gt(s * bs, s * as);
    // octahedron
    const float p1 = x + y, p2 = x + z, p3 = y + z;
    const bool g1 = C.gt(p1, 1.0f), g2 = C.gt(p2, 1.0f), t3 = C.gt(p3, 1.0f);
    const float oas = g1 ? p1 - 1.0f : 1.0f - p1;
    const float obs = g2 ? p2 - 1.0f : 1.0f - p2;
    const float score = t3 ? p3 - 1.0f : 1.0f - p3;
    const bool ale = C.le(oas, obs);
    const bool a_lt = C.lt(oas, score), b_lt = C.lt(obs, score);
    // the two extra points are a function of the region's comparison
    // outcomes: one lookup in the block's table (tetrahedron or octahedron
    // case, see tetra_case / octa_case)
    const bool tet = r0 || r1;
    const uint32_t ot = (g1 ? 1u : 0u) | (g2 ? 2u : 0u) | (t3 ? 4u : 0u) | (ale ? 8u : 0u) | (a_lt ? 16u : 0u) |
                        (b_lt ? 32u : 0u);
    const uint32_t tt = 64u + ((xy ? 1u : 0u) | (zb ? 2u : 0u) | (za ? 4u : 0u) | (n1 ? 8u : 0u) | (n2 ? 16u : 0u) |
                               (cnb ? 32u : 0u) | (r1 ? 64u : 0u));
    region = r0 ? 0 : (r1 ? 1 : 2);
    return (int)(tet ? tt : ot);
}

// Decision of a binary32-path lane from its case-table entry.
__device__ __forceinline__ void case_decision(int ci, int region, Decision &D)
{
    const float4 *t = s_extra + 2 * ci;
    const float4 a = t[0], b = t[1];
    D.region = region;
    D.w = __float_as_uint(b.z);
    D.E[0] = a.x; D.E[1] = a.y; D.E[2] = a.z; D.E[3] = a.w; D.E[4] = b.x; D.E[5] = b.y;
}

// opensimplex.py:18-21 in binary64
__device__ __forceinline__ long long fastfloor64(double x)
{
    long long xi = __double2ll_rz(x);
    return x < (double)xi ? xi - 1 : xi;
}

// The cell state the contributions need.
struct Cell {
    float dx0, dy0, dz0;
    int xb7, yb7, zb7;       // cell origin << 7 (hash base)
    int xsb, ysb, zsb;       // cell origin (trace only)
    Decision D;
    double dxd, dyd, dzd;    // binary64 path only: the displacement before rounding to binary32
};

// Binary64 decisions with the reference's operation order (opensimplex.py:
// 270-300 and the region code).  No FMA contraction: explicit _rn ops.
// Returns the cell by value: a cell passed by reference would be
// address-taken in the caller, which then keeps it in local memory on the
// common binary32 path too.
__device__ __noinline__ Cell decide_f64(double X, double Y, double Z, double s)
{
    Cell c;
    double x = __dmul_rn(X, s), y = __dmul_rn(Y, s), z = __dmul_rn(Z, s);
    double so = __dmul_rn(__dadd_rn(__dadd_rn(x, y), z), -1.0 / 6);
    double xs = __dadd_rn(x, so), ys = __dadd_rn(y, so), zs = __dadd_rn(z, so);
    long long xsb = fastfloor64(xs), ysb = fastfloor64(ys), zsb = fastfloor64(zs);
    double sq = __dmul_rn((double)(xsb + ysb + zsb), 1.0 / 3);
    double xb = __dadd_rn((double)xsb, sq), yb = __dadd_rn((double)ysb, sq), zb = __dadd_rn((double)zsb, sq);
    double xins = __dsub_rn(xs, (double)xsb), yins = __dsub_rn(ys, (double)ysb), zins = __dsub_rn(zs, (double)zsb);
    double in_sum = __dadd_rn(__dadd_rn(xins, yins), zins);
    Cmp<double, false> C;
    C.m = 0.f;
    decide<double, false>(xins, yins, zins, in_sum, C, c.D);
    pack_extra(c.D);
    c.dxd = __dsub_rn(x, xb);
    c.dyd = __dsub_rn(y, yb);
    c.dzd = __dsub_rn(z, zb);
    c.dx0 = (float)c.dxd;
    c.dy0 = (float)c.dyd;
    c.dz0 = (float)c.dzd;
    c.xsb = (int)xsb; c.ysb = (int)ysb; c.zsb = (int)zsb;
    c.xb7 = (int)((unsigned)xsb << 7);
    c.yb7 = (int)((unsigned)ysb << 7);
    c.zb7 = (int)((unsigned)zsb << 7);
    return c;
}

// What the decision from a coordinate split leaves for the displacement:
// the floors f of the skewed fractions and G = r + fx + fy + fz, so that
// dx0 = a_x - (3 fx + G) / 3 (and likewise y, z), and the case-table index.
struct Core {
    int xsb, ysb, zsb;
    int xb7, yb7, zb7;
    float fx, fy, fz, G;
    int region, ci;
};

// The decision from the split of x*scale into integers A (binary32, |A| <
// 2^22) and fractions a (|a| < 1) for each axis; `big` = max |x*scale|.
// Returns false when binary64 must decide.  The error analysis is at
// decide_f32 (a within 3.1e-8 of x*scale - A).
__device__ __forceinline__ bool decide_core(float Ax, float ax, float Ay, float ay, float Az, float az, float big,
                                            Core &o)
{
    const float T = __fadd_rn(__fadd_rn(Ax, Ay), Az);
    const float q = floorf(__fmaf_rn(T, SIXTH, 1.0f / 12.0f));
    const float r = __fmaf_rn(-6.0f, q, T);
    const float u = __fadd_rn(r, __fadd_rn(__fadd_rn(ax, ay), az));
    const float bx = __fmaf_rn(-u, SIXTH, ax), by = __fmaf_rn(-u, SIXTH, ay), bz = __fmaf_rn(-u, SIXTH, az);
    const float fx = floorf(bx), fy = floorf(by), fz = floorf(bz);
    const float xins = __fsub_rn(bx, fx), yins = __fsub_rn(by, fy), zins = __fsub_rn(bz, fz);
    const float xsbf = __fadd_rn(__fsub_rn(Ax, q), fx), ysbf = __fadd_rn(__fsub_rn(Ay, q), fy),
                zsbf = __fadd_rn(__fsub_rn(Az, q), fz);
    const int xi = __float_as_int(__fadd_rn(xsbf, MAGIC)), yi = __float_as_int(__fadd_rn(ysbf, MAGIC)),
              zi = __float_as_int(__fadd_rn(zsbf, MAGIC));
    o.xsb = xi - MAGIC_BITS; o.ysb = yi - MAGIC_BITS; o.zsb = zi - MAGIC_BITS;
    o.xb7 = xi << 7; o.yb7 = yi << 7; o.zb7 = zi << 7;
    o.fx = fx; o.fy = fy; o.fz = fz;
    o.G = __fadd_rn(r, __fadd_rn(__fadd_rn(fx, fy), fz));
    Cmp<float, true> C;
    C.m = fminf(fminf(fminf(xins, 1.0f - xins), fminf(yins, 1.0f - yins)), fminf(zins, 1.0f - zins));
    const float in_sum = __fadd_rn(__fadd_rn(xins, yins), zins);
    o.ci = decide_sel(xins, yins, zins, in_sum, C, o.region);
    return C.m >= TAU && big < PMAX;
}

// Binary32 path.  Returns false when binary64 must decide.
//
// Error of b = a - u/6 (the skewed coordinate less its integer part Ax - q)
// for |x*scale| < 2^16, each step's rounding in absolute terms:
//  * p + e = x*scale within 2^-45 |x*scale| < 2e-9: the coordinate and the
//    scale are binary32 pairs (2^-47 and 2^-48 relative), the lo*lo term is
//    dropped and the three cross terms are fused;
//  * A = round(p) and p - A are exact; a = (p - A) + e rounds once,
//    |a| < 1: <= 2^-25 (3.0e-8);
//  * T = Ax + Ay + Az is an exact integer and q = floor(T/6 + 1/12) is exact
//    (T/6 + 1/12 lies at least 1/12 from an integer; the fused product's
//    error is below |T| 2^-24 < 0.02), so r = T - 6q in 0..5 is exact;
//  * the sum of the three a (two roundings, values < 1.5): <= 1.2e-7,
//    entering b divided by 6: 2.0e-8; u = r + that, |u| < 8: 2.4e-7 / 6 =
//    4.0e-8; the errors of the a themselves: 3.0e-8 * (5/6 + 2/6) = 3.5e-8;
//  * SIXTH = 1/6 rounded, off by 5.0e-9, times |u| <= 6.5: 3.2e-8; the
//    fused b = a - u*SIXTH, |b| < 2: <= 2^-24 (6.0e-8).
// Total <= 1.9e-7 (checked by simulating these operations on random
// coordinates and scales: largest 1.3e-7).  xins = b - floor(b) is exact.
__device__ __forceinline__ bool decide_f32(float xh, float xl, float yh, float yl, float zh, float zl,
                                           float sh, float sl, Cell &c)
{
    float px = xh * sh, py = yh * sh, pz = zh * sh;
    float ex = fmaf(xh, sh, -px), ey = fmaf(yh, sh, -py), ez = fmaf(zh, sh, -pz);
    ex = fmaf(xh, sl, ex); ey = fmaf(yh, sl, ey); ez = fmaf(zh, sl, ez);
    ex = fmaf(xl, sh, ex); ey = fmaf(yl, sh, ey); ez = fmaf(zl, sh, ez);
    float big = fmaxf(fabsf(px), fmaxf(fabsf(py), fabsf(pz)));
    float Ax = (px + MAGIC) - MAGIC, Ay = (py + MAGIC) - MAGIC, Az = (pz + MAGIC) - MAGIC;
    float ax = (px - Ax) + ex, ay = (py - Ay) + ey, az = (pz - Az) + ez;
    Core o;
    const bool ok = decide_core(Ax, ax, Ay, ay, Az, az, big, o);
    c.xsb = o.xsb; c.ysb = o.ysb; c.zsb = o.zsb;
    c.xb7 = o.xb7; c.yb7 = o.yb7; c.zb7 = o.zb7;
    const float g = __fmul_rn(o.G, THIRD);
    c.dx0 = __fsub_rn(__fsub_rn(ax, o.fx), g);
    c.dy0 = __fsub_rn(__fsub_rn(ay, o.fy), g);
    c.dz0 = __fsub_rn(__fsub_rn(az, o.fz), g);
    case_decision(o.ci, o.region, c.D);
    return ok;
}

// One lattice contribution: attn^4 * (grad . d) if attn > 0.
__device__ __forceinline__ float contrib(uint32_t w, float dx, float dy, float dz, bool on)
{
    float attn = fmaf(-dx, dx, fmaf(-dy, dy, fmaf(-dz, dz, 2.0f)));
    attn = on ? fmaxf(attn, 0.0f) : 0.0f;
    float a2 = attn * attn;
    float gx = __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7442)) - GBIAS;
    float gy = __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7443)) - GBIAS;
    float gz = __uint_as_float((w & 0x7Fu) | 0x4B000000u) - GBIAS;
    float dot = fmaf(gx, dx, fmaf(gy, dy, gz * dz));
    return (a2 * a2) * dot;
}

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

__device__ __forceinline__ float gcomp(uint32_t w, uint32_t sel)
{
    return __uint_as_float(__byte_perm(w, 0x4B000000u, sel));
}

// Two lattice contributions at once in paired binary32 arithmetic (one
// FFMA2/FMUL2/FADD2 does both): acc += attn^4 * (grad . d) for slots a and
// b; ON (1 or 0) masks slots outside the region.  -attn = |d|^2 - 2 is
// clamped at 0 before squaring, so only attn > 0 counts.
__device__ __forceinline__ float2 contrib2(uint32_t wa, uint32_t wb, float2 DX, float2 DY, float2 DZ, float2 ON,
                                           float2 acc)
{
    float2 sq = __fmul2_rn(DZ, DZ);
    sq = __ffma2_rn(DY, DY, sq);
    sq = __ffma2_rn(DX, DX, sq);
    float2 na = __fadd2_rn(sq, f2(-2.0f, -2.0f));
    na = f2(fminf(na.x, 0.0f), fminf(na.y, 0.0f));
    na = __fmul2_rn(na, ON);
    const float2 a2 = __fmul2_rn(na, na);
    const float2 a4 = __fmul2_rn(a2, a2);
    const float2 nb = f2(-GBIAS, -GBIAS);
    const float2 gx = __fadd2_rn(f2(gcomp(wa, 0x7442), gcomp(wb, 0x7442)), nb);
    const float2 gy = __fadd2_rn(f2(gcomp(wa, 0x7443), gcomp(wb, 0x7443)), nb);
    const float2 gz = __fadd2_rn(f2(__uint_as_float((wa & 0x7Fu) | 0x4B000000u),
                                    __uint_as_float((wb & 0x7Fu) | 0x4B000000u)), nb);
    float2 dot = __fmul2_rn(gz, DZ);
    dot = __ffma2_rn(gy, DY, dot);
    dot = __ffma2_rn(gx, DX, dot);
    return __ffma2_rn(a4, dot, acc);
}

// noise3d(x*s) * 103 for one vertex and octave.
template <bool TRACE>
__device__ __forceinline__ float noise_raw(float xh, float xl, float yh, float yl, float zh, float zl,
                                           float sh, float sl, double X, double Y, double Z, double s,
                                           uint32_t lb, unsigned &nfb, int32_t *tr, int32_t *sl9)
{
    Cell c;
    if (!decide_f32(xh, xl, yh, yl, zh, zl, sh, sl, c)) {
        c = decide_f64(X, Y, Z, s);
        ++nfb;
    }
    const int r = c.D.region;
    const bool on0 = r != 2, onA = r != 1, onB = r != 0;
    // hash prefixes of the fixed slots
    uint32_t h0 = lk(lb, c.xb7), h1 = lk(lb, c.xb7 + 128);
    uint32_t h00 = lk(lb, (int)h0 + c.yb7), h01 = lk(lb, (int)h0 + c.yb7 + 128);
    uint32_t h10 = lk(lb, (int)h1 + c.yb7), h11 = lk(lb, (int)h1 + c.yb7 + 128);
    const int z0 = c.zb7, z1 = c.zb7 + 128;
    const float dx0 = c.dx0, dy0 = c.dy0, dz0 = c.dz0;
    // slot 0: (0,0,0) in region 0, (1,1,1) in region 1
    uint32_t w0 = lk(lb, r == 1 ? (int)h11 + z1 : (int)h00 + z0);
    const float k0 = r == 1 ? 1.0f + 1.0f : 0.0f;   // o + sum(o)/3 with o = (1,1,1): 1 + 1
    // mixed corners; displacement d = d0 - o - sum(o)/3
    const float c1 = 1.0f + THIRD, c2 = 2.0f * THIRD, c3 = 1.0f + 2.0f * THIRD;
    uint32_t w100 = lk(lb, (int)h10 + z0), w010 = lk(lb, (int)h01 + z0), w001 = lk(lb, (int)h00 + z1);
    uint32_t w110 = lk(lb, (int)h11 + z0), w101 = lk(lb, (int)h10 + z1), w011 = lk(lb, (int)h01 + z1);
    // extra points
    const Decision &D = c.D;
    const uint32_t ew = D.w;
    const int xm = c.xb7 - 128, ym = c.yb7 - 128, zm = c.zb7 - 128;
    uint32_t we0 = lk(lb, (int)lk(lb, (int)lk(lb, xm + word_step(ew, 0)) + ym + word_step(ew, 1)) + zm + word_step(ew, 2));
    uint32_t we1 = lk(lb, (int)lk(lb, (int)lk(lb, xm + word_step(ew, 3)) + ym + word_step(ew, 4)) + zm + word_step(ew, 5));
    const float2 X0 = f2(dx0, dx0), Y0 = f2(dy0, dy0), Z0 = f2(dz0, dz0);
    const float fon0 = on0 ? 1.0f : 0.0f, fA = onA ? 1.0f : 0.0f, fB = onB ? 1.0f : 0.0f;
    float2 acc = f2(0.0f, 0.0f);
    acc = contrib2(w0, w100, __fadd2_rn(X0, f2(-k0, -c1)), __fadd2_rn(Y0, f2(-k0, -THIRD)),
                   __fadd2_rn(Z0, f2(-k0, -THIRD)), f2(fon0, fA), acc);
    acc = contrib2(w010, w001, __fadd2_rn(X0, f2(-THIRD, -THIRD)), __fadd2_rn(Y0, f2(-c1, -THIRD)),
                   __fadd2_rn(Z0, f2(-THIRD, -c1)), f2(fA, fA), acc);
    acc = contrib2(w110, w101, __fadd2_rn(X0, f2(-c3, -c3)), __fadd2_rn(Y0, f2(-c3, -c2)),
                   __fadd2_rn(Z0, f2(-c2, -c3)), f2(fB, fB), acc);
    acc = contrib2(w011, we0, __fadd2_rn(X0, f2(-c2, -D.E[0])), __fadd2_rn(Y0, f2(-c3, -D.E[1])),
                   __fadd2_rn(Z0, f2(-c3, -D.E[2])), f2(fB, 1.0f), acc);
    float v = (acc.x + acc.y) + contrib(we1, dx0 - D.E[3], dy0 - D.E[4], dz0 - D.E[5], true);
    if (TRACE) {
        tr[0] = c.xsb; tr[1] = c.ysb; tr[2] = c.zsb; tr[3] = r;
        int e[6];
        for (int k = 0; k < 6; ++k) e[k] = word_offset(ew, k);
        tr[4] = c.xsb + e[0]; tr[5] = c.ysb + e[1]; tr[6] = c.zsb + e[2];
        tr[7] = c.xsb + e[3]; tr[8] = c.ysb + e[4]; tr[9] = c.zsb + e[5];
        const int o[9][3] = {{r == 1, r == 1, r == 1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0},
                             {1, 0, 1}, {0, 1, 1}, {e[0], e[1], e[2]}, {e[3], e[4], e[5]}};
        const uint32_t w[9] = {w0, w100, w010, w001, w110, w101, w011, we0, we1};
        const bool on[9] = {on0, onA, onA, onA, onB, onB, onB, true, true};
        for (int k = 0; k < 9; ++k) {
            int32_t *q = sl9 + 5 * k;
            q[0] = c.xsb + o[k][0]; q[1] = c.ysb + o[k][1]; q[2] = c.zsb + o[k][2];
            q[3] = (int32_t)(((w[k] >> 16) & 0xFF) | (((w[k] >> 24) & 0xFF) << 8) | ((w[k] & 0x7F) << 16));
            q[4] = on[k] ? 1 : 0;
        }
    }
    return v;
}


// ---------------------------------------------------------------------------
// Pair-precision noise (the batched, plain and served planet paths).
//
// Eroded planets need elevations much closer to binary64 than binary32
// gives: the erosion update branches on the sign of every neighbour height
// difference, and starting heights off by binary32 rounding (3e-7 relative)
// flip near-ties, after which water, sediment and heights leave the binary64
// trajectory (0.4 % of max |h| after 30 iterations, 13 % after 60, on a
// 100,002-vertex sphere; random errors of 1e-11 in the raw fBm sum flipped
// nothing in 100 iterations on 900,002 vertices, 1e-10 did).  This path
// takes the same decisions as the binary32 one and carries every
// continuous quantity as an unevaluated pair hi + lo of binary32s:
//  * x*scale = A + a1 + a2 + a3 exactly (A an integer): for a power-of-two
//    scale the vertex's binary32 triple scaled, otherwise the product of
//    the vertex and scale triples to ~2^-70 relative;
//  * dx0 = a - (3f + G)/3 (f, G from the decision) and every slot's offset
//    K = m/3 are anchored: hi on the 2^-21 grid, so the hi part of d =
//    dx0 - K is exact and only the lo parts round (~2^-46); d is then
//    renormalised (|lo| <= ulp(hi)/2), which keeps the cross terms 2 hi lo
//    of |d|^2 small enough to sum to ~2^-46;
//  * attn = 2 - |d|^2, attn^4, grad . d and their product with error-free
//    transforms (fma-exact products, two-sums; the running 2 - dx^2 - dy^2
//    - dz^2 uses fast two-sums, exact whenever attn > 0), two slots at a
//    time in paired binary32 lanes;
//  * the contributions, the division by 103 and the octave's
//    (noise + 1) * 0.5 * strength * radius term are summed in pairs; the
//    running sum over octaves is renormalised after every octave, so a
//    vertex gives the same bits whether its octaves run in one launch or
//    one launch each.

__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// Knuth's two-sum per lane: s + e == a + b exactly.
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2 &s, float2 &e)
{
    s = add2(a, b);
    const float2 bb = sub2(s, a);
    e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}

__device__ __forceinline__ void two_sum1(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Anchored thirds m/3, m = 0..6: hi = rint(m 2^21 / 3) 2^-21, lo = m/3 - hi
// (+-1/(3 2^21) or 0).
constexpr float ANC = 6.0f;                         // (v + 6) - 6 rounds v in [-2, 2) to the 2^-21 grid
constexpr float T1H = 699051.0f / 2097152.0f;       // 1/3
constexpr float T2H = 1398101.0f / 2097152.0f;      // 2/3
constexpr float T4H = 2796203.0f / 2097152.0f;      // 4/3
constexpr float T5H = 3495253.0f / 2097152.0f;      // 5/3
constexpr float C3L = (float)(1.0 / (3.0 * 2097152.0));   // 2^-21 / 3: |lo| of the thirds above
constexpr float C3L2 = 2.0f * C3L;

// Anchored m/3 for an integer m (|m| < 2^9): hi on the 2^-21 grid, lo.
__device__ __forceinline__ void anchor_third(int m, float &H, float &L)
{
    const int N = m * 2097152;
    const int q = N >= 0 ? (N + 1) / 3 : -((1 - N) / 3);
    H = __fmul_rn((float)q, 1.0f / 2097152.0f);
    L = __fmul_rn((float)(N - 3 * q), C3L);
}

// Pair case table of a block: entry i (as s_extra) is four float4s: the two
// extra points' offsets e + (ex + ey + ez)/3 anchored, hi parts
// (E0x, E0y, E0z, E1x), (E1y, E1z, case word, 0), doubled lo parts
// (E0x, E0y, E0z, E1x), (E1y, E1z, 0, 0).
__shared__ float4 s_extra_p[4 * 192];

__device__ __forceinline__ void anchored_offsets(uint32_t w, float *H, float *L)
{
#pragma unroll
    for (int p = 0; p < 2; ++p) {
        const int ox = word_offset(w, 3 * p), oy = word_offset(w, 3 * p + 1), oz = word_offset(w, 3 * p + 2);
        const int t = ox + oy + oz;
        anchor_third(3 * ox + t, H[3 * p], L[3 * p]);
        anchor_third(3 * oy + t, H[3 * p + 1], L[3 * p + 1]);
        anchor_third(3 * oz + t, H[3 * p + 2], L[3 * p + 2]);
    }
}

__device__ __forceinline__ void init_extra_table_pair()
{
    for (int i = threadIdx.x; i < 192; i += blockDim.x) {
        const uint32_t w = i < 64 ? octa_case(i) : tetra_case(i - 64);
        float H[6], L[6];
        anchored_offsets(w, H, L);
        s_extra_p[4 * i] = make_float4(H[0], H[1], H[2], H[3]);
        s_extra_p[4 * i + 1] = make_float4(H[4], H[5], __uint_as_float(w), 0.0f);
        s_extra_p[4 * i + 2] = make_float4(2.0f * L[0], 2.0f * L[1], 2.0f * L[2], 2.0f * L[3]);
        s_extra_p[4 * i + 3] = make_float4(2.0f * L[4], 2.0f * L[5], 0.0f, 0.0f);
    }
}

// d = dx0 - K for one axis of two slots, from the anchored dx0 (hi X0H,
// doubled lo X0L2) and offsets (K, doubled lo KL2): the hi part dx0 - K is
// exact (both on the 2^-21 grid); then renormalised by a fast two-sum
// (|hi| >= 2^-21 > |lo| or hi = 0), H + L2/2 == d with |L2/2| <=
// ulp(H)/2.  L2 = 2 lo (exact: twice the fast two-sum's exact error).
// Without NORM the anchored pair is used as it is (|lo| up to 2^-20): the
// cross terms then carry ~2^-42 of error, which octaves of small amplitude
// can afford (see noise_pair).
template <bool NORM>
__device__ __forceinline__ void slot_disp(float X0H, float X0L2, float2 K, float2 KL2, float2 &H, float2 &L2)
{
    const float2 h0 = sub2(f2(X0H, X0H), K);
    const float2 l2 = sub2(f2(X0L2, X0L2), KL2);
    if (NORM) {
        H = fma2(f2(0.5f, 0.5f), l2, h0);
        L2 = fma2(f2(-2.0f, -2.0f), sub2(H, h0), l2);
    } else {
        H = h0;
        L2 = l2;
    }
}

// Two lattice contributions (slots a, b in the lanes) in pair arithmetic,
// added to the pair accumulator (AH, AL).  X0H, X0L2: the anchored dx0 (hi,
// 2 lo); KX/KXL2 the slots' anchored offsets (hi, 2 lo); ON 1/0 masks.
template <bool NORM>
__device__ __forceinline__ void contrib2_pair(uint32_t wa, uint32_t wb, float X0H, float X0L2, float Y0H, float Y0L2,
                                              float Z0H, float Z0L2, float2 KX, float2 KXL2, float2 KY, float2 KYL2,
                                              float2 KZ, float2 KZL2, float2 ON, float2 &AH, float2 &AL)
{
    float2 Xh, X2, Yh, Y2, Zh, Z2;
    slot_disp<NORM>(X0H, X0L2, KX, KXL2, Xh, X2);
    slot_disp<NORM>(Y0H, Y0L2, KY, KYL2, Yh, Y2);
    slot_disp<NORM>(Z0H, Z0L2, KZ, KZL2, Zh, Z2);
    // attn = 2 - |d|^2: squares of the hi parts exact as p + pe, plus the
    // cross terms 2 hi lo
    const float2 px = mul2(Xh, Xh), py = mul2(Yh, Yh), pz = mul2(Zh, Zh);
    const float2 pxe = fma2(Xh, Xh, f2(-px.x, -px.y)), pye = fma2(Yh, Yh, f2(-py.x, -py.y)),
                 pze = fma2(Zh, Zh, f2(-pz.x, -pz.y));
    float2 L = add2(pxe, add2(pye, pze));
    L = fma2(Xh, X2, L);
    L = fma2(Yh, Y2, L);
    L = fma2(Zh, Z2, L);
    const float2 two = f2(2.0f, 2.0f);
    const float2 r1 = sub2(two, px), r2 = sub2(r1, py), r3 = sub2(r2, pz);
    const float2 e1 = sub2(sub2(two, r1), px), e2 = sub2(sub2(r1, r2), py), e3 = sub2(sub2(r2, r3), pz);
    const float2 al = sub2(add2(add2(e1, e2), e3), L);
    // only attn > 0 counts, and only in the region (ah = 0 zeroes the rest)
    const float2 ah = mul2(f2(fmaxf(r3.x, 0.0f), fmaxf(r3.y, 0.0f)), ON);
    // attn^2, attn^4 as pairs
    const float2 h2 = mul2(ah, ah);
    float2 l2 = fma2(ah, ah, f2(-h2.x, -h2.y));
    l2 = fma2(add2(ah, ah), al, l2);
    const float2 h4 = mul2(h2, h2);
    float2 l4 = fma2(h2, h2, f2(-h4.x, -h4.y));
    l4 = fma2(add2(h2, h2), l2, l4);
    // grad . d as a pair (dh, dl), times DSC (see below)
    const float4 ga = s_grad[wa & 31u], gb = s_grad[wb & 31u];
    const float2 gx = f2(ga.x, gb.x), gy = f2(ga.y, gb.y), gz = f2(ga.z, gb.z);
    float2 dh, dl;
    if (NORM) {
        // products exact as q + qe, summed with two-sums; DSC = 1
        const float2 qx = mul2(gx, Xh), qy = mul2(gy, Yh), qz = mul2(gz, Zh);
        const float2 qxe = fma2(gx, Xh, f2(-qx.x, -qx.y)), qye = fma2(gy, Yh, f2(-qy.x, -qy.y)),
                     qze = fma2(gz, Zh, f2(-qz.x, -qz.y));
        float2 s1, t1, t2;
        two_sum2(qx, qy, s1, t1);
        two_sum2(s1, qz, dh, t2);
        const float2 gl = fma2(gx, X2, fma2(gy, Y2, mul2(gz, Z2)));     // 2 (grad . lo)
        dl = fma2(f2(0.5f, 0.5f), gl, add2(add2(add2(qxe, qye), qze), add2(t1, t2)));
    } else {
        // hi parts on the 2^-21 grid (|d| < sqrt 2 wherever attn > 0): with
        // g_i = s_i (4 + 7 [i == a]), grad . hi = 4 (U + V) exactly, U =
        // sum s_i hi_i + 2 s_a hi_a (|U| < 8 on the grid: exact), V =
        // -s_a hi_a / 4; the lo parts' product in binary32.  DSC = 1/4.
        const uint4 sa = s_gsign[wa & 31u], sb = s_gsign[wb & 31u];
        const float2 sx = f2(__uint_as_float(__float_as_uint(Xh.x) ^ sa.x), __uint_as_float(__float_as_uint(Xh.y) ^ sb.x));
        const float2 sy = f2(__uint_as_float(__float_as_uint(Yh.x) ^ sa.y), __uint_as_float(__float_as_uint(Yh.y) ^ sb.y));
        const float2 sz = f2(__uint_as_float(__float_as_uint(Zh.x) ^ sa.z), __uint_as_float(__float_as_uint(Zh.y) ^ sb.z));
        const float2 s_a = f2(sa.w == 0u ? sx.x : (sa.w == 1u ? sy.x : sz.x), sb.w == 0u ? sx.y : (sb.w == 1u ? sy.y : sz.y));
        const float2 U = fma2(f2(2.0f, 2.0f), s_a, add2(add2(sx, sy), sz));
        const float2 V = mul2(f2(-0.25f, -0.25f), s_a);
        float2 e;
        two_sum2(U, V, dh, e);
        const float2 gl = fma2(gx, X2, fma2(gy, Y2, mul2(gz, Z2)));     // 2 (grad . lo)
        dl = fma2(f2(0.125f, 0.125f), gl, e);
    }
    // attn^4 * (grad . d)
    const float2 ch = mul2(h4, dh);
    float2 cl = fma2(h4, dh, f2(-ch.x, -ch.y));
    cl = fma2(h4, dl, fma2(l4, dh, cl));
    float2 s, e;
    two_sum2(AH, ch, s, e);
    AH = s;
    AL = add2(AL, add2(e, cl));
}

// x*scale = A + a1 + a2 + a3 for one axis: x = x1 + x2 + x3 and scale =
// s1 + s2 + s3 exact binary32 triples; |x*scale| < 2^22 for A to be exact.
__device__ __forceinline__ void coord_split(float x1, float x2, float x3, float s1, float s2, float s3, bool pow2,
                                            float &A, float &a1, float &a2, float &a3)
{
    const float p = __fmul_rn(x1, s1);
    A = __fsub_rn(__fadd_rn(p, MAGIC), MAGIC);
    a1 = __fsub_rn(p, A);
    if (pow2) {                       // scale = s1, a power of two: exact scaling
        a2 = __fmul_rn(x2, s1);
        a3 = __fmul_rn(x3, s1);
        return;
    }
    const float e11 = __fmaf_rn(x1, s1, -p);
    const float p12 = __fmul_rn(x1, s2), e12 = __fmaf_rn(x1, s2, -p12);
    const float p21 = __fmul_rn(x2, s1), e21 = __fmaf_rn(x2, s1, -p21);
    const float q = __fmaf_rn(x1, s3, __fmaf_rn(x2, s2, __fmul_rn(x3, s1)));
    float b, c, b2, c2;
    two_sum1(p12, p21, b, c);
    two_sum1(b, e11, b2, c2);
    a2 = b2;
    a3 = __fadd_rn(__fadd_rn(c, c2), __fadd_rn(__fadd_rn(e12, e21), q));
}

// Anchor a pair (h, l) with h in [-2, 2): hi on the 2^-21 grid, lo.
__device__ __forceinline__ void anchor_pair(float h, float l, float &H, float &L)
{
    H = __fsub_rn(__fadd_rn(h, ANC), ANC);
    L = __fadd_rn(__fsub_rn(h, H), l);
}

// A binary64 value in [-2, 2) anchored (binary64 decision path).
__device__ __forceinline__ void anchor_f64(double d, float &H, float &L)
{
    const float h = __double2float_rn(d);
    anchor_pair(h, __double2float_rn(__dsub_rn(d, (double)h)), H, L);
}

// Per-octave constants of the pair path.
struct OctP {
    float s1, s2, s3;     // scale as a binary32 triple
    float amph, ampl;     // 0.5 * strength * radius as a pair
    double s;             // scale (binary64 decision path)
    bool norm;            // renormalise the displacements (noise_pair<true>)
};

// noise3d(x * s) as a pair (vh, vl) of 103 * noise, for one vertex and
// octave.  x1..z3: the vertex's binary32 triples (x1 + x2 + x3 == x).
//
// A lane evaluates at most 8 lattice points: its region's fixed corners
// (tetrahedra: the corner at 0 or 1 and its three neighbours; octahedron:
// the six mixed corners) and the two extra points.  The corners are
// assigned to lanes per region (selects), so a warp runs four slot pairs:
// X1..X4 (every region), X5/X6 (octahedron only) and the extra points.
//
// NORM: renormalise the slots' displacements.  Without it the value carries
// up to ~1.5e-13 * (0.5 strength radius) of extra error, so the planet
// paths skip it only for octaves whose amplitude is at most 1/8 of the
// first one's (|error| <= 2e-14 of a field whose range is ~2 amp_0).
template <bool NORM>
__device__ __forceinline__ void noise_pair(float x1, float x2, float x3, float y1, float y2, float y3, float z1,
                                           float z2, float z3, const OctP &O, bool pow2, uint32_t lb, unsigned &nfb,
                                           float &vh, float &vl)
{
    float Ax, ax1, ax2, ax3, Ay, ay1, ay2, ay3, Az, az1, az2, az3;
    coord_split(x1, x2, x3, O.s1, O.s2, O.s3, pow2, Ax, ax1, ax2, ax3);
    coord_split(y1, y2, y3, O.s1, O.s2, O.s3, pow2, Ay, ay1, ay2, ay3);
    coord_split(z1, z2, z3, O.s1, O.s2, O.s3, pow2, Az, az1, az2, az3);
    const float ax = __fadd_rn(ax1, ax2), ay = __fadd_rn(ay1, ay2), az = __fadd_rn(az1, az2);
    const float big = fmaxf(fabsf(__fadd_rn(Ax, ax)), fmaxf(fabsf(__fadd_rn(Ay, ay)), fabsf(__fadd_rn(Az, az))));
    Core o;
    int region, xb7, yb7, zb7;
    uint32_t ew;
    float X0H, X0L2, Y0H, Y0L2, Z0H, Z0L2;
    float EH[6], EL2[6];
    if (decide_core(Ax, ax, Ay, ay, Az, az, big, o)) {
        region = o.region;
        xb7 = o.xb7; yb7 = o.yb7; zb7 = o.zb7;
        // the fraction anchored, then dx0 = a - (f + G/3)
        float GH, GL;
        anchor_third((int)o.G, GH, GL);
        const float GL2 = __fmul_rn(2.0f, GL);
        const float FXH = __fsub_rn(__fadd_rn(ax, ANC), ANC), FYH = __fsub_rn(__fadd_rn(ay, ANC), ANC),
                    FZH = __fsub_rn(__fadd_rn(az, ANC), ANC);
        const float FXL = __fadd_rn(__fadd_rn(__fsub_rn(ax1, FXH), ax2), ax3);
        const float FYL = __fadd_rn(__fadd_rn(__fsub_rn(ay1, FYH), ay2), ay3);
        const float FZL = __fadd_rn(__fadd_rn(__fsub_rn(az1, FZH), az2), az3);
        X0H = __fsub_rn(FXH, __fadd_rn(o.fx, GH));
        Y0H = __fsub_rn(FYH, __fadd_rn(o.fy, GH));
        Z0H = __fsub_rn(FZH, __fadd_rn(o.fz, GH));
        X0L2 = __fmaf_rn(2.0f, FXL, -GL2);
        Y0L2 = __fmaf_rn(2.0f, FYL, -GL2);
        Z0L2 = __fmaf_rn(2.0f, FZL, -GL2);
        const float4 *t = s_extra_p + 4 * o.ci;
        const float4 t0 = t[0], t1 = t[1], t2 = t[2], t3 = t[3];
        EH[0] = t0.x; EH[1] = t0.y; EH[2] = t0.z; EH[3] = t0.w; EH[4] = t1.x; EH[5] = t1.y;
        ew = __float_as_uint(t1.z);
        EL2[0] = t2.x; EL2[1] = t2.y; EL2[2] = t2.z; EL2[3] = t2.w; EL2[4] = t3.x; EL2[5] = t3.y;
    } else {
        // the vertex as binary64 (the triple's sum is exact)
        const double X = (double)x1 + (double)x2 + (double)x3, Y = (double)y1 + (double)y2 + (double)y3,
                     Z = (double)z1 + (double)z2 + (double)z3;
        const Cell c = decide_f64(X, Y, Z, O.s);
        ++nfb;
        region = c.D.region;
        xb7 = c.xb7; yb7 = c.yb7; zb7 = c.zb7;
        float L;
        anchor_f64(c.dxd, X0H, L);
        X0L2 = __fmul_rn(2.0f, L);
        anchor_f64(c.dyd, Y0H, L);
        Y0L2 = __fmul_rn(2.0f, L);
        anchor_f64(c.dzd, Z0H, L);
        Z0L2 = __fmul_rn(2.0f, L);
        ew = c.D.w;
        float EL[6];
        anchored_offsets(ew, EH, EL);
        for (int k = 0; k < 6; ++k) EL2[k] = __fmul_rn(2.0f, EL[k]);
    }
    const bool r1 = region == 1, r2 = region == 2;
    uint32_t h0 = lk(lb, xb7), h1 = lk(lb, xb7 + 128);
    uint32_t h00 = lk(lb, (int)h0 + yb7), h01 = lk(lb, (int)h0 + yb7 + 128);
    uint32_t h10 = lk(lb, (int)h1 + yb7), h11 = lk(lb, (int)h1 + yb7 + 128);
    const int zo0 = zb7, zo1 = zb7 + 128;
    const uint32_t w0 = lk(lb, r1 ? (int)h11 + zo1 : (int)h00 + zo0);
    const uint32_t w100 = lk(lb, (int)h10 + zo0), w010 = lk(lb, (int)h01 + zo0), w001 = lk(lb, (int)h00 + zo1);
    const uint32_t w110 = lk(lb, (int)h11 + zo0), w101 = lk(lb, (int)h10 + zo1), w011 = lk(lb, (int)h01 + zo1);
    const int xm = xb7 - 128, ym = yb7 - 128, zm = zb7 - 128;
    const uint32_t we0 = lk(lb, (int)lk(lb, (int)lk(lb, xm + word_step(ew, 0)) + ym + word_step(ew, 1)) + zm + word_step(ew, 2));
    const uint32_t we1 = lk(lb, (int)lk(lb, (int)lk(lb, xm + word_step(ew, 3)) + ym + word_step(ew, 4)) + zm + word_step(ew, 5));
    // fixed corners per lane (offsets o + (ox + oy + oz)/3 in thirds: A1 =
    // (1,0,0) -> (4,1,1)/3, A2 (1,4,1)/3, A3 (1,1,4)/3, B1 = (1,1,0) ->
    // (5,5,2)/3, B2 (5,2,5)/3, B3 (2,5,5)/3; corner 0: (0,0,0) or (2,2,2));
    // A-corners' anchored lo is -C3L, B-corners' +C3L, the corner's 0
    const float k0 = r1 ? 2.0f : 0.0f;
    const float nL2 = -C3L2, pL2 = C3L2;
    //   X1: r2 ? A1 : corner 0       X2: r2 ? A2 : (r1 ? B1 : A1)
    //   X3: r2 ? A3 : (r1 ? B2 : A2) X4: r2 ? B1 : (r1 ? B3 : A3)
    //   X5: B2, X6: B3 (octahedron only)
    const uint32_t wX1 = r2 ? w100 : w0, wX2 = r2 ? w010 : (r1 ? w110 : w100);
    const uint32_t wX3 = r2 ? w001 : (r1 ? w101 : w010), wX4 = r2 ? w110 : (r1 ? w011 : w001);
    const float2 X1X2x = f2(r2 ? T4H : k0, r2 ? T1H : (r1 ? T5H : T4H));
    const float2 X1X2y = f2(r2 ? T1H : k0, r2 ? T4H : (r1 ? T5H : T1H));
    const float2 X1X2z = f2(r2 ? T1H : k0, r2 ? T1H : (r1 ? T2H : T1H));
    const float2 X1X2l = f2(r2 ? nL2 : 0.0f, r1 ? pL2 : nL2);
    const float2 X3X4x = f2(r2 ? T1H : (r1 ? T5H : T1H), r2 ? T5H : (r1 ? T2H : T1H));
    const float2 X3X4y = f2(r2 ? T1H : (r1 ? T2H : T4H), r2 ? T5H : (r1 ? T5H : T1H));
    const float2 X3X4z = f2(r2 ? T4H : (r1 ? T5H : T1H), r2 ? T2H : (r1 ? T5H : T4H));
    const float2 X3X4l = f2(r1 ? pL2 : nL2, (r1 || r2) ? pL2 : nL2);
    const float fr2 = r2 ? 1.0f : 0.0f;
    float2 AH = f2(0.0f, 0.0f), AL = f2(0.0f, 0.0f);
    contrib2_pair<NORM>(wX1, wX2, X0H, X0L2, Y0H, Y0L2, Z0H, Z0L2, X1X2x, X1X2l, X1X2y, X1X2l, X1X2z, X1X2l, f2(1.0f, 1.0f),
                  AH, AL);
    contrib2_pair<NORM>(wX3, wX4, X0H, X0L2, Y0H, Y0L2, Z0H, Z0L2, X3X4x, X3X4l, X3X4y, X3X4l, X3X4z, X3X4l, f2(1.0f, 1.0f),
                  AH, AL);
    contrib2_pair<NORM>(w101, w011, X0H, X0L2, Y0H, Y0L2, Z0H, Z0L2, f2(T5H, T2H), f2(pL2, pL2), f2(T2H, T5H), f2(pL2, pL2),
                  f2(T5H, T5H), f2(pL2, pL2), f2(fr2, fr2), AH, AL);
    contrib2_pair<NORM>(we0, we1, X0H, X0L2, Y0H, Y0L2, Z0H, Z0L2, f2(EH[0], EH[3]), f2(EL2[0], EL2[3]), f2(EH[1], EH[4]),
                  f2(EL2[1], EL2[4]), f2(EH[2], EH[5]), f2(EL2[2], EL2[5]), f2(1.0f, 1.0f), AH, AL);
    float e;
    two_sum1(AH.x, AH.y, vh, e);
    vl = __fadd_rn(e, __fadd_rn(AL.x, AL.y));
    if (!NORM) {                      // the dot products carried a factor 1/4 (exact)
        vh = __fmul_rn(vh, 4.0f);
        vl = __fmul_rn(vl, 4.0f);
    }
}

// The octave's term (v/103 + 1) * amp added to the running pair (rh, rl),
// then renormalised (|rl| <= ulp(rh)/2).
__device__ __forceinline__ void octave_accumulate(float vh, float vl, float amph, float ampl, float &rh, float &rl)
{
    constexpr float R103 = 1.0f / 103.0f;
    const float wq = __fmul_rn(vh, R103);
    const float rem = __fmaf_rn(-wq, 103.0f, vh);                 // exact
    const float wl = __fmul_rn(__fadd_rn(rem, vl), R103);
    const float s = __fadd_rn(1.0f, wq);                          // |wq| <= 1: fast two-sum
    const float lo = __fadd_rn(__fadd_rn(__fsub_rn(1.0f, s), wq), wl);
    const float th = __fmul_rn(s, amph);
    float tl = __fmaf_rn(s, amph, -th);
    tl = __fmaf_rn(s, ampl, __fmaf_rn(lo, amph, tl));
    float sh, se;
    two_sum1(rh, th, sh, se);
    const float sl = __fadd_rn(rl, __fadd_rn(se, tl));
    rh = __fadd_rn(sh, sl);
    rl = __fsub_rn(sl, __fsub_rn(rh, sh));
}

// Split a binary64 into three binary32s x1 + x2 + x3 == v exactly, with
// integer operations (GB300's binary64 pipe is narrow): x1 = the top 24
// significant bits, x2 = the next 23 as an integer times 2^(e-46), x3 = the
// last 6 times 2^(e-52).  Needs 2^-74 <= |v| < 2^128 (the scales stay
// normal binary32s); v = 0 gives zeros.  Other magnitudes give x1 =
// (float)v and zeros: outside what the planet paths use (unit or
// radius-scaled vertices), and such a coordinate only loses its low bits.
__device__ __forceinline__ void split3_f64(double v, float &x1, float &x2, float &x3)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const uint32_t hw = (uint32_t)(b >> 32), lw = (uint32_t)b;
    const int e = (int)((hw >> 20) & 0x7FF) - 1023;
    const uint32_t sign = hw & 0x80000000u;
    if (e < -74 || e > 127) {
        x1 = (float)v;
        x2 = 0.0f;
        x3 = 0.0f;
        return;
    }
    // top 24 bits: the implicit one and 23 fraction bits (bits 51-29)
    x1 = __uint_as_float(sign | ((uint32_t)(e + 127) << 23) | ((hw & 0xFFFFFu) << 3) | (lw >> 29));
    // next 23 bits (28-6) and last 6 (5-0), as exact integers scaled by 2^(e-46) and 2^(e-52)
    const uint32_t m2 = (lw >> 6) & 0x7FFFFFu, m3 = lw & 0x3Fu;
    const float i2 = __fsub_rn(__uint_as_float(0x4B000000u | m2), 8388608.0f);
    const float i3 = __fsub_rn(__uint_as_float(0x4B000000u | m3), 8388608.0f);
    const float t2 = __fmul_rn(i2, __uint_as_float((uint32_t)(e + 81) << 23));
    const float t3 = __fmul_rn(i3, __uint_as_float((uint32_t)(e + 75) << 23));
    x2 = __uint_as_float(__float_as_uint(t2) | sign);
    x3 = __uint_as_float(__float_as_uint(t3) | sign);
}

// Ordered-key transform: unsigned comparisons of keys follow float order.
__device__ __forceinline__ uint32_t fkey(float f)
{
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b ^ 0x80000000u);
}

// Ordered 64-bit key of a normalised pair: unsigned key order = value order.
__device__ __forceinline__ unsigned long long pair_key(float h, float l)
{
    return ((unsigned long long)fkey(h) << 32) | (unsigned long long)fkey(l);
}

__device__ __forceinline__ uint32_t lane_base(const uint32_t *T)
{
    return (uint32_t)__cvta_generic_to_shared(T) + ((threadIdx.x & 31u) << 2);
}

__global__ void __launch_bounds__(256) fbm_kernel(const double *__restrict__ xyz, int64_t n,
                                                  const int32_t *__restrict__ perm,
                                                  const int32_t *__restrict__ pgi, FbmParams P,
                                                  double *__restrict__ out64, float *__restrict__ out32,
                                                  int accumulate, unsigned long long *nfb_out)
{
    extern __shared__ __align__(16) uint32_t smem[];
    build_table(smem, perm, pgi);
    init_extra_table();
    __syncthreads();
    const uint32_t lb = lane_base(smem);
    unsigned nfb = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double X = xyz[3 * i], Y = xyz[3 * i + 1], Z = xyz[3 * i + 2];
        float xh, xl, yh, yl, zh, zl;
        split_f64(X, xh, xl);
        split_f64(Y, yh, yl);
        split_f64(Z, zh, zl);
        float acc = 0.0f;
        for (int o = 0; o < P.n_oct; ++o) {
            float v = noise_raw<false>(xh, xl, yh, yl, zh, zl, P.s_hi[o], P.s_lo[o], X, Y, Z, P.s[o], lb,
                                       nfb, nullptr, nullptr);
            // (noise + 1) * 0.5 * strength * radius, noise = v / 103
            acc += fmaf(v, P.amp[o] * (1.0f / 103.0f), P.amp[o]);
        }
        if (out64) out64[i] = accumulate ? out64[i] + (double)acc : (double)acc;
        if (out32) out32[i] = accumulate ? out32[i] + acc : acc;
    }
    if (nfb_out) {
        unsigned tot = __reduce_add_sync(0xFFFFFFFFu, nfb);
        if ((threadIdx.x & 31) == 0 && tot) atomicAdd(nfb_out, (unsigned long long)tot);
    }
}

__global__ void __launch_bounds__(256) trace_kernel(const double *__restrict__ xyz, int64_t n,
                                                    const int32_t *__restrict__ perm,
                                                    const int32_t *__restrict__ pgi, double s,
                                                    float *__restrict__ value, int32_t *__restrict__ trace,
                                                    int32_t *__restrict__ slots,
                                                    unsigned long long *nfb_out)
{
    extern __shared__ __align__(16) uint32_t smem[];
    build_table(smem, perm, pgi);
    init_extra_table();
    __syncthreads();
    const uint32_t lb = lane_base(smem);
    float sh, sl;
    split_f64(s, sh, sl);
    unsigned nfb = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double X = xyz[3 * i], Y = xyz[3 * i + 1], Z = xyz[3 * i + 2];
        float xh, xl, yh, yl, zh, zl;
        split_f64(X, xh, xl);
        split_f64(Y, yh, yl);
        split_f64(Z, zh, zl);
        int32_t tr[10], s9[45];
        float v = noise_raw<true>(xh, xl, yh, yl, zh, zl, sh, sl, X, Y, Z, s, lb, nfb, tr, s9);
        value[i] = v * (1.0f / 103.0f);
        if (trace)
            for (int k = 0; k < 10; ++k) trace[10 * i + k] = tr[k];
        if (slots)
            for (int k = 0; k < 45; ++k) slots[45 * i + k] = s9[k];
    }
    if (nfb_out) {
        unsigned tot = __reduce_add_sync(0xFFFFFFFFu, nfb);
        if ((threadIdx.x & 31) == 0 && tot) atomicAdd(nfb_out, (unsigned long long)tot);
    }
}


constexpr int CHUNK = 2048;   // vertices per work item of the batched kernel

__device__ __forceinline__ int chunk_planet(const nx_fbm_planet *P, int np, int c)
{
    int lo = 0, hi = np - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (P[mid].chunk0 <= c) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Chunk ranges of a batched launch: block b takes chunks [first[b],
// first[b + 1]) in order, the ranges cut so that each block gets an equal
// share of the estimated cost (vertices x octaves, renormalised octaves
// weighted 9/8).
constexpr int FBM_SPLIT_MAX = 2048;
struct FbmSplit {
    int first[FBM_SPLIT_MAX + 1];
};

// Fold the ordered keys (kmn, kmx) of the block's sums of planet P into its
// min/max (a block barrier; the whole block calls it).
__device__ __forceinline__ void fold_minmax(const nx_fbm_planet &P, unsigned long long kmn, unsigned long long kmx,
                                            unsigned long long (*s_mm)[8])
{
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long a = __shfl_xor_sync(0xFFFFFFFFu, kmn, o);
        const unsigned long long b = __shfl_xor_sync(0xFFFFFFFFu, kmx, o);
        kmn = a < kmn ? a : kmn;
        kmx = b > kmx ? b : kmx;
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { s_mm[0][w] = kmn; s_mm[1][w] = kmx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long a0 = s_mm[0][0], a1 = s_mm[1][0];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
            a0 = s_mm[0][k] < a0 ? s_mm[0][k] : a0;
            a1 = s_mm[1][k] > a1 ? s_mm[1][k] : a1;
        }
        atomicMin(&P.minmax[0], a0);
        atomicMax(&P.minmax[1], a1);
    }
    __syncthreads();
}

// Many planets in one persistent launch: work items are chunks of CHUNK
// vertices of one planet; each block walks its contiguous range of chunks
// (so it meets few planets), rebuilding its shared table when the planet
// changes.  Sums are pairs (pair path above); the ordered keys of a block's
// sums of a planet are folded into the planet's min/max once, when the
// block leaves the planet (for the rescale to metres that follows).
__global__ void __launch_bounds__(256) fbm_batch_kernel(const nx_fbm_planet *__restrict__ planets, int np,
                                                        const __grid_constant__ FbmSplit split,
                                                        unsigned long long *nfb_out)
{
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ unsigned long long s_mm[2][8];
    init_extra_table_pair();
    init_grad_table();
    __syncthreads();
    const uint32_t lb = lane_base(smem);
    const int c0 = split.first[blockIdx.x], c1 = split.first[blockIdx.x + 1];
    int cur = -1;
    unsigned nfb = 0;
    unsigned long long kmn = ~0ull, kmx = 0ull;
    for (int c = c0; c < c1; ++c) {
        int p = cur < 0 ? chunk_planet(planets, np, c) : cur;
        while (p + 1 < np && planets[p + 1].chunk0 <= c) ++p;
        if (p != cur) {
            if (cur >= 0 && planets[cur].minmax) fold_minmax(planets[cur], kmn, kmx, s_mm);
            kmn = ~0ull;
            kmx = 0ull;
            __syncthreads();
            build_table_pair(smem, planets[p].perm, planets[p].pgi);
            __syncthreads();
            cur = p;
        }
        const nx_fbm_planet &P = planets[p];
        const int64_t base = (int64_t)(c - P.chunk0) * CHUNK;
        const bool pow2 = P.pow2 != 0;
        for (int64_t i = base + threadIdx.x; i < base + CHUNK && i < P.n; i += blockDim.x) {
            const double X = P.xyz[3 * i], Y = P.xyz[3 * i + 1], Z = P.xyz[3 * i + 2];
            float x1, x2, x3, y1, y2, y3, z1, z2, z3;
            split3_f64(X, x1, x2, x3);
            split3_f64(Y, y1, y2, y3);
            split3_f64(Z, z1, z2, z3);
            float rh = 0.0f, rl = 0.0f;
            for (int o = 0; o < P.n_octaves; ++o) {
                OctP O;
                O.s1 = P.s1[o]; O.s2 = P.s2[o]; O.s3 = P.s3[o];
                O.amph = P.amp_hi[o]; O.ampl = P.amp_lo[o]; O.s = P.s[o];
                float vh, vl;
                if ((P.norm_mask >> o) & 1u)
                    noise_pair<true>(x1, x2, x3, y1, y2, y3, z1, z2, z3, O, pow2, lb, nfb, vh, vl);
                else
                    noise_pair<false>(x1, x2, x3, y1, y2, y3, z1, z2, z3, O, pow2, lb, nfb, vh, vl);
                octave_accumulate(vh, vl, O.amph, O.ampl, rh, rl);
            }
            reinterpret_cast<float2 *>(P.out)[i] = make_float2(rh, rl);
            const unsigned long long k = pair_key(rh, rl);
            kmn = k < kmn ? k : kmn;
            kmx = k > kmx ? k : kmx;
        }
    }
    if (cur >= 0 && planets[cur].minmax) fold_minmax(planets[cur], kmn, kmx, s_mm);
    if (nfb_out) {
        unsigned tot = __reduce_add_sync(0xFFFFFFFFu, nfb);
        if ((threadIdx.x & 31) == 0 && tot) atomicAdd(nfb_out, (unsigned long long)tot);
    }
}

// Per-octave constants of a single-planet pair launch.
struct FbmPairParams {
    int n_oct;
    int pow2;
    uint32_t norm_mask;   // bit o: octave o renormalises its displacements
    float s1[NX_MAX_OCTAVES], s2[NX_MAX_OCTAVES], s3[NX_MAX_OCTAVES];
    float amph[NX_MAX_OCTAVES], ampl[NX_MAX_OCTAVES];
    double s[NX_MAX_OCTAVES];
};

// One planet, the pair path: the octaves of P (any subset of a planet's
// octaves: the plain path launches one per octave, accumulate = 1 after
// the first) added to the running pair sums in out2 (float2 per vertex),
// and/or written as binary64 (out64, = hi + lo exactly; accumulate adds to
// it).  minmax (optional): ordered keys of the resulting pair sums.
__global__ void __launch_bounds__(256) fbm_pair_kernel(const double *__restrict__ xyz, int64_t n,
                                                       const int32_t *__restrict__ perm,
                                                       const int32_t *__restrict__ pgi, FbmPairParams P,
                                                       float2 *__restrict__ out2, double *__restrict__ out64,
                                                       int accumulate, unsigned long long *minmax,
                                                       unsigned long long *nfb_out)
{
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ unsigned long long s_mm[2][8];
    build_table_pair(smem, perm, pgi);
    init_extra_table_pair();
    init_grad_table();
    __syncthreads();
    const uint32_t lb = lane_base(smem);
    unsigned nfb = 0;
    unsigned long long kmn = ~0ull, kmx = 0ull;
    const bool pow2 = P.pow2 != 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double X = xyz[3 * i], Y = xyz[3 * i + 1], Z = xyz[3 * i + 2];
        float x1, x2, x3, y1, y2, y3, z1, z2, z3;
        split3_f64(X, x1, x2, x3);
        split3_f64(Y, y1, y2, y3);
        split3_f64(Z, z1, z2, z3);
        float rh = 0.0f, rl = 0.0f;
        if (accumulate && out2) {
            const float2 v = out2[i];
            rh = v.x;
            rl = v.y;
        }
        for (int o = 0; o < P.n_oct; ++o) {
            OctP O;
            O.s1 = P.s1[o]; O.s2 = P.s2[o]; O.s3 = P.s3[o];
            O.amph = P.amph[o]; O.ampl = P.ampl[o]; O.s = P.s[o];
            float vh, vl;
            if ((P.norm_mask >> o) & 1u)
                noise_pair<true>(x1, x2, x3, y1, y2, y3, z1, z2, z3, O, pow2, lb, nfb, vh, vl);
            else
                noise_pair<false>(x1, x2, x3, y1, y2, y3, z1, z2, z3, O, pow2, lb, nfb, vh, vl);
            octave_accumulate(vh, vl, O.amph, O.ampl, rh, rl);
        }
        if (out2) out2[i] = make_float2(rh, rl);
        if (out64) {
            const double v = (double)rh + (double)rl;
            out64[i] = (accumulate && !out2) ? out64[i] + v : v;
        }
        const unsigned long long k = pair_key(rh, rl);
        kmn = k < kmn ? k : kmn;
        kmx = k > kmx ? k : kmx;
    }
    if (minmax) {
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long a = __shfl_xor_sync(0xFFFFFFFFu, kmn, o);
            const unsigned long long b = __shfl_xor_sync(0xFFFFFFFFu, kmx, o);
            kmn = a < kmn ? a : kmn;
            kmx = b > kmx ? b : kmx;
        }
        const int w = threadIdx.x >> 5;
        if ((threadIdx.x & 31) == 0) { s_mm[0][w] = kmn; s_mm[1][w] = kmx; }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long a0 = s_mm[0][0], a1 = s_mm[1][0];
            for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
                a0 = s_mm[0][k] < a0 ? s_mm[0][k] : a0;
                a1 = s_mm[1][k] > a1 ? s_mm[1][k] : a1;
            }
            atomicMin(&minmax[0], a0);
            atomicMax(&minmax[1], a1);
        }
    }
    if (nfb_out) {
        unsigned tot = __reduce_add_sync(0xFFFFFFFFu, nfb);
        if ((threadIdx.x & 31) == 0 && tot) atomicAdd(nfb_out, (unsigned long long)tot);
    }
}

int grid_for(int64_t n, int block, const void *kernel, int smem)
{
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
    if (per_sm < 1) per_sm = 1;
    int64_t need = (n + block - 1) / block;
    int64_t g = (int64_t)nx::sm_count() * per_sm;
    if (need < g) g = need;
    return (int)(g < 1 ? 1 : g);
}

bool smem_configured = false;

int configure_smem()
{
    if (smem_configured) return NX_OK;
    NX_CHECK_CUDA(cudaFuncSetAttribute(fbm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TABLE_BYTES));
    NX_CHECK_CUDA(cudaFuncSetAttribute(trace_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TABLE_BYTES));
    NX_CHECK_CUDA(cudaFuncSetAttribute(fbm_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TABLE_BYTES));
    NX_CHECK_CUDA(cudaFuncSetAttribute(fbm_pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TABLE_BYTES));
    smem_configured = true;
    return NX_OK;
}

}  // namespace

namespace nx {
void note_launch(int k);
}

NX_EXPORT int nx_fbm(const double *xyz_dev, int64_t n, const int32_t *perm_dev, const int32_t *pgi_dev,
                     int n_octaves, const double *scale, const double *strength, double radius,
                     double *elev_f64_dev, float *elev_f32_dev, int accumulate,
                     unsigned long long *n_fallback_dev, void *stream)
{
    if (n < 0) return nx::fail(NX_EINVAL, "nx_fbm: n < 0");
    if (n_octaves < 0 || n_octaves > NX_MAX_OCTAVES)
        return nx::fail(NX_EINVAL, "nx_fbm: n_octaves must be in [0, %d]", NX_MAX_OCTAVES);
    if (n == 0) return NX_OK;
    if (!xyz_dev || !perm_dev || !pgi_dev || (n_octaves > 0 && (!scale || !strength)))
        return nx::fail(NX_EINVAL, "nx_fbm: null pointer");
    if (!elev_f64_dev && !elev_f32_dev) return nx::fail(NX_EINVAL, "nx_fbm: no output");
    FbmParams P;
    P.n_oct = n_octaves;
    for (int o = 0; o < n_octaves; ++o) {
        double s = scale[o];
        float hi = (float)s;
        float lo = (float)(s - (double)hi);
        P.s_hi[o] = hi;
        P.s_lo[o] = lo;
        P.s[o] = s;
        P.amp[o] = (float)(0.5 * strength[o] * radius);
    }
    int rc = configure_smem();
    if (rc) return rc;
    int grid = grid_for(n, 256, (const void *)fbm_kernel, TABLE_BYTES);
    fbm_kernel<<<grid, 256, TABLE_BYTES, (cudaStream_t)stream>>>(xyz_dev, n, perm_dev, pgi_dev, P, elev_f64_dev,
                                                                 elev_f32_dev, accumulate, n_fallback_dev);
    NX_CHECK_LAUNCH("fbm_kernel");
    nx::note_launch(1);
    return NX_OK;
}

NX_EXPORT int nx_sample_octaves(const double *xyz_dev, int64_t n, const int32_t *perm_dev,
                                const int32_t *pgi_dev, int n_octaves, double n_init_roughness,
                                double n_init_strength, double n_roughness, double n_persistence,
                                double world_radius, double *elev_f64_dev, float *elev_f32_dev,
                                int accumulate, void *stream)
{
    if (n_octaves < 0 || n_octaves > NX_MAX_OCTAVES)
        return nx::fail(NX_EINVAL, "nx_sample_octaves: n_octaves must be in [0, %d]", NX_MAX_OCTAVES);
    double scale[NX_MAX_OCTAVES], strength[NX_MAX_OCTAVES];
    // terrain.py:35-46: the per-octave arguments, in binary64 as the reference
    double f = n_init_roughness, a = n_init_strength;
    for (int o = 0; o < n_octaves; ++o) {
        scale[o] = f / world_radius;
        strength[o] = a / world_radius;
        f *= n_roughness;
        a *= n_persistence;
    }
    return nx_fbm(xyz_dev, n, perm_dev, pgi_dev, n_octaves, scale, strength, world_radius, elev_f64_dev,
                  elev_f32_dev, accumulate, nullptr, stream);
}

NX_EXPORT int nx_noise3d_trace(const double *xyz_dev, int64_t n, const int32_t *perm_dev,
                               const int32_t *pgi_dev, double scale, float *value_dev, int32_t *trace_dev,
                               int32_t *slots_dev, unsigned long long *n_fallback_dev, void *stream)
{
    if (n < 0) return nx::fail(NX_EINVAL, "nx_noise3d_trace: n < 0");
    if (n == 0) return NX_OK;
    if (!xyz_dev || !perm_dev || !pgi_dev || !value_dev)
        return nx::fail(NX_EINVAL, "nx_noise3d_trace: null pointer");
    int rc = configure_smem();
    if (rc) return rc;
    int grid = grid_for(n, 256, (const void *)trace_kernel, TABLE_BYTES);
    trace_kernel<<<grid, 256, TABLE_BYTES, (cudaStream_t)stream>>>(xyz_dev, n, perm_dev, pgi_dev, scale,
                                                                   value_dev, trace_dev, slots_dev,
                                                                   n_fallback_dev);
    NX_CHECK_LAUNCH("trace_kernel");
    nx::note_launch(1);
    return NX_OK;
}

// scale as an exact triple of binary32s and whether it is a power of two
static void split_scale(double v, float &a, float &b, float &c)
{
    a = (float)v;
    const double r = v - (double)a;      // exact
    b = (float)r;
    c = (float)(r - (double)b);          // exact (the few bits left)
}

static bool is_pow2(double v)
{
    int e = 0;
    return v > 0.0 && std::frexp(v, &e) == 0.5;
}

// Octaves whose displacements are renormalised (bit o): those with
// |0.5 strength radius| >= ref / 8, ref = amp_ref if positive, else the
// largest amplitude among the given octaves.
static uint32_t norm_mask(int n_octaves, const double *strength, double radius, double amp_ref)
{
    double ref = amp_ref;
    if (!(ref > 0.0))
        for (int o = 0; o < n_octaves; ++o) ref = std::fmax(ref, std::fabs(0.5 * strength[o] * radius));
    uint32_t m = 0;
    for (int o = 0; o < n_octaves; ++o)
        if (std::fabs(0.5 * strength[o] * radius) >= ref / 8.0) m |= 1u << o;
    return m;
}

static int check_octaves(int n_octaves, const double *scale, const double *strength, const char *who)
{
    if (n_octaves < 0 || n_octaves > NX_MAX_OCTAVES)
        return nx::fail(NX_EINVAL, "%s: n_octaves must be in [0, %d]", who, NX_MAX_OCTAVES);
    if (n_octaves && (!scale || !strength)) return nx::fail(NX_EINVAL, "%s: null scale or strength", who);
    for (int o = 0; o < n_octaves; ++o)
        if (!std::isfinite(scale[o]) || !std::isfinite(strength[o]) || std::fabs(scale[o]) > 1e30)
            return nx::fail(NX_EINVAL, "%s: octave %d: scale and strength must be finite", who, o);
    return NX_OK;
}

NX_EXPORT int nx_fbm_planet_fill(nx_fbm_planet *planet, int n_octaves, const double *scale, const double *strength,
                                 double radius)
{
    if (!planet) return nx::fail(NX_EINVAL, "nx_fbm_planet_fill: null planet");
    int rc = check_octaves(n_octaves, scale, strength, "nx_fbm_planet_fill");
    if (rc) return rc;
    planet->n_octaves = n_octaves;
    bool pow2 = true;
    for (int o = 0; o < NX_MAX_OCTAVES; ++o) {
        const double sc = o < n_octaves ? scale[o] : 0.0;
        split_scale(sc, planet->s1[o], planet->s2[o], planet->s3[o]);
        planet->s[o] = sc;
        const double amp = o < n_octaves ? 0.5 * strength[o] * radius : 0.0;
        planet->amp_hi[o] = (float)amp;
        planet->amp_lo[o] = (float)(amp - (double)planet->amp_hi[o]);
        if (o < n_octaves && !is_pow2(sc)) pow2 = false;
    }
    planet->pow2 = pow2 ? 1 : 0;
    planet->norm_mask = norm_mask(n_octaves, strength, radius, 0.0);
    return NX_OK;
}

NX_EXPORT int nx_fbm_pair(const double *xyz_dev, int64_t n, const int32_t *perm_dev, const int32_t *pgi_dev,
                          int n_octaves, const double *scale, const double *strength, double radius, double amp_ref,
                          float *pair_dev, double *elev_f64_dev, int accumulate, unsigned long long *minmax_dev,
                          unsigned long long *n_fallback_dev, void *stream)
{
    if (n < 0) return nx::fail(NX_EINVAL, "nx_fbm_pair: n < 0");
    int rc = check_octaves(n_octaves, scale, strength, "nx_fbm_pair");
    if (rc) return rc;
    if (n == 0) return NX_OK;
    if (!xyz_dev || !perm_dev || !pgi_dev) return nx::fail(NX_EINVAL, "nx_fbm_pair: null pointer");
    if (!pair_dev && !elev_f64_dev) return nx::fail(NX_EINVAL, "nx_fbm_pair: no output");
    if (pair_dev && ((uintptr_t)pair_dev & 7u)) return nx::fail(NX_EINVAL, "nx_fbm_pair: pair output must be 8-byte aligned");
    FbmPairParams P;
    P.n_oct = n_octaves;
    bool pow2 = true;
    for (int o = 0; o < NX_MAX_OCTAVES; ++o) {
        const double sc = o < n_octaves ? scale[o] : 0.0;
        split_scale(sc, P.s1[o], P.s2[o], P.s3[o]);
        P.s[o] = sc;
        const double amp = o < n_octaves ? 0.5 * strength[o] * radius : 0.0;
        P.amph[o] = (float)amp;
        P.ampl[o] = (float)(amp - (double)P.amph[o]);
        if (o < n_octaves && !is_pow2(sc)) pow2 = false;
    }
    P.pow2 = pow2 ? 1 : 0;
    P.norm_mask = norm_mask(n_octaves, strength, radius, amp_ref);
    rc = configure_smem();
    if (rc) return rc;
    int grid = grid_for(n, 256, (const void *)fbm_pair_kernel, TABLE_BYTES);
    fbm_pair_kernel<<<grid, 256, TABLE_BYTES, (cudaStream_t)stream>>>(xyz_dev, n, perm_dev, pgi_dev, P,
                                                                      (float2 *)pair_dev, elev_f64_dev, accumulate,
                                                                      minmax_dev, n_fallback_dev);
    NX_CHECK_LAUNCH("fbm_pair_kernel");
    nx::note_launch(1);
    return NX_OK;
}

NX_EXPORT int nx_fbm_batch(const nx_fbm_planet *planets_dev, const nx_fbm_planet *planets_host, int nplanets,
                           unsigned long long *n_fallback_dev, void *stream)
{
    if (nplanets <= 0) return NX_OK;
    if (!planets_dev || !planets_host) return nx::fail(NX_EINVAL, "nx_fbm_batch: null pointer");
    int total = 0;
    for (int p = 0; p < nplanets; ++p) {
        const nx_fbm_planet &P = planets_host[p];
        if (P.n < 0 || (P.n > 0 && (!P.xyz || !P.perm || !P.pgi || !P.out)))
            return nx::fail(NX_EINVAL, "nx_fbm_batch: planet %d incomplete", p);
        if ((uintptr_t)P.out & 7u) return nx::fail(NX_EINVAL, "nx_fbm_batch: planet %d: out must be 8-byte aligned", p);
        if (P.n_octaves < 0 || P.n_octaves > NX_MAX_OCTAVES) return nx::fail(NX_EINVAL, "nx_fbm_batch: octaves");
        if (P.chunk0 != total)
            return nx::fail(NX_EINVAL, "nx_fbm_batch: planet %d chunk0 must be %d (chunks of %d vertices)", p, total,
                            CHUNK);
        total += (int)((P.n + CHUNK - 1) / CHUNK);
    }
    if (total == 0) return NX_OK;
    int rc = configure_smem();
    if (rc) return rc;
    int grid = grid_for((int64_t)total * 256, 256, (const void *)fbm_batch_kernel, TABLE_BYTES);
    if (grid > FBM_SPLIT_MAX) grid = FBM_SPLIT_MAX;
    // cut the chunks into grid ranges of equal estimated cost: a planet's
    // chunk costs its vertices x (8 per octave + 1 per renormalised octave)
    std::vector<int64_t> wchunk(nplanets), cum(nplanets + 1, 0);
    for (int p = 0; p < nplanets; ++p) {
        const nx_fbm_planet &P = planets_host[p];
        const uint32_t live = P.n_octaves >= 32 ? ~0u : ((1u << P.n_octaves) - 1u);
        wchunk[p] = 8 * (int64_t)P.n_octaves + (int64_t)__builtin_popcount(P.norm_mask & live);
        cum[p + 1] = cum[p] + wchunk[p] * P.n;
    }
    FbmSplit split;
    const int64_t tot = cum[nplanets];
    int p = 0;
    split.first[0] = 0;
    for (int b = 1; b <= grid; ++b) {
        if (b == grid || tot == 0) { split.first[b] = total; continue; }
        // first chunk whose cost prefix reaches b * tot / grid
        const int64_t t = (int64_t)((__int128)tot * b / grid);
        while (p + 1 < nplanets && cum[p + 1] <= t) ++p;
        const nx_fbm_planet &P = planets_host[p];
        const int64_t per = wchunk[p] * CHUNK;
        int64_t k = per > 0 ? (t - cum[p] + per - 1) / per : 0;
        const int64_t nch = (P.n + CHUNK - 1) / CHUNK;
        if (k > nch) k = nch;
        int c = P.chunk0 + (int)k;
        if (c < split.first[b - 1]) c = split.first[b - 1];
        split.first[b] = c;
    }
    fbm_batch_kernel<<<grid, 256, TABLE_BYTES, (cudaStream_t)stream>>>(planets_dev, nplanets, split, n_fallback_dev);
    NX_CHECK_LAUNCH("fbm_batch_kernel");
    nx::note_launch(1);
    return NX_OK;
}

NX_EXPORT int nx_fbm_chunk_size(void) { return CHUNK; }
