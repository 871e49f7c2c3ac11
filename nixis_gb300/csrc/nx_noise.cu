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
__device__ __forceinline__ void decide_sel(float x, float y, float z, float in_sum, Cmp<float, true> &C, Decision &D)
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
    const float4 *t = s_extra + 2 * (tet ? tt : ot);
    const float4 a = t[0], b = t[1];
    D.region = r0 ? 0 : (r1 ? 1 : 2);
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
    c.dx0 = (float)__dsub_rn(x, xb);
    c.dy0 = (float)__dsub_rn(y, yb);
    c.dz0 = (float)__dsub_rn(z, zb);
    c.xsb = (int)xsb; c.ysb = (int)ysb; c.zsb = (int)zsb;
    c.xb7 = (int)((unsigned)xsb << 7);
    c.yb7 = (int)((unsigned)ysb << 7);
    c.zb7 = (int)((unsigned)zsb << 7);
    return c;
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
    float T = (Ax + Ay) + Az;
    float q = floorf(fmaf(T, SIXTH, 1.0f / 12.0f));
    float r = fmaf(-6.0f, q, T);
    float u = r + ((ax + ay) + az);
    float bx = fmaf(-u, SIXTH, ax), by = fmaf(-u, SIXTH, ay), bz = fmaf(-u, SIXTH, az);
    float fx = floorf(bx), fy = floorf(by), fz = floorf(bz);
    float xins = bx - fx, yins = by - fy, zins = bz - fz;
    float xsbf = (Ax - q) + fx, ysbf = (Ay - q) + fy, zsbf = (Az - q) + fz;
    int xi = __float_as_int(xsbf + MAGIC), yi = __float_as_int(ysbf + MAGIC), zi = __float_as_int(zsbf + MAGIC);
    c.xsb = xi - MAGIC_BITS; c.ysb = yi - MAGIC_BITS; c.zsb = zi - MAGIC_BITS;
    c.xb7 = xi << 7; c.yb7 = yi << 7; c.zb7 = zi << 7;
    float g = (r + ((fx + fy) + fz)) * THIRD;
    c.dx0 = (ax - fx) - g; c.dy0 = (ay - fy) - g; c.dz0 = (az - fz) - g;
    Cmp<float, true> C;
    C.m = fminf(fminf(fminf(xins, 1.0f - xins), fminf(yins, 1.0f - yins)), fminf(zins, 1.0f - zins));
    float in_sum = (xins + yins) + zins;
    decide_sel(xins, yins, zins, in_sum, C, c.D);
    return C.m >= TAU && big < PMAX;
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

// Ordered-key transform: unsigned comparisons of keys follow float order.
__device__ __forceinline__ uint32_t fkey(float f)
{
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b ^ 0x80000000u);
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

// Many planets in one persistent launch: work items are chunks of CHUNK
// vertices of one planet, handed out round-robin; a block rebuilds its
// shared table when its next chunk belongs to another planet.  Each chunk
// also folds its min/max into the planet's ordered keys (for the rescale
// to metres that follows).
__global__ void __launch_bounds__(256) fbm_batch_kernel(const nx_fbm_planet *__restrict__ planets, int np,
                                                        int total_chunks, unsigned long long *nfb_out)
{
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ uint32_t s_mm[2][8];
    init_extra_table();
    __syncthreads();
    const uint32_t lb = lane_base(smem);
    int cur = -1;
    unsigned nfb = 0;
    for (int c = blockIdx.x; c < total_chunks; c += gridDim.x) {
        const int p = chunk_planet(planets, np, c);
        const nx_fbm_planet &P = planets[p];
        if (p != cur) {
            __syncthreads();
            build_table(smem, P.perm, P.pgi);
            __syncthreads();
            cur = p;
        }
        const int64_t base = (int64_t)(c - P.chunk0) * CHUNK;
        float mn = INFINITY, mx = -INFINITY;
        for (int64_t i = base + threadIdx.x; i < base + CHUNK && i < P.n; i += blockDim.x) {
            double X = P.xyz[3 * i], Y = P.xyz[3 * i + 1], Z = P.xyz[3 * i + 2];
            float xh, xl, yh, yl, zh, zl;
            split_f64(X, xh, xl);
            split_f64(Y, yh, yl);
            split_f64(Z, zh, zl);
            float acc = 0.0f;
            for (int o = 0; o < P.n_octaves; ++o) {
                float v = noise_raw<false>(xh, xl, yh, yl, zh, zl, P.s_hi[o], P.s_lo[o], X, Y, Z, P.s[o], lb, nfb,
                                           nullptr, nullptr);
                acc += fmaf(v, P.amp[o] * (1.0f / 103.0f), P.amp[o]);
            }
            P.out[i] = acc;
            mn = fminf(mn, acc);
            mx = fmaxf(mx, acc);
        }
        if (P.minmax) {
            for (int o = 16; o > 0; o >>= 1) {
                mn = fminf(mn, __shfl_xor_sync(0xFFFFFFFFu, mn, o));
                mx = fmaxf(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
            }
            const int w = threadIdx.x >> 5;
            if ((threadIdx.x & 31) == 0) { s_mm[0][w] = fkey(mn); s_mm[1][w] = fkey(mx); }
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t a0 = s_mm[0][0], a1 = s_mm[1][0];
                for (int k = 1; k < (int)(blockDim.x >> 5); ++k) { a0 = min(a0, s_mm[0][k]); a1 = max(a1, s_mm[1][k]); }
                atomicMin(&P.minmax[0], a0);
                atomicMax(&P.minmax[1], a1);
            }
            __syncthreads();
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

NX_EXPORT int nx_fbm_planet_fill(nx_fbm_planet *planet, int n_octaves, const double *scale, const double *strength,
                                 double radius)
{
    if (!planet || n_octaves < 0 || n_octaves > NX_MAX_OCTAVES || (n_octaves && (!scale || !strength)))
        return nx::fail(NX_EINVAL, "nx_fbm_planet_fill: bad arguments");
    planet->n_octaves = n_octaves;
    for (int o = 0; o < NX_MAX_OCTAVES; ++o) {
        double sc = o < n_octaves ? scale[o] : 0.0;
        float hi = (float)sc;
        planet->s_hi[o] = hi;
        planet->s_lo[o] = (float)(sc - (double)hi);
        planet->s[o] = sc;
        planet->amp[o] = o < n_octaves ? (float)(0.5 * strength[o] * radius) : 0.0f;
    }
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
    fbm_batch_kernel<<<grid, 256, TABLE_BYTES, (cudaStream_t)stream>>>(planets_dev, nplanets, total, n_fallback_dev);
    NX_CHECK_LAUNCH("fbm_batch_kernel");
    nx::note_launch(1);
    return NX_OK;
}

NX_EXPORT int nx_fbm_chunk_size(void) { return CHUNK; }
