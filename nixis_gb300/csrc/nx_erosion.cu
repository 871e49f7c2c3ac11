// nx_erosion.cu -- erosion variant 3 (erosion.py:172-279) for sm_103a.
//
// State per vertex: a row of 8 binary32s, (h_hi, h_lo, w_hi, w_lo) and
// (s_hi, s_lo, 0, 0), double buffered (the reference reads old arrays and
// writes copies, erosion.py:199-201, 274-277).  Height, water and sediment
// are each an unevaluated pair hi + lo of binary32s (about 48 significant
// bits).  Pairs keep the small per-iteration changes the binary64 reference
// makes, and they keep the flow choice -- the sign of h_n - h_i -- on the
// binary64 trajectory: with binary32 water and sediment the heights, which
// become sums of eroded amounts, drift by ~1e-6 relative within tens of
// iterations, enough to flip near-ties and move whole regions off the
// reference's path.  Neighbour slots are the reference's (n,6) int32 table;
// edge lengths are precomputed per slot in binary64 and kept as pairs too
// (rounded to binary32 they alone move a 100-iteration run by ~1e-4).
//
// Overflow: under the reference's update, water and sediment grow about 2x
// per iteration, past binary32's range after ~140 iterations.  The update is
// positively homogeneous (only signs of height differences and the
// capacity test s > cap*w are decided, both scale invariant), and scaling by
// a power of two commutes with binary32 rounding, so each planet carries an
// exponent K: stored values are true values * 2^-K.  When the previous
// iteration's max |value| exceeds 2^96, this iteration multiplies what it
// reads by 2^-64 and K grows by 64.  The trajectory is then exactly the one
// an overflow-free binary32 machine would compute.
//
// Batched: planets are packed back to back (each range starting at a
// multiple of 256) and sorted by iteration count, descending, so the planets
// still running at iteration t are a prefix; one launch per iteration covers
// that prefix.  Each planet alternates its two buffers so that its last
// iteration writes buffer 0.
#include "nx_common.cuh"

#include <mutex>

namespace nx {
void note_launch(int k);
}

namespace {

constexpr int BLOCK = 256;
constexpr float RESCALE_ABOVE = 7.9228163e28f;   // 2^96
constexpr int RESCALE_SHIFT = 64;

// erosion.py:205-207 (solubility, 1 - evaporation, capacity) as pairs
// hi + lo of the binary64 values
constexpr double SOL = 0.01 / 320, ONE_M_EVAP = 1.0 - 0.1 / 320, CAP = 0.2 / 320;
constexpr float SOL_H = (float)SOL, SOL_L = (float)(SOL - (double)SOL_H);
constexpr float OE_H = (float)ONE_M_EVAP, OE_L = (float)(ONE_M_EVAP - (double)OE_H);
constexpr float CAP_H = (float)CAP, CAP_L = (float)(CAP - (double)CAP_H);

}  // namespace

// nx_erosion_ctl (header): maxbits = max |h|,|w|,|s| of an iteration's
// output as float bits in 3 rotating slots; K = scale exponent, ping-pong by
// iteration parity; done = blocks finished in the current iteration (mass
// sums); err = 1 for a neighbour id out of range.
static_assert(sizeof(nx_erosion_ctl) == 32, "control block layout");
static_assert(sizeof(nx_erosion_planet) == 72, "planet descriptor layout");

namespace {

struct StepArgs {
    const nx_erosion_planet *planets;
    const int2 *blk_map;   // per block of the launch: (planet index, block within the planet)
    int t;                 // global step; a planet's iteration is t - t_start
    float4 *st0;           // rows of two float4s
    float4 *st1;
    nx_erosion_ctl *ctl;
    double *partials;      // [block][3] (mass sums only)
    double *mass;          // [iteration][mass_np][3] or null
    int mass_np;
    uint16_t *flow;        // optional: per vertex 2 bits per slot (1: neighbour higher, 2: lower)
};

// Unevaluated pair hi + lo of binary32s.
struct Pair {
    float h, l;
};

// Knuth's two-sum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// pair + pair, renormalised
__device__ __forceinline__ Pair padd(Pair a, Pair b)
{
    float s, e;
    two_sum(a.h, b.h, s, e);
    e = __fadd_rn(e, __fadd_rn(a.l, b.l));
    Pair r;
    r.h = __fadd_rn(s, e);
    r.l = __fsub_rn(e, __fsub_rn(r.h, s));
    return r;
}

// pair * (ch + cl), not renormalised
__device__ __forceinline__ Pair pmul(Pair a, float ch, float cl)
{
    Pair r;
    r.h = __fmul_rn(a.h, ch);
    float e = __fmaf_rn(a.h, ch, -r.h);
    e = __fmaf_rn(a.h, cl, e);
    r.l = __fmaf_rn(a.l, ch, e);
    return r;
}

// (wh + wl) + r for binary32 rain r, not renormalised
__device__ __forceinline__ Pair prain(float wh, float wl, float r)
{
    float s, e;
    two_sum(wh, r, s, e);
    return Pair{s, __fadd_rn(wl, e)};
}

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// One neighbour's contribution (erosion.py:223-247).  o = (h_hi, h_lo,
// w_hi, w_lo) of the neighbour, its water including this iteration's rain;
// (dh, dl) the edge length pair.  The flow choice is the sign g (+1, -1, 0)
// of h_j - h_i from the height pairs; then, as two-sums in paired binary32
// lanes (FADD2), S += g*w_j (lane x) and W += g*w_j*d (lane y); A holds the
// lanes' hi parts, L their lo parts.  Returns the flow code: 1 higher,
// 2 lower, 0 equal.
__device__ __forceinline__ unsigned erode_accum(float hh, float hl, float4 o, float dh, float dl, float2 &A, float2 &L)
{
    // (o.x - hh, o.y - hl) in one paired subtraction, then their sum
    const float2 d2 = __fadd2_rn(make_float2(o.x, o.y), make_float2(-hh, -hl));
    const float diff = __fadd_rn(d2.x, d2.y);
    const bool up = diff > 0.0f, dn = diff < 0.0f;
    // +-1 with the sign of diff; 0 where diff is 0 or NaN (no flow, as the
    // reference's slope tests decide for a NaN slope)
    const float g = fabsf(diff) > 0.0f ? __int_as_float((__float_as_int(diff) & (int)0x80000000) | 0x3F800000) : 0.0f;
    const float xh = __fmul_rn(g, o.z), xl = __fmul_rn(g, o.w);
    const float p = __fmul_rn(xh, dh);
    float pe = __fmaf_rn(xh, dh, -p);
    pe = __fmaf_rn(xh, dl, pe);
    pe = __fmaf_rn(xl, dh, pe);
    const float2 B = make_float2(xh, p);
    const float2 s = __fadd2_rn(A, B);
    const float2 bb = __fadd2_rn(s, neg2(A));
    const float2 e = __fadd2_rn(__fadd2_rn(A, neg2(__fadd2_rn(s, neg2(bb)))), __fadd2_rn(B, neg2(bb)));
    L = __fadd2_rn(L, __fadd2_rn(e, make_float2(xl, pe)));
    A = s;
    return up ? 1u : (dn ? 2u : 0u);
}

// erosion.py:261-267 from the accumulated S and W: sed = s + sol*S,
// h -= sed, s += sed, w = w_i + W*(1 - evap), then the capacity test.
// wi is the vertex's water including this iteration's rain.  (Evaluating
// these in paired lanes measured slower: assembling the lane pairs costs
// more instructions than it saves.)
__device__ __forceinline__ void erode_finish(Pair hi, Pair wi, Pair si, float2 A, float2 L, Pair &hn, Pair &wn,
                                             Pair &sn)
{
    const Pair S{A.x, L.x}, W{A.y, L.y};
    const Pair sed = padd(si, pmul(S, SOL_H, SOL_L));
    hn = padd(hi, Pair{-sed.h, -sed.l});
    sn = padd(si, sed);
    wn = padd(wi, pmul(W, OE_H, OE_L));
    const Pair c = pmul(wn, CAP_H, CAP_L);
    Pair cw;
    cw.h = __fadd_rn(c.h, c.l);
    cw.l = __fsub_rn(c.l, __fsub_rn(cw.h, c.h));
    if (__fadd_rn(__fsub_rn(sn.h, cw.h), __fsub_rn(sn.l, cw.l)) > 0.0f) {
        const Pair ex = padd(sn, Pair{-cw.h, -cw.l});
        hn = padd(hn, ex);
        sn = cw;
    }
}

__device__ __forceinline__ int find_planet(const nx_erosion_planet *P, int np, int64_t v)
{
    int lo = 0, hi = np - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (P[mid].vbeg <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ float warp_max(float v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// One erosion iteration (erosion.py:210-267) for the vertices of every
// block's planet.  No barrier on the common path: every thread reads the
// (broadcast) planet descriptor and control words itself, and each warp
// folds its max into the planet's next slot with a reduction atomic.
__global__ void __launch_bounds__(BLOCK, 4) erosion_step_kernel(StepArgs a)
{
    const int2 bm = a.blk_map[blockIdx.x];
    const int p = bm.x;
    const nx_erosion_planet P = a.planets[p];
    const int t = a.t - P.t_start;
    if (t < 0 || t >= P.iters) return;        // whole block: planet not stepping now
    nx_erosion_ctl *c = a.ctl + P.slot;
    // slots read here were written by earlier launches only (this launch
    // writes the other slots), so ordinary cached loads are safe
    const float m = __uint_as_float(__ldg(&c->maxbits[t % 3]));
    const int shift = m > RESCALE_ABOVE ? RESCALE_SHIFT : 0;
    const int K = __ldg(&c->K[t & 1]) + shift;
    const float lam = shift ? __int_as_float((127 - shift) << 23) : 1.0f;
    const float rain = scalbnf(P.rain, -K);
    if (bm.y == 0 && threadIdx.x == 0) {
        c->K[(t + 1) & 1] = K;
        c->maxbits[(t + 2) % 3] = 0u;
    }
    // buffers: read B[(iters - t) & 1], write the other; B[0] = st0
    const bool par = ((P.iters - t) & 1) != 0;
    const float4 *__restrict__ ist = par ? a.st1 : a.st0;
    float4 *__restrict__ ost = par ? a.st0 : a.st1;

    const int64_t li = (int64_t)bm.y * BLOCK + threadIdx.x;   // vertex id within the planet
    const int64_t i = P.vbeg + li;                             // state row
    float vmax = 0.0f;
    double sh = 0.0, sw = 0.0, ss = 0.0;
    if (li < P.n) {
        const int2 *nb2 = reinterpret_cast<const int2 *>(P.nbr + 6 * li);
        const float4 *el4 = reinterpret_cast<const float4 *>(P.edge + 12 * li);
        const int2 n01 = nb2[0], n23 = nb2[1], n45 = nb2[2];
        const float4 me = ist[2 * i], mb = ist[2 * i + 1];
        const float4 d01 = el4[0], d23 = el4[1], d45 = el4[2];   // (hi, lo) per slot
        const Pair hi{__fmul_rn(me.x, lam), __fmul_rn(me.y, lam)};
        const Pair wi = prain(__fmul_rn(me.z, lam), __fmul_rn(me.w, lam), rain);
        const Pair si{__fmul_rn(mb.x, lam), __fmul_rn(mb.y, lam)};
        float2 A = make_float2(0.0f, wi.h), L = make_float2(0.0f, wi.l);
        const int nbr[6] = {n01.x, n01.y, n23.x, n23.y, n45.x, n45.y};
        const float dh[6] = {d01.x, d01.z, d23.x, d23.z, d45.x, d45.z};
        const float dl[6] = {d01.y, d01.w, d23.y, d23.w, d45.y, d45.w};
        unsigned flow = 0;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const int j = nbr[k];
            if (j < 0) continue;
            if ((int64_t)j >= P.n) {
                c->err = 1;
                continue;
            }
            const float4 o = ist[2 * (P.vbeg + j)];
            const Pair wj = prain(__fmul_rn(o.z, lam), __fmul_rn(o.w, lam), rain);
            const float4 os = make_float4(__fmul_rn(o.x, lam), __fmul_rn(o.y, lam), wj.h, wj.l);
            flow |= erode_accum(hi.h, hi.l, os, dh[k], dl[k], A, L) << (2 * k);
        }
        Pair hn, wn, sn;
        erode_finish(hi, wi, si, A, L, hn, wn, sn);
        ost[2 * i] = make_float4(hn.h, hn.l, wn.h, wn.l);
        ost[2 * i + 1] = make_float4(sn.h, sn.l, 0.0f, 0.0f);
        if (a.flow) a.flow[li] = (uint16_t)flow;
        vmax = fmaxf(fabsf(hn.h), fmaxf(fabsf(wn.h), fabsf(sn.h)));
        if (a.mass) {
            sh = (double)hn.h + (double)hn.l;
            sw = (double)wn.h + (double)wn.l;
            ss = (double)sn.h + (double)sn.l;
        }
    }
    // block max -> the planet's max for the next iteration's rescale decision
    // (one atomic per block; NaN never wins fmaxf; inf still triggers a rescale)
    __shared__ float s_wmax[BLOCK / 32];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    vmax = warp_max(vmax);
    if (lane == 0) s_wmax[wid] = vmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        float bmx = s_wmax[0];
        for (int w = 1; w < BLOCK / 32; ++w) bmx = fmaxf(bmx, s_wmax[w]);
        atomicMax(&c->maxbits[(t + 1) % 3], __float_as_uint(bmx));
    }
    if (!a.mass) return;

    // per-iteration mass sums: block partials, then the planet's last block
    // reduces them in a fixed order (Neumaier), scaled back by 2^K
    __shared__ double s_wsum[BLOCK / 32][3];
    __shared__ bool s_last;
    sh = warp_sum(sh); sw = warp_sum(sw); ss = warp_sum(ss);
    if (lane == 0) { s_wsum[wid][0] = sh; s_wsum[wid][1] = sw; s_wsum[wid][2] = ss; }
    __syncthreads();
    const int64_t nblk = (P.n + BLOCK - 1) / BLOCK;
    const int64_t b0 = (int64_t)blockIdx.x - bm.y;
    if (threadIdx.x == 0) {
        double t0 = 0, t1 = 0, t2 = 0;
        for (int w = 0; w < BLOCK / 32; ++w) { t0 += s_wsum[w][0]; t1 += s_wsum[w][1]; t2 += s_wsum[w][2]; }
        double *pp = a.partials + 3 * (int64_t)blockIdx.x;
        pp[0] = t0; pp[1] = t1; pp[2] = t2;
        __threadfence();
        const unsigned prev = atomicAdd(&c->done, 1u);
        s_last = (int64_t)prev + 1 == nblk;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double acc[3] = {0, 0, 0}, cmp[3] = {0, 0, 0};
    for (int64_t b = threadIdx.x; b < nblk; b += BLOCK) {
        const volatile double *pp = a.partials + 3 * (b0 + b);
        for (int q = 0; q < 3; ++q) {
            const double x = pp[q], tt = acc[q] + x;
            cmp[q] += fabs(acc[q]) >= fabs(x) ? (acc[q] - tt) + x : (x - tt) + acc[q];
            acc[q] = tt;
        }
    }
    __syncthreads();
    for (int q = 0; q < 3; ++q) {
        const double v = warp_sum(acc[q] + cmp[q]);
        if (lane == 0) s_wsum[wid][q] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double out[3];
        for (int q = 0; q < 3; ++q) {
            double sacc = 0, e = 0;
            for (int w = 0; w < BLOCK / 32; ++w) {
                const double x = s_wsum[w][q], tt = sacc + x;
                e += fabs(sacc) >= fabs(x) ? (sacc - tt) + x : (x - tt) + sacc;
                sacc = tt;
            }
            out[q] = ldexp(sacc + e, K);
        }
        double *mrow = a.mass + 3 * ((int64_t)t * a.mass_np + p);
        mrow[0] = out[0]; mrow[1] = out[1]; mrow[2] = out[2];
        c->done = 0u;
    }
}

// ---------------------------------------------------------------------------
// Ordered key -> float (inverse of the fBm kernel's min/max keys).
__device__ __forceinline__ float unkey(uint32_t k)
{
    return __uint_as_float((k & 0x80000000u) ? (k ^ 0x80000000u) : ~k);
}

// A planet's rescale constants: its minimum as a pair, f = (hi - lo) /
// (max - min) as a pair (formed in binary64).
__device__ __forceinline__ float4 init_consts(const unsigned long long *minmax, int p, double lo, double hi)
{
    const unsigned long long kmn = minmax[2 * p], kmx = minmax[2 * p + 1];
    const float mnh = unkey((uint32_t)(kmn >> 32)), mnl = unkey((uint32_t)kmn);
    const float mxh = unkey((uint32_t)(kmx >> 32)), mxl = unkey((uint32_t)kmx);
    const double mn = (double)mnh + (double)mnl, mx = (double)mxh + (double)mxl;
    const double f = (hi - lo) / (mx - mn);
    const float fh = (float)f;
    return make_float4(mnh, mnl, fh, (float)(f - (double)fh));
}

// One vertex's starting height pair: (raw - min) * f + lo, renormalised.
__device__ __forceinline__ float2 init_height(float2 r, float4 c, float loh, float lol)
{
    // t = raw - min
    float th, te;
    {
        th = __fsub_rn(r.x, c.x);
        const float bb = __fsub_rn(th, r.x);
        te = __fadd_rn(__fsub_rn(r.x, __fsub_rn(th, bb)), __fsub_rn(-c.x, bb));
    }
    const float tl = __fadd_rn(te, __fsub_rn(r.y, c.y));
    // t * f
    const float ph = __fmul_rn(th, c.z);
    float pl = __fmaf_rn(th, c.z, -ph);
    pl = __fmaf_rn(th, c.w, __fmaf_rn(tl, c.z, pl));
    // + lo, renormalised
    float sh, se;
    {
        sh = __fadd_rn(ph, loh);
        const float bb = __fsub_rn(sh, ph);
        se = __fadd_rn(__fsub_rn(ph, __fsub_rn(sh, bb)), __fsub_rn(loh, bb));
    }
    const float sl = __fadd_rn(se, __fadd_rn(pl, lol));
    const float h = __fadd_rn(sh, sl);
    return make_float2(h, __fsub_rn(sl, __fsub_rn(h, sh)));
}

// v * 2^K as a binary64 (exact) for the cases the integer form below leaves
// out; a call, so that the common path is not if-converted into binary64
// operations (GB300's binary64 pipe is narrow).
__device__ __noinline__ double f32_scaled_slow(float v, int K)
{
    return ldexp((double)v, K);
}

// v * 2^K as a binary64 (exact) by integer operations when v is a normal
// binary32 and the result's exponent is in range; otherwise through the
// binary64 pipe.
__device__ __forceinline__ double f32_scaled(float v, int K)
{
    const uint32_t u = __float_as_uint(v);
    const int e = (int)((u >> 23) & 0xFFu);
    const int E = e + (1023 - 127) + K;
    if (e == 0 || e == 255 || E <= 0 || E >= 2047) return f32_scaled_slow(v, K);
    return __hiloint2double((int)((u & 0x80000000u) | ((uint32_t)E << 20) | ((u & 0x7FFFFFu) >> 3)), (int)(u << 29));
}

// Temporally blocked erosion: one block per (planet, tile) runs a pass of up
// to R iterations in shared memory.  It loads the tile and its halo rings
// (state * lambda), then for m = 0..len-1 updates the members and the rings
// that the remaining iterations still need (ring set shrinks by one per
// iteration), and writes the members' final state.  Per vertex the
// arithmetic is erode_accum / erode_finish in slot order, as in the
// iteration-at-a-time kernel, so the results are the same.  Global buffers
// alternate per pass; a planet makes np passes with np = iters (mod 2), so
// its state starts in buffer (iters & 1) and ends in buffer 0, like the
// iteration-at-a-time path.

__host__ __device__ __forceinline__ int tb_npass(int iters, int R)
{
    if (iters <= 0) return 0;
    int np = (iters + R - 1) / R;
    if ((np ^ iters) & 1) ++np;
    return np;
}

// Length of pass q: greedy, each later pass keeps at least one iteration.
__host__ __device__ __forceinline__ int tb_len(int iters, int R, int np, int q)
{
    int done = 0;
    for (int x = 0; x < q; ++x) {
        int l = iters - done - (np - 1 - x);
        done += l < R ? l : R;
    }
    int l = iters - done - (np - 1 - q);
    return l < R ? l : R;
}

struct TbArgs {
    const nx_erosion_planet *planets;
    const int2 *blk_map;   // (planet, tile), planets ordered by pass count, descending
    int pass;              // global pass; a planet's pass is pass - t_start
    int R;
    int smem_n;            // rows per shared state array (>= every tile's local count)
    int smem_c;            // rows of the shared tile tables (>= every tile's updatable count)
    float4 *st0;
    float4 *st1;
    nx_erosion_ctl *ctl;
    // Optional fusion of the rescale: a planet's first pass reads the raw
    // fBm pair sums (float2 per row) and rescales them to its starting
    // heights as erosion_init_kernel does (minimum and maximum keys per
    // planet index in minmax, target range [elo, ehi], starting water (w0h,
    // w0l)) instead of reading a state buffer.
    const float2 *raw = nullptr;
    const unsigned long long *minmax = nullptr;
    double elo = 0.0, ehi = 0.0;
    float w0h = 0.0f, w0l = 0.0f;
};

// Threads per block of the blocked kernel: 256, 512 or 1024 (autotuned),
// sized for 1024 resident threads per SM (64 registers each).

// Shared memory of a pass for tiles of up to n local vertices: rows
// (h_hi, h_lo, w_hi, w_lo) twice (read and write side) and (s_hi, s_lo)
// once (a vertex's sediment is read and written only by its own thread).
__host__ __device__ __forceinline__ size_t tb_smem_bytes(int n) { return (2 * sizeof(float4) + sizeof(float2)) * (size_t)n; }

// Variant 2 also holds the tile's tables for c updatable vertices: edge
// pairs (48 B) and local neighbour indices (12 B, rounded to 16-byte units).
__host__ __device__ __forceinline__ size_t tb_table_bytes(int c) { return 48 * (size_t)c + (((size_t)c * 12 + 15) & ~(size_t)15); }

// Largest dynamic shared memory of a variant-2 block: the device's opt-in
// limit less the kernel's static shared memory (set by tb_prepare).
static size_t TB_SMEM_MAX = 200 * 1024;

// One vertex's tile-table entries: local neighbour indices and edge pairs.
struct TileRow {
    uint32_t p01, p23, p45;
    float4 d01, d23, d45;
};

template <bool SHARED>
__device__ __forceinline__ TileRow tile_row(const uint32_t *lnb, const float4 *led, int l)
{
    TileRow r;
    if (SHARED) {
        r.p01 = lnb[3 * l]; r.p23 = lnb[3 * l + 1]; r.p45 = lnb[3 * l + 2];
        r.d01 = led[3 * l]; r.d23 = led[3 * l + 1]; r.d45 = led[3 * l + 2];
    } else {
        r.p01 = __ldg(lnb + 3 * l); r.p23 = __ldg(lnb + 3 * l + 1); r.p45 = __ldg(lnb + 3 * l + 2);
        r.d01 = __ldg(led + 3 * l); r.d23 = __ldg(led + 3 * l + 1); r.d45 = __ldg(led + 3 * l + 2);
    }
    return r;
}

// One vertex of a pass iteration: its row of the tile tables, the state
// rows `cur` (read) and `nxt` (written), its sediment pair in place.
__device__ __forceinline__ void tb_update(int l, const TileRow &row, const float4 *cur, float4 *nxt, float2 *sed,
                                          float rain, bool more)
{
    const float4 me = cur[l];
    const float2 ms = sed[l];
    float2 A = make_float2(0.0f, me.z), L = make_float2(0.0f, me.w);
    const uint32_t nb[6] = {row.p01 & 0xFFFFu, row.p01 >> 16, row.p23 & 0xFFFFu, row.p23 >> 16,
                            row.p45 & 0xFFFFu, row.p45 >> 16};
    const float dh[6] = {row.d01.x, row.d01.z, row.d23.x, row.d23.z, row.d45.x, row.d45.z};
    const float dl[6] = {row.d01.y, row.d01.w, row.d23.y, row.d23.w, row.d45.y, row.d45.w};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        // a missing neighbour (pentagon slot) is stored as the vertex itself:
        // equal heights contribute nothing, as the reference's skip of -1
        erode_accum(me.x, me.y, cur[nb[k]], dh[k], dl[k], A, L);
    }
    Pair hn, wn, sn;
    erode_finish(Pair{me.x, me.y}, Pair{me.z, me.w}, Pair{ms.x, ms.y}, A, L, hn, wn, sn);
    const Pair wr = more ? prain(wn.h, wn.l, rain) : wn;
    nxt[l] = make_float4(hn.h, hn.l, wr.h, wr.l);
    sed[l] = make_float2(sn.h, sn.l);
}

// PF: software-pipelined table reads (the next vertex's entries are loaded
// before the current vertex is computed; ~80 registers, so 768 threads per
// SM); otherwise each vertex loads its own entries (64 registers, 1024
// threads per SM).  SMT: the tile's tables are copied to shared memory once
// per pass (with the state) and every iteration of the pass reads them
// there.  ONE: one vertex per thread (tiles whose updatable count fits the
// block); each thread loads its table row once per pass into registers, so
// the iterations of the pass make no global reads.
// MINB > 0: at least MINB resident blocks per SM (the compiler keeps the
// registers per thread at or under 65536 / (MINB * THREADS); the per-vertex
// arithmetic fits 48 registers without spills), so more warps hide the
// latency of the table reads when the tiles' shared memory allows it.
template <int THREADS, bool PF, bool SMT = false, bool ONE = false, int MINB = 0>
__global__ void __launch_bounds__(THREADS, MINB > 0 ? MINB : (PF ? 768 : 1024) / THREADS) erosion_tb_kernel(TbArgs a)
{
    extern __shared__ float4 tsm4[];
    const int2 bm = a.blk_map[blockIdx.x];
    const nx_erosion_planet P = a.planets[bm.x];
    const int R = a.R;
    const int np = tb_npass(P.iters, R);
    const int q = a.pass - P.t_start;            // the planet's own pass
    if (q < 0 || q >= np) return;
    const int len = tb_len(P.iters, R, np, q);
    const nx_tiling TL = *P.tiling;
    nx_erosion_ctl *c = a.ctl + P.slot;
    if (TL.rings < len) {                        // tiling made for shorter passes
        if (threadIdx.x == 0) c->err = 2;
        return;
    }
    const int tile = bm.y;
    const int32_t *cnt = TL.counts + (int64_t)tile * (TL.rings + 1);
    const int T = cnt[0];
    int NL = T;
    for (int r = 1; r <= len; ++r) NL += cnt[r];
    // rescale per pass: growth is below 16x per iteration, so a max under
    // 2^(96 - 4R) stays under 2^96 through the pass
    const float m = __uint_as_float(__ldg(&c->maxbits[q % 3]));
    const float thr = __int_as_float((127 + 96 - 4 * R) << 23);
    const int shift = m > thr ? RESCALE_SHIFT : 0;
    const int K = __ldg(&c->K[q & 1]) + shift;
    const float lam = shift ? __int_as_float((127 - shift) << 23) : 1.0f;
    const float rain = scalbnf(P.rain, -K);
    if (tile == 0 && threadIdx.x == 0) {
        c->K[(q + 1) & 1] = K;
        c->maxbits[(q + 2) % 3] = 0u;
    }
    if (T == 0) return;
    const bool par = ((np - q) & 1) != 0;
    const float4 *__restrict__ ist = par ? a.st1 : a.st0;
    float4 *__restrict__ ost = par ? a.st0 : a.st1;
    // rows (h_hi, h_lo, w_hi, w_lo), the water including the rain of the
    // iteration about to read it; sediment pairs apart
    float4 *buf0 = tsm4, *buf1 = tsm4 + a.smem_n;
    float2 *sed = reinterpret_cast<float2 *>(tsm4 + 2 * a.smem_n);
    const int32_t *ids = TL.ids + (int64_t)tile * TL.nmax;
    const uint32_t *lnb = reinterpret_cast<const uint32_t *>(TL.lnbr) + (int64_t)tile * TL.cmax * 3;
    const float4 *led = reinterpret_cast<const float4 *>(TL.ledge) + (int64_t)tile * TL.cmax * 3;
    const int C0 = NL - cnt[len];                // members + rings 1..len-1: the rows this pass updates
    if (SMT) {
        // tables of rows [0, C0): edge pairs as float4s, neighbour indices as
        // 16-byte units (the tile's slice starts 16-byte aligned: cmax*12 is a
        // multiple of 16 and C0 < cmax leaves room to round up)
        float4 *sled = reinterpret_cast<float4 *>(sed + a.smem_n + (a.smem_n & 1));
        uint4 *slnb = reinterpret_cast<uint4 *>(sled + 3 * a.smem_c);
        for (int r = threadIdx.x; r < 3 * C0; r += THREADS) sled[r] = __ldg(led + r);
        const uint4 *g = reinterpret_cast<const uint4 *>(lnb);
        for (int r = threadIdx.x; r < (C0 * 3 + 3) / 4; r += THREADS) slnb[r] = __ldg(g + r);
        led = sled;
        lnb = reinterpret_cast<const uint32_t *>(slnb);
    }
    TileRow myrow;
    if (ONE) {
        if (C0 > THREADS) {                      // tile too large for one vertex per thread
            if (threadIdx.x == 0) c->err = 3;
            return;
        }
        if ((int)threadIdx.x < C0) myrow = tile_row<false>(lnb, led, threadIdx.x);
    }
    // the planet's first pass of a fused run starts from the raw fBm sums
    const bool fresh = a.raw != nullptr && q == 0;
    float4 ic = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float eloh = (float)a.elo, elol = (float)(a.elo - (double)(float)a.elo);
    if (fresh) {
        __shared__ float4 s_ic;
        if (threadIdx.x == 0) s_ic = init_consts(a.minmax, bm.x, a.elo, a.ehi);
        __syncthreads();
        ic = s_ic;
    }
    // two rows per thread per round, both gathers in flight before either
    // is stored (halves the dependent DRAM round trips of the load phase)
    for (int l0 = threadIdx.x; l0 < NL; l0 += 2 * THREADS) {
        const int l1 = l0 + THREADS;
        const bool two = l1 < NL;
        const int64_t r0 = P.vbeg + ids[l0];
        const int64_t r1 = two ? P.vbeg + ids[l1] : r0;
        float4 x0, y0, x1, y1;
        if (fresh) {
            // the state erosion_init_kernel would have written
            const float2 g0 = a.raw[r0], g1 = a.raw[r1];
            const float2 h0 = init_height(g0, ic, eloh, elol), h1 = init_height(g1, ic, eloh, elol);
            x0 = make_float4(h0.x, h0.y, a.w0h, a.w0l);
            x1 = make_float4(h1.x, h1.y, a.w0h, a.w0l);
            y0 = y1 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            x0 = ist[2 * r0]; y0 = ist[2 * r0 + 1];
            x1 = ist[2 * r1]; y1 = ist[2 * r1 + 1];
        }
        const Pair w0 = prain(__fmul_rn(x0.z, lam), __fmul_rn(x0.w, lam), rain);
        buf0[l0] = make_float4(__fmul_rn(x0.x, lam), __fmul_rn(x0.y, lam), w0.h, w0.l);
        sed[l0] = make_float2(__fmul_rn(y0.x, lam), __fmul_rn(y0.y, lam));
        if (two) {
            const Pair w1 = prain(__fmul_rn(x1.z, lam), __fmul_rn(x1.w, lam), rain);
            buf0[l1] = make_float4(__fmul_rn(x1.x, lam), __fmul_rn(x1.y, lam), w1.h, w1.l);
            sed[l1] = make_float2(__fmul_rn(y1.x, lam), __fmul_rn(y1.y, lam));
        }
    }
    __syncthreads();
    int C = C0;
    for (int mi = 0; mi < len; ++mi) {
        const float4 *cur = (mi & 1) ? buf1 : buf0;
        float4 *nxt = (mi & 1) ? buf0 : buf1;
        const bool more = mi + 1 < len;          // rain for the next iteration in the pass
        if (ONE) {
            if ((int)threadIdx.x < C) tb_update(threadIdx.x, myrow, cur, nxt, sed, rain, more);
        } else {
            TileRow nextrow;
            if (PF && (int)threadIdx.x < C) nextrow = tile_row<SMT>(lnb, led, threadIdx.x);
            for (int l = threadIdx.x; l < C; l += THREADS) {
                TileRow row;
                if (PF) {
                    row = nextrow;
                    if (l + THREADS < C) nextrow = tile_row<SMT>(lnb, led, l + THREADS);
                } else {
                    row = tile_row<SMT>(lnb, led, l);
                }
                tb_update(l, row, cur, nxt, sed, rain, more);
            }
        }
        __syncthreads();
        if (more) C -= cnt[len - 1 - mi];
    }
    const float4 *fin = (len & 1) ? buf1 : buf0;
    float vmax = 0.0f;
    for (int l = threadIdx.x; l < T; l += blockDim.x) {
        const float4 v = fin[l];
        const float2 sv = sed[l];
        const int64_t row = P.vbeg + ids[l];
        ost[2 * row] = v;
        ost[2 * row + 1] = make_float4(sv.x, sv.y, 0.0f, 0.0f);
        vmax = fmaxf(vmax, fmaxf(fabsf(v.x), fmaxf(fabsf(v.z), fabsf(sv.x))));
    }
    __shared__ float s_wmax[THREADS / 32];
    vmax = warp_max(vmax);
    if ((threadIdx.x & 31) == 0) s_wmax[threadIdx.x >> 5] = vmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        float bmx = s_wmax[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) bmx = fmaxf(bmx, s_wmax[w]);
        atomicMax(&c->maxbits[(q + 1) % 3], __float_as_uint(bmx));
    }
}

// Block map of a temporally blocked run: planets ordered by pass count
// (descending, then index), each contributing one block per tile.
__global__ void erosion_tb_map_kernel(const nx_erosion_planet *__restrict__ P, int np, int R, int2 *__restrict__ map)
{
    const int p = blockIdx.x;
    if (p >= np) return;
    __shared__ int64_t s_b0;
    const int mine = tb_npass(P[p].iters, R);
    if (threadIdx.x == 0) {
        int64_t b0 = 0;
        for (int q = 0; q < np; ++q) {
            const int other = tb_npass(P[q].iters, R);
            if (other > mine || (other == mine && q < p)) b0 += P[q].ntiles;
        }
        s_b0 = b0;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < P[p].ntiles; j += blockDim.x) map[s_b0 + j] = make_int2(p, j);
}

__global__ void erosion_tb_rebase_kernel(const nx_erosion_planet *__restrict__ P, int np, int R,
                                         nx_erosion_ctl *__restrict__ ctl)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const int n = tb_npass(P[p].iters, R);
    if (n <= 0) return;
    nx_erosion_ctl &c = ctl[P[p].slot];
    const unsigned m = c.maxbits[n % 3];
    const int K = c.K[n & 1];
    c.maxbits[0] = m;
    c.maxbits[1] = 0u;
    c.maxbits[2] = 0u;
    c.K[0] = K;
    c.K[1] = K;
}

// Block map of a launch: planet p owns blocks [sum of earlier planets'
// blocks, + ceil(n_p / BLOCK)); one block per planet fills its entries.
__global__ void erosion_blkmap_kernel(const nx_erosion_planet *__restrict__ P, int np, int2 *__restrict__ map)
{
    const int p = blockIdx.x;
    if (p >= np) return;
    __shared__ int64_t s_b0;
    if (threadIdx.x == 0) {
        int64_t b0 = 0;
        for (int q = 0; q < p; ++q) b0 += (P[q].n + BLOCK - 1) / BLOCK;
        s_b0 = b0;
    }
    __syncthreads();
    const int64_t nb = (P[p].n + BLOCK - 1) / BLOCK;
    for (int64_t j = threadIdx.x; j < nb; j += blockDim.x) map[s_b0 + j] = make_int2(p, (int)j);
}

// After a run: move each planet's final scale exponent and max into slot 0
// so the state is self-describing (K[0]) and a later run starts at t = 0.
__global__ void erosion_rebase_kernel(const nx_erosion_planet *__restrict__ P, int np, nx_erosion_ctl *__restrict__ ctl)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    int it = P[p].iters;
    if (it <= 0) return;
    nx_erosion_ctl &c = ctl[P[p].slot];
    unsigned m = c.maxbits[it % 3];
    int K = c.K[it & 1];
    c.maxbits[0] = m;
    c.maxbits[1] = 0u;
    c.maxbits[2] = 0u;
    c.K[0] = K;
    c.K[1] = K;
}

// binary64 (h, w, s) -> scaled binary32 state in buffer B[iters & 1]; sets K
// so the largest magnitude lands near 2^64 or below.
__global__ void erosion_maxabs64_kernel(const double *__restrict__ h, const double *__restrict__ w,
                                        const double *__restrict__ s, int64_t n, unsigned long long *__restrict__ mbits)
{
    double m = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double a = fabs(h[i]);
        if (w) a = fmax(a, fabs(w[i]));
        if (s) a = fmax(a, fabs(s[i]));
        m = fmax(m, a);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mbits, (unsigned long long)__double_as_longlong(m));
}

__global__ void erosion_load64_kernel(const double *__restrict__ h, const double *__restrict__ w,
                                      const double *__restrict__ s, int64_t n, const unsigned long long *__restrict__ mbits,
                                      float4 *__restrict__ st, nx_erosion_ctl *__restrict__ ctl)
{
    double m = __longlong_as_double((long long)*mbits);
    int K = 0;
    if (m > 0x1p64) K = ilogb(m) - 64;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double hv = ldexp(h[i], -K), wv = w ? ldexp(w[i], -K) : 0.0, sv = s ? ldexp(s[i], -K) : 0.0;
        const float hh = (float)hv, wh = (float)wv, sh = (float)sv;
        st[2 * i] = make_float4(hh, (float)(hv - (double)hh), wh, (float)(wv - (double)wh));
        st[2 * i + 1] = make_float4(sh, (float)(sv - (double)sh), 0.0f, 0.0f);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        float mf = (float)ldexp(m, -K);
        ctl->maxbits[0] = __float_as_uint(mf);
        ctl->maxbits[1] = 0u;
        ctl->maxbits[2] = 0u;
        ctl->K[0] = K;
        ctl->K[1] = K;
        ctl->done = 0u;
        ctl->err = 0;
    }
}

__global__ void erosion_store64_kernel(const float4 *__restrict__ st, int64_t n, const nx_erosion_ctl *__restrict__ ctl,
                                       double *__restrict__ h, double *__restrict__ w, double *__restrict__ so)
{
    const int K = ctl->K[0];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 v = st[2 * i], b = st[2 * i + 1];
        h[i] = ldexp((double)v.x + (double)v.y, K);
        if (w) w[i] = ldexp((double)v.z + (double)v.w, K);
        if (so) so[i] = ldexp((double)b.x + (double)b.y, K);
    }
}

// Rows of the packed planets handed to the init and heights kernels: units
// of 4 x 256 rows, unit u to block u mod grid (consecutive blocks sweep
// consecutive rows), thread t of a block the rows base + t + 256 k, k < 4.
// A thread finds its first row's planet by binary search and then walks to
// the next planet when its row reaches that planet's vbeg: no per-block
// search or barrier.  Rows outside every planet (alignment padding) are
// skipped.
struct PlanetWalk {
    int p;
    int64_t beg, end, next;

    __device__ __forceinline__ void seek(const nx_erosion_planet *P, int np, int64_t row)
    {
        p = find_planet(P, np, row);
        span(P, np);
    }
    __device__ __forceinline__ void span(const nx_erosion_planet *P, int np)
    {
        beg = P[p].vbeg;
        end = beg + P[p].n;
        next = p + 1 < np ? P[p + 1].vbeg : INT64_MAX;
    }
    // advance to the planet of `row` (rows increase); true if it changed
    __device__ __forceinline__ bool to(const nx_erosion_planet *P, int np, int64_t row)
    {
        if (row < next) return false;
        do {
            ++p;
            span(P, np);
        } while (row >= next);
        return true;
    }
    __device__ __forceinline__ bool has(int64_t row) const { return row >= beg && row < end; }
    // rows row + 256 k, k < WALK_UNROLL, all in this planet
    __device__ __forceinline__ bool all(int64_t row) const;
};

constexpr int WALK_UNROLL = 4;
constexpr int64_t WALK_UNIT = WALK_UNROLL * 256;

__device__ __forceinline__ bool PlanetWalk::all(int64_t row) const
{
    return row >= beg && row + (WALK_UNROLL - 1) * 256 < end;
}

int walk_grid(int64_t total)
{
    const int64_t units = (total + WALK_UNIT - 1) / WALK_UNIT;
    const int64_t cap = (int64_t)nx::sm_count() * 8;
    return (int)(units < cap ? units : cap);
}

// Planets whose rescale constants the init kernel stages in shared memory
// (beyond that each thread forms its planet's constants itself).
constexpr int INIT_SMEM_PLANETS = 1024;

// util.rescale (util.py:110-140) of the raw fBm pair sums to [lo, hi], and
// the initial state (h as a pair, water0 as a pair | 0, 0, 0, 0) in the
// buffer the planet's first iteration reads: B[iters & 1].  The reference
// computes ((x - min) / (max - min)) * (hi - lo) + lo in binary64; here
// (x - min) * f + lo with f = (hi - lo) / (max - min) formed once per
// planet in binary64 (min and max are exact as binary64) and the per-vertex
// arithmetic in pairs, within ~2^-47 of the value.  A constant field
// (max == min) gives NaN, as the reference's division does.  Rows from row0
// (256-aligned) to total.  Dynamic shared memory: a float4 per planet when
// np <= INIT_SMEM_PLANETS, else none.
__global__ void __launch_bounds__(256) erosion_init_kernel(const nx_erosion_planet *__restrict__ P, int np,
                                                           const float2 *__restrict__ raw,
                                                           const unsigned long long *__restrict__ minmax,
                                                           double lo, double hi, float w0h, float w0l,
                                                           float4 *__restrict__ st0, float4 *__restrict__ st1,
                                                           int64_t row0, int64_t total)
{
    extern __shared__ float4 s_ic[];
    const bool staged = np <= INIT_SMEM_PLANETS;
    if (staged) {
        for (int i = threadIdx.x; i < np; i += blockDim.x) s_ic[i] = init_consts(minmax, i, lo, hi);
        __syncthreads();
    }
    const float loh = (float)lo, lol = (float)(lo - (double)(float)lo);
    int64_t base = row0 + (int64_t)blockIdx.x * WALK_UNIT;
    if (base + threadIdx.x >= total) return;
    PlanetWalk W;
    W.seek(P, np, base + threadIdx.x);
    float4 c = staged ? s_ic[W.p] : init_consts(minmax, W.p, lo, hi);
    float4 *dst = (P[W.p].iters & 1) ? st1 : st0;
    for (; base < total; base += (int64_t)gridDim.x * WALK_UNIT) {
        const int64_t row = base + threadIdx.x;
        if (W.all(row)) {
            // the four rows lie in the current planet: loads in flight together
            float2 r[WALK_UNROLL];
#pragma unroll
            for (int u = 0; u < WALK_UNROLL; ++u) r[u] = raw[row + u * 256];
#pragma unroll
            for (int u = 0; u < WALK_UNROLL; ++u) {
                const float2 h = init_height(r[u], c, loh, lol);
                const int64_t x = row + u * 256;
                dst[2 * x] = make_float4(h.x, h.y, w0h, w0l);
                dst[2 * x + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
            continue;
        }
        for (int u = 0; u < WALK_UNROLL; ++u) {
            const int64_t x = row + u * 256;
            if (x >= total) break;
            if (W.to(P, np, x)) {
                c = staged ? s_ic[W.p] : init_consts(minmax, W.p, lo, hi);
                dst = (P[W.p].iters & 1) ? st1 : st0;
            }
            if (!W.has(x)) continue;
            const float2 h = init_height(raw[x], c, loh, lol);
            dst[2 * x] = make_float4(h.x, h.y, w0h, w0l);
            dst[2 * x + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
}

// Heights of every planet after its run: (h_hi + h_lo) * 2^K in binary64,
// formed as h_hi 2^K + h_lo 2^K (both exact) with one rounding: the same
// bits as rounding h_hi + h_lo and then scaling.
__global__ void __launch_bounds__(256) erosion_heights_kernel(const nx_erosion_planet *__restrict__ P, int np,
                                                              const float4 *__restrict__ st,
                                                              const nx_erosion_ctl *__restrict__ ctl,
                                                              double *__restrict__ out, int64_t total)
{
    int64_t base = (int64_t)blockIdx.x * WALK_UNIT;
    if (base + threadIdx.x >= total) return;
    PlanetWalk W;
    W.seek(P, np, base + threadIdx.x);
    int K = ctl[P[W.p].slot].K[0];
    for (; base < total; base += (int64_t)gridDim.x * WALK_UNIT) {
        const int64_t row = base + threadIdx.x;
        if (W.all(row)) {
            float2 v[WALK_UNROLL];
#pragma unroll
            for (int u = 0; u < WALK_UNROLL; ++u) {
                const float4 s = st[2 * (row + u * 256)];
                v[u] = make_float2(s.x, s.y);
            }
#pragma unroll
            for (int u = 0; u < WALK_UNROLL; ++u) out[row + u * 256] = f32_scaled(v[u].x, K) + f32_scaled(v[u].y, K);
            continue;
        }
        for (int u = 0; u < WALK_UNROLL; ++u) {
            const int64_t x = row + u * 256;
            if (x >= total) break;
            if (W.to(P, np, x)) K = ctl[P[W.p].slot].K[0];
            if (!W.has(x)) continue;
            const float4 s = st[2 * x];
            out[x] = f32_scaled(s.x, K) + f32_scaled(s.y, K);
        }
    }
}

// find_lowest (erosion.py:398-406, util.py:580-587): position, within the
// neighbours that are not -1, of the first lowest one if it is strictly
// lower than the vertex, else -1; `vid` gets that neighbour's id (or -1).
__global__ void steepest_kernel(const int32_t *__restrict__ nbr, const double *__restrict__ h, int64_t n,
                                int32_t *__restrict__ pos, int32_t *__restrict__ vid)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int m = 0, best = -1, bestv = -1;
        double low = 0.0;
        for (int k = 0; k < 6; ++k) {
            int j = nbr[6 * i + k];
            if (j == -1) continue;
            double hj = ((uint64_t)(uint32_t)j < (uint64_t)n) ? h[j] : __longlong_as_double(0x7FF8000000000000LL);
            if (m == 0 || hj < low) { low = hj; best = m; bestv = j; }
            ++m;
        }
        bool ok = m > 0 && low < h[i];
        pos[i] = ok ? best : -1;
        if (vid) vid[i] = ok ? bestv : -1;
    }
}

int grid1d(int64_t n, int block = 256)
{
    int64_t g = (n + block - 1) / block;
    int64_t cap = (int64_t)nx::sm_count() * 16;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

// Workspace: control blocks (one per slot), then per launch block 3 partial
// sums (float64) and one block-map entry (int2).
NX_EXPORT size_t nx_erosion_workspace_size(int64_t n_padded_total, int nplanets)
{
    int64_t nblk = (n_padded_total + BLOCK - 1) / BLOCK;
    if (nblk < 1) nblk = 1;
    return sizeof(nx_erosion_ctl) * (size_t)(nplanets > 0 ? nplanets : 1) + (3 * sizeof(double) + sizeof(int2)) * (size_t)nblk + 64;
}

namespace {

struct Workspace {
    nx_erosion_ctl *ctl;
    double *partials;
    int2 *blk_map;
};

Workspace carve(void *ws, int nslots, int64_t nblk)
{
    Workspace w;
    w.ctl = (nx_erosion_ctl *)ws;
    uintptr_t p = (uintptr_t)(w.ctl + nslots);
    p = (p + 15) & ~(uintptr_t)15;
    w.partials = (double *)p;
    w.blk_map = (int2 *)(w.partials + 3 * nblk);
    return w;
}

}  // namespace

NX_EXPORT int nx_erosion_load(const double *h64_dev, const double *w64_dev, const double *s64_dev, int64_t n,
                              float *st_dev, void *workspace, size_t ws_bytes, void *stream)
{
    if (n <= 0) return nx::fail(NX_EINVAL, "nx_erosion_load: n must be > 0");
    if (!h64_dev || !st_dev || !workspace) return nx::fail(NX_EINVAL, "nx_erosion_load: null pointer");
    if (ws_bytes < nx_erosion_workspace_size(n, 1)) return nx::fail(NX_EINVAL, "nx_erosion_load: workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    Workspace w = carve(workspace, 1, (n + BLOCK - 1) / BLOCK);
    unsigned long long *mb = (unsigned long long *)w.partials;   // first partial slot as scratch
    NX_CHECK_CUDA(cudaMemsetAsync(mb, 0, sizeof(unsigned long long), s));
    erosion_maxabs64_kernel<<<grid1d(n), 256, 0, s>>>(h64_dev, w64_dev, s64_dev, n, mb);
    NX_CHECK_LAUNCH("erosion_maxabs64_kernel");
    erosion_load64_kernel<<<grid1d(n), 256, 0, s>>>(h64_dev, w64_dev, s64_dev, n, mb, (float4 *)st_dev, w.ctl);
    NX_CHECK_LAUNCH("erosion_load64_kernel");
    nx::note_launch(2);
    return NX_OK;
}

static int64_t planet_blocks(const nx_erosion_planet &P) { return (P.n + BLOCK - 1) / BLOCK; }

// Temporal blocking: rings of the tilings in use (all planets of a batch
// share it) and a switch for comparisons.
static int g_tb_rings = 4;
static int g_tb_threads = 512;
static int g_tb_variant = 0;
static bool g_tb_enabled = true;

NX_EXPORT int nx_erosion_tb_config(int rings, int threads, int variant, int enabled)
{
    if (rings < 1 || rings > 8) return nx::fail(NX_EINVAL, "nx_erosion_tb_config: rings must be in [1, 8]");
    const bool ok = variant == 1 ? (threads == 256 || threads == 384)
                  : (variant == 2 || variant == 3) ? (threads == 512 || threads == 1024)
                  : variant == 0 ? (threads == 256 || threads == 512 || threads == 1024)
                  : variant == 4 ? (threads == 256 || threads == 320 || threads == 384 || threads == 640)
                  : variant == 5 ? threads == 256 : false;
    if (!ok)
        return nx::fail(NX_EINVAL, "nx_erosion_tb_config: threads %d do not go with variant %d", threads, variant);
    g_tb_rings = rings;
    g_tb_threads = threads;
    g_tb_variant = variant;
    g_tb_enabled = enabled != 0;
    return NX_OK;
}

// Shared memory of a launch of the configured variant.
static size_t tb_launch_smem(int maxnl, int maxc)
{
    size_t b = tb_smem_bytes(maxnl + (maxnl & 1));
    if (g_tb_variant == 2) b += tb_table_bytes(maxc);
    return b;
}

static cudaError_t launch_tb(int64_t grid, size_t smem, cudaStream_t s, const TbArgs &ta)
{
    if (g_tb_variant == 1) {
        if (g_tb_threads == 256) erosion_tb_kernel<256, true><<<(unsigned)grid, 256, smem, s>>>(ta);
        else erosion_tb_kernel<384, true><<<(unsigned)grid, 384, smem, s>>>(ta);
    } else if (g_tb_variant == 2) {
        if (g_tb_threads == 512) erosion_tb_kernel<512, false, true><<<(unsigned)grid, 512, smem, s>>>(ta);
        else erosion_tb_kernel<1024, false, true><<<(unsigned)grid, 1024, smem, s>>>(ta);
    } else if (g_tb_variant == 3) {
        if (g_tb_threads == 512) erosion_tb_kernel<512, false, false, true><<<(unsigned)grid, 512, smem, s>>>(ta);
        else erosion_tb_kernel<1024, false, false, true><<<(unsigned)grid, 1024, smem, s>>>(ta);
    } else if (g_tb_variant == 4) {
        switch (g_tb_threads) {
        case 256: erosion_tb_kernel<256, false, false, false, 5><<<(unsigned)grid, 256, smem, s>>>(ta); break;
        case 320: erosion_tb_kernel<320, false, false, false, 4><<<(unsigned)grid, 320, smem, s>>>(ta); break;
        case 640: erosion_tb_kernel<640, false, false, false, 2><<<(unsigned)grid, 640, smem, s>>>(ta); break;
        default: erosion_tb_kernel<384, false, false, false, 3><<<(unsigned)grid, 384, smem, s>>>(ta); break;
        }
    } else if (g_tb_variant == 5) {
        erosion_tb_kernel<256, false, false, false, 6><<<(unsigned)grid, 256, smem, s>>>(ta);
    } else {
        switch (g_tb_threads) {
        case 256: erosion_tb_kernel<256, false><<<(unsigned)grid, 256, smem, s>>>(ta); break;
        case 1024: erosion_tb_kernel<1024, false><<<(unsigned)grid, 1024, smem, s>>>(ta); break;
        default: erosion_tb_kernel<512, false><<<(unsigned)grid, 512, smem, s>>>(ta); break;
        }
    }
    return cudaGetLastError();
}

// Shared-memory limit of the blocked kernel, set once per device.
static int tb_prepare()
{
    static std::mutex mu;
    static bool done[64] = {false};
    int dev = 0;
    NX_CHECK_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return nx::fail(NX_EINVAL, "erosion: device id %d out of range", dev);
    std::lock_guard<std::mutex> lk(mu);
    if (!done[dev]) {
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<512, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<1024, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<512, false, false, true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<1024, false, false, true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<384, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<256, false, false, false, 5>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<384, false, false, false, 3>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<256, false, false, false, 6>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<320, false, false, false, 4>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<640, false, false, false, 2>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        int optin = 0;
        NX_CHECK_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        cudaFuncAttributes fa512, fa1024;
        NX_CHECK_CUDA(cudaFuncGetAttributes(&fa512, erosion_tb_kernel<512, false, true>));
        NX_CHECK_CUDA(cudaFuncGetAttributes(&fa1024, erosion_tb_kernel<1024, false, true>));
        const size_t st = fa512.sharedSizeBytes > fa1024.sharedSizeBytes ? fa512.sharedSizeBytes : fa1024.sharedSizeBytes;
        TB_SMEM_MAX = (size_t)optin > st ? (size_t)optin - st : 0;
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<512, false, true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TB_SMEM_MAX));
        NX_CHECK_CUDA(cudaFuncSetAttribute(erosion_tb_kernel<1024, false, true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TB_SMEM_MAX));
        done[dev] = true;
    }
    return NX_OK;
}

// Batch: planets packed by non-increasing iteration count, so the planets
// still running at iteration t are a prefix of the block map.  allow_tb:
// whether the descriptors' tiling fields may be read at all (the
// single-planet entry points build descriptors without a tiling and pass 0,
// so their runs never depend on those fields).
// How a batch runs: validated sizes, and whether it runs temporally blocked
// (every eroding planet has a tiling and nothing per iteration -- mass
// sums, flow bits -- is requested).
struct BatchPlan {
    bool tb = false;
    int R = 0, maxnl = 0, maxc = 0, max_it = 0;
    int64_t total = 0, nblk = 0, ntiles_all = 0;
};

static int plan_batch(const nx_erosion_planet *planets_host, int np, bool allow_tb, BatchPlan &pl)
{
    pl = BatchPlan();
    for (int p = 0; p < np; ++p) {
        const nx_erosion_planet &P = planets_host[p];
        if (P.vbeg < 0 || P.n < 0 || P.iters < 0 || P.slot != p || P.t_start != 0)
            return nx::fail(NX_EINVAL, "erosion: planet %d: bad descriptor (slot must be its index, t_start 0)", p);
        if (P.n > 0 && (!P.nbr || !P.edge)) return nx::fail(NX_EINVAL, "erosion: planet %d has no mesh", p);
        if (p > 0 && P.iters > planets_host[p - 1].iters)
            return nx::fail(NX_EINVAL, "erosion: planets must be ordered by non-increasing iterations");
        if (P.iters > pl.max_it) pl.max_it = P.iters;
        if (P.vbeg + P.n > pl.total) pl.total = P.vbeg + P.n;
        pl.nblk += planet_blocks(P);
    }
    bool tb = allow_tb && g_tb_enabled;
    for (int p = 0; p < np && tb; ++p) {
        const nx_erosion_planet &P = planets_host[p];
        if (P.iters == 0) {
            if (P.tiling && P.ntiles > 0) pl.ntiles_all += P.ntiles;
            continue;
        }
        if (!P.tiling || P.ntiles <= 0 || P.maxnl <= 0) { tb = false; break; }
        if (g_tb_variant >= 2 && P.maxc <= 0)
            return nx::fail(NX_EINVAL, "erosion: planet %d has no maxc (needed by blocked-kernel variant %d)", p,
                            g_tb_variant);
        if (g_tb_variant == 3 && P.maxc > g_tb_threads)
            return nx::fail(NX_EINVAL, "erosion: planet %d: tiles of %d updatable vertices exceed %d threads (variant 3)",
                            p, P.maxc, g_tb_threads);
        pl.ntiles_all += P.ntiles;
        if (P.maxnl > pl.maxnl) pl.maxnl = P.maxnl;
        if (P.maxc > pl.maxc) pl.maxc = P.maxc;
    }
    if (pl.maxnl == 0) tb = false;
    if (tb) {
        pl.R = g_tb_rings;
        int rc = tb_prepare();
        if (rc) return rc;
        if (tb_launch_smem(pl.maxnl, pl.maxc) > (g_tb_variant == 2 ? TB_SMEM_MAX : 200 * 1024)) tb = false;
    }
    pl.tb = tb;
    return NX_OK;
}

// fuse (blocked path only): the fusion fields of TbArgs (raw sums and
// rescale constants for the planets' first passes).
static int run_batch(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host, int np,
                     float *st_dev, float *st_tmp, double *mass_dev, uint16_t *flow_dev, void *workspace,
                     size_t ws_bytes, cudaStream_t s, bool allow_tb, const TbArgs *fuse = nullptr)
{
    if (np <= 0) return NX_OK;
    if (!planets_dev || !planets_host || !st_dev || !st_tmp || !workspace)
        return nx::fail(NX_EINVAL, "erosion: null pointer");
    BatchPlan pl;
    int rc = plan_batch(planets_host, np, allow_tb && !mass_dev && !flow_dev, pl);
    if (rc) return rc;
    const bool tb = pl.tb;
    const int R = pl.R, maxnl = pl.maxnl, maxc = pl.maxc, max_it = pl.max_it;
    const int64_t nblk = pl.nblk, ntiles_all = pl.ntiles_all;
    if (fuse && !tb) return nx::fail(NX_EINVAL, "erosion: fused steps need the blocked path");
    if (tb) {
        if (ws_bytes < nx_erosion_workspace_size((ntiles_all > nblk ? ntiles_all : nblk) * BLOCK, np))
            return nx::fail(NX_EINVAL, "erosion: workspace too small");
        Workspace w = carve(workspace, np, ntiles_all > nblk ? ntiles_all : nblk);
        erosion_tb_map_kernel<<<np, 256, 0, s>>>(planets_dev, np, R, w.blk_map);
        NX_CHECK_LAUNCH("erosion_tb_map_kernel");
        nx::note_launch(1);
        int maxpass = 0;
        for (int p = 0; p < np; ++p) {
            const int n = tb_npass(planets_host[p].iters, R);
            if (n > maxpass) maxpass = n;
        }
        TbArgs ta;
        ta.planets = planets_dev;
        ta.blk_map = w.blk_map;
        ta.R = R;
        ta.smem_n = maxnl;
        ta.smem_c = maxc;
        ta.st0 = (float4 *)st_dev;
        ta.st1 = (float4 *)st_tmp;
        ta.ctl = w.ctl;
        if (fuse) {
            ta.raw = fuse->raw;
            ta.minmax = fuse->minmax;
            ta.elo = fuse->elo;
            ta.ehi = fuse->ehi;
            ta.w0h = fuse->w0h;
            ta.w0l = fuse->w0l;
        }
        const size_t smem = tb_launch_smem(maxnl, maxc);
        for (int q = 0; q < maxpass; ++q) {
            int64_t grid = 0;
            for (int p = 0; p < np; ++p)
                if (tb_npass(planets_host[p].iters, R) > q) grid += planets_host[p].ntiles;
            if (grid <= 0) break;
            ta.pass = q;
            NX_CHECK_CUDA(launch_tb(grid, smem, s, ta));
            nx::note_launch(1);
        }
        if (maxpass > 0) {
            erosion_tb_rebase_kernel<<<(np + 127) / 128, 128, 0, s>>>(planets_dev, np, R, w.ctl);
            NX_CHECK_LAUNCH("erosion_tb_rebase_kernel");
            nx::note_launch(1);
        }
        return NX_OK;
    }
    if (ws_bytes < nx_erosion_workspace_size(nblk * BLOCK, np)) return nx::fail(NX_EINVAL, "erosion: workspace too small");
    Workspace w = carve(workspace, np, nblk);
    StepArgs a;
    a.planets = planets_dev;
    a.blk_map = w.blk_map;
    a.st0 = (float4 *)st_dev;
    a.st1 = (float4 *)st_tmp;
    a.ctl = w.ctl;
    a.partials = w.partials;
    a.mass = mass_dev;
    a.mass_np = np;
    a.flow = flow_dev;
    if (max_it > 0) {
        erosion_blkmap_kernel<<<np, 256, 0, s>>>(planets_dev, np, w.blk_map);
        NX_CHECK_LAUNCH("erosion_blkmap_kernel");
        nx::note_launch(1);
    }
    int last = np - 1;
    int64_t grid = nblk;
    for (int t = 0; t < max_it; ++t) {
        while (last >= 0 && planets_host[last].iters <= t) {
            grid -= planet_blocks(planets_host[last]);
            --last;
        }
        if (last < 0 || grid <= 0) break;
        a.t = t;
        erosion_step_kernel<<<(unsigned)grid, BLOCK, 0, s>>>(a);
        NX_CHECK_LAUNCH("erosion_step_kernel");
        nx::note_launch(1);
    }
    if (max_it > 0) {
        erosion_rebase_kernel<<<(np + 127) / 128, 128, 0, s>>>(planets_dev, np, w.ctl);
        NX_CHECK_LAUNCH("erosion_rebase_kernel");
        nx::note_launch(1);
    }
    return NX_OK;
}

// Serving: one launch advances every listed planet by one iteration, each
// at its own iteration t - t_start (planets outside [0, iters) are skipped).
NX_EXPORT int nx_erosion_ticks(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host,
                               int nplanets, int t, int nticks, float *st_dev, float *st_tmp_dev, void *workspace,
                               size_t ws_bytes, int nslots, int remap, void *stream);

NX_EXPORT int nx_erosion_tick(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host, int nplanets,
                              int t, float *st_dev, float *st_tmp_dev, void *workspace, size_t ws_bytes, int nslots,
                              int remap, void *stream)
{
    return nx_erosion_ticks(planets_dev, planets_host, nplanets, t, 1, st_dev, st_tmp_dev, workspace, ws_bytes, nslots,
                            remap, stream);
}

NX_EXPORT int nx_erosion_ticks(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host,
                               int nplanets, int t, int nticks, float *st_dev, float *st_tmp_dev, void *workspace,
                               size_t ws_bytes, int nslots, int remap, void *stream)
{
    if (nplanets <= 0) return NX_OK;
    if (!planets_dev || !planets_host || !st_dev || !st_tmp_dev || !workspace || nslots <= 0)
        return nx::fail(NX_EINVAL, "nx_erosion_tick: bad arguments");
    int64_t nblk = 0;
    for (int p = 0; p < nplanets; ++p) {
        const nx_erosion_planet &P = planets_host[p];
        if (P.vbeg < 0 || P.n < 0 || P.iters < 0 || P.slot < 0 || P.slot >= nslots || (P.n > 0 && (!P.nbr || !P.edge)))
            return nx::fail(NX_EINVAL, "nx_erosion_tick: planet %d: bad descriptor", p);
        nblk += planet_blocks(P);
    }
    if (ws_bytes < nx_erosion_workspace_size(nblk * BLOCK, nslots))
        return nx::fail(NX_EINVAL, "nx_erosion_tick: workspace too small");
    if (nblk == 0) return NX_OK;
    cudaStream_t s = (cudaStream_t)stream;
    Workspace w = carve(workspace, nslots, nblk);
    if (remap) {
        erosion_blkmap_kernel<<<nplanets, 256, 0, s>>>(planets_dev, nplanets, w.blk_map);
        NX_CHECK_LAUNCH("erosion_blkmap_kernel");
        nx::note_launch(1);
    }
    StepArgs a;
    a.planets = planets_dev;
    a.blk_map = w.blk_map;
    a.t = t;
    a.st0 = (float4 *)st_dev;
    a.st1 = (float4 *)st_tmp_dev;
    a.ctl = w.ctl;
    a.partials = w.partials;
    a.mass = nullptr;
    a.mass_np = 0;
    a.flow = nullptr;
    for (int q = 0; q < nticks; ++q) {
        a.t = t + q;
        erosion_step_kernel<<<(unsigned)nblk, BLOCK, 0, s>>>(a);
        NX_CHECK_LAUNCH("erosion_step_kernel");
        nx::note_launch(1);
    }
    return NX_OK;
}

// Serving, temporally blocked: each launch advances every listed planet by
// one pass (up to R iterations), planet p at its own pass
// pass - t_start; planets outside [0, npass) skip.
NX_EXPORT int nx_erosion_passes(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host,
                                int nplanets, int pass, int npasses, float *st_dev, float *st_tmp_dev, void *workspace,
                                size_t ws_bytes, int nslots, int remap, void *stream)
{
    if (nplanets <= 0 || npasses <= 0) return NX_OK;
    if (!planets_dev || !planets_host || !st_dev || !st_tmp_dev || !workspace || nslots <= 0)
        return nx::fail(NX_EINVAL, "nx_erosion_passes: bad arguments");
    int64_t ntiles = 0;
    int maxnl = 0, maxc = 0;
    for (int p = 0; p < nplanets; ++p) {
        const nx_erosion_planet &P = planets_host[p];
        if (P.vbeg < 0 || P.n < 0 || P.iters < 0 || P.slot < 0 || P.slot >= nslots || (P.n > 0 && (!P.nbr || !P.edge)))
            return nx::fail(NX_EINVAL, "nx_erosion_passes: planet %d: bad descriptor", p);
        if (!P.tiling || P.ntiles <= 0 || P.maxnl <= 0)
            return nx::fail(NX_EINVAL, "nx_erosion_passes: planet %d has no tiling", p);
        if (g_tb_variant >= 2 && P.maxc <= 0)
            return nx::fail(NX_EINVAL, "nx_erosion_passes: planet %d has no maxc (needed by variant %d)", p, g_tb_variant);
        if (g_tb_variant == 3 && P.maxc > g_tb_threads)
            return nx::fail(NX_EINVAL, "nx_erosion_passes: planet %d: tiles exceed %d threads (variant 3)", p,
                            g_tb_threads);
        ntiles += P.ntiles;
        if (P.maxnl > maxnl) maxnl = P.maxnl;
        if (P.maxc > maxc) maxc = P.maxc;
    }
    int rc = tb_prepare();
    if (rc) return rc;
    if (tb_launch_smem(maxnl, maxc) > (g_tb_variant == 2 ? TB_SMEM_MAX : 200 * 1024))
        return nx::fail(NX_EINVAL, "nx_erosion_passes: tiles too large");
    if (ws_bytes < nx_erosion_workspace_size(ntiles * BLOCK, nslots))
        return nx::fail(NX_EINVAL, "nx_erosion_passes: workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    Workspace w = carve(workspace, nslots, ntiles);
    const int R = g_tb_rings;
    if (remap) {
        erosion_tb_map_kernel<<<nplanets, 256, 0, s>>>(planets_dev, nplanets, R, w.blk_map);
        NX_CHECK_LAUNCH("erosion_tb_map_kernel");
        nx::note_launch(1);
    }
    TbArgs ta;
    ta.planets = planets_dev;
    ta.blk_map = w.blk_map;
    ta.R = R;
    ta.smem_n = maxnl;
    ta.smem_c = maxc;
    ta.st0 = (float4 *)st_dev;
    ta.st1 = (float4 *)st_tmp_dev;
    ta.ctl = w.ctl;
    for (int q = 0; q < npasses; ++q) {
        ta.pass = pass + q;
        NX_CHECK_CUDA(launch_tb(ntiles, tb_launch_smem(maxnl, maxc), s, ta));
        nx::note_launch(1);
    }
    return NX_OK;
}

// Passes a planet of `iters` iterations makes (temporally blocked runs).
NX_EXPORT int nx_erosion_npass(int iters) { return tb_npass(iters, g_tb_rings); }

// After a planet's last iteration: its final scale exponent into K[0].
NX_EXPORT int nx_erosion_finish(const nx_erosion_planet *planets_dev, int nplanets, void *workspace, void *stream)
{
    if (nplanets <= 0) return NX_OK;
    if (!planets_dev || !workspace) return nx::fail(NX_EINVAL, "nx_erosion_finish: null pointer");
    erosion_rebase_kernel<<<(nplanets + 127) / 128, 128, 0, (cudaStream_t)stream>>>(planets_dev, nplanets,
                                                                                    (nx_erosion_ctl *)workspace);
    NX_CHECK_LAUNCH("erosion_rebase_kernel");
    nx::note_launch(1);
    return NX_OK;
}

// The same after a planet's last blocked pass (nx_erosion_passes): its
// control slots rotate per pass, so the final ones are those of its pass
// count, not of its iteration count.
NX_EXPORT int nx_erosion_finish_passes(const nx_erosion_planet *planets_dev, int nplanets, void *workspace,
                                       void *stream)
{
    if (nplanets <= 0) return NX_OK;
    if (!planets_dev || !workspace) return nx::fail(NX_EINVAL, "nx_erosion_finish_passes: null pointer");
    erosion_tb_rebase_kernel<<<(nplanets + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
        planets_dev, nplanets, g_tb_rings, (nx_erosion_ctl *)workspace);
    NX_CHECK_LAUNCH("erosion_tb_rebase_kernel");
    nx::note_launch(1);
    return NX_OK;
}

NX_EXPORT int nx_erosion_steps(const int32_t *nbr_dev, const float *edge_dev, int64_t n, float *st_dev,
                               float *st_tmp_dev, int iters, float rain, nx_erosion_planet *planet_dev,
                               double *mass_dev, uint16_t *flow_dev, void *workspace, size_t ws_bytes, void *stream)
{
    if (n <= 0 || iters < 0) return nx::fail(NX_EINVAL, "nx_erosion_steps: bad n or iters");
    if (!planet_dev) return nx::fail(NX_EINVAL, "nx_erosion_steps: planet descriptor (device) required");
    nx_erosion_planet P = {};   // no tiling: every field not set below is zero
    P.vbeg = 0;
    P.n = n;
    P.nbr = nbr_dev;
    P.edge = edge_dev;
    P.iters = iters;
    P.rain = rain;
    P.t_start = 0;
    P.slot = 0;
    cudaStream_t s = (cudaStream_t)stream;
    NX_CHECK_CUDA(cudaMemcpyAsync(planet_dev, &P, sizeof(P), cudaMemcpyHostToDevice, s));
    // state enters in buffer 0; with an odd count the first iteration reads buffer 1
    if (iters & 1)
        NX_CHECK_CUDA(cudaMemcpyAsync(st_tmp_dev, st_dev, 2 * sizeof(float4) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    return run_batch(planet_dev, &P, 1, st_dev, st_tmp_dev, mass_dev, flow_dev, workspace, ws_bytes, s, false);
}

NX_EXPORT int nx_erosion_batch(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host, int nplanets,
                               float *st_dev, float *st_tmp_dev, double *mass_dev, void *workspace, size_t ws_bytes,
                               void *stream)
{
    return run_batch(planets_dev, planets_host, nplanets, st_dev, st_tmp_dev, mass_dev, nullptr, workspace, ws_bytes,
                     (cudaStream_t)stream, true);
}

NX_EXPORT int nx_erosion_ctl_init(void *workspace, size_t ws_bytes, int nplanets, void *stream)
{
    if (!workspace || nplanets <= 0) return nx::fail(NX_EINVAL, "nx_erosion_ctl_init: bad arguments");
    if (ws_bytes < sizeof(nx_erosion_ctl) * (size_t)nplanets) return nx::fail(NX_EINVAL, "nx_erosion_ctl_init: workspace too small");
    NX_CHECK_CUDA(cudaMemsetAsync(workspace, 0, sizeof(nx_erosion_ctl) * (size_t)nplanets, (cudaStream_t)stream));
    return NX_OK;
}

NX_EXPORT int nx_erosion_store(const float *st_dev, int64_t n, const void *workspace, double *h64_dev, double *w64_dev,
                               double *s64_dev, void *stream)
{
    if (n <= 0 || !st_dev || !workspace || !h64_dev) return nx::fail(NX_EINVAL, "nx_erosion_store: bad arguments");
    const nx_erosion_ctl *ctl = (const nx_erosion_ctl *)workspace;
    erosion_store64_kernel<<<grid1d(n), 256, 0, (cudaStream_t)stream>>>((const float4 *)st_dev, n, ctl, h64_dev, w64_dev,
                                                                         s64_dev);
    NX_CHECK_LAUNCH("erosion_store64_kernel");
    nx::note_launch(1);
    return NX_OK;
}
NX_EXPORT int nx_steepest_descent(const int32_t *nbr_dev, const double *h_dev, int64_t n, int32_t *pos_dev,
                                  int32_t *vid_dev, void *stream)
{
    if (n < 0 || (n > 0 && (!nbr_dev || !h_dev || !pos_dev))) return nx::fail(NX_EINVAL, "nx_steepest_descent: bad arguments");
    if (n == 0) return NX_OK;
    steepest_kernel<<<grid1d(n), 256, 0, (cudaStream_t)stream>>>(nbr_dev, h_dev, n, pos_dev, vid_dev);
    NX_CHECK_LAUNCH("steepest_kernel");
    nx::note_launch(1);
    return NX_OK;
}

static int check_packed(const nx_erosion_planet *ph, int np, int64_t *total)
{
    int64_t t = 0;
    for (int p = 0; p < np; ++p) {
        if (ph[p].vbeg % BLOCK || ph[p].vbeg < t || ph[p].n < 0)
            return nx::fail(NX_EINVAL, "erosion batch: planet %d rows must be packed and %d-aligned", p, BLOCK);
        t = ph[p].vbeg + ph[p].n;
    }
    *total = t;
    return NX_OK;
}

NX_EXPORT int nx_erosion_init_batch(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host,
                                    int nplanets, const float *raw_dev, const unsigned long long *minmax_dev,
                                    double elev_lo, double elev_hi, double water0, float *st_dev, float *st_tmp_dev,
                                    void *stream)
{
    if (nplanets <= 0) return NX_OK;
    if (!planets_dev || !planets_host || !raw_dev || !minmax_dev || !st_dev || !st_tmp_dev)
        return nx::fail(NX_EINVAL, "nx_erosion_init_batch: null pointer");
    int64_t total = 0;
    int rc = check_packed(planets_host, nplanets, &total);
    if (rc) return rc;
    if (total == 0) return NX_OK;
    const float w0h = (float)water0, w0l = (float)(water0 - (double)w0h);
    if ((uintptr_t)raw_dev & 7u) return nx::fail(NX_EINVAL, "nx_erosion_init_batch: raw pairs must be 8-byte aligned");
    const size_t smem = nplanets <= INIT_SMEM_PLANETS ? sizeof(float4) * (size_t)nplanets : 0;
    erosion_init_kernel<<<walk_grid(total), 256, smem, (cudaStream_t)stream>>>(
        planets_dev, nplanets, (const float2 *)raw_dev, minmax_dev, elev_lo, elev_hi, w0h, w0l, (float4 *)st_dev,
        (float4 *)st_tmp_dev, 0, total);
    NX_CHECK_LAUNCH("erosion_init_kernel");
    nx::note_launch(1);
    return NX_OK;
}

NX_EXPORT int nx_erosion_heights_batch(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host,
                                       int nplanets, const float *st_dev, const void *workspace, double *out_dev,
                                       void *stream)
{
    if (nplanets <= 0) return NX_OK;
    if (!planets_dev || !planets_host || !st_dev || !workspace || !out_dev)
        return nx::fail(NX_EINVAL, "nx_erosion_heights_batch: null pointer");
    int64_t total = 0;
    int rc = check_packed(planets_host, nplanets, &total);
    if (rc) return rc;
    if (total == 0) return NX_OK;
    erosion_heights_kernel<<<walk_grid(total), 256, 0, (cudaStream_t)stream>>>(
        planets_dev, nplanets, (const float4 *)st_dev, (const nx_erosion_ctl *)workspace, out_dev, total);
    NX_CHECK_LAUNCH("erosion_heights_kernel");
    nx::note_launch(1);
    return NX_OK;
}

// The batch after its fBm in one call: rescale, erosion, heights.  On the
// blocked path the rescale runs in each eroding planet's first pass (its
// load phase reads the raw sums), so the starting state is never written to
// HBM; planets without iterations (the last ones of the non-increasing
// order) get their state from one rescale launch.  Otherwise the rescale
// runs as its own kernel first.  The heights kernel follows either way.
NX_EXPORT int nx_erosion_run_batch(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host,
                                   int nplanets, const float *raw_dev, const unsigned long long *minmax_dev,
                                   double elev_lo, double elev_hi, double water0, float *st_dev, float *st_tmp_dev,
                                   double *heights_dev, void *workspace, size_t ws_bytes, void *stream)
{
    if (nplanets <= 0) return NX_OK;
    if (!planets_dev || !planets_host || !raw_dev || !minmax_dev || !st_dev || !st_tmp_dev || !heights_dev ||
        !workspace)
        return nx::fail(NX_EINVAL, "nx_erosion_run_batch: null pointer");
    if ((uintptr_t)raw_dev & 7u) return nx::fail(NX_EINVAL, "nx_erosion_run_batch: raw pairs must be 8-byte aligned");
    int64_t total = 0;
    int rc = check_packed(planets_host, nplanets, &total);
    if (rc) return rc;
    BatchPlan pl;
    rc = plan_batch(planets_host, nplanets, true, pl);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (!pl.tb) {
        rc = nx_erosion_init_batch(planets_dev, planets_host, nplanets, raw_dev, minmax_dev, elev_lo, elev_hi, water0,
                                   st_dev, st_tmp_dev, stream);
        if (rc) return rc;
        rc = run_batch(planets_dev, planets_host, nplanets, st_dev, st_tmp_dev, nullptr, nullptr, workspace, ws_bytes, s,
                       true);
        if (rc) return rc;
        return nx_erosion_heights_batch(planets_dev, planets_host, nplanets, st_dev, workspace, heights_dev, stream);
    }
    const float w0h = (float)water0, w0l = (float)(water0 - (double)w0h);
    int dry = nplanets;
    while (dry > 0 && planets_host[dry - 1].iters == 0) --dry;
    if (dry < nplanets && total > planets_host[dry].vbeg) {
        const int nd = nplanets - dry;
        const int64_t row0 = planets_host[dry].vbeg;
        const size_t smem = nd <= INIT_SMEM_PLANETS ? sizeof(float4) * (size_t)nd : 0;
        erosion_init_kernel<<<walk_grid(total - row0), 256, smem, s>>>(
            planets_dev + dry, nd, (const float2 *)raw_dev, minmax_dev + 2 * dry, elev_lo, elev_hi, w0h, w0l,
            (float4 *)st_dev, (float4 *)st_tmp_dev, row0, total);
        NX_CHECK_LAUNCH("erosion_init_kernel");
        nx::note_launch(1);
    }
    TbArgs f;
    f.raw = (const float2 *)raw_dev;
    f.minmax = minmax_dev;
    f.elo = elev_lo;
    f.ehi = elev_hi;
    f.w0h = w0h;
    f.w0l = w0l;
    rc = run_batch(planets_dev, planets_host, nplanets, st_dev, st_tmp_dev, nullptr, nullptr, workspace, ws_bytes, s,
                     true, &f);
    if (rc) return rc;
    return nx_erosion_heights_batch(planets_dev, planets_host, nplanets, st_dev, workspace, heights_dev, stream);
}

// ---------------------------------------------------------------------------
// Erosion without allocation.
//
// Some callers cannot allocate device memory at the point where they run
// erosion: code that lives inside a host application's own device-memory
// pool (where a direct cudaMalloc bypasses the owner's budget), and loops
// that must not stall, since cudaMalloc/cudaFree synchronise the device.
// nx_erosion_steps_noalloc takes the same mesh and state buffers as
// nx_erosion_steps but keeps its scratch -- the planet descriptor, the
// control block, the per-block mass partials and the second state buffer --
// in the fixed device array below, sized for NX_NOALLOC_MAX_VERTICES
// vertices.  Every GPU that loads the library holds this array until the
// process exits.

namespace {

constexpr int64_t NOALLOC_MAX_N = NX_NOALLOC_MAX_VERTICES;
constexpr size_t NOALLOC_HEAD = 512;    // descriptor (72 B) at 0, control block (32 B) at 256, padded
constexpr size_t NOALLOC_PARTIALS = (3 * sizeof(double) + sizeof(int2)) * (size_t)((NOALLOC_MAX_N + BLOCK - 1) / BLOCK);
constexpr size_t NOALLOC_STATE = 32 * (size_t)NOALLOC_MAX_N;
constexpr size_t NOALLOC_BYTES = NOALLOC_HEAD + NOALLOC_PARTIALS + NOALLOC_STATE;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {nullptr};

// Device address of g_noalloc_scratch on the current device (looked up once
// per device; the host-side symbol is only a stand-in for it).  The cached
// address belongs to the device's primary context: it stays valid for the
// life of the process unless that context is destroyed (cudaDeviceReset),
// after which the library must not be called on that device again.
int noalloc_scratch(unsigned char **out)
{
    int dev = 0;
    NX_CHECK_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return nx::fail(NX_EINVAL, "nx_erosion_steps_noalloc: device id %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return nx::check_cuda(e, "nx_erosion_steps_noalloc: cudaGetSymbolAddress");
        g_noalloc_ptr[dev] = p;
    }
    *out = (unsigned char *)g_noalloc_ptr[dev];
    return NX_OK;
}

// Writes the planet descriptor and zeroes the control block (scale exponent
// 0, no rescale pending, mass counter and error flag cleared): the scratch
// keeps whatever the previous call left there.
__global__ void noalloc_prepare_kernel(nx_erosion_planet P, nx_erosion_planet *desc, nx_erosion_ctl *ctl)
{
    *desc = P;
    ctl->maxbits[0] = 0u;
    ctl->maxbits[1] = 0u;
    ctl->maxbits[2] = 0u;
    ctl->K[0] = 0;
    ctl->K[1] = 0;
    ctl->done = 0u;
    ctl->err = 0;
    ctl->pad = 0;
}

__global__ void noalloc_status_kernel(const nx_erosion_ctl *ctl, int32_t *status)
{
    status[0] = ctl->K[0];
    status[1] = ctl->err;
}

}  // namespace

NX_EXPORT int nx_erosion_steps_noalloc(const int32_t *nbr_dev, const float *edge_dev, int64_t n, float *st_dev,
                                       int iters, float rain, double *mass_dev, int32_t *status_dev, void *stream)
{
    if (n <= 0 || iters < 0) return nx::fail(NX_EINVAL, "nx_erosion_steps_noalloc: bad n or iters");
    if (n > NOALLOC_MAX_N)
        return nx::fail(NX_EINVAL, "nx_erosion_steps_noalloc: %lld vertices exceed the fixed scratch of %lld vertices",
                        (long long)n, (long long)NOALLOC_MAX_N);
    if (!nbr_dev || !edge_dev || !st_dev) return nx::fail(NX_EINVAL, "nx_erosion_steps_noalloc: null pointer");
    unsigned char *base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc) return rc;
    // scratch layout: descriptor at 0; control block at 256, followed (16-byte
    // aligned, as the workspace carving expects) by the per-block partials and
    // block map; second state buffer after NOALLOC_HEAD + NOALLOC_PARTIALS
    nx_erosion_planet *desc = (nx_erosion_planet *)base;
    nx_erosion_ctl *ctl = (nx_erosion_ctl *)(base + 256);
    float *st_tmp = (float *)(base + NOALLOC_HEAD + NOALLOC_PARTIALS);
    nx_erosion_planet P = {};   // no tiling: every field not set below is zero
    P.vbeg = 0;
    P.n = n;
    P.nbr = nbr_dev;
    P.edge = edge_dev;
    P.iters = iters;
    P.rain = rain;
    P.t_start = 0;
    P.slot = 0;
    cudaStream_t s = (cudaStream_t)stream;
    noalloc_prepare_kernel<<<1, 1, 0, s>>>(P, desc, ctl);
    NX_CHECK_LAUNCH("noalloc_prepare_kernel");
    nx::note_launch(1);
    if (iters & 1)
        NX_CHECK_CUDA(cudaMemcpyAsync(st_tmp, st_dev, 32 * (size_t)n, cudaMemcpyDeviceToDevice, s));
    size_t ws_bytes = nx_erosion_workspace_size(n, 1);
    static_assert(256 + sizeof(nx_erosion_ctl) + 16 + NOALLOC_PARTIALS <= NOALLOC_HEAD + NOALLOC_PARTIALS,
                  "partials fit before the second state buffer");
    static_assert((NOALLOC_HEAD + NOALLOC_PARTIALS) % 256 == 0, "state buffer alignment");
    rc = run_batch(desc, &P, 1, st_dev, st_tmp, mass_dev, nullptr, (void *)ctl, ws_bytes, s, false);
    if (rc) return rc;
    if (status_dev) {
        noalloc_status_kernel<<<1, 1, 0, s>>>(ctl, status_dev);
        NX_CHECK_LAUNCH("noalloc_status_kernel");
        nx::note_launch(1);
    }
    return NX_OK;
}
