// nx_shape.cu -- the post-noise height shaping of nixis.py:330-364 on the GPU:
// util.rescale (util.py:110-176, all of its forms), util.find_percent_val
// (util.py:556-566), terrain.make_bool_elevation_mask (terrain.py:61-72) and
// util.power_rescale (util.py:179-250), in binary64 with the reference's
// operation order.
//
// Reductions are exact and order independent: min and max as atomics on
// ordered 64-bit keys.  power_rescale finds the masked range with a running
// update, `if x < lo: lo = x  elif x > hi: hi = x` from lo = max(x),
// hi = min(x) (util.py:203-214); a value that is a new running minimum is
// never considered for the maximum.  So hi = max(min(x), max of the selected
// values that are not below every earlier selected value and max(x)).  It is
// computed exactly: per chunk of CHUNK elements the selected minimum, an
// exclusive prefix minimum over chunks, then per element its exclusive
// prefix minimum (block scan) decides whether it counts for hi.
//
// All scalars (ranges, the ocean level) stay in the workspace on the device:
// a shaping run makes no host round trip.
#include "nx_common.cuh"

namespace nx {
void note_launch(int k);
}

namespace {

constexpr int THREADS = 256;
constexpr int PER_THREAD = 16;
constexpr int CHUNK = THREADS * PER_THREAD;   // elements per scan block

// Ordered key of a binary64 (-0 taken as +0, as the reference's
// comparisons see them equal).
__device__ __forceinline__ unsigned long long dkey(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v + 0.0);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ double dunkey(unsigned long long k)
{
    const unsigned long long b = (k & 0x8000000000000000ull) ? (k & ~0x8000000000000000ull) : ~k;
    return __longlong_as_double((long long)b);
}

// Workspace: keys and scalars, then one selected-minimum key per chunk.
struct Ws {
    unsigned long long kmin, kmax;     // min, max of the input
    unsigned long long klo, khi;       // power_rescale's masked range
    double level;                      // ocean level (find_percent_val)
    double pad[3];
};

__device__ __forceinline__ unsigned long long warp_min(unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = w < v ? w : v;
    }
    return v;
}

__device__ __forceinline__ unsigned long long warp_max(unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

__global__ void init_ws_kernel(Ws *w)
{
    w->kmin = ~0ull;
    w->kmax = 0ull;
    w->klo = ~0ull;
    w->khi = 0ull;
}

// np.min / np.max (util.py:125-126, 195-196)
__global__ void __launch_bounds__(THREADS) minmax_kernel(const double *__restrict__ x, int64_t n, Ws *w)
{
    unsigned long long lo = ~0ull, hi = 0ull;
    for (int64_t i = (int64_t)blockIdx.x * THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * THREADS) {
        const unsigned long long k = dkey(x[i]);
        lo = k < lo ? k : lo;
        hi = k > hi ? k : hi;
    }
    lo = warp_min(lo);
    hi = warp_max(hi);
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&w->kmin, lo);
        atomicMax(&w->kmax, hi);
    }
}

// util.rescale.  form: 0 plain, 1 with mid, 2 mode 'lower', 3 mode 'upper'.
// u_min / u_max widen the input range (util.py:128-131).
struct RescaleArgs {
    double lower, upper, mid, u_min, u_max;
    int form, has_umin, has_umax;
};

__global__ void __launch_bounds__(THREADS) rescale_kernel(const double *__restrict__ x, int64_t n, const Ws *w,
                                                          RescaleArgs a, double *__restrict__ out)
{
    double x_min = dunkey(w->kmin), x_max = dunkey(w->kmax);
    if (a.has_umin && a.u_min < x_min) x_min = a.u_min;
    if (a.has_umax && a.u_max > x_max) x_max = a.u_max;
    for (int64_t i = (int64_t)blockIdx.x * THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * THREADS) {
        const double v = x[i];
        double r = v;
        if (a.form == 0) {
            const double x_range = __dsub_rn(x_max, x_min), new_range = __dsub_rn(a.upper, a.lower);
            r = __dadd_rn(__dmul_rn(__ddiv_rn(__dsub_rn(v, x_min), x_range), new_range), a.lower);
        } else if (a.form == 1) {
            if (v <= a.mid) {
                const double xr = __dsub_rn(a.mid, x_min), nr = __dsub_rn(a.mid, a.lower);
                r = __dadd_rn(__dmul_rn(__ddiv_rn(__dsub_rn(v, x_min), xr), nr), a.lower);
            } else {
                const double xr = __dsub_rn(x_max, a.mid), nr = __dsub_rn(a.upper, a.mid);
                r = __dadd_rn(__dmul_rn(__ddiv_rn(__dsub_rn(v, a.mid), xr), nr), a.mid);
            }
        } else if (a.form == 2) {
            if (v <= a.mid) {
                const double xr = __dsub_rn(a.mid, x_min), nr = __dsub_rn(a.mid, a.lower);
                r = __dadd_rn(__dmul_rn(__ddiv_rn(__dsub_rn(v, x_min), xr), nr), a.lower);
            }
        } else {
            if (v >= a.mid) {
                const double xr = __dsub_rn(x_max, a.mid), nr = __dsub_rn(a.upper, a.mid);
                r = __dadd_rn(__dmul_rn(__ddiv_rn(__dsub_rn(v, a.mid), xr), nr), a.mid);
            }
        }
        out[i] = r;
    }
}

// x - ocean level (nixis.py:362), the level read from the workspace
__global__ void __launch_bounds__(THREADS) shift_kernel(const double *__restrict__ x, int64_t n, const Ws *w,
                                                        double *__restrict__ out)
{
    const double lv = w->level;
    for (int64_t i = (int64_t)blockIdx.x * THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * THREADS)
        out[i] = __dsub_rn(x[i], lv);
}

// find_percent_val (util.py:556-566) of the workspace's min and max
__global__ void level_kernel(Ws *w, double percent)
{
    if (!(0.0 < percent && percent < 100.0)) percent = 50.0;
    const double mn = dunkey(w->kmin), mx = dunkey(w->kmax);
    w->level = __dadd_rn(mn, __ddiv_rn(__dmul_rn(__dsub_rn(mx, mn), percent), 100.0));
}

// make_bool_elevation_mask (terrain.py:61-72): height <= level; level from
// the argument or (use_ws) the workspace
__global__ void __launch_bounds__(THREADS) mask_kernel(const double *__restrict__ h, int64_t n, double level,
                                                       const Ws *w, int use_ws, uint8_t *__restrict__ mask)
{
    const double lv = use_ws ? w->level : level;
    for (int64_t i = (int64_t)blockIdx.x * THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * THREADS)
        mask[i] = h[i] <= lv ? 1 : 0;
}

__device__ __forceinline__ bool selected(const uint8_t *mask, int64_t i, int mode)
{
    const bool m = mask[i] != 0;
    return mode == 1 ? m : !m;
}

// power_rescale pass 1: per chunk, the minimum key of the selected values
__global__ void __launch_bounds__(THREADS) chunk_min_kernel(const double *__restrict__ x, const uint8_t *__restrict__ mask,
                                                            int64_t n, int mode, unsigned long long *__restrict__ cmin)
{
    const int64_t c = blockIdx.x;
    const int64_t b = c * CHUNK;
    unsigned long long lo = ~0ull;
    for (int64_t i = b + threadIdx.x; i < b + CHUNK && i < n; i += THREADS)
        if (selected(mask, i, mode)) {
            const unsigned long long k = dkey(x[i]);
            lo = k < lo ? k : lo;
        }
    __shared__ unsigned long long s[THREADS / 32];
    lo = warp_min(lo);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = lo;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = s[0];
        for (int k = 1; k < THREADS / 32; ++k) m = s[k] < m ? s[k] : m;
        cmin[c] = m;
    }
}

// pass 2: exclusive prefix minimum over chunks, starting from max(x); one
// block, each thread a run of consecutive chunks
constexpr int SCAN_THREADS = 1024;

__global__ void __launch_bounds__(SCAN_THREADS) chunk_scan_kernel(unsigned long long *cmin, int64_t nchunks, const Ws *w)
{
    const int64_t per = (nchunks + SCAN_THREADS - 1) / SCAN_THREADS;
    const int64_t b = (int64_t)threadIdx.x * per;
    const int64_t e = b + per < nchunks ? b + per : nchunks;
    unsigned long long local = ~0ull;
    for (int64_t c = b; c < e; ++c) local = cmin[c] < local ? cmin[c] : local;
    __shared__ unsigned long long s_warp[SCAN_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long inc = local;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long v = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc = v < inc ? v : inc;
    }
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    unsigned long long before = w->kmax;
    for (int k = 0; k < wid; ++k) before = s_warp[k] < before ? s_warp[k] : before;
    const unsigned long long ex = __shfl_up_sync(0xFFFFFFFFu, inc, 1);
    if (lane > 0) before = ex < before ? ex : before;
    for (int64_t c = b; c < e; ++c) {
        const unsigned long long v = cmin[c];
        cmin[c] = before;
        before = v < before ? v : before;
    }
}

// pass 3: per element, the running minimum before it; selected values not
// below it count for the maximum; the selected minimum as well
__global__ void __launch_bounds__(THREADS) chunk_range_kernel(const double *__restrict__ x, const uint8_t *__restrict__ mask,
                                                              int64_t n, int mode,
                                                              const unsigned long long *__restrict__ carry, Ws *w)
{
    const int64_t c = blockIdx.x;
    const int64_t b = c * CHUNK + (int64_t)threadIdx.x * PER_THREAD;   // this thread's run of PER_THREAD
    unsigned long long key[PER_THREAD];
    unsigned sel = 0;
    unsigned long long tmin = ~0ull;
#pragma unroll
    for (int k = 0; k < PER_THREAD; ++k) {
        const int64_t i = b + k;
        key[k] = ~0ull;
        if (i < n && selected(mask, i, mode)) {
            key[k] = dkey(x[i]);
            sel |= 1u << k;
            tmin = key[k] < tmin ? key[k] : tmin;
        }
    }
    // exclusive prefix minimum of the threads' minima, in thread order
    __shared__ unsigned long long s_warp[THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long inc = tmin;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long v = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc = v < inc ? v : inc;
    }
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    unsigned long long before = carry[c];
    for (int k = 0; k < wid; ++k) before = s_warp[k] < before ? s_warp[k] : before;
    unsigned long long ex = __shfl_up_sync(0xFFFFFFFFu, inc, 1);
    if (lane > 0) before = ex < before ? ex : before;
    // walk this thread's run
    unsigned long long hi = 0ull, lo = ~0ull;
#pragma unroll
    for (int k = 0; k < PER_THREAD; ++k) {
        if (sel & (1u << k)) {
            if (key[k] < before) before = key[k];        // new running minimum: not a candidate
            else hi = key[k] > hi ? key[k] : hi;
            lo = key[k] < lo ? key[k] : lo;
        }
    }
    hi = warp_max(hi);
    lo = warp_min(lo);
    if (lane == 0) {
        if (hi) atomicMax(&w->khi, hi);
        atomicMin(&w->klo, lo);
    }
}

// pass 4: the map (util.py:223-248).  lo = min(max(x), selected min);
// hi = max(min(x), candidates).
__global__ void __launch_bounds__(THREADS) power_map_kernel(const double *__restrict__ x, const uint8_t *__restrict__ mask,
                                                            int64_t n, int mode, double power, const Ws *w,
                                                            double *__restrict__ out)
{
    const unsigned long long kl = w->klo < w->kmax ? w->klo : w->kmax;
    const unsigned long long kh = w->khi > w->kmin ? w->khi : w->kmin;
    const double lo = dunkey(kl), hi = dunkey(kh);
    const double range = __dsub_rn(hi, lo);
    for (int64_t i = (int64_t)blockIdx.x * THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * THREADS) {
        double v = x[i];
        if (mode >= 0 && selected(mask, i, mode)) {
            // ((x - lo) / range) * 1.0 + 0.0, then ** power, then
            // ((v - 0.0) / 1.0) * range + lo
            double t = __dadd_rn(__dmul_rn(__ddiv_rn(__dsub_rn(v, lo), range), 1.0), 0.0);
            if (power == 2.0) t = __dmul_rn(t, t);
            else if (power == 0.5) t = __dsqrt_rn(t);
            else if (power != 1.0) t = pow(t, power);
            v = __dadd_rn(__dmul_rn(__ddiv_rn(__dsub_rn(t, 0.0), 1.0), range), lo);
        }
        out[i] = v;
    }
}

int grid_for(int64_t n)
{
    int64_t g = (n + THREADS - 1) / THREADS;
    const int64_t cap = (int64_t)nx::sm_count() * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

int64_t nchunks_of(int64_t n) { return (n + CHUNK - 1) / CHUNK; }

int launch_minmax(const double *x, int64_t n, Ws *w, cudaStream_t s)
{
    init_ws_kernel<<<1, 1, 0, s>>>(w);
    NX_CHECK_LAUNCH("init_ws_kernel");
    minmax_kernel<<<grid_for(n), THREADS, 0, s>>>(x, n, w);
    NX_CHECK_LAUNCH("minmax_kernel");
    nx::note_launch(2);
    return NX_OK;
}

int launch_rescale(const double *x, int64_t n, const RescaleArgs &a, double *out, Ws *w, cudaStream_t s)
{
    int rc = launch_minmax(x, n, w, s);
    if (rc) return rc;
    rescale_kernel<<<grid_for(n), THREADS, 0, s>>>(x, n, w, a, out);
    NX_CHECK_LAUNCH("rescale_kernel");
    nx::note_launch(1);
    return NX_OK;
}

int launch_power(const double *x, int64_t n, const uint8_t *mask, int mode, double power, double *out, Ws *w,
                 cudaStream_t s)
{
    int rc = launch_minmax(x, n, w, s);
    if (rc) return rc;
    const int64_t nc = nchunks_of(n);
    unsigned long long *cmin = reinterpret_cast<unsigned long long *>(w + 1);
    if (mode >= 0) {
        chunk_min_kernel<<<(unsigned)nc, THREADS, 0, s>>>(x, mask, n, mode, cmin);
        NX_CHECK_LAUNCH("chunk_min_kernel");
        chunk_scan_kernel<<<1, SCAN_THREADS, 0, s>>>(cmin, nc, w);
        NX_CHECK_LAUNCH("chunk_scan_kernel");
        chunk_range_kernel<<<(unsigned)nc, THREADS, 0, s>>>(x, mask, n, mode, cmin, w);
        NX_CHECK_LAUNCH("chunk_range_kernel");
        nx::note_launch(3);
    }
    power_map_kernel<<<grid_for(n), THREADS, 0, s>>>(x, mask, n, mode, power, w, out);
    NX_CHECK_LAUNCH("power_map_kernel");
    nx::note_launch(1);
    return NX_OK;
}

int check_ws(void *ws, size_t ws_bytes, int64_t n, const char *who);

}  // namespace

NX_EXPORT size_t nx_shape_workspace_size(int64_t n)
{
    return sizeof(Ws) + sizeof(unsigned long long) * (size_t)(nchunks_of(n > 0 ? n : 1)) + 64;
}

namespace {
int check_ws(void *ws, size_t ws_bytes, int64_t n, const char *who)
{
    if (!ws) return nx::fail(NX_EINVAL, "%s: null workspace", who);
    if (((uintptr_t)ws) % 16) return nx::fail(NX_EINVAL, "%s: workspace must be 16-byte aligned", who);
    if (ws_bytes < nx_shape_workspace_size(n)) return nx::fail(NX_EINVAL, "%s: workspace too small", who);
    return NX_OK;
}
}  // namespace

NX_EXPORT int nx_rescale(const double *x_dev, int64_t n, double lower, double upper, double mid, int form,
                         double u_min, int has_umin, double u_max, int has_umax, double *out_dev, void *ws,
                         size_t ws_bytes, void *stream)
{
    if (n <= 0) return nx::fail(NX_EINVAL, "nx_rescale: n must be > 0");
    if (!x_dev || !out_dev) return nx::fail(NX_EINVAL, "nx_rescale: null pointer");
    if (form < 0 || form > 3) return nx::fail(NX_EINVAL, "nx_rescale: form must be 0-3");
    int rc = check_ws(ws, ws_bytes, n, "nx_rescale");
    if (rc) return rc;
    RescaleArgs a;
    a.lower = lower; a.upper = upper; a.mid = mid; a.u_min = u_min; a.u_max = u_max;
    a.form = form; a.has_umin = has_umin != 0; a.has_umax = has_umax != 0;
    return launch_rescale(x_dev, n, a, out_dev, (Ws *)ws, (cudaStream_t)stream);
}

NX_EXPORT int nx_power_rescale(const double *x_dev, int64_t n, const uint8_t *mask_dev, int mode, double power,
                               double *out_dev, void *ws, size_t ws_bytes, void *stream)
{
    if (n <= 0) return nx::fail(NX_EINVAL, "nx_power_rescale: n must be > 0");
    if (!x_dev || !out_dev) return nx::fail(NX_EINVAL, "nx_power_rescale: null pointer");
    if (mode != -1 && mode != 0 && mode != 1) return nx::fail(NX_EINVAL, "nx_power_rescale: mode must be -1, 0 or 1");
    if (mode >= 0 && !mask_dev) return nx::fail(NX_EINVAL, "nx_power_rescale: mode %d needs a mask", mode);
    int rc = check_ws(ws, ws_bytes, n, "nx_power_rescale");
    if (rc) return rc;
    return launch_power(x_dev, n, mask_dev, mode, power, out_dev, (Ws *)ws, (cudaStream_t)stream);
}

NX_EXPORT int nx_elevation_mask(const double *h_dev, int64_t n, double level, uint8_t *mask_dev, void *stream)
{
    if (n < 0 || (n > 0 && (!h_dev || !mask_dev))) return nx::fail(NX_EINVAL, "nx_elevation_mask: bad arguments");
    if (n == 0) return NX_OK;
    mask_kernel<<<grid_for(n), THREADS, 0, (cudaStream_t)stream>>>(h_dev, n, level, nullptr, 0, mask_dev);
    NX_CHECK_LAUNCH("mask_kernel");
    nx::note_launch(1);
    return NX_OK;
}

// nixis.py:332-364 with h1..h5 as there: h1 = rescale(h, min_alt, max_alt);
// level = find_percent_val(min h1, max h1, ocean_percent); ocean = h1 <= level;
// h2 = power_rescale(h1, ocean, 1, 0.5); h3 = power_rescale(h2, ocean, 0, 2.0);
// h5 = rescale(h3 - level, min_alt, max_alt, mid=0).  out_dev gets h5,
// mask_dev (optional) the ocean mask, level_dev (optional) the level.
// tmp_dev: a second array of n doubles.
NX_EXPORT int nx_shape_heights(const double *h_dev, int64_t n, double min_alt, double max_alt, double ocean_percent,
                               double *out_dev, double *tmp_dev, uint8_t *mask_dev, double *level_dev, void *ws,
                               size_t ws_bytes, void *stream)
{
    if (n <= 0) return nx::fail(NX_EINVAL, "nx_shape_heights: n must be > 0");
    if (!h_dev || !out_dev || !tmp_dev || !mask_dev) return nx::fail(NX_EINVAL, "nx_shape_heights: null pointer");
    int rc = check_ws(ws, ws_bytes, n, "nx_shape_heights");
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    Ws *w = (Ws *)ws;
    RescaleArgs a;
    a.lower = min_alt; a.upper = max_alt; a.mid = 0.0; a.u_min = 0.0; a.u_max = 0.0;
    a.form = 0; a.has_umin = 0; a.has_umax = 0;
    rc = launch_rescale(h_dev, n, a, out_dev, w, s);                   // h1 -> out
    if (rc) return rc;
    rc = launch_minmax(out_dev, n, w, s);
    if (rc) return rc;
    level_kernel<<<1, 1, 0, s>>>(w, ocean_percent);
    NX_CHECK_LAUNCH("level_kernel");
    mask_kernel<<<grid_for(n), THREADS, 0, s>>>(out_dev, n, 0.0, w, 1, mask_dev);
    NX_CHECK_LAUNCH("mask_kernel");
    nx::note_launch(2);
    if (level_dev) NX_CHECK_CUDA(cudaMemcpyAsync(level_dev, &w->level, sizeof(double), cudaMemcpyDeviceToDevice, s));
    // (the min/max resets below leave the level in place)
    rc = launch_power(out_dev, n, mask_dev, 1, 0.5, tmp_dev, w, s);    // h2 -> tmp
    if (rc) return rc;
    rc = launch_power(tmp_dev, n, mask_dev, 0, 2.0, out_dev, w, s);    // h3 -> out
    if (rc) return rc;
    shift_kernel<<<grid_for(n), THREADS, 0, s>>>(out_dev, n, w, tmp_dev);   // h4 -> tmp
    NX_CHECK_LAUNCH("shift_kernel");
    nx::note_launch(1);
    a.form = 1;
    return launch_rescale(tmp_dev, n, a, out_dev, w, s);              // h5 -> out
}
