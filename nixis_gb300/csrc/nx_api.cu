// nx_api.cu -- error reporting, device queries and host-side table setup.
#include "nx_common.cuh"

#include <atomic>
#include <cstdarg>
#include <cstring>
#include <mutex>

namespace nx {

static thread_local char g_err[512] = "";
static std::atomic<unsigned long long> g_launches{0};

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int check_cuda(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return NX_OK;
    set_error("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? NX_ENOMEM : NX_ECUDA;
}

int sm_count()
{
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    if (!cache[dev]) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) v = 1;
        cache[dev] = v;
    }
    return cache[dev];
}

void note_launch(int k) { g_launches.fetch_add((unsigned long long)k, std::memory_order_relaxed); }

}  // namespace nx

NX_EXPORT const char *nx_last_error(void) { return nx::g_err; }

NX_EXPORT int nx_version(void) { return 10100; }

NX_EXPORT unsigned long long nx_launch_count(void) { return nx::g_launches.load(); }

// opensimplex.init (opensimplex.py:90-107).  `over` (opensimplex.py:110-112)
// is compiled by numba with signature int32(int32): each LCG state is cut to
// its low 32 bits, sign-extended; the 64-bit multiply-add itself wraps.
// The index r is a floor-mod, non-negative for the positive modulus.
NX_EXPORT int nx_perm_init(int64_t seed, int32_t *perm, int32_t *pgi)
{
    if (!perm || !pgi) return nx::fail(NX_EINVAL, "nx_perm_init: null pointer");
    auto step = [](int64_t state) -> int64_t {
        uint64_t v = (uint64_t)state * 6364136223846793005ULL + 1442695040888963407ULL;
        return (int64_t)(int32_t)(uint32_t)(v & 0xFFFFFFFFu);
    };
    int32_t pool[256];
    for (int i = 0; i < 256; ++i) pool[i] = i;
    int64_t st = step(step(step(seed)));
    for (int i = 255; i >= 0; --i) {
        st = step(st);
        int64_t m = (int64_t)i + 1;
        int64_t r = (st + 31) % m;
        if (r < 0) r += m;
        perm[i] = pool[r];
        pgi[i] = (perm[i] % 24) * 3;   // int((perm % 24.0) * 3) for perm in [0, 255]
        pool[r] = pool[i];
    }
    return NX_OK;
}
