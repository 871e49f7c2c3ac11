// nx_image.cu -- equirectangular map sampling (util.py:290-366, nixis.py:270-302):
// the pixel positions of make_ll_arr and the inverse-distance weighting of
// make_gray_array, in binary64 with the reference's operation order.  The
// three nearest vertices of each pixel come from nx_nearest3 (nx_mesh.cu).
#include "nx_common.cuh"

namespace nx {
void note_launch(int k);
}

namespace {

constexpr double PI = 3.141592653589793;

// make_ll_arr (util.py:290-310): row h at latitude max(90 - h*180/(height-1),
// -90), column w at longitude max(-180 + w*360/width, -180), through
// util.latlon2xyz (util.py:79-88).
__global__ void __launch_bounds__(256) make_ll_kernel(int width, int height, double radius, double *__restrict__ out)
{
    const int64_t np = (int64_t)width * height;
    const double latpercent = 180.0 / (double)(height - 1), lonpercent = 360.0 / (double)width;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        const int h = (int)(p / width), w = (int)(p - (int64_t)h * width);
        const double lat = fmax(__dsub_rn(90.0, __dmul_rn((double)h, latpercent)), -90.0);
        const double lon = fmax(__dadd_rn(-180.0, __dmul_rn((double)w, lonpercent)), -180.0);
        const double a = __dmul_rn(lat, PI / 180), b = __dmul_rn(lon, PI / 180);
        out[3 * p] = __dmul_rn(__dmul_rn(radius, cos(a)), cos(b));
        out[3 * p + 1] = __dmul_rn(__dmul_rn(radius, cos(a)), sin(b));
        out[3 * p + 2] = __dmul_rn(radius, sin(a));
    }
}

// make_gray_array (util.py:342-366) per pixel: weights 1 / ((d + 1e-5) / sum d)
// normalised by their sum, the weighted colours summed in slot order and
// truncated toward zero (Python int()).
__global__ void __launch_bounds__(256) gray_kernel(const double *__restrict__ dist, const int64_t *__restrict__ idx,
                                                   int64_t np, const double *__restrict__ colors, int64_t nc,
                                                   double *__restrict__ out, int *__restrict__ err)
{
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        const double *d = dist + 3 * p;
        const double sd = __dadd_rn(__dadd_rn(d[0], d[1]), d[2]);
        double ws[3];
        for (int k = 0; k < 3; ++k) ws[k] = __ddiv_rn(1.0, __ddiv_rn(__dadd_rn(d[k], 0.00001), sd));
        const double t = __dadd_rn(__dadd_rn(ws[0], ws[1]), ws[2]);
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) {
            const int64_t v = idx[3 * p + k];
            if (v < 0 || v >= nc) {
                atomicOr(err, 1);
                continue;
            }
            acc = __dadd_rn(acc, __dmul_rn(colors[v], __ddiv_rn(ws[k], t)));
        }
        out[p] = trunc(acc);
    }
}

int grid_for(int64_t n)
{
    int64_t g = (n + 255) / 256;
    const int64_t cap = (int64_t)nx::sm_count() * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

NX_EXPORT int nx_make_ll(int width, int height, double radius, double *out_dev, void *stream)
{
    if (width < 1 || height < 2 || !out_dev) return nx::fail(NX_EINVAL, "nx_make_ll: bad arguments");
    make_ll_kernel<<<grid_for((int64_t)width * height), 256, 0, (cudaStream_t)stream>>>(width, height, radius, out_dev);
    NX_CHECK_LAUNCH("make_ll_kernel");
    nx::note_launch(1);
    return NX_OK;
}

NX_EXPORT int nx_sample_gray(const double *dist_dev, const int64_t *idx_dev, int64_t npix, const double *colors_dev,
                             int64_t ncolors, double *out_dev, int *err_dev, void *stream)
{
    if (npix < 0 || (npix > 0 && (!dist_dev || !idx_dev || !colors_dev || !out_dev || !err_dev)))
        return nx::fail(NX_EINVAL, "nx_sample_gray: bad arguments");
    if (npix == 0) return NX_OK;
    gray_kernel<<<grid_for(npix), 256, 0, (cudaStream_t)stream>>>(dist_dev, idx_dev, npix, colors_dev, ncolors, out_dev,
                                                                  err_dev);
    NX_CHECK_LAUNCH("gray_kernel");
    nx::note_launch(1);
    return NX_OK;
}
