// nx_mesh.cu -- icosphere generation, adjacency and per-slot edge lengths.
//
// The reference gets its sphere from meshzoo.icosa_sphere (util.py:43) and
// its neighbour table from build_adjacency + sort_adjacency (util.py:591-662).
// meshzoo is not available, so the vertex layout here is this project's own
// (documented in nixis_gb300/icosphere.py); the adjacency kernels implement
// the reference's two functions for any consistently wound triangle mesh, so
// the neighbour table equals what the reference computes from the same
// triangles.
#include <algorithm>
#include <climits>
#include <cmath>

#include "nx_common.cuh"

namespace nx {
void note_launch(int k);
}

namespace {

struct IcoTables {
    double corner[12][3];
    int face[20][3];
    int fedge[20][3][2];   // per face side (AB, AC, BC): edge id, 1 if it runs low->high corner
    int edge[30][2];
    double inv[20][3][3];  // per face: inverse of the matrix with columns A, B, C
};

__constant__ IcoTables c_ico;

// Home face of every corner and edge (the lowest-numbered face containing
// it), used to give every vertex one (face, i, j) grid position for tiling.
struct IcoHome {
    int corner_face[12], corner_which[12];        // which: 0 = A, 1 = B, 2 = C of that face
    int edge_face[30], edge_side[30], edge_fwd[30];  // side: 0 = AB, 1 = AC, 2 = BC
};

__constant__ IcoHome c_home;

// Point = normalise(w0*A + w1*B + w2*C), sums in the written order, no FMA.
__device__ __forceinline__ void blend3(const double *A, const double *B, const double *C, double w0, double w1,
                                       double w2, double *out)
{
    double p[3];
    for (int c = 0; c < 3; ++c)
        p[c] = __dadd_rn(__dadd_rn(__dmul_rn(w0, A[c]), __dmul_rn(w1, B[c])), __dmul_rn(w2, C[c]));
    double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(p[0], p[0]), __dmul_rn(p[1], p[1])), __dmul_rn(p[2], p[2])));
    for (int c = 0; c < 3; ++c) out[c] = __ddiv_rn(p[c], r);
}

__device__ __forceinline__ void blend2(const double *A, const double *B, double w0, double w1, double *out)
{
    double p[3];
    for (int c = 0; c < 3; ++c) p[c] = __dadd_rn(__dmul_rn(w0, A[c]), __dmul_rn(w1, B[c]));
    double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(p[0], p[0]), __dmul_rn(p[1], p[1])), __dmul_rn(p[2], p[2])));
    for (int c = 0; c < 3; ++c) out[c] = __ddiv_rn(p[c], r);
}

// Face-interior offset q -> (face, i, j): rows i = 1..k-2 hold k-1-i points.
__device__ __forceinline__ void interior_fij(int64_t q, int k, int &f, int &i, int &j)
{
    const int64_t npf = (int64_t)(k - 1) * (k - 2) / 2;
    f = (int)(q / npf);
    const int64_t off = q - (int64_t)f * npf;
    // binary32 estimate of the row; the loops below make it exact
    const float kk = (float)k;
    const float disc = (2.0f * kk - 3.0f) * (2.0f * kk - 3.0f) - 8.0f * (float)off;
    int ii = (int)floorf(((2.0f * kk - 3.0f) - sqrtf(fmaxf(disc, 0.0f))) * 0.5f) + 1;
    if (ii < 1) ii = 1;
    if (ii > k - 2) ii = k - 2;
    auto start = [&](int a) -> int64_t { return (int64_t)(a - 1) * (k - 1) - (int64_t)(a - 1) * a / 2; };
    while (ii > 1 && start(ii) > off) --ii;
    while (ii < k - 2 && start(ii + 1) <= off) ++ii;
    i = ii;
    j = (int)(off - start(ii)) + 1;
}

__global__ void ico_vertices_kernel(int k, int64_t nv, double *__restrict__ xyz)
{
    const int64_t ne = (int64_t)30 * (k - 1);
    const int64_t npf = (int64_t)(k - 1) * (k - 2) / 2;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
        double out[3];
        if (v < 12) {
            for (int c = 0; c < 3; ++c) out[c] = c_ico.corner[v][c];
        } else if (v < 12 + ne) {
            int64_t q = v - 12;
            int e = (int)(q / (k - 1));
            int t = (int)(q - (int64_t)e * (k - 1)) + 1;
            blend2(c_ico.corner[c_ico.edge[e][0]], c_ico.corner[c_ico.edge[e][1]], (double)(k - t), (double)t, out);
        } else {
            int64_t q = v - 12 - ne;
            int f = (int)(q / npf);
            int64_t off = q - (int64_t)f * npf;
            // row i (1..k-2) holds k-1-i points; invert the running offset
            // (i-1)(k-1) - (i-1)i/2 with a binary32 estimate plus correction.
            const float kk = (float)k;
            const float disc = (2.0f * kk - 3.0f) * (2.0f * kk - 3.0f) - 8.0f * (float)off;
            int i0 = (int)floorf(((2.0f * kk - 3.0f) - sqrtf(fmaxf(disc, 0.0f))) * 0.5f);
            int i = i0 + 1;
            if (i < 1) i = 1;
            if (i > k - 2) i = k - 2;
            auto start = [&](int ii) -> int64_t { return (int64_t)(ii - 1) * (k - 1) - (int64_t)(ii - 1) * ii / 2; };
            while (i > 1 && start(i) > off) --i;
            while (i < k - 2 && start(i + 1) <= off) ++i;
            int j = (int)(off - start(i)) + 1;
            const int *F = c_ico.face[f];
            blend3(c_ico.corner[F[0]], c_ico.corner[F[1]], c_ico.corner[F[2]], (double)(k - i - j), (double)i,
                   (double)j, out);
        }
        xyz[3 * v] = out[0];
        xyz[3 * v + 1] = out[1];
        xyz[3 * v + 2] = out[2];
    }
}

// Vertex id of face point (i, j); layout in icosphere.py.
__device__ __forceinline__ int32_t face_vid(int f, int i, int j, int k)
{
    const int *F = c_ico.face[f];
    if (i == 0 && j == 0) return F[0];
    if (i == k && j == 0) return F[1];
    if (i == 0 && j == k) return F[2];
    int side, pos;
    if (j == 0) { side = 0; pos = i; }
    else if (i == 0) { side = 1; pos = j; }
    else if (i + j == k) { side = 2; pos = j; }
    else {
        int64_t npf = (int64_t)(k - 1) * (k - 2) / 2;
        int64_t off = (int64_t)(i - 1) * (k - 1) - (int64_t)(i - 1) * i / 2 + (j - 1);
        return (int32_t)(12 + (int64_t)30 * (k - 1) + (int64_t)f * npf + off);
    }
    int e = c_ico.fedge[f][side][0];
    int t = c_ico.fedge[f][side][1] ? pos : k - pos;
    return (int32_t)(12 + (int64_t)e * (k - 1) + t - 1);
}

// Triangles of one face row-pair: triangle index within the face for
// (i, j): rows before i hold sum_{i'<i} (2(k-i') - 1) = i(2k - i) triangles.
__global__ void ico_triangles_kernel(int k, int64_t nt, int32_t *__restrict__ tris)
{
    const int64_t per_face = (int64_t)k * k;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
        int f = (int)(t / per_face);
        int64_t q = t - (int64_t)f * per_face;
        // find row i with i(2k-i) <= q < (i+1)(2k-i-1)
        double kk = (double)k;
        int i = (int)floor(kk - sqrt(kk * kk - (double)q));
        if (i < 0) i = 0;
        if (i > k - 1) i = k - 1;
        while (i > 0 && (int64_t)i * (2 * k - i) > q) --i;
        while (i < k - 1 && (int64_t)(i + 1) * (2 * k - i - 1) <= q) ++i;
        int64_t r = q - (int64_t)i * (2 * k - i);   // 0 .. 2(k-i)-2
        int j = (int)(r / 2);
        bool down = (r & 1) != 0;
        int32_t a, b, c;
        if (!down) {
            a = face_vid(f, i, j, k); b = face_vid(f, i + 1, j, k); c = face_vid(f, i, j + 1, k);
        } else {
            a = face_vid(f, i + 1, j, k); b = face_vid(f, i + 1, j + 1, k); c = face_vid(f, i, j + 1, k);
        }
        tris[3 * t] = a;
        tris[3 * t + 1] = b;
        tris[3 * t + 2] = c;
    }
}

// build_adjacency (util.py:591-613): every triangle t appends t1 to t0's row,
// t2 to t1's, t0 to t2's, in triangle order.  Records (t, neighbour) are
// gathered with an atomic slot per vertex, then each row is ordered by t.
__global__ void adj_records_kernel(const int32_t *__restrict__ tris, int64_t nt, int64_t nv,
                                   unsigned *__restrict__ cnt, unsigned long long *__restrict__ rec,
                                   int *__restrict__ err)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
        for (int e = 0; e < 3; ++e) {
            int32_t a = tris[3 * t + e], b = tris[3 * t + (e + 1) % 3];
            if ((uint64_t)(uint32_t)a >= (uint64_t)nv || (uint64_t)(uint32_t)b >= (uint64_t)nv) {
                atomicOr(err, 1);
                continue;
            }
            unsigned s = atomicAdd(&cnt[a], 1u);
            if (s >= 6) {
                atomicOr(err, 2);
                continue;
            }
            rec[6 * (int64_t)a + s] = ((unsigned long long)t << 32) | (uint32_t)b;
        }
    }
}

__device__ __forceinline__ void cswap(unsigned long long &a, unsigned long long &b)
{
    const unsigned long long lo = a < b ? a : b, hi = a < b ? b : a;
    a = lo;
    b = hi;
}

__global__ void adj_rows_kernel(int64_t nv, const unsigned *__restrict__ cnt,
                                const unsigned long long *__restrict__ rec, int32_t *__restrict__ adj)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
        unsigned c = cnt[v];
        if (c > 6) c = 6;
        unsigned long long r[6];
#pragma unroll
        for (int s = 0; s < 6; ++s) r[s] = s < (int)c ? rec[6 * v + s] : ~0ull;
        // by triangle index: a 12-comparator sorting network for 6 keys
        // (fixed indices, so the keys stay in registers)
        cswap(r[0], r[5]); cswap(r[1], r[3]); cswap(r[2], r[4]);
        cswap(r[1], r[2]); cswap(r[3], r[4]);
        cswap(r[0], r[3]); cswap(r[2], r[5]);
        cswap(r[0], r[1]); cswap(r[2], r[3]); cswap(r[4], r[5]);
        cswap(r[1], r[2]); cswap(r[3], r[4]);
#pragma unroll
        for (int s = 0; s < 6; ++s) adj[6 * v + s] = s < (int)c ? (int32_t)(uint32_t)r[s] : -1;
    }
}

__device__ __forceinline__ bool row_has(const int32_t *row, int32_t v)
{
    bool f = false;
    for (int s = 0; s < 6; ++s) f |= row[s] == v;
    return f;
}

// sort_adjacency (util.py:638-662) with next_vert (util.py:623-629): walk the
// neighbours of each vertex into a ring starting at slot 0.  Reads the
// unsorted rows `in`, writes `out` (membership tests do not depend on order).
__global__ void adj_sort_kernel(int64_t nv, const int32_t *__restrict__ in, int32_t *__restrict__ out)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
        int32_t row[6], vis[6];
        for (int s = 0; s < 6; ++s) { row[s] = in[6 * v + s]; vis[s] = -1; }
        int deg = v < 12 ? 5 : 6;
        int32_t pv = (int32_t)v, cur = row[0];
        for (int i = 0; i < deg - 1; ++i) {
            vis[i] = cur;
            int32_t nxt = -1;
            if (cur >= 0 && (int64_t)cur < nv) {
                const int32_t *other = in + 6 * (int64_t)cur;
                int32_t o[6];
                for (int s = 0; s < 6; ++s) o[s] = other[s];
                for (int s = 0; s < 6; ++s) {
                    int32_t c = row[s];
                    if (row_has(o, c) && c != pv) { nxt = c; break; }
                }
            }
            cur = nxt;
            pv = vis[i];
        }
        vis[deg - 1] = cur;
        for (int s = 0; s < 6; ++s) out[6 * v + s] = vis[s];
    }
}

__device__ __forceinline__ double edge_len(const double *xyz, int64_t v, int64_t j)
{
    const double dx = __dsub_rn(xyz[3 * v], xyz[3 * j]);
    const double dy = __dsub_rn(xyz[3 * v + 1], xyz[3 * j + 1]);
    const double dz = __dsub_rn(xyz[3 * v + 2], xyz[3 * j + 2]);
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

__device__ __forceinline__ float2 edge_pair(double d)
{
    const float hi = (float)d;
    return make_float2(hi, (float)(d - (double)hi));
}

// erosion.py:38-40 in binary64 (squares by multiplication), split into a
// pair hi + lo of binary32s: el[2q] = hi, el[2q+1] = lo.  |v_i - v_j| and
// |v_j - v_i| are the same number (the differences only change sign), so
// the binary64 arithmetic -- slow at GB300's binary64 rate -- runs once per
// edge: this pass fills the slots whose neighbour has the larger id (or is
// the vertex itself), edge_mirror_kernel copies them into the reverse slots.
// Each warp takes 64 consecutive slots at a time and gathers the ones that
// need a distance (about half) into consecutive lanes through shared
// memory, so the binary64 instructions run with the warp's lanes busy
// instead of half of them masked off.
__global__ void __launch_bounds__(256) edge_len_kernel(const double *__restrict__ xyz, const int32_t *__restrict__ nbr,
                                                       int64_t nv, float2 *__restrict__ el, int *__restrict__ err)
{
    __shared__ int64_t s_q[8][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t nq = 6 * nv;
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = wid * 64; base < nq; base += nw * 64) {
        int cnt = 0;
        for (int h = 0; h < 2; ++h) {
            const int64_t q = base + 32 * h + lane;
            bool work = false;
            if (q < nq) {
                const int32_t j = nbr[q];
                if (j >= 0 && (int64_t)j < nv) {
                    work = (int64_t)j >= q / 6;                  // j < v: filled by the mirror pass
                } else {
                    if (j != -1 && err) atomicOr(err, 1);
                    el[q] = make_float2(0.0f, 0.0f);
                }
            }
            const unsigned m = __ballot_sync(0xFFFFFFFFu, work);
            if (work) s_q[w][cnt + __popc(m & ((1u << lane) - 1u))] = q;
            cnt += __popc(m);
        }
        __syncwarp();
        for (int r = lane; r < cnt; r += 32) {
            const int64_t q = s_q[w][r];
            el[q] = edge_pair(edge_len(xyz, q / 6, nbr[q]));
        }
        __syncwarp();
    }
}

// Slots whose neighbour j has the smaller id take the pair of j's slot that
// points back; a table that is not symmetric gets the distance computed.
__global__ void edge_mirror_kernel(const double *__restrict__ xyz, const int32_t *__restrict__ nbr, int64_t nv,
                                   float2 *__restrict__ el)
{
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 6 * nv; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = q / 6;
        const int32_t j = nbr[q];
        if (j < 0 || (int64_t)j >= nv || (int64_t)j >= v) continue;
        int m = -1;
        for (int s = 0; s < 6; ++s)
            if (nbr[6 * (int64_t)j + s] == (int32_t)v) { m = s; break; }
        el[q] = m >= 0 ? el[6 * (int64_t)j + m] : edge_pair(edge_len(xyz, v, j));
    }
}

int grid1d(int64_t n, int block = 256)
{
    int64_t g = (n + block - 1) / block;
    int64_t cap = (int64_t)nx::sm_count() * 16;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

bool g_tables_ready[64] = {false};

int upload_tables(const double *corners, const int *faces, const int *fedge, const int *edges)
{
    int dev = 0;
    NX_CHECK_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && g_tables_ready[dev]) return NX_OK;
    IcoTables t;
    for (int i = 0; i < 12; ++i)
        for (int c = 0; c < 3; ++c) t.corner[i][c] = corners[3 * i + c];
    for (int f = 0; f < 20; ++f)
        for (int c = 0; c < 3; ++c) {
            t.face[f][c] = faces[3 * f + c];
            t.fedge[f][c][0] = fedge[6 * f + 2 * c];
            t.fedge[f][c][1] = fedge[6 * f + 2 * c + 1];
        }
    for (int e = 0; e < 30; ++e) {
        t.edge[e][0] = edges[2 * e];
        t.edge[e][1] = edges[2 * e + 1];
    }
    for (int f = 0; f < 20; ++f) {
        // M = [A B C] (columns); inverse by cofactors
        double m[3][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) m[r][c] = t.corner[t.face[f][c]][r];
        const double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1], c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2],
                     c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
        const double det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
        t.inv[f][0][0] = c00 / det;
        t.inv[f][1][0] = c01 / det;
        t.inv[f][2][0] = c02 / det;
        t.inv[f][0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / det;
        t.inv[f][1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / det;
        t.inv[f][2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / det;
        t.inv[f][0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / det;
        t.inv[f][1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / det;
        t.inv[f][2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / det;
    }
    NX_CHECK_CUDA(cudaMemcpyToSymbol(c_ico, &t, sizeof(t)));
    IcoHome h;
    for (int c = 0; c < 12; ++c) {
        h.corner_face[c] = -1;
        for (int f = 0; f < 20 && h.corner_face[c] < 0; ++f)
            for (int w = 0; w < 3; ++w)
                if (t.face[f][w] == c) { h.corner_face[c] = f; h.corner_which[c] = w; break; }
    }
    for (int e = 0; e < 30; ++e) {
        h.edge_face[e] = -1;
        for (int f = 0; f < 20 && h.edge_face[e] < 0; ++f)
            for (int sd = 0; sd < 3; ++sd)
                if (t.fedge[f][sd][0] == e) { h.edge_face[e] = f; h.edge_side[e] = sd; h.edge_fwd[e] = t.fedge[f][sd][1]; break; }
    }
    NX_CHECK_CUDA(cudaMemcpyToSymbol(c_home, &h, sizeof(h)));
    if (dev >= 0 && dev < 64) g_tables_ready[dev] = true;
    return NX_OK;
}

}  // namespace

NX_EXPORT int nx_icosphere_tables(const double *corners, const int32_t *faces, const int32_t *face_edges,
                                  const int32_t *edges)
{
    if (!corners || !faces || !face_edges || !edges) return nx::fail(NX_EINVAL, "nx_icosphere_tables: null pointer");
    int dev = 0;
    NX_CHECK_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64) g_tables_ready[dev] = false;
    return upload_tables(corners, faces, face_edges, edges);
}

NX_EXPORT int nx_icosphere(int k, double *xyz_dev, int32_t *tris_dev, void *stream)
{
    if (k < 1 || (int64_t)10 * k * k + 2 > 0x7FFFFFFFLL) return nx::fail(NX_EINVAL, "nx_icosphere: bad divisions %d", k);
    int dev = 0;
    NX_CHECK_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64 || !g_tables_ready[dev])
        return nx::fail(NX_EINVAL, "nx_icosphere: call nx_icosphere_tables first on this device");
    int64_t nv = (int64_t)10 * k * k + 2, nt = (int64_t)20 * k * k;
    cudaStream_t s = (cudaStream_t)stream;
    if (xyz_dev) {
        ico_vertices_kernel<<<grid1d(nv), 256, 0, s>>>(k, nv, xyz_dev);
        NX_CHECK_LAUNCH("ico_vertices_kernel");
        nx::note_launch(1);
    }
    if (tris_dev) {
        ico_triangles_kernel<<<grid1d(nt), 256, 0, s>>>(k, nt, tris_dev);
        NX_CHECK_LAUNCH("ico_triangles_kernel");
        nx::note_launch(1);
    }
    return NX_OK;
}

NX_EXPORT size_t nx_adjacency_workspace_size(int64_t nv)
{
    return (size_t)nv * (6 * sizeof(unsigned long long) + sizeof(unsigned)) + 256;
}

NX_EXPORT int nx_build_adjacency(const int32_t *tris_dev, int64_t nt, int64_t nv, int32_t *adj_dev, void *workspace,
                                 size_t ws_bytes, int *err_dev, void *stream)
{
    if (nt < 0 || nv < 0 || (nt + 4) / 2 != nv) return nx::fail(NX_EINVAL, "nx_build_adjacency: need nv = (nt+4)/2");
    if (nv == 0) return NX_OK;
    if (!tris_dev || !adj_dev || !workspace || !err_dev) return nx::fail(NX_EINVAL, "nx_build_adjacency: null pointer");
    if (ws_bytes < nx_adjacency_workspace_size(nv)) return nx::fail(NX_EINVAL, "nx_build_adjacency: workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long *rec = (unsigned long long *)workspace;
    unsigned *cnt = (unsigned *)(rec + 6 * nv);
    NX_CHECK_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned) * (size_t)nv, s));
    adj_records_kernel<<<grid1d(nt), 256, 0, s>>>(tris_dev, nt, nv, cnt, rec, err_dev);
    NX_CHECK_LAUNCH("adj_records_kernel");
    adj_rows_kernel<<<grid1d(nv), 256, 0, s>>>(nv, cnt, rec, adj_dev);
    NX_CHECK_LAUNCH("adj_rows_kernel");
    nx::note_launch(2);
    return NX_OK;
}

NX_EXPORT int nx_sort_adjacency(const int32_t *adj_in_dev, int32_t *adj_out_dev, int64_t nv, void *stream)
{
    if (nv < 0) return nx::fail(NX_EINVAL, "nx_sort_adjacency: nv < 0");
    if (nv == 0) return NX_OK;
    if (!adj_in_dev || !adj_out_dev || adj_in_dev == adj_out_dev)
        return nx::fail(NX_EINVAL, "nx_sort_adjacency: need distinct input and output rows");
    adj_sort_kernel<<<grid1d(nv), 256, 0, (cudaStream_t)stream>>>(nv, adj_in_dev, adj_out_dev);
    NX_CHECK_LAUNCH("adj_sort_kernel");
    nx::note_launch(1);
    return NX_OK;
}

NX_EXPORT int nx_edge_lengths(const double *xyz_dev, const int32_t *nbr_dev, int64_t nv, float *edge_dev,
                              int *err_dev, void *stream)
{
    if (nv < 0) return nx::fail(NX_EINVAL, "nx_edge_lengths: nv < 0");
    if (nv == 0) return NX_OK;
    if (!xyz_dev || !nbr_dev || !edge_dev) return nx::fail(NX_EINVAL, "nx_edge_lengths: null pointer");
    edge_len_kernel<<<grid1d(3 * nv), 256, 0, (cudaStream_t)stream>>>(xyz_dev, nbr_dev, nv, (float2 *)edge_dev, err_dev);
    NX_CHECK_LAUNCH("edge_len_kernel");
    edge_mirror_kernel<<<grid1d(6 * nv), 256, 0, (cudaStream_t)stream>>>(xyz_dev, nbr_dev, nv, (float2 *)edge_dev);
    NX_CHECK_LAUNCH("edge_mirror_kernel");
    nx::note_launch(1);
    nx::note_launch(1);
    return NX_OK;
}


// ---------------------------------------------------------------------------
// Tiling for temporally blocked erosion.
//
// Every vertex gets one grid position (face, i, j) in its home face (corners
// and edge vertices belong to the lowest-numbered face containing them);
// tile (f, i / B, j / B) collects it.  For each tile a block then collects
// the R rings of neighbours around it (breadth first over the neighbour
// table, with a shared-memory hash set), numbers them locally (members,
// ring 1, ..., ring R) and stores, for every vertex that a pass can update
// (members and rings 1..R-1), its six neighbours as local indices and its
// six edge lengths.

namespace {

__device__ __forceinline__ void home_of(int64_t v, int k, int &f, int &i, int &j)
{
    const int64_t ne = (int64_t)30 * (k - 1);
    if (v < 12) {
        f = c_home.corner_face[v];
        const int w = c_home.corner_which[v];
        i = w == 1 ? k : 0;
        j = w == 2 ? k : 0;
    } else if (v < 12 + ne) {
        const int64_t q = v - 12;
        const int e = (int)(q / (k - 1));
        const int t = (int)(q - (int64_t)e * (k - 1)) + 1;
        f = c_home.edge_face[e];
        const int pos = c_home.edge_fwd[e] ? t : k - t;
        const int sd = c_home.edge_side[e];
        if (sd == 0) { i = pos; j = 0; }
        else if (sd == 1) { i = 0; j = pos; }
        else { i = k - pos; j = pos; }
    } else {
        interior_fij(v - 12 - ne, k, f, i, j);
    }
}

__device__ __forceinline__ int64_t tile_of(int f, int i, int j, int B, int M)
{
    const int ti = i / B, tj = j / B;
    const int64_t tpf = (int64_t)(M + 1) * (M + 2) / 2;
    return (int64_t)f * tpf + (int64_t)ti * (M + 1) - (int64_t)ti * (ti - 1) / 2 + tj;
}

__global__ void tile_assign_kernel(int k, int B, int64_t nv, int R, int nmax, int32_t *__restrict__ counts,
                                   int32_t *__restrict__ ids, int *__restrict__ err)
{
    const int M = k / B;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
        int f, i, j;
        home_of(v, k, f, i, j);
        const int64_t t = tile_of(f, i, j, B, M);
        const int pos = atomicAdd(&counts[t * (R + 1)], 1);
        if (pos < nmax) ids[t * nmax + pos] = (int32_t)v;
        else atomicOr(err, 1);
    }
}

}  // namespace

// Hexagonal tiles.  On the face grid's lattice (neighbours (+-1, 0),
// (0, +-1), (+1, -1), (-1, +1)) the vertices within graph distance rho of a
// point c, max(|i - ci|, |j - cj|, |i + j - ci - cj|) <= rho, form a hexagon
// of N = 3 rho^2 + 3 rho + 1 points, and these hexagons tile the lattice
// exactly with centres c = m a + n b, a = (2 rho + 1, -rho), b = (rho,
// rho + 1) (det [a b] = N).  A hexagon is the set with the fewest vertices
// within R of it for its size, so hexagonal tiles carry fewer halo vertices
// per member than squares.  Per face the tiles are the (m, n) whose hexagon
// meets the face triangle {i, j >= 0, i + j <= k}; for each m these form one
// run of n, numbered row by row.
constexpr int HEX_ROWS_MAX = 1024;
struct HexRows {
    int rho, N;
    int m0, nrows;          // rows m = m0 .. m0 + nrows - 1
    int per_face;           // tiles per face
    int nlo[HEX_ROWS_MAX];  // first n of each row
    int base[HEX_ROWS_MAX + 1];   // local index of each row's first tile; base[nrows] = per_face
};

static inline int hex_points(int r) { return 3 * r * r + 3 * r + 1; }

// Whether the hexagon of radius rho centred at (ci, cj) holds a point of
// the face triangle: integer i, j with |i - ci|, |j - cj|, |i + j - ci - cj|
// <= rho and i, j >= 0, i + j <= k.  Every sum between ilo + jlo and
// ihi + jhi is reachable, so the box and the sum band must overlap.
static bool hex_meets_face(long long ci, long long cj, int rho, int k)
{
    const long long ilo = std::max(ci - rho, 0LL), ihi = std::min(ci + rho, (long long)k);
    const long long jlo = std::max(cj - rho, 0LL), jhi = std::min(cj + rho, (long long)k);
    const long long slo = std::max(ci + cj - rho, 0LL), shi = std::min(ci + cj + rho, (long long)k);
    return ilo <= ihi && jlo <= jhi && slo <= shi && std::max(slo, ilo + jlo) <= std::min(shi, ihi + jhi);
}

// Host: the row table of hexagonal tiles of radius rho on divisions k.
static int hex_rows(int k, int rho, HexRows &H)
{
    H.rho = rho;
    H.N = hex_points(rho);
    // lattice coordinates of a grid point: (m, n) = [a b]^-1 (i, j) =
    // ((rho + 1) i - rho j, rho i + (2 rho + 1) j) / N; over the triangle's
    // corners, widened by one centre on every side
    const double N = H.N;
    const double cm[3] = {0.0, (rho + 1.0) * k / N, -(double)rho * k / N};
    const double cn[3] = {0.0, (double)rho * k / N, (2.0 * rho + 1.0) * k / N};
    const int mlo = (int)std::floor(std::min(cm[0], std::min(cm[1], cm[2]))) - 2;
    const int mhi = (int)std::ceil(std::max(cm[0], std::max(cm[1], cm[2]))) + 2;
    const int nlo = (int)std::floor(std::min(cn[0], std::min(cn[1], cn[2]))) - 2;
    const int nhi = (int)std::ceil(std::max(cn[0], std::max(cn[1], cn[2]))) + 2;
    H.nrows = 0;
    H.m0 = 0;
    int total = 0;
    for (int m = mlo; m <= mhi; ++m) {
        int first = INT_MAX, last = INT_MIN;
        for (int n = nlo; n <= nhi; ++n) {
            const long long ci = (long long)m * (2 * rho + 1) + (long long)n * rho;
            const long long cj = -(long long)m * rho + (long long)n * (rho + 1);
            if (hex_meets_face(ci, cj, rho, k)) {
                if (first == INT_MAX) first = n;
                else if (n != last + 1)
                    return nx::fail(NX_EINVAL, "hexagonal tiling: row %d of divisions %d is not one run", m, k);
                last = n;
            }
        }
        if (first == INT_MAX) {
            if (H.nrows > 0) break;      // past the last row
            continue;
        }
        if (H.nrows == 0) H.m0 = m;
        else if (m != H.m0 + H.nrows)
            return nx::fail(NX_EINVAL, "hexagonal tiling: rows of divisions %d are not contiguous", k);
        if (H.nrows >= HEX_ROWS_MAX)
            return nx::fail(NX_EINVAL, "hexagonal tiling: more than %d rows (divisions %d, radius %d)", HEX_ROWS_MAX, k, rho);
        H.nlo[H.nrows] = first;
        H.base[H.nrows] = total;
        total += last - first + 1;
        ++H.nrows;
    }
    H.base[H.nrows] = total;
    H.per_face = total;
    return total > 0 ? NX_OK : nx::fail(NX_EINVAL, "hexagonal tiling: no tiles");
}

namespace {

__device__ __forceinline__ int floor_div(int a, int b) { return a >= 0 ? a / b : -((b - 1 - a) / b); }

// Tile of a grid point: the centre within rho is one of the four lattice
// points at the floors of its lattice coordinates and their +1 neighbours.
__device__ __forceinline__ int64_t hex_tile_of(int f, int i, int j, const HexRows &H)
{
    const int rho = H.rho;
    const int m0 = floor_div((rho + 1) * i - rho * j, H.N), n0 = floor_div(rho * i + (2 * rho + 1) * j, H.N);
    for (int q = 0; q < 4; ++q) {
        const int m = m0 + (q & 1), n = n0 + (q >> 1);
        const int di = i - (m * (2 * rho + 1) + n * rho), dj = j - (-m * rho + n * (rho + 1));
        if (max(abs(di), max(abs(dj), abs(di + dj))) <= rho) {
            const int r = m - H.m0;
            if (r < 0 || r >= H.nrows) return -1;
            const int loc = H.base[r] + n - H.nlo[r];
            if (n < H.nlo[r] || loc >= H.base[r + 1]) return -1;
            return (int64_t)f * H.per_face + loc;
        }
    }
    return -1;
}

__global__ void tile_assign_hex_kernel(int k, int64_t nv, int R, int nmax, int32_t *__restrict__ counts,
                                       int32_t *__restrict__ ids, int *__restrict__ err,
                                       const __grid_constant__ HexRows H)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
        int f, i, j;
        home_of(v, k, f, i, j);
        const int64_t t = hex_tile_of(f, i, j, H);
        if (t < 0) {
            atomicOr(err, 2);
            continue;
        }
        const int pos = atomicAdd(&counts[t * (R + 1)], 1);
        if (pos < nmax) ids[t * nmax + pos] = (int32_t)v;
        else atomicOr(err, 1);
    }
}

// Per-tile hash set of vertex ids in shared memory: 2^bits entries, the
// smallest power of two with at least twice the tile's local bound (load
// factor <= 1/2), linear probing.
struct HashSet {
    int bits;
    uint32_t mask;
};

__host__ __device__ __forceinline__ int hash_bits_for(int nmax)
{
    int b = 6;
    while ((1 << b) < 2 * nmax) ++b;
    return b;
}

__device__ __forceinline__ uint32_t hslot(const HashSet &H, int32_t v)
{
    return ((uint32_t)v * 2654435761u) >> (32 - H.bits);
}

// Insert v (bounded probing); returns its local index, assigning the next
// one if v is new.  -1 if the set or the list is full.
__device__ __forceinline__ int hinsert(const HashSet &H, int32_t *key, int32_t *val, int32_t *list, int *cnt, int nmax,
                                       int32_t v)
{
    uint32_t h = hslot(H, v);
    for (uint32_t probe = 0; probe <= H.mask; ++probe) {
        const int32_t old = atomicCAS(&key[h], -1, v);
        if (old == -1) {
            const int idx = atomicAdd(cnt, 1);
            if (idx >= nmax) { val[h] = -1; return -1; }
            list[idx] = v;
            val[h] = idx;
            return idx;
        }
        if (old == v) return 0;       // present (its index is read after a barrier)
        h = (h + 1) & H.mask;
    }
    return -1;
}

__device__ __forceinline__ int hfind(const HashSet &H, const int32_t *key, const int32_t *val, int32_t v)
{
    uint32_t h = hslot(H, v);
    for (uint32_t probe = 0; probe <= H.mask; ++probe) {
        const int32_t kk = key[h];
        if (kk == v) return val[h];
        if (kk == -1) return -1;
        h = (h + 1) & H.mask;
    }
    return -1;
}

__global__ void __launch_bounds__(512) tile_rings_kernel(const int32_t *__restrict__ nbr, const float *__restrict__ edge,
                                                         int64_t nv, int R, int nmax, int cmax, int32_t *__restrict__ counts,
                                                         int32_t *__restrict__ ids, uint16_t *__restrict__ lnbr,
                                                         float *__restrict__ ledge, int *__restrict__ err)
{
    extern __shared__ int32_t sh[];
    HashSet H;
    H.bits = hash_bits_for(nmax);
    H.mask = (1u << H.bits) - 1u;
    const int hcap = 1 << H.bits;
    int32_t *key = sh;                      // hcap
    int32_t *val = key + hcap;              // hcap
    int32_t *list = val + hcap;             // local vertices; list + nmax: sort scratch
    __shared__ int s_cnt, s_bad;
    __shared__ int s_ring[16];
    const int64_t tile = blockIdx.x;
    int32_t *tc = counts + tile * (R + 1);
    int32_t *tid = ids + tile * nmax;
    int T = tc[0];
    if (T > nmax) T = nmax;
    int P2 = 1;
    while (P2 < T) P2 <<= 1;
    for (int q = threadIdx.x; q < hcap; q += blockDim.x) key[q] = -1;
    for (int q = threadIdx.x; q < P2; q += blockDim.x) list[q] = q < T ? tid[q] : 0x7FFFFFFF;
    if (threadIdx.x == 0) { s_cnt = 0; s_bad = 0; }
    __syncthreads();
    // members in ascending id order (row segments -> coalesced accesses)
    for (int size = 2; size <= P2; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int q = threadIdx.x; q < P2; q += blockDim.x) {
                const int o = q ^ stride;
                if (o > q) {
                    const bool up = (q & size) == 0;
                    const int32_t a = list[q], b = list[o];
                    if ((a > b) == up) { list[q] = b; list[o] = a; }
                }
            }
            __syncthreads();
        }
    for (int q = threadIdx.x; q < T; q += blockDim.x) {
        // members take local indices 0..T-1 in sorted order
        const int32_t v = list[q];
        uint32_t h = hslot(H, v);
        for (uint32_t probe = 0; probe <= H.mask; ++probe) {
            if (atomicCAS(&key[h], -1, v) == -1) { val[h] = q; break; }
            h = (h + 1) & H.mask;
        }
    }
    if (threadIdx.x == 0) s_cnt = T;
    __syncthreads();
    int beg = 0, end = T;
    for (int r = 1; r <= R; ++r) {
        const int nwork = (end - beg) * 6;
        // two slots per thread per round, both reads issued first (the
        // ring's order is fixed by the sort below, not by insertion order)
        for (int w0 = threadIdx.x; w0 < nwork; w0 += 2 * blockDim.x) {
            int32_t jv[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int w = w0 + u * blockDim.x;
                jv[u] = w < nwork ? nbr[6 * (int64_t)list[beg + w / 6] + (w % 6)] : -1;
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int32_t j = jv[u];
                if (j < 0) continue;
                if ((int64_t)j >= nv) { s_bad = 1; continue; }
                if (hinsert(H, key, val, list, &s_cnt, nmax, j) < 0) s_bad = 1;
            }
        }
        __syncthreads();
        beg = end;
        end = min(s_cnt, nmax);
        if (threadIdx.x == 0) s_ring[r] = end - beg;
        __syncthreads();
    }
    const int NL = end;
    // each ring in ascending id order too (neighbouring vertices get nearby
    // local indices: fewer shared-memory bank conflicts in the erosion pass),
    // then the hash values follow the new positions
    {
        int32_t *scr = list + nmax;        // scratch of nmax entries
        int rb = T;
        for (int r = 1; r <= R; ++r) {
            const int re = rb + s_ring[r];
            const int ln = re - rb;
            // rank sort (the ids of a ring are distinct): each entry's
            // position is the number of smaller ids, read as broadcasts
            for (int q = threadIdx.x; q < ln; q += blockDim.x) {
                const int32_t v = list[rb + q];
                int rank = 0;
                for (int x = 0; x < ln; ++x) rank += list[rb + x] < v ? 1 : 0;
                scr[rank] = v;
            }
            __syncthreads();
            for (int q = threadIdx.x; q < ln; q += blockDim.x) {
                const int32_t v = scr[q];
                list[rb + q] = v;
                uint32_t h = hslot(H, v);
                for (uint32_t probe = 0; probe <= H.mask; ++probe) {
                    if (key[h] == v) { val[h] = rb + q; break; }
                    h = (h + 1) & H.mask;
                }
            }
            __syncthreads();
            rb = re;
        }
    }
    int C0 = T;
    for (int r = 1; r < R; ++r) C0 += s_ring[r];
    if (C0 > cmax) { if (threadIdx.x == 0) s_bad = 1; C0 = cmax; }
    __syncthreads();
    for (int q = threadIdx.x; q < NL; q += blockDim.x) tid[q] = list[q];
    // four slots per thread per round, their global reads issued before any
    // hash probe (independent loads in flight instead of a dependent chain)
    constexpr int U = 4;
    const int nslot = C0 * 6;
    for (int w0 = threadIdx.x; w0 < nslot; w0 += U * blockDim.x) {
        int32_t jv[U];
        float2 ev[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int w = w0 + u * blockDim.x;
            if (w < nslot) {
                const int64_t g = 6 * (int64_t)list[w / 6] + w % 6;
                jv[u] = nbr[g];
                ev[u] = reinterpret_cast<const float2 *>(edge)[g];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int w = w0 + u * blockDim.x;
            if (w < nslot) {
                const int q = w / 6, sl = w % 6;
                // a missing neighbour (-1, pentagon slot) points at the vertex
                // itself: the erosion update then sees equal heights and adds
                // nothing
                int loc = q;
                if (jv[u] >= 0) {
                    loc = hfind(H, key, val, jv[u]);
                    if (loc < 0) { s_bad = 1; loc = q; }
                }
                lnbr[((int64_t)tile * cmax + q) * 6 + sl] = (uint16_t)loc;
                reinterpret_cast<float2 *>(ledge)[((int64_t)tile * cmax + q) * 6 + sl] = ev[u];
            }
        }
    }
    if (threadIdx.x == 0) {
        tc[0] = T;
        for (int r = 1; r <= R; ++r) tc[r] = s_ring[r];
        atomicMax(&err[1], NL);
        atomicMax(&err[2], C0);
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_bad) atomicOr(err, 2);
}

}  // namespace

static_assert(sizeof(nx_tiling) == 48, "tiling descriptor layout");

// Local and updatable capacities of tiles whose members lie within graph
// distance `reach` of a point or square (see nx_tiling_shape).
static int tile_caps(int64_t nm, int64_t cm, int32_t *nmax, int32_t *cmax)
{
    cm = (cm + 3) & ~(int64_t)3;                     // cm*12 B: 16-byte units
    if (cm > nm) cm = nm & ~(int64_t)3;
    if (nm > 4096) return nx::fail(NX_EINVAL, "nx_tiling_shape: tile too large (%lld local vertices)", (long long)nm);
    *nmax = (int32_t)nm;
    *cmax = (int32_t)cm;
    return NX_OK;
}

NX_EXPORT int nx_tiling_shape(int k, int tile, int rings, int32_t *ntiles, int32_t *nmax, int32_t *cmax)
{
    if (k < 1 || rings < 1 || rings > 8 || !ntiles || !nmax || !cmax || (tile >= 0 && tile < 2) || tile < -64 ||
        tile == -1)
        return nx::fail(NX_EINVAL, "nx_tiling_shape: bad arguments");
    if (tile < 0) {
        // hexagons of radius rho: the vertices within R of a tile lie within
        // rho + R of its centre (on the flat lattice of a face and across an
        // edge onto the next face; around the twelve five-neighbour corners
        // the count only drops), at most hex_points(rho + R); 6(rho + R) of
        // slack as for squares
        const int rho = -tile;
        HexRows H;
        int rc = hex_rows(k, rho, H);
        if (rc) return rc;
        const int64_t nt = (int64_t)20 * H.per_face;
        if (nt > 0x7FFFFFFF) return nx::fail(NX_EINVAL, "nx_tiling_shape: too many tiles");
        rc = tile_caps(hex_points(rho + rings) + 6 * (rho + rings), hex_points(rho + rings - 1) + 6 * (rho + rings - 1),
                       nmax, cmax);
        if (rc) return rc;
        *ntiles = (int32_t)nt;
        return NX_OK;
    }
    const int M = k / tile;
    const int64_t nt = (int64_t)20 * (M + 1) * (M + 2) / 2;
    // A tile holds at most B x B members of one face grid.  On the lattice
    // of the face grids (six neighbours: (+-1, 0), (0, +-1), (+1, -1),
    // (-1, +1)) the vertices within graph distance R of a B x B square form
    // the square widened by R on every side less two corners, fewer than
    // (B + 2R)^2; at the twelve five-neighbour corners the count only drops.
    // The bounds keep 4(B + 2R) of slack (overflow is still detected and
    // reported by the build); the updatable set (rings below R) uses R - 1.
    const int64_t B = tile, D = B + 2 * (int64_t)rings, Dc = D - 2;
    if (nt > 0x7FFFFFFF) return nx::fail(NX_EINVAL, "nx_tiling_shape: too many tiles");
    const int rc = tile_caps(D * D + 4 * D, Dc * Dc + 4 * Dc, nmax, cmax);
    if (rc) return rc;
    *ntiles = (int32_t)nt;
    return NX_OK;
}

NX_EXPORT int nx_tiling_build(int k, int tile, int rings, const int32_t *nbr_dev, const float *edge_dev,
                              int32_t *counts_dev, int32_t *ids_dev, uint16_t *lnbr_dev, float *ledge_dev, int *err_dev,
                              void *stream)
{
    int32_t nt = 0, nmax = 0, cmax = 0;
    int rc = nx_tiling_shape(k, tile, rings, &nt, &nmax, &cmax);
    if (rc) return rc;
    if (!nbr_dev || !edge_dev || !counts_dev || !ids_dev || !lnbr_dev || !ledge_dev || !err_dev)
        return nx::fail(NX_EINVAL, "nx_tiling_build: null pointer");
    int dev = 0;
    NX_CHECK_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64 || !g_tables_ready[dev]) return nx::fail(NX_EINVAL, "nx_tiling_build: call nx_icosphere_tables first");
    const int64_t nv = (int64_t)10 * k * k + 2;
    cudaStream_t s = (cudaStream_t)stream;
    NX_CHECK_CUDA(cudaMemsetAsync(counts_dev, 0, sizeof(int32_t) * (size_t)nt * (rings + 1), s));
    if (tile < 0) {
        HexRows H;
        rc = hex_rows(k, -tile, H);
        if (rc) return rc;
        tile_assign_hex_kernel<<<grid1d(nv), 256, 0, s>>>(k, nv, rings, nmax, counts_dev, ids_dev, err_dev, H);
        NX_CHECK_LAUNCH("tile_assign_hex_kernel");
    } else {
        tile_assign_kernel<<<grid1d(nv), 256, 0, s>>>(k, tile, nv, rings, nmax, counts_dev, ids_dev, err_dev);
        NX_CHECK_LAUNCH("tile_assign_kernel");
    }
    int P2 = 1;
    while (P2 < nmax) P2 <<= 1;
    // hash keys + values, the local list (padded for sorting) and a scratch
    const size_t smem = sizeof(int32_t) * (2 * ((size_t)1 << hash_bits_for(nmax)) + 2 * (size_t)P2);
    NX_CHECK_CUDA(cudaFuncSetAttribute(tile_rings_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    tile_rings_kernel<<<nt, 512, smem, s>>>(nbr_dev, edge_dev, nv, rings, nmax, cmax, counts_dev, ids_dev, lnbr_dev,
                                            ledge_dev, err_dev);
    NX_CHECK_LAUNCH("tile_rings_kernel");
    nx::note_launch(2);
    return NX_OK;
}

// ---------------------------------------------------------------------------
// Nearest three vertices of query points (the reference's KD-tree
// query(k=3), nixis.py:278-283), by point location in the icosphere's own
// structure: the face whose corner matrix gives the query direction the
// largest smallest barycentric weight, the grid triangle of the flat face
// point (the spherical triangles are radial projections of the flat ones),
// then the exact distances to that triangle's vertices and all their
// neighbours.  On the icosphere's near-equilateral triangles the three
// nearest vertices of a point are always among them (checked against brute
// force in the tests).  Distances sqrt((dx*dx + dy*dy) + dz*dz), ascending,
// ties by vertex id.

namespace {

__global__ void __launch_bounds__(256) nearest3_kernel(int k, const double *__restrict__ xyz,
                                                       const int32_t *__restrict__ nbr, int64_t nv,
                                                       const double *__restrict__ q, int64_t nq,
                                                       double *__restrict__ dist, int64_t *__restrict__ idx)
{
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nq; p += (int64_t)gridDim.x * blockDim.x) {
        const double qx = q[3 * p], qy = q[3 * p + 1], qz = q[3 * p + 2];
        int bf = 0;
        double bw[3] = {0, 0, 0}, bs = -INFINITY;
        for (int f = 0; f < 20; ++f) {
            double w[3];
            for (int r = 0; r < 3; ++r) w[r] = c_ico.inv[f][r][0] * qx + c_ico.inv[f][r][1] * qy + c_ico.inv[f][r][2] * qz;
            const double sc = fmin(w[0], fmin(w[1], w[2]));
            if (sc > bs) { bs = sc; bf = f; bw[0] = w[0]; bw[1] = w[1]; bw[2] = w[2]; }
        }
        const double tot = bw[0] + bw[1] + bw[2];
        const double fi = fmin(fmax(bw[1] / tot, 0.0), 1.0) * k, fj = fmin(fmax(bw[2] / tot, 0.0), 1.0) * k;
        int i0 = (int)floor(fi), j0 = (int)floor(fj);
        if (i0 > k - 1) i0 = k - 1;
        if (i0 < 0) i0 = 0;
        if (j0 > k - 1 - i0) j0 = k - 1 - i0;
        if (j0 < 0) j0 = 0;
        const bool up = (fi - i0) + (fj - j0) <= 1.0 || i0 + j0 == k - 1;
        int32_t tri[3];
        if (up) {
            tri[0] = face_vid(bf, i0, j0, k); tri[1] = face_vid(bf, i0 + 1, j0, k); tri[2] = face_vid(bf, i0, j0 + 1, k);
        } else {
            tri[0] = face_vid(bf, i0 + 1, j0, k); tri[1] = face_vid(bf, i0 + 1, j0 + 1, k);
            tri[2] = face_vid(bf, i0, j0 + 1, k);
        }
        double bd[3] = {INFINITY, INFINITY, INFINITY};
        int64_t bi[3] = {-1, -1, -1};
        for (int c = 0; c < 21; ++c) {
            const int32_t v = c < 3 ? tri[c] : nbr[6 * (int64_t)tri[(c - 3) / 6] + (c - 3) % 6];
            if (v < 0 || (int64_t)v >= nv) continue;
            if (v == bi[0] || v == bi[1] || v == bi[2]) continue;
            const double dx = __dsub_rn(qx, xyz[3 * (int64_t)v]), dy = __dsub_rn(qy, xyz[3 * (int64_t)v + 1]),
                         dz = __dsub_rn(qz, xyz[3 * (int64_t)v + 2]);
            const double d = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
            int m = 3;
            while (m > 0 && (d < bd[m - 1] || (d == bd[m - 1] && v < bi[m - 1]))) --m;
            if (m < 3) {
                for (int r = 2; r > m; --r) { bd[r] = bd[r - 1]; bi[r] = bi[r - 1]; }
                bd[m] = d;
                bi[m] = v;
            }
        }
        for (int m = 0; m < 3; ++m) {
            dist[3 * p + m] = bd[m];
            idx[3 * p + m] = bi[m];
        }
    }
}

}  // namespace

NX_EXPORT int nx_nearest3(int k, const double *xyz_dev, const int32_t *nbr_dev, int64_t nv, const double *q_dev,
                          int64_t nq, double *dist_dev, int64_t *idx_dev, void *stream)
{
    if (k < 1 || nv != 10 * (int64_t)k * k + 2 || nq < 0) return nx::fail(NX_EINVAL, "nx_nearest3: bad sizes");
    if (nq == 0) return NX_OK;
    if (!xyz_dev || !nbr_dev || !q_dev || !dist_dev || !idx_dev) return nx::fail(NX_EINVAL, "nx_nearest3: null pointer");
    int dev = 0;
    NX_CHECK_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64 || !g_tables_ready[dev]) return nx::fail(NX_EINVAL, "nx_nearest3: icosphere tables not set");
    nearest3_kernel<<<grid1d(nq), 256, 0, (cudaStream_t)stream>>>(k, xyz_dev, nbr_dev, nv, q_dev, nq, dist_dev, idx_dev);
    NX_CHECK_LAUNCH("nearest3_kernel");
    nx::note_launch(1);
    return NX_OK;
}
