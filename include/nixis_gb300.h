/*
 * nixis_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the Nixis
 * per-vertex terrain hot path: fractal OpenSimplex-3D noise, erosion
 * (variant 3) and insolation accumulation, plus the icosphere/adjacency
 * generator that feeds them, the batched and served multi-planet paths,
 * and the next functions around them: height shaping (rescale,
 * power_rescale, percentiles, masks), latitude-table insolation, starting
 * surface temperatures and equirectangular map sampling.
 *
 * Conventions
 *  - Every function returns an int status: NX_OK (0) or one of the NX_E*
 *    codes; nx_last_error() gives a message for the calling host thread.
 *    Nothing throws across the ABI.
 *  - Pointers named *_dev are device pointers owned by the caller; the
 *    library never frees them.  `stream` is a cudaStream_t (NULL = legacy
 *    default stream).  Calls are stream ordered and do not synchronise the
 *    device unless stated.
 *  - Layouts follow the reference: vertices float64 (n,3) row-major,
 *    neighbours int32 (n,6) with -1 in unused slots, fields (n,).
 *
 * Reference citations are paths within the MightyBOBcnc/nixis project.
 */
#ifndef NIXIS_GB300_H
#define NIXIS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NX_OK 0
#define NX_EINVAL 1   /* bad argument (null pointer, size, range) */
#define NX_ENOMEM 2   /* device memory exhausted or budget exceeded */
#define NX_ECUDA 3    /* CUDA runtime error */
#define NX_ETIMEOUT 4 /* a bounded device-side wait gave up */
#define NX_ERANGE 5   /* input outside the supported numeric range */

#define NX_MAX_OCTAVES 32

/* Message for the last failing call on this host thread ("" if none). */
const char *nx_last_error(void);

/* Library version, major*10000 + minor*100 + patch. */
int nx_version(void);

/* Number of kernels this library has launched in this process (all
 * entry points); used to report launch counts. */
unsigned long long nx_launch_count(void);

/* ------------------------------------------------------------------ */
/* OpenSimplex tables                                                  */
/* ------------------------------------------------------------------ */

/* Replaces opensimplex.init (opensimplex.py:90-107), host only.
 * perm, pgi: host int32[256].  Bit-exact with the reference, including
 * the int32 truncation of `over` (opensimplex.py:110-112). */
int nx_perm_init(int64_t seed, int32_t *perm, int32_t *pgi);

/* ------------------------------------------------------------------ */
/* Noise                                                               */
/* ------------------------------------------------------------------ */

/* Fused fBm over octaves; the kernel behind terrain.sample_octaves
 * (terrain.py:32-59) and terrain.sample_noise (terrain.py:12-28).
 * For every vertex v:
 *   acc = sum_o (noise3d(v * scale[o]) + 1) * 0.5 * strength[o] * radius
 * (opensimplex.noise3d, opensimplex.py:266-759), computed in binary32
 * with the lattice cell, region and extra lattice points decided exactly
 * as binary64 would.  scale/strength: host double[n_octaves].
 * Output: elev_f64_dev (if not NULL) gets acc (accumulate=0) or
 * elev += acc (accumulate=1); elev_f32_dev likewise.  perm_dev/pgi_dev:
 * device int32[256].  n_fallback_dev (optional, device uint64) counts
 * vertex-octaves whose decisions needed the binary64 path. */
int nx_fbm(const double *xyz_dev, int64_t n, const int32_t *perm_dev, const int32_t *pgi_dev,
           int n_octaves, const double *scale, const double *strength, double radius,
           double *elev_f64_dev, float *elev_f32_dev, int accumulate,
           unsigned long long *n_fallback_dev, void *stream);

/* terrain.sample_octaves (terrain.py:32-59) argument convention: octave o
 * uses scale = f_o / world_radius and strength = a_o / world_radius with
 * f_0 = n_init_roughness, a_0 = n_init_strength, f *= n_roughness,
 * a *= n_persistence, exactly as the reference computes them. */
int nx_sample_octaves(const double *xyz_dev, int64_t n, const int32_t *perm_dev,
                      const int32_t *pgi_dev, int n_octaves, double n_init_roughness,
                      double n_init_strength, double n_roughness, double n_persistence,
                      double world_radius, double *elev_f64_dev, float *elev_f32_dev,
                      int accumulate, void *stream);

/* Single-octave noise3d with the integer decisions exposed (test/debug).
 * value_dev: float[n] = noise3d(v * scale); trace_dev (optional):
 * int32[n*10] = [xsb, ysb, zsb, region(0 tetra@0, 1 tetra@1, 2 octa),
 * ext0 xyz, ext1 xyz]; slots_dev (optional): int32[n*9*5], per evaluated
 * lattice point [x, y, z, gradient index (perm_grad_index_3D value),
 * used(0/1)]. */
int nx_noise3d_trace(const double *xyz_dev, int64_t n, const int32_t *perm_dev,
                     const int32_t *pgi_dev, double scale, float *value_dev, int32_t *trace_dev,
                     int32_t *slots_dev, unsigned long long *n_fallback_dev, void *stream);


/* fBm in pair precision: the kernel behind the planet paths (batched,
 * plain, served) and terrain.sample_octaves' binary64 output.  Same sum as
 * nx_fbm, with the same exactly-decided lattice cells, regions and extra
 * points, but every continuous quantity carried as an unevaluated pair
 * hi + lo of binary32s: results lie within ~1e-13 of the binary64
 * reference's sums (eroded planets need this: the erosion update branches
 * on the sign of neighbour height differences, which binary32 noise flips).
 * pair_dev (optional, 8-byte aligned): float[2n], vertex v's running sum as
 * (hi, lo) -- written (accumulate = 0) or added to (accumulate = 1);
 * elev_f64_dev (optional): the sum as binary64 (= hi + lo exactly), or
 * added to it when accumulate = 1 and pair_dev is NULL.  minmax_dev
 * (optional, device uint64[2], caller sets {~0, 0}): atomically folded
 * min and max ordered keys of the resulting pair sums, key(h, l) =
 * (fkey(h) << 32) | fkey(l) with fkey(f) = f >= 0 ? bits ^ 0x80000000 :
 * ~bits.  A running sum is renormalised after every octave, so one launch
 * over all octaves and one launch per octave give the same bits, given the
 * same amp_ref: octaves whose amplitude 0.5*strength*radius is below
 * amp_ref/8 take a cheaper displacement form (amp_ref <= 0: the largest
 * amplitude among this call's octaves; a planet evaluated one octave per
 * call passes its first octave's amplitude). */
int nx_fbm_pair(const double *xyz_dev, int64_t n, const int32_t *perm_dev, const int32_t *pgi_dev, int n_octaves,
                const double *scale, const double *strength, double radius, double amp_ref, float *pair_dev,
                double *elev_f64_dev, int accumulate, unsigned long long *minmax_dev,
                unsigned long long *n_fallback_dev, void *stream);

/* One planet of a batched fBm launch (device-resident array of these);
 * the batch runs the pair path of nx_fbm_pair. */
typedef struct nx_fbm_planet {
    const double *xyz;      /* (n,3) float64 vertices (its mesh) */
    int64_t n;
    const int32_t *perm;    /* device int32[256] tables of its seed */
    const int32_t *pgi;
    float *out;             /* float[2n], 8-byte aligned: (hi, lo) pair sums over octaves */
    unsigned long long *minmax; /* optional: min, max ordered keys as in nx_fbm_pair; caller sets {~0, 0} */
    int32_t n_octaves;
    int32_t chunk0;         /* index of its first chunk: sum of ceil(n/chunk) of earlier planets */
    int32_t pow2;           /* filled: 1 when every scale is a power of two */
    uint32_t norm_mask;     /* filled: bit o set when octave o renormalises (amplitude >= 1/8 of the largest) */
    float s1[NX_MAX_OCTAVES];     /* filled by nx_fbm_planet_fill: scale[o] = s1 + s2 + s3 exactly */
    float s2[NX_MAX_OCTAVES];
    float s3[NX_MAX_OCTAVES];
    float amp_hi[NX_MAX_OCTAVES]; /* 0.5 * strength[o] * radius as a pair */
    float amp_lo[NX_MAX_OCTAVES];
    double s[NX_MAX_OCTAVES];
} nx_fbm_planet;

/* Host: fill a planet's octave constants (same meaning as nx_fbm). */
int nx_fbm_planet_fill(nx_fbm_planet *planet, int n_octaves, const double *scale, const double *strength,
                       double radius);

/* Vertices per work item of nx_fbm_batch (for chunk0). */
int nx_fbm_chunk_size(void);

/* fBm of many planets (uneven sizes, seeds, octave counts) in one
 * persistent launch; planets_dev/planets_host: the same array on device
 * and host. */
int nx_fbm_batch(const nx_fbm_planet *planets_dev, const nx_fbm_planet *planets_host, int nplanets,
                 unsigned long long *n_fallback_dev, void *stream);

/* ------------------------------------------------------------------ */
/* Mesh: icosphere, adjacency, edge lengths                            */
/* ------------------------------------------------------------------ */

/* Upload the icosahedron tables (12 corners as float64[36], faces int32[60],
 * per face side edge id and direction int32[120], edges int32[60]) for the
 * current device; nixis_gb300/icosphere.py defines them.  Once per device. */
int nx_icosphere_tables(const double *corners, const int32_t *faces, const int32_t *face_edges,
                        const int32_t *edges);

/* Icosphere with k divisions (replaces meshzoo.icosa_sphere at util.py:43):
 * xyz_dev float64[(10k^2+2)*3] and/or tris_dev int32[20k^2*3] (either may be
 * NULL).  Corners are vertices 0-11; layout in nixis_gb300/icosphere.py. */
int nx_icosphere(int k, double *xyz_dev, int32_t *tris_dev, void *stream);

/* Workspace bytes for nx_build_adjacency. */
size_t nx_adjacency_workspace_size(int64_t nv);

/* util.build_adjacency (util.py:591-613) for nv = (nt+4)/2 vertices:
 * adj_dev int32[nv*6], row order = triangle order, -1 padding.  err_dev
 * (device int, caller zeroes it) gets bit 0 for an out-of-range vertex id,
 * bit 1 for a vertex with more than 6 neighbours. */
int nx_build_adjacency(const int32_t *tris_dev, int64_t nt, int64_t nv, int32_t *adj_dev, void *workspace,
                       size_t ws_bytes, int *err_dev, void *stream);

/* util.sort_adjacency (util.py:638-662), out of place: rows of adj_in are
 * walked into rings (vertices 0-11 have 5 neighbours) and written to adj_out. */
int nx_sort_adjacency(const int32_t *adj_in_dev, int32_t *adj_out_dev, int64_t nv, void *stream);

/* Per-slot neighbour distance |v_i - v_j| in binary64 (erosion.calc_distance,
 * erosion.py:38-40) split into a pair hi + lo of binary32s: edge_dev
 * float[nv*6*2], (hi, lo) per slot, 0 for -1 slots.
 * err_dev (optional) gets bit 0 for an out-of-range neighbour id. */
int nx_edge_lengths(const double *xyz_dev, const int32_t *nbr_dev, int64_t nv, float *edge_dev, int *err_dev,
                    void *stream);

/* Tiling of a mesh for temporally blocked erosion: every vertex belongs to
 * one tile of its home face's grid -- for tile > 0 a tile x tile square,
 * for tile < 0 a hexagon of the grid points within graph distance -tile
 * (2..64) of a centre (hexagons carry fewer halo vertices per member); each
 * tile lists its members, then `rings` rings of neighbours (local numbering),
 * and, for members and rings 1..rings-1, the six neighbours as local
 * indices and the six edge lengths. */
typedef struct nx_tiling {
    int32_t ntiles;
    int32_t rings;
    int32_t nmax;              /* local vertices per tile (capacity) */
    int32_t cmax;              /* updatable vertices per tile (capacity) */
    const int32_t *counts;     /* ntiles x (rings + 1): members, then each ring's size */
    const int32_t *ids;        /* ntiles x nmax global vertex ids */
    const uint16_t *lnbr;      /* ntiles x cmax x 6 local neighbour indices, 0xFFFF = none */
    const float *ledge;        /* ntiles x cmax x 6 edge lengths, (hi, lo) pairs */
} nx_tiling;

/* Host: sizes of the tiling of divisions k (tile: square side, or minus
 * the hexagon radius). */
int nx_tiling_shape(int k, int tile, int rings, int32_t *ntiles, int32_t *nmax, int32_t *cmax);

/* Build a tiling from the mesh's neighbour table and edge lengths into
 * caller buffers sized by nx_tiling_shape (counts int32[ntiles*(rings+1)],
 * ids int32[ntiles*nmax], lnbr uint16[ntiles*cmax*6], ledge
 * float[ntiles*cmax*6*2]).  err_dev (device int[3], caller zeroes it):
 * [0] bit 0 = a tile exceeded nmax members, bit 1 = a halo or neighbour
 * problem; [1] largest local vertex count; [2] largest updatable count. */
int nx_tiling_build(int k, int tile, int rings, const int32_t *nbr_dev, const float *edge_dev,
                    int32_t *counts_dev, int32_t *ids_dev, uint16_t *lnbr_dev, float *ledge_dev, int *err_dev,
                    void *stream);

/* ------------------------------------------------------------------ */
/* Erosion (variant 3)                                                 */
/* ------------------------------------------------------------------ */

/* One planet of an erosion launch.  Its state occupies rows [vbeg, vbeg+n)
 * of the state buffers; nbr (n,6) local neighbour ids and edge (n,6,2)
 * per-slot lengths (pairs, as nx_edge_lengths writes them) are its mesh (device pointers, shared by planets of
 * equal divisions).  `rain` is added to every water value before each
 * iteration (erode_terrain3 adds 0.3/320, erosion.py:182-183; 0 gives bare
 * erosion_iteration3 steps).  Its iteration t runs at global step
 * t_start + t; `slot` is its control block in the workspace.  Batches
 * (nx_erosion_batch) use t_start = 0, slot = index, and order planets by
 * non-increasing `iters`. */
typedef struct nx_erosion_planet {
    int64_t vbeg;
    int64_t n;
    const int32_t *nbr;
    const float *edge;
    int32_t iters;
    float rain;
    int32_t t_start;
    int32_t slot;
    const nx_tiling *tiling;   /* device copy of the mesh's tiling, or NULL */
    int32_t ntiles;            /* its ntiles (read on the host) */
    int32_t maxnl;             /* its largest local vertex count */
    int32_t maxc;              /* its largest updatable count (tables held in shared memory) */
    int32_t pad;
} nx_erosion_planet;

/* Workspace bytes for erosion over n_padded_total state rows (a bound on
 * 256 x the blocks a launch covers) and nplanets control blocks (control
 * words, per-block partial sums and block map). */
size_t nx_erosion_workspace_size(int64_t n_padded_total, int nplanets);

/* Zero the per-planet control words (scale exponent 0) of a workspace. */
int nx_erosion_ctl_init(void *workspace, size_t ws_bytes, int nplanets, void *stream);

/* Erosion state: a row of 8 floats per vertex, (h_hi, h_lo, w_hi, w_lo,
 * s_hi, s_lo, 0, 0): height, water and sediment each an unevaluated sum
 * hi + lo of binary32s; values are true values * 2^-K for the planet's
 * scale exponent K (below). */

/* Load binary64 fields (the reference's r_buff/heights, wat, sed; w/s may
 * be NULL for zeros) into the state st_dev float[8n], choosing a
 * power-of-two scale so every value fits. */
int nx_erosion_load(const double *h64_dev, const double *w64_dev, const double *s64_dev, int64_t n, float *st_dev,
                    void *workspace, size_t ws_bytes, void *stream);

/* `iters` Jacobi iterations of erosion.erosion_iteration3 (erosion.py:
 * 197-279) on one planet, result left in st_dev.  st_tmp_dev: second
 * buffer of the same size.  planet_dev: device scratch for one
 * nx_erosion_planet.  mass_dev (optional): float64[iters*3] per-iteration
 * (sum h, sum w, sum s), compensated, in true units.  flow_dev (optional):
 * uint16[n], per slot k bits 2k..2k+1 = 1 if the neighbour is higher, 2 if
 * lower (the reference's slope > 0 / < 0 choice), of the last iteration. */
int nx_erosion_steps(const int32_t *nbr_dev, const float *edge_dev, int64_t n, float *st_dev, float *st_tmp_dev,
                     int iters, float rain, nx_erosion_planet *planet_dev, double *mass_dev, uint16_t *flow_dev,
                     void *workspace, size_t ws_bytes, void *stream);

/* Batched erosion: every planet runs its own iteration count.  If every
 * planet has a tiling (with tiling->rings = R) and neither mass sums nor
 * flow bits are requested, iterations run temporally blocked: one launch per
 * pass of up to R iterations, each block updating one tile in shared
 * memory; otherwise one launch per iteration over the planets still
 * running.  Both give the same results.  A planet's state starts
 * in buffer (iters & 1) -- 0: st_dev, 1: st_tmp_dev -- and ends in st_dev.
 * mass_dev (optional): float64[max_iters][nplanets][3].  Call
 * nx_erosion_ctl_init first. */
int nx_erosion_batch(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host, int nplanets,
                     float *st_dev, float *st_tmp_dev, double *mass_dev, void *workspace, size_t ws_bytes,
                     void *stream);

/* Serving: one launch that advances every listed planet (any order) by one
 * iteration, planet p at its own iteration t - t_start (planets outside
 * [0, iters) skip).  Control blocks are workspace slots [0, nslots);
 * zero a planet's slot (32 bytes at 32*slot) before its first iteration.
 * remap = 1 rebuilds the launch's block map (whenever the list changed). */
int nx_erosion_tick(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host, int nplanets, int t,
                    float *st_dev, float *st_tmp_dev, void *workspace, size_t ws_bytes, int nslots, int remap,
                    void *stream);

/* nticks consecutive ticks t, t+1, ... (one launch each) over the same
 * planet list; a planet whose iterations end inside the range is skipped
 * by the later launches and keeps its final state. */
int nx_erosion_ticks(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host, int nplanets, int t,
                     int nticks, float *st_dev, float *st_tmp_dev, void *workspace, size_t ws_bytes, int nslots,
                     int remap, void *stream);

/* Serving, temporally blocked: npasses launches over the same planet list,
 * launch q advancing every listed planet by one pass of up to R iterations
 * (R = the rings of nx_erosion_tb_config), planet p at its own pass
 * pass + q - t_start (planets outside [0, nx_erosion_npass(iters)) skip).
 * Every planet needs a tiling with R rings (a tiling with fewer sets err = 2
 * in its control block and leaves the state).  Same results as
 * nx_erosion_ticks; call nx_erosion_finish after a planet's last pass.
 * remap = 1 rebuilds the launch's block map (whenever the list changed). */
int nx_erosion_passes(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host, int nplanets,
                      int pass, int npasses, float *st_dev, float *st_tmp_dev, void *workspace, size_t ws_bytes,
                      int nslots, int remap, void *stream);

/* Number of passes a temporally blocked run of `iters` iterations makes
 * (iters rounded up to passes of R, plus one if needed so that the count has
 * the parity of iters: a run ends in the buffer it started from iff iters
 * is even, as with one launch per iteration). */
int nx_erosion_npass(int iters);

/* After each listed planet's last iteration: record its final scale
 * exponent in its control block's K[0] (read by nx_erosion_store and
 * nx_erosion_heights_batch). */
int nx_erosion_finish(const nx_erosion_planet *planets_dev, int nplanets, void *workspace, void *stream);

/* The same after each listed planet's last blocked pass (nx_erosion_passes,
 * with the rings currently configured): the control slots rotate per pass,
 * so the final exponent and maximum are those of the planet's pass count. */
int nx_erosion_finish_passes(const nx_erosion_planet *planets_dev, int nplanets, void *workspace, void *stream);

/* Temporal blocking settings (process wide, default 4 rings, 512 threads,
 * variant 0, enabled): the ring count of the tilings that batches use
 * (passes have up to that many iterations), threads per block of the
 * blocked kernel, the kernel variant -- 0: tile tables read from global
 * memory each iteration (256, 512 or 1024 threads); 1: the same with the
 * next vertex's entries loaded ahead (256 or 384); 2: the tile's tables
 * copied to shared memory once per pass (512 or 1024; needs maxc in the
 * planet descriptors); 3: one vertex per thread, its table row held in
 * registers for the pass (512 or 1024; every tile's updatable count maxc
 * must fit the block); 4: variant 0 compiled for more resident blocks per
 * SM (256 threads: 5 blocks, 320: 4, 384: 3, 640: 2; at most 1280
 * threads x 48 registers or 1152 x 56), for tiles whose shared memory lets
 * that many blocks reside; 5: the same for 6 blocks of 256 (40 registers)
 * -- and whether batches with tilings use it (1) or
 * run one iteration per launch (0).  The autotuner (nixis_gb300.autotune)
 * picks these and the tile side per device. */
int nx_erosion_tb_config(int rings, int threads, int variant, int enabled);

/* Write one planet's state back as binary64 true values (hi + lo of each
 * field times 2^K, K from the workspace's first control block).  w64_dev /
 * s64_dev may be NULL. */
int nx_erosion_store(const float *st_dev, int64_t n, const void *workspace, double *h64_dev, double *w64_dev,
                     double *s64_dev, void *stream);

/* Layout of a workspace's per-planet control block (32 bytes, planet p at
 * byte 32*p): after a run, K[0] is the planet's scale exponent (stored
 * value = true value * 2^-K[0]) and err = 1 flags a neighbour id outside
 * the planet's range, err = 2 a tiling with fewer rings than a pass. */
typedef struct nx_erosion_ctl {
    uint32_t maxbits[3];
    int32_t K[2];
    uint32_t done;
    int32_t err;
    int32_t pad;
} nx_erosion_ctl;

/* Initial state of a batch from raw fBm pair sums (nx_fbm_batch /
 * nx_fbm_pair output rows, float[2 * rows], and their min/max keys, 2 per
 * planet): h = util.rescale(raw, elev_lo, elev_hi) (util.py:110-140) as a
 * pair, (raw - min) * ((hi - lo) / (max - min)) + lo with the factor
 * formed in binary64, w = water0 (as a pair), s = 0, written to buffer
 * (iters & 1). */
int nx_erosion_init_batch(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host,
                          int nplanets, const float *raw_dev, const unsigned long long *minmax_dev, double elev_lo,
                          double elev_hi, double water0, float *st_dev, float *st_tmp_dev, void *stream);

/* Heights of every planet of a finished batch into out_dev (packed rows):
 * (h_hi + h_lo) * 2^K in binary64, finite for every iteration count (the
 * reference's heights grow without bound: binary32 metres overflow past
 * ~130 iterations). */
int nx_erosion_heights_batch(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host,
                             int nplanets, const float *st_dev, const void *workspace, double *out_dev,
                             void *stream);

/* nx_erosion_init_batch, nx_erosion_batch and nx_erosion_heights_batch in
 * one call, with the same results (state in st_dev, heights in
 * heights_dev).  On the temporally blocked path the rescale runs inside each
 * eroding planet's first pass (its load phase reads the raw pair sums), so
 * the starting state is never written to HBM; planets with no iterations get
 * their state from one rescale launch.  Call nx_erosion_ctl_init first. */
int nx_erosion_run_batch(const nx_erosion_planet *planets_dev, const nx_erosion_planet *planets_host, int nplanets,
                         const float *raw_dev, const unsigned long long *minmax_dev, double elev_lo, double elev_hi,
                         double water0, float *st_dev, float *st_tmp_dev, double *heights_dev, void *workspace,
                         size_t ws_bytes, void *stream);

/* Latitude-table insolation (climate.py:503-597).  Tables for n_tilts
 * tilts (degrees, device float64[n_tilts]) into tables_dev
 * float[n_tilts * 181]: entry i is latitude i for i <= 90, i - 181 above,
 * each the binary32 running sum over 360 rotations of one degree from -180
 * (calc_insolation_slice). */
int nx_insolation_slices(const double *tilts_dev, int n_tilts, double radius, float *tables_dev, void *stream);

/* Every vertex's insolation interpolated between the entries of floor(lat)
 * and ceil(lat) (interpolate_insolation), summed in binary32 over n_tables
 * tables in order (calc_yearly_insolation: 360 tables); accumulate = 1 adds
 * to out_dev. */
int nx_interpolate_insolation(const double *xyz_dev, int64_t n, double radius, const float *tables_dev, int n_tables,
                              float *out_dev, int accumulate, void *stream);

/* Starting surface temperatures (climate.assign_surface_temp,
 * climate.py:345-411): out_dev float[n], vertex v's value
 * max(cos(|lat - tilt| * pi / 180), 0) with lat from util.xyz2latlon.  The
 * reference's altitude term rescales the altitudes to [0, 0], which is 0
 * (NaN for a constant field) everywhere, so it never enters the result. */
int nx_surface_temp(const double *xyz_dev, int64_t n, double radius, double tilt, float *out_dev, void *stream);

/* ------------------------------------------------------------------ */
/* Equirectangular maps (util.py:290-366, nixis.py:270-302)            */
/* ------------------------------------------------------------------ */

/* util.make_ll_arr: out_dev double[height*width*3], pixel (h, w) at
 * latitude max(90 - h*180/(height-1), -90), longitude
 * max(-180 + w*360/width, -180) on the sphere of the radius. */
int nx_make_ll(int width, int height, double radius, double *out_dev, void *stream);

/* The 3 nearest vertices of nq query points (replaces the reference's
 * KDTree(points).query(queries, k=3)): xyz_dev/nbr_dev the icosphere of
 * divisions k made by nx_icosphere / nx_build_adjacency / nx_sort_adjacency
 * (any radius; nv = 10k^2+2); dist_dev double[nq*3] ascending, idx_dev
 * int64[nq*3] (ties by vertex id).  Needs nx_icosphere_tables. */
int nx_nearest3(int k, const double *xyz_dev, const int32_t *nbr_dev, int64_t nv, const double *q_dev, int64_t nq,
                double *dist_dev, int64_t *idx_dev, void *stream);

/* util.make_gray_array per pixel: inverse-distance weighting of the 3
 * neighbours' colours (double[ncolors]), truncated toward zero, into
 * out_dev double[npix]; err_dev (device int, caller zeroes it) gets bit 0 for
 * an index outside the colours. */
int nx_sample_gray(const double *dist_dev, const int64_t *idx_dev, int64_t npix, const double *colors_dev,
                   int64_t ncolors, double *out_dev, int *err_dev, void *stream);

/* ------------------------------------------------------------------ */
/* Height shaping (nixis.py:332-364), binary64                         */
/* ------------------------------------------------------------------ */

/* Workspace bytes for the shaping calls on n values (16-byte aligned). */
size_t nx_shape_workspace_size(int64_t n);

/* util.rescale (util.py:110-176): form 0 plain min/max normalisation to
 * [lower, upper]; 1 with mid (each side of mid mapped separately); 2 mode
 * 'lower' (only x <= mid); 3 mode 'upper' (only x >= mid).  has_umin /
 * has_umax: u_min / u_max widen the input range.  Min and max are found on
 * the device (all reads finish before the first write: out_dev may equal
 * x_dev). */
int nx_rescale(const double *x_dev, int64_t n, double lower, double upper, double mid, int form, double u_min,
               int has_umin, double u_max, int has_umax, double *out_dev, void *ws, size_t ws_bytes, void *stream);

/* util.power_rescale (util.py:179-250): mode 1 rescales the values where
 * mask_dev is non-zero, 0 where it is zero, -1 none (copy); the masked range
 * is the reference's running min/max update. */
int nx_power_rescale(const double *x_dev, int64_t n, const uint8_t *mask_dev, int mode, double power, double *out_dev,
                     void *ws, size_t ws_bytes, void *stream);

/* terrain.make_bool_elevation_mask (terrain.py:61-72): mask = h <= level. */
int nx_elevation_mask(const double *h_dev, int64_t n, double level, uint8_t *mask_dev, void *stream);

/* nixis.py:332-364 on the device: rescale to [min_alt, max_alt], ocean level
 * = util.find_percent_val(min, max, ocean_percent), ocean mask, power_rescale
 * (ocean, 0.5) then (land, 2.0), minus the level, rescale about 0.
 * out_dev: the heights; tmp_dev: n doubles of scratch; mask_dev: the ocean
 * mask; level_dev (optional, device double): the level. */
int nx_shape_heights(const double *h_dev, int64_t n, double min_alt, double max_alt, double ocean_percent,
                     double *out_dev, double *tmp_dev, uint8_t *mask_dev, double *level_dev, void *ws,
                     size_t ws_bytes, void *stream);

/* Erosion for callers that cannot allocate device memory.  No counterpart
 * in the reference (whose erosion is host code).  Some callers run inside
 * a host application's own device-memory pool, where a direct cudaMalloc
 * bypasses the owner's budget, or in loops that must not stall, since
 * cudaMalloc and cudaFree synchronise the device.  This entry point runs
 * `iters` iterations like nx_erosion_steps on one planet of at most
 * NX_NOALLOC_MAX_VERTICES vertices (larger n returns NX_EINVAL) without
 * allocating: its scratch (second state buffer, control block, partial
 * sums) is a fixed array inside the library, about 8.4 MB, which every GPU
 * that loads the library keeps until the process exits.  The caller passes
 * the mesh, the state st_dev (8-float rows as in nx_erosion_load, true
 * values with scale exponent 0, magnitudes below 2^96) and the outputs:
 * the state is updated in place, mass_dev (optional) as in
 * nx_erosion_steps, status_dev (optional, device int32[2]) gets the final
 * scale exponent K and the neighbour-range error flag.  The first call on
 * each device looks up the array's device address in that device's
 * primary context and keeps it for the life of the process (make that
 * first call before any stream capture; after cudaDeviceReset the cached
 * address is stale, so do not call it on that device again).  All calls
 * share the one array and each call resets what must start at zero; calls
 * whose work overlaps on the GPU (other streams, other threads) race on it
 * and must be serialised by the caller. */
#define NX_NOALLOC_MAX_VERTICES 262144
int nx_erosion_steps_noalloc(const int32_t *nbr_dev, const float *edge_dev, int64_t n, float *st_dev, int iters,
                             float rain, double *mass_dev, int32_t *status_dev, void *stream);

/* erosion.find_lowest (erosion.py:398-406) for every vertex: pos_dev gets
 * the position, among the neighbours that are not -1, of the first lowest
 * one if it is strictly lower than the vertex, else -1; vid_dev (optional)
 * that neighbour's id or -1. */
int nx_steepest_descent(const int32_t *nbr_dev, const double *h_dev, int64_t n, int32_t *pos_dev, int32_t *vid_dev,
                        void *stream);

/* ------------------------------------------------------------------ */
/* Insolation                                                          */
/* ------------------------------------------------------------------ */

/* Host: the (cos, sin) table for a schedule of sun positions -- rotations
 * in degrees (about z) and tilts in degrees (about y), the arguments of
 * climate.sample_insolation (climate.py:415-444).  table_host must hold
 * 2*(n_rot + n_tilt) floats.  If the rotations come in pairs h and
 * h + n_rot/2 that differ by exactly 180 degrees, only the first half is
 * tabulated (*pairs = 1).  *n_rot_entries gets the number of rotation
 * entries written; tilt entries follow them. */
int nx_insolation_plan(const double *rot_deg, int n_rot, const double *tilt_deg, int n_tilt, float *table_host,
                       int *n_rot_entries, int *pairs);

/* Sum over every (tilt, rotation) pair of sample_insolation's term
 * max(cos|lat|,0)*max(cos lon,0) (climate.py:442, util.py:59-75):
 * out_dev[v] = sum (accumulate=0) or out_dev[v] += sum.  table_dev: the
 * plan's table on the device.  Binary32 terms; per-tilt partial sums with
 * a compensated total. */
int nx_insolation(const double *xyz_dev, int64_t n, double radius, const float *table_dev, int n_rot_entries,
                  int pairs, int n_tilt, float *out_dev, int accumulate, void *stream);

/* One planet of a batched insolation launch: its vertices and radius; its
 * sums go to packed output rows [vbeg, vbeg + n) (vbeg a multiple of 256). */
typedef struct nx_inso_planet {
    const double *xyz;
    int64_t n;
    int64_t vbeg;
    double radius;
} nx_inso_planet;

/* nx_insolation for many planets (same schedule) in one launch. */
int nx_insolation_batch(const nx_inso_planet *planets_dev, const nx_inso_planet *planets_host, int nplanets,
                        const float *table_dev, int n_rot_entries, int pairs, int n_tilt, float *out_dev,
                        void *stream);

#ifdef __cplusplus
}
#endif

#endif /* NIXIS_GB300_H */
