/*
 * nixis_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the Nixis
 * per-vertex terrain hot path: fractal OpenSimplex-3D noise, erosion
 * (variant 3) and insolation accumulation, plus the icosphere/adjacency
 * generator that feeds them.
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

#ifdef __cplusplus
}
#endif

#endif /* NIXIS_GB300_H */
