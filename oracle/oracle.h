/*
 * oracle.h -- CPU oracle of the ray-tracing core.  TEST INFRASTRUCTURE ONLY.
 *
 * This is a scalar C++ restatement of what the GPU kernels compute, used by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as
 * the checker.  Nothing in the product links or calls it.
 *
 * Parity anchors:
 *   - raygen / miss / closest-hit and the SBT record rule restate the
 *     reference sample's GLSL and host code
 *     (vulkan-raytraced-triangle/main.cpp:1033-1091, 1260-1262, 1306-1317);
 *     they are pinned by known-answer pixels of the sample's own scene
 *     (tests/golden/).
 *   - BVH build and traversal: the reference performs them inside the Vulkan
 *     driver (main.cpp:808, 932, 1047), closed code with no tests, so they are
 *     parity unpinned against the reference; the oracle pins the GPU build
 *     bit-exactly and its hits are checked against an FP64 brute force.
 */
#ifndef RT_ORACLE_H
#define RT_ORACLE_H

#include <stdint.h>
#include "../include/rtcore.h"
#include "../include/rtcore_accel.h"
#include "../include/rtcore_pt.h"
#include "../include/rtcore_cache.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Host-memory geometry description: same fields as rt_geometry_triangles,
 * pointers are host pointers. */
typedef rt_geometry_triangles orc_geometry;

/* Sizes of the buffers orc_build_blas / orc_build_tlas need. */
uint64_t orc_blas_accel_bytes(const uint32_t *tri_counts, uint32_t n_geoms);
uint64_t orc_tlas_accel_bytes(uint32_t n_instances);

/* Intermediate results of the LBVH stages, for stage-by-stage comparison.
 * Any pointer may be NULL.  keys/ids: sorted Morton keys and the input index
 * of each; nodes: binary internal nodes as (left, right, first, last) with
 * bit 31 of left/right set for a leaf reference. */
typedef struct orc_lbvh_debug {
    uint64_t *keys_unsorted; /* n */
    uint64_t *keys_sorted;   /* n */
    uint32_t *ids_sorted;    /* n */
    uint32_t *bin_nodes;     /* 4 * (n - 1) */
} orc_lbvh_debug;

/* Builds a bottom-level structure into host memory `accel` (zeroed by the
 * caller, orc_blas_accel_bytes long).  Returns 0 or an RT_ERR_* code. */
int orc_build_blas(const orc_geometry *geoms, uint32_t n_geoms, uint32_t flags,
                   void *accel, uint64_t accel_bytes, orc_lbvh_debug *dbg);

/* Builds a top-level structure; instances[i].accel_ref are host pointers to
 * bottom-level buffers built by orc_build_blas. */
int orc_build_tlas(const rt_instance *instances, uint32_t n, uint32_t flags,
                   void *accel, uint64_t accel_bytes);

/* Refit restatement (rt_refit_blas / rt_refit_tlas): recomputes the leaf
 * records and every box of `accel` from new inputs in the existing tree,
 * nodes in reverse breadth-first order.  Returns 0, RT_ERR_INVALID_ARG when
 * the structure does not match the inputs (left unchanged), or the build's
 * RT_ERR_BOUNDS status for an index beyond max_vertex. */
int orc_refit_blas(const orc_geometry *geoms, uint32_t n_geoms, void *accel);
int orc_refit_tlas(const rt_instance *instances, uint32_t n, void *accel);

/* Closest-hit / any-hit traversal of the BVH8 in `accel` (host memory),
 * mirroring the GPU kernel's visiting order.  stats (nullable) receives
 * [nodes visited, triangles tested] summed over rays.  n_threads 0 = all. */
void orc_trace_closest(const void *accel, const rt_ray *rays, rt_hit *hits,
                       rt_hit_ext *hits_ext, uint32_t n, uint32_t n_threads,
                       uint64_t *stats);
void orc_trace_any(const void *accel, const rt_ray *rays, uint8_t *occluded,
                   uint32_t n, uint32_t n_threads, uint64_t *stats);

/* Brute force over the raw build input (one bottom-level structure without
 * instancing).  precision 32: the same watertight FP32 test and tie rule as
 * the traversal; precision 64: the same algorithm in double. */
void orc_brute_closest(const orc_geometry *geoms, uint32_t n_geoms,
                       const rt_ray *rays, rt_hit *hits, uint32_t n,
                       int precision, uint32_t n_threads);

/* Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013) as the GPU
 * computes it.  Returns 1 on a hit inside [tmin, tmax]. */
int orc_intersect_tri(const float org[3], const float dir[3], float tmin,
                      float tmax, const float v0[3], const float v1[3],
                      const float v2[3], float *t, float *u, float *v);

/* The sample's raygen for launch id (x, y) of a width x height launch. */
void orc_raygen(const rt_camera *cam, uint32_t width, uint32_t height,
                uint32_t x, uint32_t y, float org[3], float dir[3]);

/* vkCmdTraceRaysKHR with the sample's programs, on the CPU: fills
 * out_rgba32f (host, width*height*4).  sbt colours are host memory. */
int orc_trace_rays(const rt_pipeline *p, const float *sbt_colors,
                   uint32_t sbt_count, uint32_t sbt_stride, const void *accel,
                   const rt_camera *cam, float *out_rgba32f, uint32_t width,
                   uint32_t height, uint32_t n_threads);

/* The path tracer of rtcore_pt.h on the CPU, pixel by pixel: adds the
 * samples to accum (host, width*height*4) exactly as rt_path_trace does.
 * tri_material, materials and lights are host arrays. */
int orc_path_trace(const void *accel, const uint32_t *tri_material, const rt_material *materials,
                   uint32_t n_materials, const rt_pt_light *lights, uint32_t n_lights, const rt_pt_params *p,
                   float *accum, uint32_t n_threads);

/* What one path of orc_path_trace_pixels brought back (88 bytes).  kind:
 * 0 the path never reached a second reflective vertex (or the plain form),
 * 1 it ended there in a cache query, 2 it is a training path.  L: the
 * path's radiance (for a query path: before the cache's contribution);
 * L_before, t1, rec: radiance, throughput and the cache input (position,
 * direction toward the first vertex, normal, albedo) at the second vertex. */
typedef struct orc_path_record {
    uint32_t kind;
    float L[3];
    float L_before[3];
    float t1[3];
    rt_cache_input rec;
} orc_path_record;

/* The same paths for a list of pixels only: out[k * spp + s] is sample
 * sample_offset + s of pixels[k].  train_stride 0: the plain path tracer;
 * otherwise the learned form of rt_path_trace_cached with that training
 * stride (training pixels (pixel + offset) % stride == 0 per sample). */
int orc_path_trace_pixels(const void *accel, const uint32_t *tri_material, const rt_material *materials,
                          uint32_t n_materials, const rt_pt_light *lights, uint32_t n_lights, const rt_pt_params *p,
                          uint32_t train_stride, const uint32_t *pixels, uint32_t n_pixels, orc_path_record *out,
                          uint32_t n_threads);

/* The seeded workload generators of rtcore_scene.h (rt_scene_soup,
 * rt_scene_incoherent_rays) restated, so that a CPU-only run can make the
 * same inputs without the product library. */
int orc_scene_soup(uint64_t seed, uint32_t n_tris, float *v, uint32_t *idx);
int orc_scene_incoherent_rays(uint64_t seed, uint32_t n, const float lo[3], const float hi[3], float tmax,
                              rt_ray *rays);

/* sin and cos of the oracle's polynomial, for tests of their accuracy. */
void orc_sincos_q(float x, float *s, float *c);

/* Stable LSD radix sort of (key, value) pairs on `bits` low key bits. */
void orc_sort_pairs(uint64_t *keys, uint32_t *vals, uint32_t n, uint32_t bits);

/* Number of hardware threads the oracle uses when n_threads == 0. */
uint32_t orc_hw_threads(void);

#ifdef __cplusplus
}
#endif
#endif
