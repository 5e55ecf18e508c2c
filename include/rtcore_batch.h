/*
 * rtcore_batch.h -- batched path tracing: many scenes and cameras of uneven
 * triangle count and resolution traced by one launch, and the autotuner that
 * chooses the launch shapes.
 *
 * No counterpart in the reference, whose sample records one
 * vkCmdTraceRaysKHR for one image into a command buffer every frame and
 * submits it (render(), vulkan-raytraced-triangle/main.cpp:1322-1422; the
 * trace at :1349).  The GB300 form of a recorded command buffer is a plan
 * captured in a CUDA graph, here covering many scenes at once: the wavefront
 * path tracer of rtcore_pt.h over the concatenated pixels of all scenes, so
 * that small scenes and the thin tails of deep bounces share the GPU instead
 * of leaving it idle between per-scene launches.
 *
 * Results: each scene's accum receives exactly what rt_path_trace would add
 * for that scene with the same camera, size, seed, sample offset, spp, depth
 * and ray_eps -- bit for bit (per-pixel random streams and float operations
 * do not depend on the batch).
 */
#ifndef RTCORE_BATCH_H
#define RTCORE_BATCH_H

#include "rtcore.h"
#include "rtcore_pt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One scene of a batch (80 bytes). */
typedef struct rt_batch_scene {
    rt_pt_scene scene;        /* bottom-level structure, materials, lights  */
    rt_camera camera;
    uint32_t width, height;   /* 0 x 0: the scene is skipped               */
    float *accum;             /* device, width*height*4 floats, added to as
                                 by rt_path_trace                           */
} rt_batch_scene;

typedef struct rt_batch_params {
    uint32_t spp;             /* samples per pixel per launch               */
    uint32_t max_depth;       /* path vertices, 1..64                        */
    uint32_t rr_depth;        /* Russian roulette from this vertex on        */
    uint32_t flags;           /* 0 or RT_PT_OCTANT_BINNING (rtcore_pt.h)     */
    uint64_t seed;
    float ray_eps;
    uint32_t reserved;        /* 0                                           */
} rt_batch_params;

/* Launch shapes.  Zero in any field selects the default. */
typedef struct rt_batch_tuning {
    uint32_t trace_threads;        /* traversal block size: 128 or 256       */
    uint32_t trace_blocks_per_sm;  /* persistent traversal blocks per SM     */
    uint32_t stack_ring;           /* shared-memory stack entries per ray:
                                      8, 16 or 32 (deeper entries spill to
                                      local memory)                          */
    uint32_t refill;               /* a traversal warp refills when at least
                                      this many of its lanes are idle (1-32) */
    uint32_t shade_threads;        /* block size of the shading kernels:
                                      128, 256 or 512                        */
    uint32_t wave_paths;           /* paths in flight per wave (the queue
                                      capacity); 0 = every pixel of every
                                      scene in one wave                      */
    uint32_t bvh_width;            /* children per node the scenes'
                                      structures were built with
                                      (RT_BUILD_WIDTH, 4..8): a build-time
                                      choice recorded with the launch shapes;
                                      the plan traces any width              */
    uint32_t reserved;
} rt_batch_tuning;

typedef struct rt_batch_plan rt_batch_plan;

#define RT_BATCH_GRAPH 1u          /* capture the plan in a CUDA graph        */
#define RT_BATCH_DISCARD 2u        /* trace but add nothing to accum (timing
                                      runs of the autotuner)                 */

/* The defaults: 128 / 8 / 16 / 4 / 256 / 0 / 8. */
rt_status rt_batch_default_tuning(rt_batch_tuning *t);

/* Scratch bytes of a plan.  t == NULL: enough for every tuning the
 * autotuner tries (one wave holding every pixel). */
rt_status rt_batch_scratch_bytes(const rt_batch_scene *scenes, uint32_t n_scenes, const rt_batch_params *p,
                                 const rt_batch_tuning *t, uint64_t *bytes);

/*
 * Records one launch of the batch: p->spp samples of every pixel of every
 * scene.  The scene table is copied; the buffers it points to (structures,
 * materials, lights, accum) and the scratch (256-byte aligned, caller-owned)
 * must stay valid while the plan is used.  flags: RT_BATCH_GRAPH captures the
 * launch sequence once into a CUDA graph (one cudaGraphLaunch per launch);
 * without it every launch issues the kernels on the stream directly.
 */
rt_status rt_batch_plan_create(rt_context *ctx, const rt_batch_scene *scenes, uint32_t n_scenes,
                               const rt_batch_params *p, const rt_batch_tuning *t, void *scratch,
                               uint64_t scratch_bytes, uint32_t flags, rt_batch_plan **plan);

/* Traces samples [sample_offset, sample_offset + spp) of every pixel and adds
 * them to each scene's accum.  Asynchronous on `stream`. */
rt_status rt_batch_launch(rt_batch_plan *plan, rt_stream stream, uint32_t sample_offset);

/* Extension and shadow rays traced by the plan's last launch (synchronises
 * `stream`). */
rt_status rt_batch_ray_counts(rt_batch_plan *plan, rt_stream stream, uint64_t *extension_rays,
                              uint64_t *shadow_rays);

/* Kernel launches (graph nodes) one launch of the plan issues. */
rt_status rt_batch_plan_launches(const rt_batch_plan *plan, uint32_t *kernels);

rt_status rt_batch_plan_destroy(rt_batch_plan *plan);

/*
 * Autotuner.  Times candidate tunings on this batch (one sample per pixel,
 * graph launches, CUDA events, the best of three launches after a warm-up),
 * walking one parameter at a time from the defaults and keeping each
 * improvement of more than 1 %, and returns the fastest in *best (its time in
 * *best_ms).
 * The returned bvh_width is the width the structures were built with; the
 * width itself is chosen by rebuilding and timing (rtcore.batch --widths).
 * With a cache_path, the result is looked up first and stored after tuning
 * in a JSON file keyed by rt_batch_tuning_key; flags RT_TUNE_FORCE re-tunes
 * even when the key is present.  scratch: rt_batch_scratch_bytes(..., NULL).
 */
#define RT_TUNE_FORCE 1u
rt_status rt_batch_autotune(rt_context *ctx, const rt_batch_scene *scenes, uint32_t n_scenes,
                            const rt_batch_params *p, void *scratch, uint64_t scratch_bytes, const char *cache_path,
                            uint32_t flags, rt_batch_tuning *best, float *best_ms);

/* Cache key of a batch on this context's device: the device, the scene-count,
 * triangle-count and pixel-count buckets (powers of two) and the depth, e.g.
 * "sm103-152/n2^6/tris2^25/px2^27/d8".  Triangle counts are read from the
 * structures' headers (synchronous). */
rt_status rt_batch_tuning_key(rt_context *ctx, const rt_batch_scene *scenes, uint32_t n_scenes,
                              const rt_batch_params *p, char *key, uint32_t key_bytes);

/* The JSON tuning cache (host only): lookup returns RT_ERR_NOT_FOUND when the
 * file or the key is absent; store adds the key's entry or updates its
 * tuning fields and time (keeping its other fields, such as the autotuner's
 * trial list) and rewrites the file atomically. */
rt_status rt_batch_tuning_cache_lookup(const char *path, const char *key, rt_batch_tuning *t, float *ms);
rt_status rt_batch_tuning_cache_store(const char *path, const char *key, const rt_batch_tuning *t, float ms);

#ifdef __cplusplus
}
#endif
#endif
