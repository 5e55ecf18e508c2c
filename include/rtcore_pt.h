/*
 * rtcore_pt.h -- wavefront path tracer of the GB300 ray-tracing core.
 *
 * No counterpart in the reference: its sample shades one bounce with a
 * constant closest-hit colour (vulkan-raytraced-triangle/main.cpp:1080-1091).
 * The path tracer reuses the sample's pinhole camera model (main.cpp:1036-1045)
 * with a per-sample sub-pixel jitter, and traces with the same BVH8 kernels.
 *
 * Light transport: Lambertian surfaces, next-event estimation to emissive
 * triangles (area sampling), one-sided emitters (along the triangle's
 * geometric normal, (v1-v0) x (v2-v0)), Russian roulette from rr_depth on,
 * at most max_depth path vertices.  Random numbers: one PCG32 stream per pixel
 * and sample (state seeded from the sample index, stream = pixel index), six
 * draws per path vertex (light pick, 2 for the light point, 2 for the BSDF,
 * roulette) and two for the camera jitter, consumed whether used or not.
 */
#ifndef RTCORE_PT_H
#define RTCORE_PT_H

#include "rtcore.h"
#include "rtcore_scene.h"

#ifdef __cplusplus
extern "C" {
#endif

/* An emissive triangle for next-event estimation (48 bytes). */
typedef struct rt_pt_light {
    float v0[3], v1[3], v2[3];
    float emission[3];
} rt_pt_light;

typedef struct rt_pt_scene {
    uint64_t accel;                 /* bottom-level rt_accel_address        */
    const uint32_t *tri_material;   /* device, material of each build-input
                                       triangle                            */
    const rt_material *materials;   /* device                               */
    uint32_t n_materials;
    const rt_pt_light *lights;      /* device                               */
    uint32_t n_lights;
} rt_pt_scene;

typedef struct rt_pt_params {
    rt_camera camera;
    uint32_t width, height;
    uint32_t spp;            /* samples per pixel traced by this call        */
    uint32_t sample_offset;  /* index of the first sample (progressive use) */
    uint32_t max_depth;      /* path vertices, >= 1                          */
    uint32_t rr_depth;       /* Russian roulette from this vertex index on   */
    uint64_t seed;
    float ray_eps;           /* secondary-ray offset along the normal        */
    uint32_t flags;          /* 0 or RT_PT_OCTANT_BINNING                    */
} rt_pt_params;

/* Traces the bounce rays of each path vertex grouped by direction octant (the
 * shading kernel ranks each ray within its octant with one warp-level match
 * and one atomic per octant present in the warp; a scatter pass places the
 * octants one after the other), so the lanes of a traversal warp share a
 * child visiting order.  The images do not depend on the order.  Off by
 * default: on the GB300 the rays' spatial order (pixel order) is worth more
 * to the traversal than their directional order -- 2M-triangle box at
 * 1920x1080, 4 spp per call: 6.72 ms per sample in shading order, 7.01 ms
 * binned. */
#define RT_PT_OCTANT_BINNING 1u

/* Scratch bytes of rt_path_trace for these parameters.  A call traces up to
 * four samples of every pixel together (at most 2^23 paths per wave), so the
 * size grows with min(spp, 4): about 220 bytes per pixel and sample of a
 * wave; the image does not depend on it. */
rt_status rt_pt_scratch_bytes(const rt_pt_params *p, uint64_t *bytes);

/*
 * Traces p->spp samples per pixel and ADDS them to accum (device,
 * width*height*4 floats, row-major): rgb += sum of sample radiances,
 * a += number of samples.  Zero accum before the first call; divide rgb by a
 * to resolve.  Asynchronous on `stream`.
 */
rt_status rt_path_trace(rt_context *ctx, rt_stream stream, const rt_pt_scene *scene, const rt_pt_params *p,
                        float *accum, void *scratch, uint64_t scratch_bytes);

/*
 * Learned form: the MLP radiance cache of rtcore_cache.h ends paths at their
 * second vertex.  Per sample, about train_paths pixels (an exact residue
 * class of the pixel index, re-drawn every sample) are training paths: they
 * continue as plain path tracing, and the radiance their tail brings back
 * through the second vertex (divided by the throughput there) is a training
 * target for (position, direction toward the first vertex, normal, albedo).
 * Every other path adds throughput x max(cache, 0) at its second vertex and
 * stops.  A wave holds up to four of the call's samples (see
 * rt_pt_scratch_bytes): its paths query the cache as it stood before the
 * wave, and after the wave the cache takes ceil(training paths / train_batch)
 * Adam steps on the wave's training paths (train_batch 0: no training), so a
 * call of one sample trains after every sample.  The cache's
 * emission is not included: direct light reaches the first vertex through
 * next-event estimation only, as in the plain form.
 */
typedef struct rt_pt_cache_params {
    void *cache;            /* rt_cache state (device)            */
    uint32_t train_paths;   /* training paths per sample, > 0     */
    uint32_t train_batch;   /* Adam batch, multiple of 64, or 0   */
} rt_pt_cache_params;

rt_status rt_pt_cached_scratch_bytes(const rt_pt_params *p, const rt_pt_cache_params *cp, uint64_t *bytes);

rt_status rt_path_trace_cached(rt_context *ctx, rt_stream stream, const rt_pt_scene *scene, const rt_pt_params *p,
                               const rt_pt_cache_params *cp, float *accum, void *scratch, uint64_t scratch_bytes);

/* Extension rays (camera + bounce) and shadow rays traced by the last
 * rt_path_trace call that used `scratch` with these parameters and light
 * count (synchronises `stream`). */
rt_status rt_pt_ray_counts(rt_context *ctx, rt_stream stream, const rt_pt_params *p, uint32_t n_lights,
                           const void *scratch, uint64_t *extension_rays, uint64_t *shadow_rays);

#ifdef __cplusplus
}
#endif
#endif
