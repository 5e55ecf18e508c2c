/*
 * rtcore_cache.h -- online-trained MLP radiance cache.
 *
 * No counterpart in the reference (its sample has no path tracer).  The cache
 * maps a path vertex (position, outgoing direction, normal, albedo) to the
 * radiance scattered there toward the direction.  Network: frequency-encoded
 * position (12 octaves of sin/cos per axis, positions normalised to the scene
 * box), raw direction, normal and albedo = 81 inputs (padded to 96);
 * 5 hidden layers of 64 ReLU units; 3 linear outputs.  BF16 weights on the
 * tensor cores with FP32 accumulation; FP32 master weights; Adam.
 * Loss: relative L2, (y' - y)^2 / (y'^2 + 0.01) with y' held constant in the
 * gradient, averaged over samples and channels.
 *
 * All cache state (FP32 parameters, gradients, Adam moments, BF16 copy,
 * step counter, configuration) lives in one caller-owned device buffer of
 * rt_cache_bytes() bytes.
 */
#ifndef RTCORE_CACHE_H
#define RTCORE_CACHE_H

#include "rtcore.h"

#ifdef __cplusplus
extern "C" {
#endif

#define RT_CACHE_INPUTS 81
#define RT_CACHE_HIDDEN 64
#define RT_CACHE_LAYERS 5
#define RT_CACHE_OUTPUTS 3

/* One query / training input (48 bytes). */
typedef struct rt_cache_input {
    float pos[3];
    float dir[3];    /* unit direction the radiance leaves in */
    float normal[3];
    float albedo[3];
} rt_cache_input;

typedef struct rt_cache_config {
    float scene_lo[3];
    float scene_hi[3];
    float lr;        /* Adam learning rate (1e-3) */
    float beta1;     /* 0.9 */
    float beta2;     /* 0.99 */
    float eps;       /* 1e-8 */
    uint32_t seed;   /* weight initialisation */
    uint32_t reserved;
} rt_cache_config;

/* Bytes of the cache state buffer (256-byte aligned by the caller). */
rt_status rt_cache_bytes(uint64_t *bytes);

/* Number of FP32 parameters in the padded layout rt_cache_get_params uses. */
uint32_t rt_cache_param_count(void);

/* Resets the state: He-uniform weights from cfg->seed (PCG32), zero biases,
 * zero Adam moments, step 0.  Synchronous (uploads from the host). */
rt_status rt_cache_init(rt_context *ctx, rt_stream stream, void *cache, const rt_cache_config *cfg);

/* out[i] = (r, g, b, 0) predicted for in[i]; n inputs, device arrays. */
rt_status rt_cache_query(rt_context *ctx, rt_stream stream, const void *cache, const rt_cache_input *in,
                         float *out_rgba, uint32_t n);

/* One pass over n training samples in batches of `batch` (multiple of 64):
 * per batch one forward/backward and one Adam step.  targets are float4
 * (r, g, b, ignored).  loss_out (device, nullable) receives the mean loss of
 * the last batch. */
rt_status rt_cache_train(rt_context *ctx, rt_stream stream, void *cache, const rt_cache_input *in,
                         const float *targets, uint32_t n, uint32_t batch, float *loss_out);

/* Gradient of the loss over the first n samples at the current weights
 * (FP32, padded layout), without updating: for gradient checks. */
rt_status rt_cache_gradient(rt_context *ctx, rt_stream stream, void *cache, const rt_cache_input *in,
                            const float *targets, uint32_t n, float *grad_out);

/* Copies the FP32 master parameters (padded layout) out of / into the
 * state; setting also refreshes the BF16 copy.  Device pointers. */
rt_status rt_cache_get_params(rt_context *ctx, rt_stream stream, const void *cache, float *params);
rt_status rt_cache_set_params(rt_context *ctx, rt_stream stream, void *cache, const float *params);

/* Checkpoint: the whole state (FP32 weights, Adam moments and step, the
 * encoding box, the optimiser constants) to / from a file: a 64-byte header
 * ("RTMC", format version, parameter count, state bytes, FNV-1a 64 checksum of
 * the state) and the state bytes.  Load rejects a file of another format,
 * size or checksum with RT_ERR_INVALID_ARG and leaves the cache unchanged.
 * Both synchronise `stream`. */
rt_status rt_cache_save(rt_context *ctx, rt_stream stream, const void *cache, const char *path);
rt_status rt_cache_load(rt_context *ctx, rt_stream stream, void *cache, const char *path);

#ifdef __cplusplus
}
#endif
#endif
