// rt_trace_multi.cu -- persistent BVH8 traversal over rays of many scenes.
//
// The batched path tracer (rt_pt.cu, rtcore_batch.h) traces the queues of
// all scenes of a batch in one launch: ray i belongs to scene ray_scene[i],
// whose structure a lane picks up from a 32-byte view table when it takes the
// ray.  Queue entries are appended in pixel order, so neighbouring rays -- and
// the lanes of a warp -- mostly share a scene.  Instantiated for the launch
// shapes the autotuner chooses among: 128 or 256 threads per block and a
// shared-memory stack ring of 8, 16 or 32 entries per ray.
#include "rt_internal.h"
#include "rt_traverse.cuh"

namespace rtc {
namespace {

template <bool ANY, int THREADS, bool MIXED = false>
void launch_ring(const BatchArgs &a, uint32_t ring, uint32_t blocks, cudaStream_t st) {
    switch (ring) {
    case 8: k_trace_blas<ANY, false, true, THREADS, 8, MIXED><<<blocks, THREADS, 0, st>>>(a); break;
    case 32: k_trace_blas<ANY, false, true, THREADS, 32, MIXED><<<blocks, THREADS, 0, st>>>(a); break;
    default: k_trace_blas<ANY, false, true, THREADS, 16, MIXED><<<blocks, THREADS, 0, st>>>(a); break;
    }
}

template <bool ANY, int THREADS, bool MIXED = false>
const void *kernel_ring(uint32_t ring) {
    switch (ring) {
    case 8: return (const void *)k_trace_blas<ANY, false, true, THREADS, 8, MIXED>;
    case 32: return (const void *)k_trace_blas<ANY, false, true, THREADS, 32, MIXED>;
    default: return (const void *)k_trace_blas<ANY, false, true, THREADS, 16, MIXED>;
    }
}

bool valid_shape(const TraceShape &shape) {
    return (shape.threads == 128u || shape.threads == 256u) &&
           (shape.ring == 8u || shape.ring == 16u || shape.ring == 32u) && shape.refill != 0u && shape.refill <= 32u &&
           shape.blocks_per_sm != 0u;
}

}  // namespace

int prepare_queue_trace_multi(rt_context *ctx, const TraceShape &shape) {
    if (!valid_shape(shape)) return set_error(ctx, RT_ERR_INVALID_ARG, "multi-scene traversal: unsupported launch shape");
    const void *k[3] = {shape.threads == 256u ? kernel_ring<false, 256>(shape.ring) : kernel_ring<false, 128>(shape.ring),
                        shape.threads == 256u ? kernel_ring<true, 256>(shape.ring) : kernel_ring<true, 128>(shape.ring),
                        shape.threads == 256u ? kernel_ring<false, 256, true>(shape.ring)
                                              : kernel_ring<false, 128, true>(shape.ring)};
    cudaFuncAttributes fa;
    for (const void *f : k) RT_CUDA_CTX(ctx, cudaFuncGetAttributes(&fa, f));
    return RT_OK;
}

int launch_queue_trace_multi(rt_context *ctx, cudaStream_t st, const void *views, uint32_t n_scenes,
                             const uint32_t *ray_scene, const void *rays, void *hits, uint8_t *occluded,
                             const uint32_t *n_dev, uint32_t max_n, uint32_t *counter, bool any,
                             const TraceShape &shape) {
    if (max_n == 0) return RT_OK;
    if (!valid_shape(shape))
        return set_error(ctx, RT_ERR_INVALID_ARG, "multi-scene traversal: unsupported launch shape");
    BatchArgs a{};
    a.scenes = static_cast<const TravScene *>(views);
    a.ray_scene = ray_scene;
    a.n_scenes = n_scenes;
    a.rays = static_cast<const float4 *>(rays);
    a.hits = static_cast<float4 *>(hits);
    a.occluded = occluded;
    a.n = max_n;
    a.refill = shape.refill;
    a.counter = counter;
    a.err = ctx->d_err;
    a.n_dev = n_dev;
    a.out_rec = 1;
    uint32_t blocks = shape.blocks_per_sm * (uint32_t)ctx->sm_count;
    const uint32_t need = (max_n + shape.threads - 1u) / shape.threads;
    if (blocks > need) blocks = need;
    if (shape.threads == 256u) {
        if (any) launch_ring<true, 256>(a, shape.ring, blocks, st);
        else launch_ring<false, 256>(a, shape.ring, blocks, st);
    } else {
        if (any) launch_ring<true, 128>(a, shape.ring, blocks, st);
        else launch_ring<false, 128>(a, shape.ring, blocks, st);
    }
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}

// Two queues in one launch (see k_trace_blas, MIXED): the closest-hit rays
// (ray_scene/rays/n_dev, to hits), then the any-hit rays (ray_scene2/rays2/
// n_dev2, to occluded), each at most max_n.
int launch_queue_trace_multi_mixed(rt_context *ctx, cudaStream_t st, const void *views, uint32_t n_scenes,
                                   const uint32_t *ray_scene, const void *rays, void *hits, const uint32_t *n_dev,
                                   const uint32_t *ray_scene2, const void *rays2, uint8_t *occluded,
                                   const uint32_t *n_dev2, uint32_t max_n, uint32_t *counter,
                                   const TraceShape &shape) {
    if (max_n == 0) return RT_OK;
    if (!valid_shape(shape))
        return set_error(ctx, RT_ERR_INVALID_ARG, "multi-scene traversal: unsupported launch shape");
    BatchArgs a{};
    a.scenes = static_cast<const TravScene *>(views);
    a.ray_scene = ray_scene;
    a.n_scenes = n_scenes;
    a.rays = static_cast<const float4 *>(rays);
    a.hits = static_cast<float4 *>(hits);
    a.n = max_n;
    a.n_dev = n_dev;
    a.ray_scene2 = ray_scene2;
    a.rays2 = static_cast<const float4 *>(rays2);
    a.occluded = occluded;
    a.n_dev2 = n_dev2;
    a.n2 = max_n;
    a.refill = shape.refill;
    a.counter = counter;
    a.err = ctx->d_err;
    a.out_rec = 1;
    uint32_t blocks = shape.blocks_per_sm * (uint32_t)ctx->sm_count;
    const uint32_t need = (uint32_t)(((uint64_t)max_n * 2u + shape.threads - 1u) / shape.threads);
    if (blocks > need) blocks = need;
    if (shape.threads == 256u) launch_ring<false, 256, true>(a, shape.ring, blocks, st);
    else launch_ring<false, 128, true>(a, shape.ring, blocks, st);
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}

}  // namespace rtc
