// rt_internal.h -- host-side internals shared by the translation units of
// librtcore: the context object, error plumbing and cross-file launchers.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>

#include <cuda_runtime.h>

#include "../../include/rtcore.h"
#include "../../include/rtcore_accel.h"
#include "../../include/rtcore_cache.h"
#include "rt_device.cuh"

// Library-owned state of one device.  Replaces the Vulkan instance/device
// bring-up of the sample (createVkInstance/createVkDevice, main.cpp:242-388).
struct rt_context {
    int device = 0;
    int sm_count = 0;
    int cc_major = 0, cc_minor = 0;
    size_t smem_optin = 0;
    // d_err[0]: first device-side error code (negated RT_ERR_*), d_err[1]:
    // detail word.  Cleared by rt_sync.
    uint32_t *d_err = nullptr;
    // Work-stealing counters for persistent kernels, used round-robin.
    uint32_t *d_counters = nullptr;
    uint32_t counter_next = 0;
    rt_trace_tuning tuning{};
    std::string last_error;
    // Host-memory ray API (rt_trace_*_host): two copy streams and, per
    // device slot of the copy ring, the events that order copy in ->
    // traversal -> copy out -> reuse; created on first use.
    static constexpr int kHostSlots = 4;
    static constexpr int kHostTraceStreams = 3;
    bool host_ready = false;
    cudaStream_t h2d = nullptr, d2h = nullptr, htr[kHostTraceStreams] = {};
    cudaEvent_t ev_loaded[kHostSlots] = {}, ev_traced[kHostSlots] = {}, ev_free[kHostSlots] = {};
    cudaEvent_t ev_start = nullptr;
    uint32_t slot_next = 0;
    uint32_t host_transfer = 0;  // RT_HOST_TRANSFER_*
    int pageable_state = 0;      // 0 not queried, 1 pageable memory reachable in place, 2 not
    const void *host_scratch = nullptr;  // the ring the events above refer to
    uint64_t host_scratch_bytes = 0;
    // Polls of a predecessor tile's status the onesweep look-back makes
    // before it gives up with RT_ERR_TIMEOUT (rt_debug_set_sort_spin_limit).
    static constexpr uint32_t kSortSpinLimit = 1u << 22;
    uint32_t sort_spin_limit = kSortSpinLimit;
    uint32_t sort_withhold = 0;  // rt_debug_set_sort_withhold
};

namespace rtc {

constexpr uint32_t kNumCounters = 256;

inline uint64_t align_up(uint64_t x, uint64_t a) { return (x + a - 1u) / a * a; }

// Records a host-side error on the context and returns the code.
int set_error(rt_context *ctx, int code, const char *msg);
int set_cuda_error(rt_context *ctx, cudaError_t e, const char *where);

// Next work counter (zeroed on `stream` before it is handed out).
uint32_t *acquire_counter(rt_context *ctx, cudaStream_t stream);

// aspect_y = tan(radians(yFov) * 0.5), aspect_x = aspect_y * W / H of the
// sample's raygen (main.cpp:1039-1040): radians and the halving in float as
// GLSL evaluates them, tan in double rounded once, on the host.
inline void camera_aspects(const rt_camera *cam, uint32_t w, uint32_t h, float *ay, float *ax) {
    const float half = (cam->y_fov_degree * (float)(3.14159265358979323846 / 180.0)) * 0.5f;
    *ay = (float)std::tan((double)half);
    *ax = (*ay * (float)w) / (float)h;
}

// Queue-driven BLAS traversal (rt_trace.cu) used by the path tracer.
int launch_queue_trace(rt_context *ctx, cudaStream_t st, const uint8_t *accel, const void *rays, void *hits,
                       uint8_t *occluded, const uint32_t *n_dev, uint32_t max_n, uint32_t *counter, bool any);
int launch_queue_trace_mixed(rt_context *ctx, cudaStream_t st, const uint8_t *accel, const void *rays, void *hits,
                             const uint32_t *n_dev, const void *rays2, uint8_t *occluded, const uint32_t *n_dev2,
                             uint32_t max_n, uint32_t *counter);

// Launch shape of the multi-scene traversal (rt_trace_multi.cu).
struct TraceShape {
    uint32_t threads;        // 128 or 256
    uint32_t blocks_per_sm;
    uint32_t ring;           // 8, 16 or 32 shared-memory stack entries per ray
    uint32_t refill;         // 1..32
};

// Queue-driven traversal over rays of many scenes: ray i belongs to scene
// ray_scene[i], whose 32-byte traversal view is views[ray_scene[i]]
// (TravScene of rt_traverse.cuh).  Closest hits carry the leaf-record index.
int launch_queue_trace_multi(rt_context *ctx, cudaStream_t st, const void *views, uint32_t n_scenes,
                             const uint32_t *ray_scene, const void *rays, void *hits, uint8_t *occluded,
                             const uint32_t *n_dev, uint32_t max_n, uint32_t *counter, bool any,
                             const TraceShape &shape);
int launch_queue_trace_multi_mixed(rt_context *ctx, cudaStream_t st, const void *views, uint32_t n_scenes,
                                   const uint32_t *ray_scene, const void *rays, void *hits, const uint32_t *n_dev,
                                   const uint32_t *ray_scene2, const void *rays2, uint8_t *occluded,
                                   const uint32_t *n_dev2, uint32_t max_n, uint32_t *counter,
                                   const TraceShape &shape);

// Loads the two traversal kernels of a shape (before a graph capture).
int prepare_queue_trace_multi(rt_context *ctx, const TraceShape &shape);

// MLP cache launchers whose row counts live on the device (rt_mlp.cu).
int cache_query_dev(rt_context *ctx, cudaStream_t st, const void *cache, const rt_cache_input *in, float *out,
                    const uint32_t *n_dev, uint32_t max_n);
int cache_train_dev(rt_context *ctx, cudaStream_t st, void *cache, const rt_cache_input *in, const float *targets,
                    const uint32_t *n_dev, uint32_t max_n, uint32_t batch);

// Sort (rt_sort.cu)
uint64_t sort_scratch_bytes(uint32_t n, int passes);
int sort_pairs(const rt_context *ctx, cudaStream_t stream, uint64_t *keys0, uint32_t *vals0, uint64_t *keys1,
               uint32_t *vals1, uint32_t n, int key_bits, void *scratch, bool hist_done, uint32_t *err,
               uint32_t withhold = 0u);
uint32_t *sort_hist_ptr(void *scratch);

// Forgets the cached device address of the allocation-free build's static
// scratch array on `device` (rt_build.cu); rt_context_create calls it so that
// a context made after a device reset looks the address up again.
void static_scratch_forget(int device);

}  // namespace rtc

#define RT_CUDA_TRY(expr)                                  \
    do {                                                   \
        cudaError_t rt_e_ = (expr);                        \
        if (rt_e_ != cudaSuccess) return RT_ERR_CUDA;      \
    } while (0)

#define RT_CUDA_CTX(ctx, expr)                                               \
    do {                                                                     \
        cudaError_t rt_e_ = (expr);                                          \
        if (rt_e_ != cudaSuccess) return rtc::set_cuda_error(ctx, rt_e_, #expr); \
    } while (0)
