// rt_context.cu -- context lifetime, error reporting, synchronisation and the
// image writers of the ray-tracing core.
//
// The context stands in for the Vulkan instance/device/queue the sample
// creates (createVkInstance / createVkDevice, vulkan-raytraced-triangle/
// main.cpp:242-388); rt_sync stands in for vkQueueWaitIdle (main.cpp:820, 942,
// 998) and the frame fence (main.cpp:1333, 1411).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "rt_internal.h"

namespace rtc {

int set_error(rt_context *ctx, int code, const char *msg) {
    if (ctx) ctx->last_error = msg ? msg : "";
    return code;
}

int set_cuda_error(rt_context *ctx, cudaError_t e, const char *where) {
    if (ctx) {
        ctx->last_error = std::string(where) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    }
    if (e == cudaErrorNoKernelImageForDevice || e == cudaErrorInvalidDevice || e == cudaErrorNoDevice)
        return RT_ERR_NO_DEVICE;
    return RT_ERR_CUDA;
}

uint32_t *acquire_counter(rt_context *ctx, cudaStream_t stream) {
    uint32_t *c = ctx->d_counters + (ctx->counter_next++ % kNumCounters);
    if (cudaMemsetAsync(c, 0, sizeof(uint32_t), stream) != cudaSuccess) return nullptr;
    return c;
}

}  // namespace rtc

using namespace rtc;

extern "C" uint32_t rt_abi_version(void) { return RTCORE_ABI_VERSION; }

extern "C" rt_status rt_context_create(int device, rt_context **out) {
    if (!out) return RT_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return RT_ERR_NO_DEVICE;
    if (device < 0 || device >= count) return RT_ERR_INVALID_ARG;
    rt_context *ctx = new (std::nothrow) rt_context();
    if (!ctx) return RT_ERR_OOM;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    cudaDeviceProp prop;
    if (e == cudaSuccess) e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) {
        delete ctx;
        return RT_ERR_NO_DEVICE;
    }
    ctx->sm_count = prop.multiProcessorCount;
    ctx->cc_major = prop.major;
    ctx->cc_minor = prop.minor;
    ctx->smem_optin = prop.sharedMemPerBlockOptin;
    // The kernels are built for sm_103a only.
    if (prop.major != 10 || prop.minor != 3) {
        delete ctx;
        return RT_ERR_NO_DEVICE;
    }
    // Library-owned bookkeeping: error word + work counters.
    void *p = nullptr;
    if (cudaMalloc(&p, (2u + kNumCounters) * sizeof(uint32_t)) != cudaSuccess) {
        delete ctx;
        return RT_ERR_OOM;
    }
    ctx->d_err = static_cast<uint32_t *>(p);
    ctx->d_counters = ctx->d_err + 2;
    if (cudaMemset(p, 0, (2u + kNumCounters) * sizeof(uint32_t)) != cudaSuccess) {
        cudaFree(p);
        delete ctx;
        return RT_ERR_CUDA;
    }
    ctx->tuning.block_threads = 128;
    ctx->tuning.blocks_per_sm = 9;
    // refill a warp once 4 lanes are idle: best for incoherent rays in a
    // sweep of 1..32 on the 1M-triangle soup (primary rays are flat from 4
    // to 16)
    ctx->tuning.batch_rays = 4;
    *out = ctx;
    return RT_OK;
}

extern "C" rt_status rt_context_destroy(rt_context *ctx) {
    if (!ctx) return RT_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->host_ready) {
        cudaStreamSynchronize(ctx->h2d);
        cudaStreamSynchronize(ctx->d2h);
        for (int k = 0; k < rt_context::kHostTraceStreams; ++k) {
            cudaStreamSynchronize(ctx->htr[k]);
            cudaStreamDestroy(ctx->htr[k]);
        }
        cudaEventDestroy(ctx->ev_start);
        for (int s = 0; s < rt_context::kHostSlots; ++s) {
            cudaEventDestroy(ctx->ev_loaded[s]);
            cudaEventDestroy(ctx->ev_traced[s]);
            cudaEventDestroy(ctx->ev_free[s]);
        }
        cudaStreamDestroy(ctx->h2d);
        cudaStreamDestroy(ctx->d2h);
    }
    if (ctx->d_err) cudaFree(ctx->d_err);
    delete ctx;
    return RT_OK;
}

extern "C" const char *rt_last_error_string(rt_context *ctx) {
    if (!ctx) return "null context";
    return ctx->last_error.c_str();
}

extern "C" rt_status rt_sync(rt_context *ctx, rt_stream stream) {
    if (!ctx) return RT_ERR_INVALID_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    RT_CUDA_CTX(ctx, cudaStreamSynchronize(st));
    uint32_t w[2] = {0, 0};
    RT_CUDA_CTX(ctx, cudaMemcpy(w, ctx->d_err, sizeof(w), cudaMemcpyDeviceToHost));
    if (w[0]) {
        RT_CUDA_CTX(ctx, cudaMemset(ctx->d_err, 0, sizeof(w)));
        char msg[128];
        std::snprintf(msg, sizeof(msg), "device-side error %d (detail 0x%08x)", -(int)w[0], w[1]);
        return set_error(ctx, -(int)w[0], msg);
    }
    return RT_OK;
}

extern "C" rt_status rt_set_trace_tuning(rt_context *ctx, const rt_trace_tuning *t) {
    if (!ctx || !t) return RT_ERR_INVALID_ARG;
    if (t->block_threads != 128u) return set_error(ctx, RT_ERR_UNSUPPORTED, "traversal blocks are 128 threads");
    if (t->blocks_per_sm == 0 || t->blocks_per_sm > 16u) return set_error(ctx, RT_ERR_INVALID_ARG, "blocks_per_sm in 1..16");
    if (t->batch_rays == 0 || t->batch_rays > 32u) return set_error(ctx, RT_ERR_INVALID_ARG, "batch_rays in 1..32");
    ctx->tuning = *t;
    return RT_OK;
}

extern "C" rt_status rt_get_trace_tuning(rt_context *ctx, rt_trace_tuning *t) {
    if (!ctx || !t) return RT_ERR_INVALID_ARG;
    *t = ctx->tuning;
    return RT_OK;
}

// R8G8B8A8_UNORM conversion: clamp to [0,1], scale by 255, round to nearest.
static inline unsigned char unorm8(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 1.0f) return 255;
    return (unsigned char)std::lround(v * 255.0f);
}

extern "C" rt_status rt_write_ppm(const float *rgba, uint32_t width, uint32_t height, const char *path) {
    if (!rgba || !path || width == 0 || height == 0) return RT_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "wb");
    if (!f) return RT_ERR_INVALID_ARG;
    std::fprintf(f, "P6\n%u %u\n255\n", width, height);
    std::vector<unsigned char> row((size_t)width * 3u);
    for (uint32_t y = 0; y < height; ++y) {
        for (uint32_t x = 0; x < width; ++x)
            for (int c = 0; c < 3; ++c) row[(size_t)x * 3u + c] = unorm8(rgba[((size_t)y * width + x) * 4u + c]);
        if (std::fwrite(row.data(), 1, row.size(), f) != row.size()) {
            std::fclose(f);
            return RT_ERR_INVALID_ARG;
        }
    }
    return std::fclose(f) == 0 ? RT_OK : RT_ERR_INVALID_ARG;
}

extern "C" rt_status rt_write_pfm(const float *rgba, uint32_t width, uint32_t height, const char *path) {
    if (!rgba || !path || width == 0 || height == 0) return RT_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "wb");
    if (!f) return RT_ERR_INVALID_ARG;
    std::fprintf(f, "PF\n%u %u\n-1.0\n", width, height);
    std::vector<float> row((size_t)width * 3u);
    for (uint32_t yy = 0; yy < height; ++yy) {
        uint32_t y = height - 1u - yy;  // PFM stores the bottom row first
        for (uint32_t x = 0; x < width; ++x)
            for (int c = 0; c < 3; ++c) row[(size_t)x * 3u + c] = rgba[((size_t)y * width + x) * 4u + c];
        if (std::fwrite(row.data(), sizeof(float), row.size(), f) != row.size()) {
            std::fclose(f);
            return RT_ERR_INVALID_ARG;
        }
    }
    return std::fclose(f) == 0 ? RT_OK : RT_ERR_INVALID_ARG;
}
