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

namespace rtc {
namespace {

// Bandwidth probe: reads the buffer `passes` times, four independent 16-byte
// loads per thread and step, cached in L2 only (ld.global.cg), so that a
// buffer smaller than L2 measures L2 read bandwidth and a larger one HBM.
// The XOR of everything read decides one store nobody expects, which keeps
// the loads alive.
__global__ void __launch_bounds__(512) k_read_sweep(const uint4 *__restrict__ buf, uint64_t n16, uint32_t passes,
                                                    uint32_t *sink) {
    uint32_t acc = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t r = 0; r < passes; ++r) {
        uint64_t i = t;
        for (; i + 3u * stride < n16; i += 4u * stride) {
            const uint4 a = __ldcg(buf + i), b = __ldcg(buf + i + stride);
            const uint4 c = __ldcg(buf + i + 2u * stride), d = __ldcg(buf + i + 3u * stride);
            acc ^= (a.x ^ b.y) ^ (c.z ^ d.w);
        }
        for (; i < n16; i += stride) acc ^= __ldcg(buf + i).x;
    }
    if (acc == 0x9e3779b9u) sink[0] = acc;
}

}  // namespace
}  // namespace rtc

using namespace rtc;

extern "C" rt_status rt_debug_read_sweep(rt_context *ctx, rt_stream stream, const void *buf, uint64_t bytes,
                                         uint32_t passes) {
    if (!ctx || (bytes && !buf) || (bytes & 15u) || (reinterpret_cast<uintptr_t>(buf) & 15u))
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_debug_read_sweep: a 16-byte aligned buffer of 16-byte units");
    if (bytes == 0 || passes == 0) return RT_OK;
    k_read_sweep<<<(unsigned)ctx->sm_count * 4u, 512, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const uint4 *>(buf), bytes / 16u, passes, ctx->d_counters + kNumCounters);
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}

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
    static_scratch_forget(device);
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
    // Library-owned bookkeeping: error word + work counters + the bandwidth
    // probe's sink word.
    void *p = nullptr;
    if (cudaMalloc(&p, (3u + kNumCounters) * sizeof(uint32_t)) != cudaSuccess) {
        delete ctx;
        return RT_ERR_OOM;
    }
    ctx->d_err = static_cast<uint32_t *>(p);
    ctx->d_counters = ctx->d_err + 2;
    if (cudaMemset(p, 0, (3u + kNumCounters) * sizeof(uint32_t)) != cudaSuccess) {
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
