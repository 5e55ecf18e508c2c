// rt_sort.cu -- onesweep LSD radix sort of (uint64 key, uint32 value) pairs.
//
// The acceleration-structure build of the reference happens inside the
// Vulkan driver (vkCmdBuildAccelerationStructuresKHR,
// vulkan-raytraced-triangle/main.cpp:808); its Morton-order sort is one of the
// driver-hidden steps made explicit here.
//
// Algorithm: Adinets & Merrill, "Onesweep: A Faster Least Significant Digit
// Radix Sort for GPUs" (2022).  One histogram kernel counts the 8-bit digits
// of every pass in a single read; each pass is then one kernel in which tiles
// rank their keys locally (warp multisplit by ballots), publish per-digit
// counts, resolve their global offsets by decoupled look-back over earlier
// tiles, and scatter through shared memory.  Tiles are numbered in launch
// order by an atomic counter, so a tile only waits on tiles already owned by
// running blocks.  Every wait is bounded: on expiry the kernel records
// RT_ERR_TIMEOUT and carries on, so the host sees an error instead of a hang.
// The sort is stable, hence its output equals std::stable_sort by key.
#include <cuda_runtime.h>

#include "rt_internal.h"
#include "../../include/rtcore_debug.h"

namespace rtc {

namespace {

constexpr int kSortThreads = 512;
constexpr int kSortWarps = kSortThreads / 32;
// 14 keys per thread: tiles of 7,168 keys, 140 tiles for 1M keys, one wave
// of one 98 KB block per SM on 152 SMs (8 keys per thread: 245 tiles, two
// waves, 1M-key soup build 0.807 ms; 16: 123 tiles, 0.792 ms then and equal
// to 14 now on the soup; 14: 2M box 1.317 -> 1.306 ms)
constexpr int kSortItems = 14;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kRankGroup = 8;  // keys ranked together (their votes, atomics and shuffles back to back)
constexpr int kRadix = 256;
// Statuses read per look-back round trip.  Tiles of one wave publish their
// aggregates at about the same time, so a walk of one predecessor per round
// trip crossed about half the wave serially.
constexpr int kLookWindow = 8;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagIncl = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;

constexpr size_t kSortSmemBytes =
    (size_t)kSortTile * 8u + (size_t)kSortTile * 4u + (size_t)kSortWarps * kRadix * 4u;

// Digit mask of pass p when sorting on the low key_bits bits.
__host__ __device__ __forceinline__ uint32_t digit_mask(int key_bits, int p) {
    int left = key_bits - 8 * p;
    return left >= 8 ? 0xffu : ((1u << left) - 1u);
}

__global__ void __launch_bounds__(256) k_sort_hist(const uint64_t *__restrict__ keys, uint32_t n, int key_bits,
                                                    uint32_t *__restrict__ hist) {
    const int passes = (key_bits + 7) / 8;
    __shared__ uint32_t sh[8][kRadix];
    for (int i = threadIdx.x; i < 8 * kRadix; i += blockDim.x) (&sh[0][0])[i] = 0u;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint64_t k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][(k >> (8 * p)) & digit_mask(key_bits, p)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x) {
        uint32_t c = (&sh[0][0])[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// Exclusive scan of 256 values held one per thread by threads 0..255 of the
// block (all threads of the block must call it).  Returns the exclusive
// prefix for threads < 256 and writes the total to *total.
__device__ __forceinline__ uint32_t block_scan256(uint32_t v, uint32_t *s_warp, uint32_t *total) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    uint32_t x = (t < kRadix) ? v : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (t < kRadix && lane == 31) s_warp[w] = x;
    __syncthreads();
    if (t == 0) {
        uint32_t s = 0;
        for (int i = 0; i < kRadix / 32; ++i) { uint32_t c = s_warp[i]; s_warp[i] = s; s += c; }
        s_warp[kRadix / 32] = s;
    }
    __syncthreads();
    uint32_t excl = (t < kRadix) ? (x - v + s_warp[w]) : 0u;
    if (total) *total = s_warp[kRadix / 32];
    __syncthreads();
    return excl;
}

__global__ void __launch_bounds__(kSortThreads) k_onesweep(const uint64_t *__restrict__ kin,
                                                            const uint32_t *__restrict__ vin,
                                                            uint64_t *__restrict__ kout,
                                                            uint32_t *__restrict__ vout, uint32_t n, int shift, uint32_t dmask,
                                                            const uint32_t *__restrict__ hist,
                                                            uint32_t *__restrict__ status,
                                                            uint32_t *__restrict__ tile_counter, uint32_t *err,
                                                            uint32_t spin_limit, uint32_t withhold) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint64_t *s_keys = reinterpret_cast<uint64_t *>(smem);
    uint32_t *s_vals = reinterpret_cast<uint32_t *>(s_keys + kSortTile);
    uint32_t *s_whist = s_vals + kSortTile;  // [warp][digit]
    __shared__ uint32_t s_digit_excl[kRadix];
    __shared__ uint32_t s_global[kRadix];
    __shared__ uint32_t s_warp[kRadix / 32 + 1];
    __shared__ uint32_t s_tile;

    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (t == 0) s_tile = atomicAdd(tile_counter, 1u);
    for (int i = t; i < kSortWarps * kRadix; i += kSortThreads) s_whist[i] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * (uint32_t)kSortTile;

    uint64_t k[kSortItems];
    uint32_t v[kSortItems];
    uint32_t rank[kSortItems];
    const uint32_t wbase = base + (uint32_t)w * 32u * kSortItems;
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        uint32_t idx = wbase + (uint32_t)j * 32u + (uint32_t)lane;
        bool valid = idx < n;
        k[j] = valid ? kin[idx] : 0ull;
        v[j] = valid ? vin[idx] : 0u;
    }
    const uint32_t lt = (1u << lane) - 1u;
    // Peers of each key (the valid lanes holding the same digit) from eight
    // ballots on the digit's bits: vote instructions in registers, where
    // match.any took about 0.5 us per round with a warp's ~30 distinct
    // digits (7.7 of a tile's 17 us).  Eight keys per group: their peer
    // masks first, then the leaders' shared-memory atomics back to back
    // (applied in issue order, which keeps the ranks in input order), then
    // the shuffles of the old counts, so no key waits on the one before it.
#pragma unroll
    for (int j0 = 0; j0 < kSortItems; j0 += kRankGroup) {
        uint32_t pm[kRankGroup], old[kRankGroup];
#pragma unroll
        for (int jj = 0; jj < kRankGroup; ++jj) {
            const int j = j0 + jj;
            if (j >= kSortItems) break;  // a last, shorter group
            const uint32_t d = (uint32_t)(k[j] >> shift) & dmask;
            uint32_t peers = __ballot_sync(0xffffffffu, wbase + (uint32_t)j * 32u + (uint32_t)lane < n);
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const uint32_t bb = __ballot_sync(0xffffffffu, (d >> b) & 1u);
                peers &= ((d >> b) & 1u) ? bb : ~bb;
            }
            pm[jj] = peers;
        }
#pragma unroll
        for (int jj = 0; jj < kRankGroup; ++jj) {
            const int j = j0 + jj;
            if (j >= kSortItems) break;
            const uint32_t d = (uint32_t)(k[j] >> shift) & dmask;
            old[jj] = 0u;
            if ((int)(__ffs(pm[jj]) - 1) == lane)
                old[jj] = atomicAdd(&s_whist[w * kRadix + d], (uint32_t)__popc(pm[jj]));
        }
#pragma unroll
        for (int jj = 0; jj < kRankGroup; ++jj) {
            const int j = j0 + jj;
            if (j >= kSortItems) break;
            const int leader = pm[jj] ? __ffs(pm[jj]) - 1 : lane;
            rank[j] = __shfl_sync(0xffffffffu, old[jj], leader) + (uint32_t)__popc(pm[jj] & lt);
        }
    }
    __syncthreads();

    // per digit: exclusive over warps, block total
    uint32_t total = 0;
    if (t < kRadix) {
        uint32_t s = 0;
        for (int ww = 0; ww < kSortWarps; ++ww) {
            uint32_t c = s_whist[ww * kRadix + t];
            s_whist[ww * kRadix + t] = s;
            s += c;
        }
        total = s;
    }
    uint32_t dex = block_scan256(total, s_warp, nullptr);
    uint32_t gex = block_scan256(t < kRadix ? hist[t] : 0u, s_warp, nullptr);
    if (t < kRadix) {
        s_digit_excl[t] = dex;
        volatile uint32_t *st = status;
        uint32_t prefix = 0;
        if (tile == 0) {
            if (!withhold) st[t] = kFlagIncl | total;
        } else {
            st[(size_t)tile * kRadix + t] = kFlagAgg | total;
            __threadfence();
            // kLookWindow predecessors per round trip, nearest first: their
            // aggregates add up until an inclusive prefix ends the walk; a
            // predecessor not yet published is polled alone (bounded).
            int64_t p = (int64_t)tile - 1;
            bool done = false;
            while (!done) {
                uint32_t sw[kLookWindow];
#pragma unroll
                for (int i = 0; i < kLookWindow; ++i) sw[i] = p - i >= 0 ? st[(size_t)(p - i) * kRadix + t] : 0u;
                int used = 0;
#pragma unroll
                for (int i = 0; i < kLookWindow; ++i) {
                    if (done || used < i || (sw[i] & ~kValueMask) == 0u) continue;
                    prefix += sw[i] & kValueMask;
                    done = (sw[i] & ~kValueMask) == kFlagIncl;
                    used = i + 1;
                }
                if (done) break;
                p -= used;  // p >= 0: tile 0 publishes an inclusive prefix
                if (used == kLookWindow) continue;
                uint32_t s = 0u, spins = 0;
                do {
                    s = st[(size_t)p * kRadix + t];
                } while ((s & ~kValueMask) == 0u && ++spins < spin_limit);
                if ((s & ~kValueMask) == 0u) {
                    report_error(err, RT_ERR_TIMEOUT, 0x50000000u | (uint32_t)tile);
                    break;
                }
            }
            st[(size_t)tile * kRadix + t] = kFlagIncl | ((prefix + total) & kValueMask);
        }
        s_global[t] = gex + prefix;
    }
    __syncthreads();

#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        uint32_t idx = wbase + (uint32_t)j * 32u + (uint32_t)lane;
        if (idx < n) {
            uint32_t d = (uint32_t)(k[j] >> shift) & dmask;
            uint32_t pos = s_digit_excl[d] + s_whist[w * kRadix + d] + rank[j];
            s_keys[pos] = k[j];
            s_vals[pos] = v[j];
        }
    }
    __syncthreads();
    const uint32_t tile_n = (n - base) < (uint32_t)kSortTile ? (n - base) : (uint32_t)kSortTile;
    for (uint32_t i = (uint32_t)t; i < tile_n; i += kSortThreads) {
        uint64_t key = s_keys[i];
        uint32_t d = (uint32_t)(key >> shift) & dmask;
        uint32_t o = s_global[d] + (i - s_digit_excl[d]);
        if (o < n) {
            kout[o] = key;
            vout[o] = s_vals[i];
        } else {
            report_error(err, RT_ERR_BOUNDS, 0x51000000u | (uint32_t)tile);
        }
    }
}

}  // namespace

uint64_t sort_scratch_bytes(uint32_t n, int passes) {
    uint64_t tiles = ((uint64_t)n + kSortTile - 1) / kSortTile;
    if (tiles == 0) tiles = 1;
    // histograms (8 x 256) + tile counters (8) + status (passes x tiles x 256)
    return align_up(8u * kRadix * 4u, 256) + align_up(8u * 4u, 256) +
           align_up((uint64_t)passes * tiles * kRadix * 4u, 256);
}

// Sorts (keys0, vals0) on the low 8*passes key bits, using (keys1, vals1) as
// the ping-pong buffer.  After an even number of passes the result is back in
// keys0/vals0.  `keys_hist_done`: the caller already accumulated the digit
// histograms into the scratch (fused with key generation).
int sort_pairs(const rt_context *ctx, cudaStream_t stream, uint64_t *keys0, uint32_t *vals0, uint64_t *keys1,
               uint32_t *vals1, uint32_t n, int key_bits, void *scratch, bool hist_done, uint32_t *err,
               uint32_t withhold) {
    if (n == 0) return RT_OK;
    const int passes = (key_bits + 7) / 8;
    if (n > kValueMask) return RT_ERR_UNSUPPORTED;
    uint8_t *s = static_cast<uint8_t *>(scratch);
    uint32_t *hist = reinterpret_cast<uint32_t *>(s);
    uint32_t *counters = reinterpret_cast<uint32_t *>(s + align_up(8u * kRadix * 4u, 256));
    uint32_t *status = reinterpret_cast<uint32_t *>(s + align_up(8u * kRadix * 4u, 256) + align_up(8u * 4u, 256));
    uint64_t tiles = ((uint64_t)n + kSortTile - 1) / kSortTile;
    // counters and status must start at zero; the histogram too unless the
    // caller filled it.
    if (!hist_done) {
        RT_CUDA_TRY(cudaMemsetAsync(hist, 0, 8u * kRadix * 4u, stream));
        int blocks = (int)((n + 255u) / 256u);
        int cap = ctx->sm_count * 8;
        if (blocks > cap) blocks = cap;
        k_sort_hist<<<blocks, 256, 0, stream>>>(keys0, n, key_bits, hist);
        RT_CUDA_TRY(cudaGetLastError());
    }
    RT_CUDA_TRY(cudaMemsetAsync(counters, 0, 8u * 4u, stream));
    RT_CUDA_TRY(cudaMemsetAsync(status, 0, (size_t)passes * tiles * kRadix * 4u, stream));
    RT_CUDA_TRY(cudaFuncSetAttribute(k_onesweep, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kSortSmemBytes));
    for (int p = 0; p < passes; ++p) {
        const uint64_t *ki = (p & 1) ? keys1 : keys0;
        const uint32_t *vi = (p & 1) ? vals1 : vals0;
        uint64_t *ko = (p & 1) ? keys0 : keys1;
        uint32_t *vo = (p & 1) ? vals0 : vals1;
        k_onesweep<<<(unsigned)tiles, kSortThreads, kSortSmemBytes, stream>>>(
            ki, vi, ko, vo, n, 8 * p, digit_mask(key_bits, p), hist + p * kRadix, status + (size_t)p * tiles * kRadix, counters + p, err,
            ctx->sort_spin_limit, withhold);
        RT_CUDA_TRY(cudaGetLastError());
    }
    if (passes & 1) {
        RT_CUDA_TRY(cudaMemcpyAsync(keys0, keys1, (size_t)n * 8u, cudaMemcpyDeviceToDevice, stream));
        RT_CUDA_TRY(cudaMemcpyAsync(vals0, vals1, (size_t)n * 4u, cudaMemcpyDeviceToDevice, stream));
    }
    return RT_OK;
}

uint32_t *sort_hist_ptr(void *scratch) { return static_cast<uint32_t *>(scratch); }

}  // namespace rtc

// ---------------------------------------------------------------------------
// C ABI: standalone pair sort (used for ray reordering and tested on its own)
// ---------------------------------------------------------------------------
extern "C" rt_status rt_get_sort_scratch_bytes(uint32_t n, uint32_t key_bits, uint64_t *out) {
    if (!out || key_bits == 0 || key_bits > 64) return RT_ERR_INVALID_ARG;
    int passes = (int)((key_bits + 7u) / 8u);
    *out = rtc::align_up((uint64_t)n * 12u, 256) + rtc::sort_scratch_bytes(n, passes);
    return RT_OK;
}

extern "C" rt_status rt_debug_set_sort_spin_limit(rt_context *ctx, uint32_t spins) {
    if (!ctx) return RT_ERR_INVALID_ARG;
    ctx->sort_spin_limit = spins ? spins : rt_context::kSortSpinLimit;
    return RT_OK;
}

extern "C" rt_status rt_debug_set_sort_withhold(rt_context *ctx, int withhold) {
    if (!ctx) return RT_ERR_INVALID_ARG;
    ctx->sort_withhold = withhold ? 1u : 0u;
    return RT_OK;
}

extern "C" rt_status rt_sort_pairs(rt_context *ctx, rt_stream stream, uint64_t *keys, uint32_t *vals, uint32_t n,
                                   uint32_t key_bits, void *scratch, uint64_t scratch_bytes) {
    if (!ctx || (n && (!keys || !vals || !scratch)) || key_bits == 0 || key_bits > 64)
        return rtc::set_error(ctx, RT_ERR_INVALID_ARG, "rt_sort_pairs: bad argument");
    uint64_t need = 0;
    rt_get_sort_scratch_bytes(n, key_bits, &need);
    if (scratch_bytes < need) return rtc::set_error(ctx, RT_ERR_OOM, "rt_sort_pairs: scratch too small");
    int passes = (int)((key_bits + 7u) / 8u);
    uint8_t *s = static_cast<uint8_t *>(scratch);
    uint64_t *k1 = reinterpret_cast<uint64_t *>(s);
    uint32_t *v1 = reinterpret_cast<uint32_t *>(s + (size_t)n * 8u);
    void *sort_s = s + rtc::align_up((uint64_t)n * 12u, 256);
    int st = rtc::sort_pairs(ctx, static_cast<cudaStream_t>(stream), keys, vals, k1, v1, n, (int)key_bits, sort_s, false,
                             ctx->d_err, ctx->sort_withhold);
    if (st) return rtc::set_error(ctx, st, "rt_sort_pairs: launch failed");
    return RT_OK;
}
