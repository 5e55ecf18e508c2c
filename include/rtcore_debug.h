/*
 * rtcore_debug.h -- utility and inspection entry points of librtcore.
 *
 * The reference has no counterpart for these: its sort and tree build are
 * hidden inside vkCmdBuildAccelerationStructuresKHR
 * (vulkan-raytraced-triangle/main.cpp:808).  They expose the stages of the
 * build so that each can be compared with the CPU restatement, the sort as a
 * stand-alone primitive (ray reordering uses it), the sort's bounded wait for
 * tests of its timeout, and the learned path tracer's intermediate arrays.
 */
#ifndef RTCORE_DEBUG_H
#define RTCORE_DEBUG_H

#include "rtcore.h"
#include "rtcore_pt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Scratch bytes rt_sort_pairs needs for n pairs sorted on key_bits bits. */
rt_status rt_get_sort_scratch_bytes(uint32_t n, uint32_t key_bits, uint64_t *out);

/* Stable LSD radix sort (onesweep) of n (uint64 key, uint32 value) device
 * pairs on the low key_bits bits, in place.  n < 2^30. */
rt_status rt_sort_pairs(rt_context *ctx, rt_stream stream, uint64_t *keys, uint32_t *vals, uint32_t n,
                        uint32_t key_bits, void *scratch, uint64_t scratch_bytes);

/* Byte offsets, within the scratch buffer of a finished BLAS build of n_tris
 * triangles, of the sorted Morton keys (uint64), the sorted build-input
 * triangle ids (uint32) and the binary radix-tree nodes (uint32 x4:
 * left, right, first, last; bit 31 marks a leaf reference; internal node i
 * is the one that splits between sorted keys i and i + 1). */
rt_status rt_debug_blas_scratch_layout(uint32_t n_tris, uint32_t flags, uint64_t *keys_off, uint64_t *ids_off,
                                       uint64_t *bin_off);

/* Sets how many times the onesweep look-back of this context's sorts (the
 * build's and rt_sort_pairs') polls a predecessor tile's status before it
 * gives up: the tile then records RT_ERR_TIMEOUT (reported by rt_sync),
 * publishes what it has and finishes, with every write still inside the
 * output.  0 restores the default (2^22 polls).  For tests of the timeout
 * path; a small limit makes the sort's output wrong. */
rt_status rt_debug_set_sort_spin_limit(rt_context *ctx, uint32_t spins);

/* When `withhold` is nonzero, the first tile of every onesweep pass of this
 * context's rt_sort_pairs calls (not its builds) publishes no status, so the tile after it waits on a
 * status that nothing sets until its poll limit runs out (RT_ERR_TIMEOUT):
 * a bounded wait made to expire on purpose, with every write still inside
 * the output.  0 restores normal sorts.  For tests of the timeout path; the
 * sort's output is wrong while it is set. */
rt_status rt_debug_set_sort_withhold(rt_context *ctx, int withhold);

/* Bandwidth probe: reads the device buffer [buf, buf + bytes) `passes` times
 * with 16-byte loads cached in L2 only; the caller times it (CUDA events on
 * `stream`).  A buffer well below the L2 size (129 MB on a GB300) measures L2
 * read bandwidth, the denominator of the traversal's L2 roofline.  bytes and
 * buf 16-byte aligned. */
rt_status rt_debug_read_sweep(rt_context *ctx, rt_stream stream, const void *buf, uint64_t bytes, uint32_t passes);

/* Whether rt_trace_closest_host / rt_trace_any_host would read and write the
 * host range [p, p + bytes) in place (*in_place = 1) or stage it through
 * copies (0): the range must be mapped from end to end, in memory the device
 * reaches at the same address.  Touches none of the range's bytes. */
rt_status rt_debug_host_in_place(rt_context *ctx, const void *p, uint64_t bytes, int *in_place);

/* Byte offsets, within the scratch of a finished rt_path_trace_cached call
 * with these parameters and light count, of the learned form's arrays of the
 * call's last wave: the numbers of cache queries and training samples
 * (uint32), then per query its rt_cache_input, the throughput at the second
 * vertex (float4), the path index within the wave (uint32: sample j of pixel
 * p is j * pixels + p) and the cache's answer (float4), and per training
 * sample its rt_cache_input, throughput (float4), radiance before the second
 * vertex (float4), path index (uint32) and target (float4). */
typedef struct rt_debug_pt_cache_offsets {
    uint64_t query_count, query_in, query_t1, query_path, query_out;
    uint64_t train_count, train_in, train_t1, train_before, train_path, train_target;
} rt_debug_pt_cache_offsets;

rt_status rt_debug_pt_cache_layout(const rt_pt_params *p, const rt_pt_cache_params *cp, uint32_t n_lights,
                                   rt_debug_pt_cache_offsets *out);

#ifdef __cplusplus
}
#endif
#endif
