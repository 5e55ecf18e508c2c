/*
 * rtcore_debug.h -- utility and inspection entry points of librtcore.
 *
 * The reference has no counterpart for these: its sort and tree build are
 * hidden inside vkCmdBuildAccelerationStructuresKHR
 * (vulkan-raytraced-triangle/main.cpp:808).  They expose the stages of the
 * build so that each can be compared with the CPU restatement, and the sort
 * as a stand-alone primitive (ray reordering uses it).
 */
#ifndef RTCORE_DEBUG_H
#define RTCORE_DEBUG_H

#include "rtcore.h"

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
 * left, right, first, last; bit 31 marks a leaf reference). */
rt_status rt_debug_blas_scratch_layout(uint32_t n_tris, uint32_t flags, uint64_t *keys_off, uint64_t *ids_off,
                                       uint64_t *bin_off);

#ifdef __cplusplus
}
#endif
#endif
