/*
 * rtcore_accel.h -- byte layout of a built acceleration structure.
 *
 * Vulkan keeps this layout opaque inside the driver
 * (vkCmdBuildAccelerationStructuresKHR, vulkan-raytraced-triangle/main.cpp:808
 * and :932).  It is spelled out here because the build is bit-exact against
 * the CPU oracle, which writes the same bytes, and because tests compare the
 * two buffers directly.  Callers only need rt_build_sizes and the handle.
 *
 *   [0, 256)                      rt_accel_header
 *   [node_offset, +80*capacity)   rt_bvh8_node[], node 0 is the root
 *   [prim_offset, ...)            leaf records in node (breadth-first) order:
 *                                 BLAS: rt_tri_record   (48 B) per triangle
 *                                 TLAS: rt_inst_record  (80 B) per instance
 *   [geom_offset, ...)            BLAS only: uint32 first-triangle index of
 *                                 each geometry, n_geoms + 1 entries
 *
 * Wide node = compressed 8-wide BVH node with 8-bit quantised child boxes
 * relative to a per-node origin and per-axis power-of-two scale
 * (Ylitie, Karras, Laine: "Efficient Incoherent Ray Traversal on GPUs Through
 * Compressed Wide BVHs", HPG 2017).  Field order is this project's own.
 */
#ifndef RTCORE_ACCEL_H
#define RTCORE_ACCEL_H

#include <stdint.h>

#define RT_ACCEL_MAGIC 0x53415452u /* "RTAS" little-endian */
#define RT_ACCEL_VERSION 1u
#define RT_ACCEL_KIND_BLAS 1u
#define RT_ACCEL_KIND_TLAS 2u
#define RT_ACCEL_HEADER_BYTES 256u
#define RT_BVH_WIDTH 8
#define RT_MAX_LEAF_PRIMS 3 /* unary count in meta bits 5..7 */

/* Surface-area-heuristic constants of the binary-tree leaf decision.
 * cost(leaf of c prims) = c * RT_SAH_PRIM; cost(split) = RT_SAH_NODE +
 * (A(l) cost(l) + A(r) cost(r)) / A(n), A = half surface area. */
#define RT_SAH_PRIM 1.0f
#define RT_SAH_NODE 0.3f

/* A primitive whose box is longer, on its longest axis, than this fraction of
 * the longest axis of the centroid bounds is "large": its sort key gets the
 * bit above the Morton code (bit 63 of the 63-bit keys, bit 31 of the 30-bit
 * ones), so the radix tree's root separates the large primitives from the
 * rest and the small primitives' node boxes are not stretched by them (the
 * walls of a room around small objects).  0.25 is exact in binary. */
#define RT_LARGE_PRIM_FRACTION 0.25f

/* Smallest / largest per-axis exponent of a node's quantisation grid. */
#define RT_QEXP_MIN (-100)
#define RT_QEXP_MAX (100)

/* Zero ray-direction components are replaced by +-2^-80 before the
 * reciprocal of the box test (the triangle test uses the raw direction). */
#define RT_DIR_EPS 8.2718061255302767e-25f /* 2^-80 */

typedef struct rt_accel_header {
    uint32_t magic;         /* RT_ACCEL_MAGIC                           */
    uint32_t version;       /* RT_ACCEL_VERSION                         */
    uint32_t kind;          /* RT_ACCEL_KIND_*                          */
    uint32_t prim_count;    /* triangles or instances                   */
    uint32_t node_count;    /* wide nodes written (device-written)      */
    uint32_t geom_count;    /* BLAS geometries                          */
    uint32_t build_flags;
    uint32_t status;        /* 0, or an RT_ERR_* code (device-written)  */
    uint32_t depth;         /* wide-tree levels (device-written)        */
    uint32_t morton_bits;   /* 30 or 63                                 */
    uint32_t node_capacity; /* wide nodes the buffer holds              */
    uint32_t reserved0;
    float bounds_lo[4];     /* root box (device-written), w unused      */
    float bounds_hi[4];
    uint64_t node_offset;   /* bytes from the header to node 0          */
    uint64_t prim_offset;   /* bytes from the header to leaf record 0   */
    uint64_t geom_offset;   /* bytes from the header to geometry table  */
    uint64_t total_bytes;   /* size the buffer was laid out for         */
    uint8_t reserved[256 - 112];
} rt_accel_header;

/*
 * 80-byte wide node (five 16-byte words):
 *   w0: origin.x origin.y origin.z | exp_x exp_y exp_z imask
 *   w1: child_base | prim_base | meta[0..3] | meta[4..7]
 *   w2: qlo_x[8] qlo_y[8]
 *   w3: qlo_z[8] qhi_x[8]
 *   w4: qhi_y[8] qhi_z[8]
 * Slot s is
 *   empty    : meta[s] == 0 and its box is inverted (qlo = 255, qhi = 0),
 *   internal : bit s of imask; node index = child_base + popcount(imask &
 *              ((1 << s) - 1)),
 *   leaf     : meta[s] = (unary count << 5) | offset, the leaf's records are
 *              prim_base + offset ... + count - 1 (count 1..3 -> 1, 3, 7).
 * Child box along axis a: [origin_a + qlo_a * 2^exp_a, origin_a + qhi_a *
 * 2^exp_a], conservative in exact arithmetic.
 * Slot choice: the child in slot s is the one nearest the node's far side
 * for rays whose direction-sign octant is s (bit0: x<0, bit1: y<0, bit2:
 * z<0); traversal visits internal children in order of (slot ^ octant).
 */
typedef struct rt_bvh8_node {
    float origin[3];
    int8_t exp[3];
    uint8_t imask;
    uint32_t child_base;
    uint32_t prim_base;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
} rt_bvh8_node;

/* Triangle leaf record, 48 bytes: vertices after the geometry transform.
 *   v0.w = bits of the build-input triangle index (across geometries)
 *   v1.w = bits of the geometry index
 *   v2.w = bits of the primitive index within the geometry */
typedef struct rt_tri_record {
    float v0[4];
    float v1[4];
    float v2[4];
} rt_tri_record;

/* Instance leaf record, 80 bytes.
 *   world_to_object: inverse of the instance transform, 3x4 row-major
 *   accel_ref: bottom-level address, custom_index_and_mask and
 *   sbt_offset_and_flags copied from rt_instance, instance_id = its index. */
typedef struct rt_inst_record {
    float world_to_object[3][4];
    uint64_t accel_ref;
    uint32_t custom_index_and_mask;
    uint32_t sbt_offset_and_flags;
    uint32_t instance_id;
    uint32_t reserved[3];
} rt_inst_record;

#ifdef __cplusplus
static_assert(sizeof(rt_accel_header) == 256, "header size");
static_assert(sizeof(rt_bvh8_node) == 80, "node size");
static_assert(sizeof(rt_tri_record) == 48, "tri size");
static_assert(sizeof(rt_inst_record) == 80, "instance size");
#endif

#endif /* RTCORE_ACCEL_H */
