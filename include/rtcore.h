/*
 * rtcore.h -- C ABI of the GB300 software ray-tracing core.
 *
 * The core is a headless drop-in for the ray-tracing sample of
 * Ray-Studio2/build-up-phase (vulkan-raytraced-triangle/main.cpp, identical to
 * vulkan-raytracing-basic/main.cpp).  That sample drives the Vulkan KHR
 * acceleration-structure and ray-tracing-pipeline entry points directly from
 * main(); every entry point below names the Vulkan call it replaces and the
 * sample line that calls it.
 *
 * Conventions
 *   - Every function returns rt_status: 0 on success, a negative RT_ERR_* code
 *     otherwise.  No C++ exception and no C++ type crosses this boundary.
 *   - Pointers documented as "device" are CUDA device pointers owned by the
 *     caller (the sample owns every VkBuffer the same way, main.cpp:534-575).
 *     The library owns only the rt_context and its small bookkeeping buffers.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  All work is
 *     stream-ordered and asynchronous; rt_sync() replaces vkQueueWaitIdle
 *     (main.cpp:820, 942, 998) and the per-frame fence (main.cpp:1333, 1411).
 *   - One host thread drives a context at a time.  Calls made on one context
 *     from several streams must not overlap in time on the device.
 */
#ifndef RTCORE_H
#define RTCORE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RTCORE_ABI_VERSION 1u

typedef int rt_status;
enum {
    RT_OK = 0,
    RT_ERR_INVALID_ARG = -1, /* bad pointer, size, flag or handle           */
    RT_ERR_OOM = -2,         /* a caller buffer is smaller than required     */
    RT_ERR_CUDA = -3,        /* a CUDA runtime call failed                   */
    RT_ERR_TIMEOUT = -4,     /* a bounded device-side wait ran out           */
    RT_ERR_BOUNDS = -5,      /* a device-side bounds check fired             */
    RT_ERR_UNSUPPORTED = -6, /* valid request the library does not implement */
    RT_ERR_NO_DEVICE = -7,   /* no CUDA device / kernel image for it         */
    RT_ERR_NOT_FOUND = -8    /* a lookup (tuning cache) found no entry       */
};

typedef struct rt_context rt_context;
typedef void *rt_stream; /* cudaStream_t */

/* ------------------------------------------------------------------------ */
/* Plain data types (bit layouts shared with the device)                    */
/* ------------------------------------------------------------------------ */

/* VkTransformMatrixKHR: 3x4 row-major affine transform (main.cpp:684-695). */
typedef struct rt_transform3x4 {
    float m[3][4];
} rt_transform3x4;

/* Index types (VkIndexType subset). */
enum { RT_INDEX_UINT32 = 1, RT_INDEX_NONE = 0 };

/* Geometry flags (VkGeometryFlagBitsKHR subset). */
enum { RT_GEOMETRY_OPAQUE = 1u };

/*
 * One triangle geometry of a bottom-level build: the data of
 * VkAccelerationStructureGeometryTrianglesDataKHR (main.cpp:726-742) plus the
 * primitive count of its VkAccelerationStructureBuildRangeInfoKHR
 * (main.cpp:795-804).  vertices/indices/transform are device pointers.
 * The transform, when given, is applied to the vertices at build time, as
 * Vulkan does with transformData.
 */
typedef struct rt_geometry_triangles {
    const void *vertices;            /* device, R32G32B32_SFLOAT           */
    uint64_t vertex_stride;          /* bytes between vertices (>= 12)     */
    uint32_t max_vertex;             /* highest vertex index referenced    */
    uint32_t index_type;             /* RT_INDEX_UINT32 or RT_INDEX_NONE   */
    const uint32_t *indices;         /* device, 3 per triangle (or NULL)   */
    uint32_t tri_count;              /* primitiveCount                     */
    uint32_t flags;                  /* RT_GEOMETRY_OPAQUE                 */
    const rt_transform3x4 *transform;/* device or NULL (identity)          */
} rt_geometry_triangles;

/*
 * Top-level instance: the exact 64-byte layout of
 * VkAccelerationStructureInstanceKHR (main.cpp:835-858).
 *   custom_index_and_mask: instanceCustomIndex in bits 0..23, mask in 24..31
 *   sbt_offset_and_flags : instanceShaderBindingTableRecordOffset in bits
 *                          0..23, VkGeometryInstanceFlagsKHR in 24..31
 *   accel_ref            : rt_accel_address() of a bottom-level build
 */
typedef struct rt_instance {
    rt_transform3x4 transform;
    uint32_t custom_index_and_mask;
    uint32_t sbt_offset_and_flags;
    uint64_t accel_ref;
} rt_instance;

/* Build flags (VkBuildAccelerationStructureFlagBitsKHR subset + ours). */
enum {
    RT_BUILD_PREFER_FAST_TRACE = 1u << 0, /* accepted; the only mode   */
    RT_BUILD_MORTON30 = 1u << 8,          /* 30-bit keys, 4 sort passes */
    RT_BUILD_MORTON63 = 1u << 9           /* 63-bit keys, 8 passes (default) */
};
/* Children per wide node: RT_BUILD_WIDTH(w), w in 4..8 (bits 16-19; 0 = 8).
 * The node format stays the 8-slot one; a narrower tree is deeper with fewer
 * child tests per node. */
#define RT_BUILD_WIDTH(w) ((uint32_t)(w) << 16)
#define RT_BUILD_WIDTH_MASK (0xfu << 16)

/* vkGetAccelerationStructureBuildSizesKHR output (main.cpp:756-762). */
typedef struct rt_build_sizes {
    uint64_t accel_bytes;
    uint64_t scratch_bytes;
} rt_build_sizes;

/* Camera uniform of the sample: struct Data {cameraPos[3]; yFov_degree}
 * (main.cpp:1003-1016, GLSL block main.cpp:1025-1029).  16 bytes. */
typedef struct rt_camera {
    float position[3];
    float y_fov_degree;
} rt_camera;

/* Ray flags (gl_RayFlags*EXT subset). */
enum {
    RT_RAY_FLAG_OPAQUE = 1u << 0,
    RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT = 1u << 2,
    RT_RAY_FLAG_SKIP_CLOSEST_HIT = 1u << 3
};

/* Closest-hit programs available to a pipeline. */
enum {
    /* The sample's closest-hit shader (main.cpp:1080-1091): barycentric
     * colour when PrimitiveID==1 && InstanceID==1 && CustomIndex==100 &&
     * GeometryIndex==1, else the colour of the hit group's SBT record. */
    RT_CHIT_SAMPLE = 0,
    RT_CHIT_BARYCENTRIC = 1, /* (1-u-v, u, v) for every hit            */
    RT_CHIT_SBT_COLOR = 2    /* always the SBT record colour           */
};

/*
 * A ray-tracing pipeline: the fixed programs of the sample
 * (createRayTracingPipeline, main.cpp:1093-1172) and the constant arguments
 * its raygen passes to traceRayEXT (main.cpp:1047-1052).
 */
typedef struct rt_pipeline {
    uint32_t chit;              /* RT_CHIT_*                             */
    uint32_t ray_flags;         /* gl_RayFlagsOpaqueEXT                  */
    uint32_t cull_mask;         /* 0xff                                  */
    uint32_t sbt_record_offset; /* 0                                     */
    uint32_t sbt_record_stride; /* 1                                     */
    uint32_t miss_index;        /* 0                                     */
    float tmin;                 /* 0.0                                   */
    float tmax;                 /* 100.0                                 */
    float miss_color[3];        /* (0, 0, 0.2) (main.cpp:1063-1066)      */
    uint32_t max_recursion;     /* 1 (main.cpp:1168)                     */
} rt_pipeline;

/*
 * Hit-group shader binding table: the HitgCustomData {float color[3]}
 * records that follow each 32-byte handle (main.cpp:1248-1250, 1306-1317).
 * The record used for a hit is
 *   instance.sbt_offset + geometry_index * sbt_record_stride + sbt_record_offset
 * (Vulkan indexing rule quoted at main.cpp:1260-1262).
 */
typedef struct rt_sbt {
    const float *hit_colors;  /* device, record i at hit_colors[i*stride]   */
    uint32_t hit_record_count;
    uint32_t hit_record_stride; /* in floats, >= 3                          */
} rt_sbt;

/* Ray for the lower-level batch API.  32 bytes. */
typedef struct rt_ray {
    float org[3];
    float tmin;
    float dir[3]; /* need not be normalised; t is in units of |dir| */
    float tmax;
} rt_ray;

/* Closest-hit record.  16 bytes.  prim is the triangle's index in the
 * bottom-level build input, counted across geometries in order; a miss has
 * prim == RT_NO_HIT and t == +inf.  u, v are the barycentrics of vertex 1 and
 * vertex 2 (hitAttributeEXT vec2 attribs, main.cpp:1078). */
typedef struct rt_hit {
    float t;
    uint32_t prim;
    float u;
    float v;
} rt_hit;
#define RT_NO_HIT 0xffffffffu

/* Full hit record (ids the sample's closest-hit shader reads). 32 bytes. */
typedef struct rt_hit_ext {
    float t;
    float u;
    float v;
    uint32_t instance_id;     /* gl_InstanceID                 */
    uint32_t custom_index;    /* gl_InstanceCustomIndexEXT     */
    uint32_t geometry_index;  /* gl_GeometryIndexEXT           */
    uint32_t primitive_id;    /* gl_PrimitiveID                */
    uint32_t sbt_record;      /* hit-group record selected     */
} rt_hit_ext;

/* ------------------------------------------------------------------------ */
/* Context                                                                  */
/* ------------------------------------------------------------------------ */

/* Replaces createVkInstance/createVkDevice (main.cpp:242-388). */
rt_status rt_context_create(int device, rt_context **out);
rt_status rt_context_destroy(rt_context *ctx);
/* Text of the last error reported on this context ("" if none). */
const char *rt_last_error_string(rt_context *ctx);
/* Waits for `stream` and returns the first device-side error (timeout,
 * bounds) recorded by this context's kernels since the previous rt_sync.
 * Replaces vkQueueWaitIdle (main.cpp:820, 942, 998). */
rt_status rt_sync(rt_context *ctx, rt_stream stream);
/* ABI version of the loaded library (RTCORE_ABI_VERSION). */
uint32_t rt_abi_version(void);

/* ------------------------------------------------------------------------ */
/* Acceleration structures                                                  */
/* ------------------------------------------------------------------------ */

/* vkGetAccelerationStructureBuildSizesKHR for a bottom-level build
 * (main.cpp:756-762): tri_counts[i] is the maximum primitive count of
 * geometry i. */
rt_status rt_get_blas_build_sizes(rt_context *ctx, const uint32_t *tri_counts,
                                  uint32_t n_geoms, uint32_t flags,
                                  rt_build_sizes *out);
/* Same for a top-level build over n_instances (main.cpp:892-897). */
rt_status rt_get_tlas_build_sizes(rt_context *ctx, uint32_t n_instances,
                                  uint32_t flags, rt_build_sizes *out);

/*
 * vkCmdBuildAccelerationStructuresKHR for one bottom-level structure
 * (main.cpp:788-811).  `geoms` is a host array of n_geoms descriptors whose
 * pointers are device pointers.  `accel` and `scratch` are device buffers of
 * at least the sizes rt_get_blas_build_sizes returned; `accel` must be
 * 256-byte aligned.  Asynchronous on `stream`; the structure is usable by any
 * later work on the same stream.
 */
rt_status rt_build_blas(rt_context *ctx, rt_stream stream,
                        const rt_geometry_triangles *geoms, uint32_t n_geoms,
                        uint32_t flags, void *accel, uint64_t accel_bytes,
                        void *scratch, uint64_t scratch_bytes);

/*
 * rt_build_blas without a scratch buffer, for callers that cannot allocate
 * device memory: for instance a plugin that is handed its input and output
 * buffers by an engine that owns all device memory, or a frame loop that must
 * not call cudaMalloc/cudaFree because they can synchronise the device and
 * stall other streams.  This call itself allocates nothing.  It has no
 * counterpart in the reference (whose Vulkan sample allocates its scratch
 * buffer with vkAllocateMemory).
 *
 * The scratch is one fixed 40 MiB array compiled into the library, held in
 * device memory of every GPU that loads the library until the process
 * exits; it limits a build to RT_STATIC_SCRATCH_MAX_TRIS triangles (larger
 * inputs return RT_ERR_UNSUPPORTED -- use rt_build_blas).  The first call on
 * each device looks up the array's device address, so make that first call
 * before any stream capture.  Every call shares the array: calls whose work
 * overlaps on the GPU race and give undefined results; order them on one
 * stream (or with events).  Output is byte-identical to rt_build_blas.
 */
#define RT_STATIC_SCRATCH_MAX_TRIS 131072u
rt_status rt_build_blas_static_scratch(rt_context *ctx, rt_stream stream,
                                       const rt_geometry_triangles *geoms,
                                       uint32_t n_geoms, uint32_t flags,
                                       void *accel, uint64_t accel_bytes);

/*
 * vkCmdBuildAccelerationStructuresKHR for one top-level structure
 * (main.cpp:920-940).  `instances` is a device array of n rt_instance whose
 * accel_ref fields point at completed bottom-level builds.
 */
rt_status rt_build_tlas(rt_context *ctx, rt_stream stream,
                        const rt_instance *instances, uint32_t n,
                        uint32_t flags, void *accel, uint64_t accel_bytes,
                        void *scratch, uint64_t scratch_bytes);

/*
 * Refit: the update mode of a build (VK_BUILD_ACCELERATION_STRUCTURE_MODE_UPDATE_KHR;
 * the sample builds once, main.cpp:808, :932).  Takes the inputs of the build
 * that made `accel` with new vertex positions or geometry transforms (BLAS:
 * same geometry and triangle counts) or new instance transforms and
 * references (TLAS: same instance count), recomputes every leaf record and
 * box and keeps the tree.  For animation whose motion keeps the tree
 * reasonable; rebuild when it degrades.  A BLAS refit moves its bounds, so the
 * TLASes that reference it need a refit or a rebuild after it.  A structure
 * that does not match the inputs is left unchanged and RT_ERR_INVALID_ARG
 * surfaces at rt_sync.  scratch: rt_get_refit_scratch_bytes(primitives),
 * about 72 bytes per primitive.
 */
rt_status rt_get_refit_scratch_bytes(uint32_t prim_count, uint64_t *bytes);
rt_status rt_refit_blas(rt_context *ctx, rt_stream stream, const rt_geometry_triangles *geoms, uint32_t n_geoms,
                        void *accel, uint64_t accel_bytes, void *scratch, uint64_t scratch_bytes);
rt_status rt_refit_tlas(rt_context *ctx, rt_stream stream, const rt_instance *instances, uint32_t n,
                        void *accel, uint64_t accel_bytes, void *scratch, uint64_t scratch_bytes);

/* vkGetAccelerationStructureDeviceAddressKHR (main.cpp:665-672): the handle
 * by which instances and trace calls name a built structure. */
uint64_t rt_accel_address(const void *accel);

/* Reads the header of a built structure (synchronises `stream`): node count
 * and the build's device-side status. */
rt_status rt_accel_info(rt_context *ctx, rt_stream stream, const void *accel,
                        uint32_t *node_count, uint32_t *prim_count,
                        uint32_t *tree_depth);

/* ------------------------------------------------------------------------ */
/* Ray tracing                                                              */
/* ------------------------------------------------------------------------ */

/*
 * vkCmdTraceRaysKHR(rgen, miss, hit, call, width, height, depth)
 * (main.cpp:1349-1355) with the sample's raygen (main.cpp:1033-1055): one
 * pinhole ray per pixel through its centre, closest-hit or miss program,
 * imageStore of vec4(hitValue, 0.0).  `out_rgba32f` is a device buffer of
 * width*height*4 floats, row-major, pixel (x, y) at index y*width + x.
 * `accel` is an rt_accel_address (top- or bottom-level).  depth must be 1.
 */
rt_status rt_trace_rays(rt_context *ctx, rt_stream stream,
                        const rt_pipeline *pipeline, const rt_sbt *sbt,
                        uint64_t accel, const rt_camera *camera,
                        float *out_rgba32f, uint32_t width, uint32_t height,
                        uint32_t depth);

/* Closest-hit query for n rays (device arrays).  `accel` may be top- or
 * bottom-level.  `hits_ext` (nullable) receives the full id record. */
rt_status rt_trace_closest(rt_context *ctx, rt_stream stream, uint64_t accel,
                           const rt_ray *rays, rt_hit *hits,
                           rt_hit_ext *hits_ext, uint32_t n);

/* Any-hit (occlusion) query: occluded[i] = 1 if some triangle is hit with
 * t in [tmin, tmax], else 0.  Terminates each ray on its first hit. */
rt_status rt_trace_any(rt_context *ctx, rt_stream stream, uint64_t accel,
                       const rt_ray *rays, uint8_t *occluded, uint32_t n);

/*
 * The same traversals with the rays and results in HOST memory (pinned for
 * the copies to overlap): the rays go to the device and the results come
 * back.  When both buffers are 16-byte aligned and the device reaches them
 * at the same address -- pinned or registered host memory under unified
 * addressing (cudaHostAlloc / cudaHostRegister), or any host memory on a
 * device that accesses pageable memory through the host page tables (a
 * Grace-Blackwell system, over NVLink-C2C) -- one traversal launch reads the
 * rays and writes the results in place and `scratch` is not touched.
 * Otherwise the rays go in and
 * the results come back in chunks (2^18 rays first, then doubling up to 2^20
 * or what a slot holds) through a ring of four slots in
 * `scratch` (rt_trace_host_scratch_bytes(n): enough for chunks of n rays; a
 * smaller scratch means smaller chunks), the copies of neighbouring chunks
 * running on the context's two copy streams and the chunks traced on three
 * trace streams of the context, so consecutive traversals overlap too.  The
 * call's work starts after what `stream` holds when it is made.  Calls that
 * share a scratch buffer (closest and any hit alike) overlap each other's
 * copies.  Asynchronous: the results are in host memory when `stream` reaches
 * the end of the call.  The
 * form a caller holding rays in host memory (the sample's CPU-side data, a
 * plugin) uses in place of traceRayEXT batches (main.cpp:1047-1052).
 */
rt_status rt_trace_host_scratch_bytes(uint32_t n, int any_hit, uint64_t *bytes);
/* How the host-memory calls move rays and results: RT_HOST_TRANSFER_AUTO
 * (default) reads and writes the buffers in place where the device reaches
 * them and stages the others through the scratch ring;
 * RT_HOST_TRANSFER_STAGED always stages. */
enum { RT_HOST_TRANSFER_AUTO = 0, RT_HOST_TRANSFER_STAGED = 1 };
rt_status rt_set_host_transfer(rt_context *ctx, uint32_t mode);
rt_status rt_trace_closest_host(rt_context *ctx, rt_stream stream, uint64_t accel, const rt_ray *rays,
                                rt_hit *hits, uint32_t n, void *scratch, uint64_t scratch_bytes);
rt_status rt_trace_any_host(rt_context *ctx, rt_stream stream, uint64_t accel, const rt_ray *rays,
                            uint8_t *occluded, uint32_t n, void *scratch, uint64_t scratch_bytes);

/* Pinhole primary rays of the sample's raygen (main.cpp:1036-1052) for a
 * width x height launch, written to a device array (row-major), tmin/tmax as
 * given.  Used to feed the batch API with the sample's camera model. */
rt_status rt_generate_primary_rays(rt_context *ctx, rt_stream stream,
                                   const rt_camera *camera, uint32_t width,
                                   uint32_t height, float tmin, float tmax,
                                   rt_ray *rays);

/* Traversal statistics over n rays: sums of BVH8 nodes visited and
 * triangles tested (uint64 each, device pointer to 2 values), for the
 * algorithmic-bytes roofline.  Runs an instrumented copy of the closest-hit
 * kernel; not for timing. */
rt_status rt_trace_stats(rt_context *ctx, rt_stream stream, uint64_t accel,
                         const rt_ray *rays, uint32_t n, int any_hit,
                         unsigned long long *counters);

/* ------------------------------------------------------------------------ */
/* Tuning                                                                    */
/* ------------------------------------------------------------------------ */

/* Launch shape of the traversal kernel.  blocks_per_sm applies to every
 * single-structure traversal (ray-query calls and rt_path_trace; any-hit
 * launches use at most 8); batch_rays to the ray-query calls only -- the path
 * tracer's queue traversals refill at 8 idle lanes, the batch uses its own
 * autotuned shape.  Defaults: 128, 9, 4. */
typedef struct rt_trace_tuning {
    uint32_t block_threads;   /* threads per block of the traversal kernel */
    uint32_t blocks_per_sm;   /* persistent blocks per SM                  */
    uint32_t batch_rays;      /* a warp refills its idle lanes (one atomic
                                 fetch) once at least this many are idle    */
    uint32_t reserved;
} rt_trace_tuning;
rt_status rt_set_trace_tuning(rt_context *ctx, const rt_trace_tuning *t);
rt_status rt_get_trace_tuning(rt_context *ctx, rt_trace_tuning *t);

/* ------------------------------------------------------------------------ */
/* Host helpers                                                             */
/* ------------------------------------------------------------------------ */

/* Writes an 8-bit binary PPM (P6) of a host RGBA32F image; each channel is
 * clamped to [0,1] and rounded to nearest as an R8G8B8A8_UNORM store does
 * (main.cpp:953).  Alpha is dropped. */
rt_status rt_write_ppm(const float *host_rgba32f, uint32_t width,
                       uint32_t height, const char *path);

/* Writes a little-endian PFM ("PF") of the RGB channels, bottom row first,
 * for lossless FP32 comparisons. */
rt_status rt_write_pfm(const float *host_rgba32f, uint32_t width,
                       uint32_t height, const char *path);

#ifdef __cplusplus
}
#endif
#endif /* RTCORE_H */
