// rt_traverse.cuh -- the persistent BVH8 traversal kernel.
//
// Replaces the RT-core traversal behind traceRayEXT of the reference sample
// (vulkan-raytraced-triangle/main.cpp:1047-1052).  Included by rt_trace.cu
// (one structure per launch: the ray-query API and the path tracer) and by
// rt_trace_multi.cu (many scenes per launch: the batched path tracer, where
// each ray carries the index of its scene).
//
// Persistent warps walk a ray array.  A warp refills its idle lanes from a
// global counter (atomic work stealing) whenever at least `refill` of them
// have finished; each lane walks the compressed BVH8 with 16-byte node loads
// and keeps its traversal stack in a shared-memory ring of RING entries whose
// bottom spills to local memory.
//
// Visiting order (identical in the CPU restatement, so hits and statistics
// agree exactly): a node's leaf records first, in ascending record order,
// then its internal children in ascending (slot ^ ray octant); remaining
// siblings are pushed as one group.  Closest hit = smallest t, ties broken by
// the smallest triangle index.
#pragma once

#include <cuda_runtime.h>

#include "../../include/rtcore.h"
#include "../../include/rtcore_accel.h"
#include "rt_device.cuh"

namespace rtc {
namespace {

constexpr int kTraceThreads = 128;  // block size of the single-structure kernels
// Shared-memory stack entries per ray of the single-structure kernels: 8 KB
// per block, so nine blocks leave more of the SM's L1 to node fetches than
// 16 entries did (1M soup: 2,150 -> 2,159 M rays/s; path tracer 6.33 -> 6.29
// ms per sample); deeper entries spill to local memory.
constexpr int kRing = 8;
constexpr uint32_t kAnyBlocksPerSm = 1024u / kTraceThreads;  // resident blocks the any-hit kernel is bounded for
constexpr int kMaxDepth = 64;       // total stack entries per ray
constexpr uint32_t kNone = 0xffffffffu;

struct Hit {
    float t, u, v;
    uint32_t rec;     // leaf-record index of the best triangle
    uint32_t tri;     // build-input triangle index
    uint32_t inst;    // instance index (0 for a bare BLAS)
    bool found;
};

__device__ __forceinline__ uint4 ldg4(const uint4 *p) { return __ldg(p); }

// Traversal view of one bottom-level structure (32 bytes), written on the
// device from the structure's header.  node_count 0 marks a structure whose
// rays all miss (empty, or not a bottom-level structure).
struct TravScene {
    const uint4 *nodes;
    const uint4 *prims;
    uint32_t node_count;
    uint32_t prim_count;
    uint32_t pad[2];
};
static_assert(sizeof(TravScene) == 32, "TravScene is read as two 16-byte words");

struct BatchArgs {
    const uint8_t *accel;       // the structure (single-structure kernels)
    const TravScene *scenes;    // per-scene views (multi-scene kernels)
    const uint32_t *ray_scene;  // scene index of each ray (multi-scene kernels)
    uint32_t n_scenes;
    const float4 *rays;      // 2 float4 per ray
    float4 *hits;            // closest: 1 float4 per ray (t, prim bits, u, v)
    rt_hit_ext *hits_ext;    // nullable
    uint8_t *occluded;       // any-hit output
    uint32_t n;
    uint32_t refill;         // refill when at least this many lanes are idle
    uint32_t *counter;
    uint32_t *err;
    unsigned long long *stats;
    const uint32_t *n_dev;   // when set: the ray count, read on the device
    uint32_t out_rec;        // closest hit: write the leaf-record index
    // mixed launches: a second queue of any-hit rays after the closest-hit
    // queue above (rays2[i] is ray n1 + i of the launch; results to occluded)
    const float4 *rays2;
    const uint32_t *ray_scene2;
    const uint32_t *n_dev2;
    uint32_t n2;
};

// MIXED: one launch over two queues -- the closest-hit rays (rays, n_dev;
// results to hits) and then the any-hit rays (rays2, n_dev2; results to
// occluded) -- each ray walked exactly as in a launch of its own kind; the
// path tracer traces a depth's shadow rays and the next depth's extension
// rays together, so the two share one launch tail.
// Register budget: the closest-hit and mixed single-structure kernels fit
// nine 128-thread blocks per SM (56 registers; 36 warps against 32 at 64
// registers: 2,093 -> 2,111 M rays/s on the 1M soup, 6.72 -> 6.58 ms per
// path-traced sample).  The any-hit and multi-scene kernels keep eight
// blocks and 64 registers: any-hit shadow rays run 1,287 M rays/s there
// against 1,202 at nine blocks, and the multi-scene kernels spill at 56.
// The box test pairs the z planes too (isect_node<true>) where it pays: in
// the 64-register kernels, and in the mixed kernel despite 20 bytes of spill
// (path tracer 6.30 -> 6.23 ms per sample; the closest-hit kernel loses 2 %
// with it).
template <bool ANY, bool STATS, bool MULTI, int THREADS, int RING, bool MIXED = false>
__global__ void __launch_bounds__(THREADS, ((MULTI || ANY) ? 1024 : 1152) / THREADS) k_trace_blas(const BatchArgs a) {
    static_assert((RING & (RING - 1)) == 0 && RING <= kMaxDepth, "RING is a power of two");
    __shared__ uint2 s_stack[RING][THREADS];
    const uint4 *nodes = nullptr, *prims = nullptr;
    // A tree walk visits each node at most once: more visits, or a node index
    // past the end, can only come from a corrupt structure.
    uint32_t max_visits = 0;
    bool empty = true;
    if (!MULTI) {
        const rt_accel_header *hd = reinterpret_cast<const rt_accel_header *>(a.accel);
        if (hd->kind != RT_ACCEL_KIND_BLAS) return;  // k_trace_inst handles it
        nodes = reinterpret_cast<const uint4 *>(a.accel + hd->node_offset);
        prims = reinterpret_cast<const uint4 *>(a.accel + hd->prim_offset);
        empty = hd->prim_count == 0;
        max_visits = hd->node_count;
    }
    const int tid = threadIdx.x, lane = tid & 31;

    bool active = false, exhausted = false;
    uint32_t ray_idx = 0;
    Ray r;
    float tmin = 0.f;
    Hit h;
    h.t = 0.f; h.u = 0.f; h.v = 0.f; h.rec = kNone; h.tri = kNone; h.inst = 0; h.found = false;
    uint32_t node = 0;
    bool pending = false;
    uint2 g = make_uint2(0u, 0u);
    int sp = 0, lo = 0;
    uint2 spill[kMaxDepth];
    unsigned long long n_nodes = 0, n_tris = 0;
    uint32_t visits = 0;
    const uint32_t n1 = a.n_dev ? min(*a.n_dev, a.n) : a.n;
    const uint32_t n_rays = MIXED ? n1 + min(*a.n_dev2, a.n2) : n1;
    bool any_ray = ANY;  // this lane's ray is an any-hit ray

    for (;;) {
        // ---- refill idle lanes from the global counter
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        if (!exhausted && __popc(idle) >= (int)a.refill) {
            const uint32_t cnt = __popc(idle);
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(a.counter, cnt);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + cnt >= n_rays) exhausted = true;
            if (!active) {
                uint32_t idx = base + __popc(idle & ((1u << lane) - 1u));
                if (idx < n_rays) {
                    const float4 *ray_src = a.rays;
                    const uint32_t *scene_src = a.ray_scene;
                    if (MIXED) {
                        any_ray = idx >= n1;
                        if (any_ray) {
                            idx -= n1;
                            ray_src = a.rays2;
                            scene_src = a.ray_scene2;
                        }
                    }
                    if (MULTI) {
                        const uint32_t s = __ldg(scene_src + idx);
                        if (s < a.n_scenes) {
                            const uint4 *tv = reinterpret_cast<const uint4 *>(a.scenes + s);
                            const uint4 t0 = ldg4(tv), t1 = ldg4(tv + 1);
                            nodes = reinterpret_cast<const uint4 *>(((uint64_t)t0.y << 32) | t0.x);
                            prims = reinterpret_cast<const uint4 *>(((uint64_t)t0.w << 32) | t0.z);
                            max_visits = t1.x;
                            empty = t1.x == 0u || t1.y == 0u;
                        } else {
                            report_error(a.err, RT_ERR_BOUNDS, 0x77000000u | (s & 0xffffffu));
                            empty = true;
                        }
                    }
                    const float4 r0 = __ldg(ray_src + 2u * idx), r1 = __ldg(ray_src + 2u * idx + 1u);
                    const float o[3] = {r0.x, r0.y, r0.z}, d[3] = {r1.x, r1.y, r1.z};
                    ray_setup(r, o, d);
                    tmin = r0.w;
                    h.t = r1.w; h.u = 0.f; h.v = 0.f; h.rec = kNone; h.tri = kNone; h.found = false;
                    ray_idx = idx;
                    active = true;
                    node = 0;          // start at the root
                    visits = 0;
                    pending = !empty;  // an empty structure resolves as a miss
                    g = make_uint2(0u, 0u);
                    sp = 0;
                    lo = 0;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (exhausted) break;
            continue;
        }
        // ---- traversal steps until too many lanes are idle
        for (;;) {
            if (active) {
                bool finish = false;
                if (pending && (visits >= max_visits || node >= max_visits)) {
                    report_error(a.err, RT_ERR_BOUNDS, 0x76000000u | ray_idx);
                    pending = false;
                    finish = true;
                }
                if (pending) {
                    pending = false;
                    ++visits;
                    NodeWords nd = load_node(nodes, node);
                    uint32_t nh, ph;
                    isect_node<ANY || MULTI || MIXED>(r, nd, tmin, h.t, nh, ph);
                    if (STATS) n_nodes++;
                    const uint32_t pbase = nd.w1.y;
                    while (ph) {
                        const uint32_t i = __ffs(ph) - 1;
                        ph &= ph - 1u;
                        const uint4 *rec = prims + (size_t)(pbase + i) * 3u;
                        const uint4 q0 = ldg4(rec), q1 = ldg4(rec + 1), q2 = ldg4(rec + 2);
                        if (STATS) n_tris++;
                        float t, u, v;
                        if (!isect_tri(r,
                                       make_float4(__uint_as_float(q0.x), __uint_as_float(q0.y),
                                                   __uint_as_float(q0.z), 0.f),
                                       make_float4(__uint_as_float(q1.x), __uint_as_float(q1.y),
                                                   __uint_as_float(q1.z), 0.f),
                                       make_float4(__uint_as_float(q2.x), __uint_as_float(q2.y),
                                                   __uint_as_float(q2.z), 0.f),
                                       tmin, h.t, t, u, v))
                            continue;
                        if (ANY || (MIXED && any_ray)) {
                            h.t = t; h.found = true;
                            finish = true;
                            break;
                        }
                        if (t < h.t || (t == h.t && q0.w < h.tri)) {
                            h.t = t; h.u = u; h.v = v; h.rec = pbase + i; h.tri = q0.w; h.found = true;
                        }
                    }
                    g = make_uint2(nd.w1.x, nh | ((nd.w0.w >> 24) << 8));
                }
                // ---- next node: from the current group, else pop
                while (!finish) {
                    if (g.y & 0xffu) {
                        const uint32_t k = __ffs(g.y & 0xffu) - 1;
                        g.y &= ~(1u << k);
                        const uint32_t s = k ^ r.oct;
                        node = g.x + __popc((g.y >> 8) & ((1u << s) - 1u));
                        pending = true;
                        if (g.y & 0xffu) {
                            if (sp >= kMaxDepth) {
                                report_error(a.err, RT_ERR_BOUNDS, 0x72000000u | ray_idx);
                                finish = true;
                                break;
                            }
                            if (sp - lo == RING) {
                                spill[lo] = s_stack[lo & (RING - 1)][tid];
                                ++lo;
                            }
                            s_stack[sp & (RING - 1)][tid] = g;
                            ++sp;
                        }
                        break;
                    }
                    if (sp == 0) { finish = true; break; }
                    --sp;
                    if (sp >= lo) {
                        g = s_stack[sp & (RING - 1)][tid];
                    } else {
                        g = spill[sp];
                        lo = sp;
                    }
                }
                if (finish) {
                    // ---- write the result
                    if (ANY || (MIXED && any_ray)) {
                        if (a.occluded) a.occluded[ray_idx] = h.found ? 1u : 0u;
                    } else {
                        float4 out;
                        if (h.found) out = make_float4(h.t, __uint_as_float(a.out_rec ? h.rec : h.tri), h.u, h.v);
                        else out = make_float4(kInf, __uint_as_float(kNone), 0.f, 0.f);
                        if (a.hits) a.hits[ray_idx] = out;
                        if (!MULTI && a.hits_ext) {
                            rt_hit_ext x;
                            x.t = out.x; x.u = out.z; x.v = out.w;
                            x.instance_id = h.found ? 0u : kNone;
                            x.custom_index = 0;
                            x.geometry_index = h.found ? ldg4(prims + (size_t)h.rec * 3u + 1).w : 0u;
                            x.primitive_id = h.found ? ldg4(prims + (size_t)h.rec * 3u + 2).w : kNone;
                            x.sbt_record = x.geometry_index;
                            a.hits_ext[ray_idx] = x;
                        }
                    }
                    active = false;
                    pending = false;
                }
            }
            const uint32_t act = __ballot_sync(0xffffffffu, active);
            if (act == 0u) break;
            if (!exhausted && (uint32_t)__popc(~act) >= a.refill) break;
        }
    }
    if (STATS) {
        for (int o = 16; o > 0; o >>= 1) {
            n_nodes += __shfl_xor_sync(0xffffffffu, n_nodes, o);
            n_tris += __shfl_xor_sync(0xffffffffu, n_tris, o);
        }
        if (lane == 0) {
            atomicAdd(a.stats, n_nodes);
            atomicAdd(a.stats + 1, n_tris);
        }
    }
}

}  // namespace
}  // namespace rtc
