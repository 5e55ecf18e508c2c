// rt_trace.cu -- BVH8 traversal kernels and the ray-tracing pipeline.
//
// Replaces traceRayEXT / vkCmdTraceRaysKHR of the reference sample
// (vulkan-raytraced-triangle/main.cpp:1047-1052 and :1349-1355), which run on
// RT cores inside the driver.  The GB300 has no RT cores, so traversal runs
// on the SMs:
//
//   k_trace_blas (rt_traverse.cuh)  persistent warps over a ray array
//                   with atomic work stealing and a shared-memory stack ring.
//   k_trace_inst    two-level structures (instances): persistent warps as
//                   above, a lane walking an instance's BLAS with its
//                   object-space ray between TLAS steps.
//                   Both kernels are launched; each returns at once when the
//                   structure in the header is not its kind.
//   k_pipeline      the sample's raygen + traceRayEXT + closest-hit / miss +
//                   imageStore, one thread per launch id.
//
// Visiting order (identical in the CPU restatement, so hits and statistics
// agree exactly): a node's leaf records first, in ascending record order,
// then its internal children in ascending (slot ^ ray octant); remaining
// siblings are pushed as one group.  Closest hit = smallest t, ties broken by
// the smallest (instance, triangle) key.
#include <cmath>
#include <cuda.h>
#include <cuda_runtime.h>
#include <sys/mman.h>
#include <unistd.h>

#include "rt_internal.h"
#include "../../include/rtcore_debug.h"
#include "rt_traverse.cuh"

namespace rtc {

namespace {

__device__ __forceinline__ bool key_less(float t, uint64_t key, float bt, uint64_t bkey) {
    return t < bt || (t == bt && key < bkey);
}

// ---------------------------------------------------------------------------
// Simple per-thread traversal (local-memory stack) for the sample pipeline
// (k_pipeline): one thread per pixel, both structure kinds.  Same visiting
// order as the persistent kernels.
// ---------------------------------------------------------------------------

struct LocalStack {
    uint2 e[kMaxDepth];
    int sp;
};

template <bool ANY>
__device__ bool traverse_blas_simple(const uint8_t *accel, const Ray &r, float tmin, Hit &h, uint64_t &hkey,
                                     uint32_t inst, uint32_t *err, unsigned long long *stats) {
    const rt_accel_header *hd = reinterpret_cast<const rt_accel_header *>(accel);
    if (hd->prim_count == 0) return false;
    const uint4 *nodes = reinterpret_cast<const uint4 *>(accel + hd->node_offset);
    const uint4 *prims = reinterpret_cast<const uint4 *>(accel + hd->prim_offset);
    LocalStack st;
    st.sp = 0;
    uint32_t node = 0;
    // A tree walk visits each node at most once; more visits (or a node
    // index past the end) can only come from a corrupt structure.
    const uint32_t max_visits = hd->node_count;
    for (uint32_t visits = 0;; ++visits) {
        if (visits >= max_visits || node >= max_visits) {
            report_error(err, RT_ERR_BOUNDS, 0x74000000u | node);
            return h.found;
        }
        NodeWords nd = load_node(nodes, node);
        uint32_t nh, ph;
        isect_node(r, nd, tmin, h.t, nh, ph);
        if (stats) stats[0]++;
        const uint32_t pbase = nd.w1.y;
        while (ph) {
            uint32_t i = __ffs(ph) - 1;
            ph &= ph - 1u;
            const uint4 *rec = prims + (size_t)(pbase + i) * 3u;
            uint4 a = ldg4(rec), b = ldg4(rec + 1), c = ldg4(rec + 2);
            if (stats) stats[1]++;
            float t, u, v;
            if (!isect_tri(r, make_float4(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z), 0.f),
                           make_float4(__uint_as_float(b.x), __uint_as_float(b.y), __uint_as_float(b.z), 0.f),
                           make_float4(__uint_as_float(c.x), __uint_as_float(c.y), __uint_as_float(c.z), 0.f),
                           tmin, h.t, t, u, v))
                continue;
            uint64_t key = ((uint64_t)inst << 32) | a.w;
            if (ANY) {
                h.t = t; h.u = u; h.v = v; h.rec = pbase + i; h.tri = a.w; h.inst = inst; h.found = true;
                return true;
            }
            if (key_less(t, key, h.t, hkey)) {
                h.t = t; h.u = u; h.v = v; h.rec = pbase + i; h.tri = a.w; h.inst = inst; h.found = true;
                hkey = key;
            }
        }
        uint2 g = make_uint2(nd.w1.x, nh | ((nd.w0.w >> 24) << 8));
        for (;;) {
            if (g.y & 0xffu) {
                uint32_t k = __ffs(g.y & 0xffu) - 1;
                g.y &= ~(1u << k);
                uint32_t s = k ^ r.oct;
                node = g.x + __popc((g.y >> 8) & ((1u << s) - 1u));
                if (g.y & 0xffu) {
                    if (st.sp >= kMaxDepth) {
                        report_error(err, RT_ERR_BOUNDS, 0x70000000u);
                        return h.found;
                    }
                    st.e[st.sp++] = g;
                }
                break;
            }
            if (st.sp == 0) return false;
            g = st.e[--st.sp];
        }
    }
}

struct InstRec {
    float w2o[12];
    uint64_t accel_ref;
    uint32_t cim, sof, id;
};

__device__ __forceinline__ InstRec load_inst(const uint4 *prims, uint32_t i) {
    const uint4 *p = prims + (size_t)i * 5u;
    uint4 a = ldg4(p), b = ldg4(p + 1), c = ldg4(p + 2), d = ldg4(p + 3), e = ldg4(p + 4);
    InstRec r;
    r.w2o[0] = __uint_as_float(a.x); r.w2o[1] = __uint_as_float(a.y); r.w2o[2] = __uint_as_float(a.z);
    r.w2o[3] = __uint_as_float(a.w); r.w2o[4] = __uint_as_float(b.x); r.w2o[5] = __uint_as_float(b.y);
    r.w2o[6] = __uint_as_float(b.z); r.w2o[7] = __uint_as_float(b.w); r.w2o[8] = __uint_as_float(c.x);
    r.w2o[9] = __uint_as_float(c.y); r.w2o[10] = __uint_as_float(c.z); r.w2o[11] = __uint_as_float(c.w);
    r.accel_ref = (uint64_t)d.x | ((uint64_t)d.y << 32);
    r.cim = d.z;
    r.sof = d.w;
    r.id = e.x;
    return r;
}

struct HitIds {
    uint32_t custom, sbt_off, geom, prim;
};

// Full closest/any traversal of a top- or bottom-level structure.
template <bool ANY>
__device__ bool trace_ray(const uint8_t *accel, const float o[3], const float d[3], float tmin, float tmax,
                          uint32_t cull_mask, Hit &h, HitIds &ids, uint32_t *err, unsigned long long *stats) {
    const rt_accel_header *hd = reinterpret_cast<const rt_accel_header *>(accel);
    h.t = tmax; h.u = 0.f; h.v = 0.f; h.rec = kNone; h.tri = kNone; h.inst = 0; h.found = false;
    ids.custom = 0; ids.sbt_off = 0; ids.geom = 0; ids.prim = 0;
    uint64_t hkey = ~0ull;
    Ray r;
    ray_setup(r, o, d);
    const uint8_t *hit_blas = accel;
    if (hd->kind == RT_ACCEL_KIND_BLAS) {
        bool any = traverse_blas_simple<ANY>(accel, r, tmin, h, hkey, 0u, err, stats);
        if (h.found) {
            const uint4 *prims = reinterpret_cast<const uint4 *>(accel + hd->prim_offset);
            ids.geom = ldg4(prims + (size_t)h.rec * 3u + 1).w;
            ids.prim = ldg4(prims + (size_t)h.rec * 3u + 2).w;
        }
        return ANY ? any : h.found;
    }
    if (hd->prim_count == 0) return false;
    const uint4 *nodes = reinterpret_cast<const uint4 *>(accel + hd->node_offset);
    const uint4 *prims = reinterpret_cast<const uint4 *>(accel + hd->prim_offset);
    LocalStack st;
    st.sp = 0;
    uint32_t node = 0;
    bool done = false;
    for (uint32_t visits = 0; !done; ++visits) {
        if (visits >= hd->node_count || node >= hd->node_count) {
            report_error(err, RT_ERR_BOUNDS, 0x75000000u | node);
            break;
        }
        NodeWords nd = load_node(nodes, node);
        uint32_t nh, ph;
        isect_node(r, nd, tmin, h.t, nh, ph);
        if (stats) stats[0]++;
        const uint32_t pbase = nd.w1.y;
        while (ph && !(ANY && h.found)) {
            uint32_t i = __ffs(ph) - 1;
            ph &= ph - 1u;
            InstRec ir = load_inst(prims, pbase + i);
            if (((ir.cim >> 24) & cull_mask) == 0u) continue;
            float o2[3], d2[3];
            xform_point(ir.w2o, o, o2);
            xform_vector(ir.w2o, d, d2);
            Ray r2;
            ray_setup(r2, o2, d2);
            const uint8_t *blas = reinterpret_cast<const uint8_t *>(ir.accel_ref);
            bool hit = traverse_blas_simple<ANY>(blas, r2, tmin, h, hkey, ir.id, err, stats);
            // instances occur once in a TLAS: a best hit carrying this id
            // was found in this instance's BLAS
            if (h.found && h.inst == ir.id) {
                ids.custom = ir.cim & 0xffffffu;
                ids.sbt_off = ir.sof & 0xffffffu;
                hit_blas = blas;
            }
            if (ANY && hit) break;
        }
        if (ANY && h.found) break;
        uint2 g = make_uint2(nd.w1.x, nh | ((nd.w0.w >> 24) << 8));
        for (;;) {
            if (g.y & 0xffu) {
                uint32_t k = __ffs(g.y & 0xffu) - 1;
                g.y &= ~(1u << k);
                uint32_t s = k ^ r.oct;
                node = g.x + __popc((g.y >> 8) & ((1u << s) - 1u));
                if (g.y & 0xffu) {
                    if (st.sp >= kMaxDepth) {
                        report_error(err, RT_ERR_BOUNDS, 0x71000000u);
                        done = true;
                        break;
                    }
                    st.e[st.sp++] = g;
                }
                break;
            }
            if (st.sp == 0) { done = true; break; }
            g = st.e[--st.sp];
        }
    }
    if (h.found && hit_blas) {
        const rt_accel_header *bh = reinterpret_cast<const rt_accel_header *>(hit_blas);
        const uint4 *bp = reinterpret_cast<const uint4 *>(hit_blas + bh->prim_offset);
        ids.geom = ldg4(bp + (size_t)h.rec * 3u + 1).w;
        ids.prim = ldg4(bp + (size_t)h.rec * 3u + 2).w;
    }
    return h.found;
}


// Two-level structures (instances), persistent like k_trace_blas: warps
// refill idle lanes from the work counter, stacks live in a shared-memory
// ring whose bottom spills to local memory.  At an instance a lane saves the
// TLAS node's remaining work on its stack -- the node's internal children,
// its instances not yet walked, then a return marker -- and walks the
// instance's BLAS with the object-space ray; popping the marker restores the
// world ray.  The visiting order is trace_ray's: a TLAS node's instances in
// ascending record order, each BLAS in full, then the node's internal
// children; closest hit = smallest t, ties broken by the smallest
// (instance id, triangle) key.  Launched beside k_trace_blas; each kernel
// returns at once when the structure is not its kind.
constexpr uint32_t kInstGroup = 0x40000000u;   // stack entry: instances of a TLAS node still to walk
constexpr uint32_t kReturnTop = 0x80000000u;   // stack entry: back to the TLAS
constexpr int kInstDepth = 128;                // stack entries per ray (both levels)
constexpr uint32_t kInstBlocksPerSm = 6;  // 80 registers (7 blocks: 72 and 72 bytes of spill, 2 % slower)

__device__ __forceinline__ bool inst_key_less(float t, uint32_t inst, uint32_t tri, const Hit &h) {
    return t < h.t || (t == h.t && (!h.found || inst < h.inst || (inst == h.inst && tri < h.tri)));
}

template <bool ANY, bool STATS>
__global__ void __launch_bounds__(kTraceThreads, kInstBlocksPerSm) k_trace_inst(const BatchArgs a) {
    const rt_accel_header *hd = reinterpret_cast<const rt_accel_header *>(a.accel);
    if (hd->kind != RT_ACCEL_KIND_TLAS) return;
    const uint4 *tnodes = reinterpret_cast<const uint4 *>(a.accel + hd->node_offset);
    const uint4 *tprims = reinterpret_cast<const uint4 *>(a.accel + hd->prim_offset);
    const uint32_t t_count = hd->node_count;
    const bool t_empty = hd->prim_count == 0;
    __shared__ uint2 s_stack[kRing][kTraceThreads];
    const int tid = threadIdx.x, lane = tid & 31;

    bool active = false, exhausted = false;
    uint32_t ray_idx = 0;
    float wo[3] = {0.f, 0.f, 0.f}, wd[3] = {0.f, 0.f, 0.f};  // the world ray
    Ray r;  // the current level's ray
    float tmin = 0.f;
    Hit h;
    h.t = 0.f; h.u = 0.f; h.v = 0.f; h.rec = kNone; h.tri = kNone; h.inst = 0; h.found = false;
    uint32_t h_irec = kNone;  // TLAS record of the best hit's instance
    uint32_t node = 0;
    bool pending = false, in_blas = false;
    const uint4 *bnodes = nullptr, *bprims = nullptr;
    uint32_t b_count = 0, inst_id = 0, inst_rec = 0, visits_t = 0, visits_b = 0;
    uint2 g = make_uint2(0u, 0u), ig = make_uint2(0u, 0u);
    int sp = 0, lo = 0;
    uint2 spill[kInstDepth];
    unsigned long long n_nodes = 0, n_tris = 0;
    const uint32_t n_rays = a.n;

    auto push = [&](uint2 e) {
        if (sp - lo == kRing) {
            spill[lo] = s_stack[lo & (kRing - 1)][tid];
            ++lo;
        }
        s_stack[sp & (kRing - 1)][tid] = e;
        ++sp;
    };

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
                const uint32_t idx = base + __popc(idle & ((1u << lane) - 1u));
                if (idx < n_rays) {
                    const float4 r0 = __ldg(a.rays + 2u * idx), r1 = __ldg(a.rays + 2u * idx + 1u);
                    wo[0] = r0.x; wo[1] = r0.y; wo[2] = r0.z;
                    wd[0] = r1.x; wd[1] = r1.y; wd[2] = r1.z;
                    ray_setup(r, wo, wd);
                    tmin = r0.w;
                    h.t = r1.w; h.u = 0.f; h.v = 0.f; h.rec = kNone; h.tri = kNone; h.inst = 0; h.found = false;
                    h_irec = kNone;
                    ray_idx = idx;
                    active = true;
                    in_blas = false;
                    node = 0;
                    pending = !t_empty;
                    visits_t = 0;
                    g = make_uint2(0u, 0u);
                    ig = make_uint2(0u, 0u);
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
                if (pending) {
                    pending = false;
                    const uint32_t count = in_blas ? b_count : t_count;
                    const uint32_t visits = in_blas ? visits_b : visits_t;
                    if (visits >= count || node >= count) {
                        report_error(a.err, RT_ERR_BOUNDS, (in_blas ? 0x74000000u : 0x75000000u) | (node & 0xffffffu));
                        finish = true;
                    } else {
                        if (in_blas) ++visits_b;
                        else ++visits_t;
                        NodeWords nd = load_node(in_blas ? bnodes : tnodes, node);
                        uint32_t nh, ph;
                        isect_node<true>(r, nd, tmin, h.t, nh, ph);
                        if (STATS) n_nodes++;
                        g = make_uint2(nd.w1.x, nh | ((nd.w0.w >> 24) << 8));
                        if (!in_blas) {
                            ig = make_uint2(nd.w1.y, ph);  // the node's instances, walked first
                        } else {
                            const uint32_t pbase = nd.w1.y;
                            while (ph) {
                                const uint32_t i = __ffs(ph) - 1;
                                ph &= ph - 1u;
                                const uint4 *rec = bprims + (size_t)(pbase + i) * 3u;
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
                                if (ANY || inst_key_less(t, inst_id, q0.w, h)) {
                                    h.t = t; h.u = u; h.v = v; h.rec = pbase + i; h.tri = q0.w; h.inst = inst_id;
                                    h_irec = inst_rec;
                                    h.found = true;
                                }
                                if (ANY) {
                                    finish = true;
                                    break;
                                }
                            }
                        }
                    }
                }
                // ---- next: an instance of the current TLAS node, else a node
                while (!finish) {
                    if (!in_blas && ig.y) {
                        const uint32_t i = __ffs(ig.y) - 1;
                        ig.y &= ig.y - 1u;
                        const uint32_t rec = ig.x + i;
                        const InstRec ir = load_inst(tprims, rec);
                        if (((ir.cim >> 24) & 0xffu) == 0u) continue;  // masked out (cull mask 0xFF)
                        const uint8_t *blas = reinterpret_cast<const uint8_t *>(ir.accel_ref);
                        const rt_accel_header *bh = reinterpret_cast<const rt_accel_header *>(blas);
                        if (bh->prim_count == 0) continue;
                        if (sp + 3 > kInstDepth) {
                            report_error(a.err, RT_ERR_BOUNDS, 0x71000000u);
                            finish = true;
                            break;
                        }
                        // save the TLAS node's remaining work under a return marker
                        if (g.y & 0xffu) push(g);
                        if (ig.y) push(make_uint2(ig.x, ig.y | kInstGroup));
                        push(make_uint2(0u, kReturnTop));
                        g = make_uint2(0u, 0u);
                        ig = make_uint2(0u, 0u);
                        float o2[3], d2[3];
                        xform_point(ir.w2o, wo, o2);
                        xform_vector(ir.w2o, wd, d2);
                        ray_setup(r, o2, d2);
                        in_blas = true;
                        bnodes = reinterpret_cast<const uint4 *>(blas + bh->node_offset);
                        bprims = reinterpret_cast<const uint4 *>(blas + bh->prim_offset);
                        b_count = bh->node_count;
                        visits_b = 0;
                        inst_id = ir.id;
                        inst_rec = rec;
                        node = 0;
                        pending = true;
                        break;
                    }
                    if (g.y & 0xffu) {
                        const uint32_t k = __ffs(g.y & 0xffu) - 1;
                        g.y &= ~(1u << k);
                        const uint32_t s = k ^ r.oct;
                        node = g.x + __popc((g.y >> 8) & ((1u << s) - 1u));
                        pending = true;
                        if (g.y & 0xffu) {
                            if (sp >= kInstDepth) {
                                report_error(a.err, RT_ERR_BOUNDS, in_blas ? 0x70000000u : 0x71000000u);
                                finish = true;
                                break;
                            }
                            push(g);
                        }
                        break;
                    }
                    if (sp == 0) { finish = true; break; }
                    --sp;
                    uint2 e;
                    if (sp >= lo) {
                        e = s_stack[sp & (kRing - 1)][tid];
                    } else {
                        e = spill[sp];
                        lo = sp;
                    }
                    if (e.y & kReturnTop) {
                        // the TLAS work saved under the marker (if any) needs
                        // the world ray back; with none left the walk is done
                        if (sp == 0) { finish = true; break; }
                        ray_setup(r, wo, wd);
                        in_blas = false;
                    } else if (e.y & kInstGroup) {
                        ig = make_uint2(e.x, e.y & ~kInstGroup);
                    } else {
                        g = e;
                    }
                }
                if (finish) {
                    // ---- write the result
                    if (ANY) {
                        if (a.occluded) a.occluded[ray_idx] = h.found ? 1u : 0u;
                    } else {
                        const float4 out = h.found ? make_float4(h.t, __uint_as_float(h.tri), h.u, h.v)
                                                   : make_float4(kInf, __uint_as_float(kNone), 0.f, 0.f);
                        if (a.hits) a.hits[ray_idx] = out;
                        if (a.hits_ext) {
                            rt_hit_ext x;
                            x.t = out.x; x.u = out.z; x.v = out.w;
                            x.instance_id = h.found ? h.inst : kNone;
                            x.custom_index = 0u;
                            x.geometry_index = 0u;
                            x.primitive_id = kNone;
                            x.sbt_record = 0u;
                            if (h.found) {
                                const InstRec ir = load_inst(tprims, h_irec);
                                const uint8_t *blas = reinterpret_cast<const uint8_t *>(ir.accel_ref);
                                const rt_accel_header *bh = reinterpret_cast<const rt_accel_header *>(blas);
                                const uint4 *bp = reinterpret_cast<const uint4 *>(blas + bh->prim_offset);
                                x.custom_index = ir.cim & 0xffffffu;
                                x.geometry_index = ldg4(bp + (size_t)h.rec * 3u + 1).w;
                                x.primitive_id = ldg4(bp + (size_t)h.rec * 3u + 2).w;
                                x.sbt_record = (ir.sof & 0xffffffu) + x.geometry_index;
                            }
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

// ---------------------------------------------------------------------------
// Sample pipeline: raygen + trace + closest-hit/miss + imageStore
// ---------------------------------------------------------------------------

struct PipelineArgs {
    const uint8_t *accel;
    float cam[3];
    float ay, ax;   // aspect_y, aspect_x of the raygen (host-computed)
    uint32_t width, height;
    uint32_t chit, ray_flags, cull_mask, sbt_record_offset, sbt_record_stride;
    float tmin, tmax;
    float miss[3];
    const float *sbt;
    uint32_t sbt_count, sbt_stride;
    float4 *out;
    rt_ray *rays_out;  // when set: write the primary rays instead of tracing
    uint32_t *err;
};

// The sample's raygen (main.cpp:1036-1045), one IEEE operation at a time.
__device__ __forceinline__ void raygen(const PipelineArgs &a, uint32_t x, uint32_t y, float dir[3]) {
    const float sx = (float)x + 0.5f, sy = (float)y + 0.5f;
    const float ndx = (sx / (float)a.width) * 2.0f - 1.0f;
    const float ndy = (sy / (float)a.height) * 2.0f - 1.0f;
    const float p = ndx * a.ax, q = ndy * a.ay;
    dir[0] = (p * 1.0f + q * 0.0f) + 0.0f;
    dir[1] = (p * 0.0f + q * -1.0f) + 0.0f;
    dir[2] = (p * 0.0f + q * 0.0f) + -1.0f;
}

__global__ void __launch_bounds__(128) k_pipeline(const PipelineArgs a) {
    const uint32_t x = blockIdx.x * 16u + (threadIdx.x & 15u);
    const uint32_t y = blockIdx.y * 8u + (threadIdx.x >> 4);
    if (x >= a.width || y >= a.height) return;
    float dir[3];
    raygen(a, x, y, dir);
    const size_t pix = (size_t)y * a.width + x;
    if (a.rays_out) {
        rt_ray rr;
        rr.org[0] = a.cam[0]; rr.org[1] = a.cam[1]; rr.org[2] = a.cam[2];
        rr.dir[0] = dir[0]; rr.dir[1] = dir[1]; rr.dir[2] = dir[2];
        rr.tmin = a.tmin;
        rr.tmax = a.tmax;
        a.rays_out[pix] = rr;
        return;
    }
    Hit h;
    HitIds ids;
    float c[3];
    if (a.ray_flags & RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT)
        trace_ray<true>(a.accel, a.cam, dir, a.tmin, a.tmax, a.cull_mask & 0xffu, h, ids, a.err, nullptr);
    else
        trace_ray<false>(a.accel, a.cam, dir, a.tmin, a.tmax, a.cull_mask & 0xffu, h, ids, a.err, nullptr);
    if (!h.found) {
        c[0] = a.miss[0]; c[1] = a.miss[1]; c[2] = a.miss[2];
    } else if (a.ray_flags & RT_RAY_FLAG_SKIP_CLOSEST_HIT) {
        c[0] = c[1] = c[2] = 0.0f;
    } else {
        const uint32_t rec = ids.sbt_off + ids.geom * a.sbt_record_stride + a.sbt_record_offset;
        const bool bary = a.chit == RT_CHIT_BARYCENTRIC ||
                          (a.chit == RT_CHIT_SAMPLE && ids.prim == 1u && h.inst == 1u && ids.custom == 100u &&
                           ids.geom == 1u);
        if (bary) {
            c[0] = (1.0f - h.u) - h.v; c[1] = h.u; c[2] = h.v;
        } else if (rec < a.sbt_count) {
            c[0] = a.sbt[(size_t)rec * a.sbt_stride + 0];
            c[1] = a.sbt[(size_t)rec * a.sbt_stride + 1];
            c[2] = a.sbt[(size_t)rec * a.sbt_stride + 2];
        } else {
            c[0] = c[1] = c[2] = 0.0f;
            report_error(a.err, RT_ERR_BOUNDS, 0x73000000u | rec);
        }
    }
    a.out[pix] = make_float4(c[0], c[1], c[2], 0.0f);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

int launch_batch(rt_context *ctx, cudaStream_t st, uint64_t accel, const rt_ray *rays, rt_hit *hits,
                 rt_hit_ext *hits_ext, uint8_t *occ, uint32_t n, bool any, unsigned long long *stats) {
    if (n == 0) return RT_OK;
    BatchArgs a{};
    a.accel = reinterpret_cast<const uint8_t *>(accel);
    a.rays = reinterpret_cast<const float4 *>(rays);
    a.hits = reinterpret_cast<float4 *>(hits);
    a.hits_ext = hits_ext;
    a.occluded = occ;
    a.n = n;
    a.refill = ctx->tuning.batch_rays ? ctx->tuning.batch_rays : 4u;
    if (a.refill > 32u) a.refill = 32u;
    a.err = ctx->d_err;
    a.stats = stats;
    a.n_dev = nullptr;
    a.out_rec = 0;
    a.counter = acquire_counter(ctx, st);
    if (!a.counter) return set_error(ctx, RT_ERR_CUDA, "work counter reset failed");
    uint32_t per_sm = ctx->tuning.blocks_per_sm ? ctx->tuning.blocks_per_sm : 8u;
    if (any && per_sm > kAnyBlocksPerSm) per_sm = kAnyBlocksPerSm;
    uint32_t blocks = per_sm * (uint32_t)ctx->sm_count;
    uint32_t need = (n + kTraceThreads - 1) / kTraceThreads;
    if (blocks > need) blocks = need;
    // Both kernels are launched; the one that does not match the structure's
    // kind returns immediately.
    uint32_t tl_blocks = kInstBlocksPerSm * (uint32_t)ctx->sm_count;
    if (tl_blocks > need) tl_blocks = need;
    if (stats) {
        if (any) {
            k_trace_blas<true, true, false, kTraceThreads, kRing><<<blocks, kTraceThreads, 0, st>>>(a);
            k_trace_inst<true, true><<<tl_blocks, kTraceThreads, 0, st>>>(a);
        } else {
            k_trace_blas<false, true, false, kTraceThreads, kRing><<<blocks, kTraceThreads, 0, st>>>(a);
            k_trace_inst<false, true><<<tl_blocks, kTraceThreads, 0, st>>>(a);
        }
    } else {
        if (any) {
            k_trace_blas<true, false, false, kTraceThreads, kRing><<<blocks, kTraceThreads, 0, st>>>(a);
            k_trace_inst<true, false><<<tl_blocks, kTraceThreads, 0, st>>>(a);
        } else {
            k_trace_blas<false, false, false, kTraceThreads, kRing><<<blocks, kTraceThreads, 0, st>>>(a);
            k_trace_inst<false, false><<<tl_blocks, kTraceThreads, 0, st>>>(a);
        }
    }
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}

}  // namespace

// Refill threshold of the path tracer's queue traversals: a warp refills once
// eight of its lanes are idle (2M box, 4 spp per call: 6.91 / 6.56 / 6.45 /
// 6.43 ms per sample at 2 / 4 / 6 / 8; the ray-query calls keep the context's
// batch_rays, whose default 4 is best for the soup's primary + incoherent
// rays; re-checked with the packed box test and the 8-entry ring: 6.26 /
// 6.23 / 6.33 ms at 6 / 8 / 12).  The batch's autotuner chose 8 as well.
constexpr uint32_t kQueueRefill = 8u;

// Queue-driven BLAS traversal for the wavefront path tracer: the ray count is
// read on the device from *n_dev (at most max_n), the work counter is
// `counter` (zeroed by the caller on the stream), and closest hits carry the
// leaf-record index.  Capturable in a CUDA graph (no host reads, no
// allocation).
int launch_queue_trace(rt_context *ctx, cudaStream_t st, const uint8_t *accel, const void *rays, void *hits,
                       uint8_t *occluded, const uint32_t *n_dev, uint32_t max_n, uint32_t *counter, bool any) {
    if (max_n == 0) return RT_OK;
    BatchArgs a{};
    a.accel = accel;
    a.rays = static_cast<const float4 *>(rays);
    a.hits = static_cast<float4 *>(hits);
    a.hits_ext = nullptr;
    a.occluded = occluded;
    a.n = max_n;
    a.refill = kQueueRefill;
    a.err = ctx->d_err;
    a.stats = nullptr;
    a.n_dev = n_dev;
    a.out_rec = 1;
    a.counter = counter;
    uint32_t per_sm = ctx->tuning.blocks_per_sm ? ctx->tuning.blocks_per_sm : 8u;
    if (any && per_sm > kAnyBlocksPerSm) per_sm = kAnyBlocksPerSm;
    uint32_t blocks = per_sm * (uint32_t)ctx->sm_count;
    uint32_t need = (max_n + kTraceThreads - 1) / kTraceThreads;
    if (blocks > need) blocks = need;
    if (any) k_trace_blas<true, false, false, kTraceThreads, kRing><<<blocks, kTraceThreads, 0, st>>>(a);
    else k_trace_blas<false, false, false, kTraceThreads, kRing><<<blocks, kTraceThreads, 0, st>>>(a);
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}

// One launch over two queues of at most max_n rays each: closest hits for
// rays/n_dev (leaf-record index out, to hits), then any hits for
// rays2/n_dev2 (to occluded).  Capturable like launch_queue_trace.
int launch_queue_trace_mixed(rt_context *ctx, cudaStream_t st, const uint8_t *accel, const void *rays, void *hits,
                             const uint32_t *n_dev, const void *rays2, uint8_t *occluded, const uint32_t *n_dev2,
                             uint32_t max_n, uint32_t *counter) {
    if (max_n == 0) return RT_OK;
    BatchArgs a{};
    a.accel = accel;
    a.rays = static_cast<const float4 *>(rays);
    a.hits = static_cast<float4 *>(hits);
    a.occluded = occluded;
    a.n = max_n;
    a.n_dev = n_dev;
    a.rays2 = static_cast<const float4 *>(rays2);
    a.n_dev2 = n_dev2;
    a.n2 = max_n;
    a.refill = kQueueRefill;
    a.err = ctx->d_err;
    a.out_rec = 1;
    a.counter = counter;
    uint32_t per_sm = ctx->tuning.blocks_per_sm ? ctx->tuning.blocks_per_sm : 8u;
    uint32_t blocks = per_sm * (uint32_t)ctx->sm_count;
    const uint32_t need = (uint32_t)(((uint64_t)max_n * 2u + kTraceThreads - 1) / kTraceThreads);
    if (blocks > need) blocks = need;
    k_trace_blas<false, false, false, kTraceThreads, kRing, true><<<blocks, kTraceThreads, 0, st>>>(a);
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}

namespace {


}  // namespace
}  // namespace rtc

using namespace rtc;

extern "C" rt_status rt_trace_closest(rt_context *ctx, rt_stream stream, uint64_t accel, const rt_ray *rays,
                                      rt_hit *hits, rt_hit_ext *hits_ext, uint32_t n) {
    if (!ctx || !accel || (n && (!rays || !hits))) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_trace_closest: null argument");
    return launch_batch(ctx, static_cast<cudaStream_t>(stream), accel, rays, hits, hits_ext, nullptr, n, false,
                        nullptr);
}

extern "C" rt_status rt_trace_any(rt_context *ctx, rt_stream stream, uint64_t accel, const rt_ray *rays,
                                  uint8_t *occluded, uint32_t n) {
    if (!ctx || !accel || (n && (!rays || !occluded))) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_trace_any: null argument");
    return launch_batch(ctx, static_cast<cudaStream_t>(stream), accel, rays, nullptr, nullptr, occluded, n, true,
                        nullptr);
}

// ---------------------------------------------------------------------------
// Rays and results staged through the scratch (pageable memory the device
// cannot reach, misaligned buffers, RT_HOST_TRANSFER_STAGED): a ring of four
// device slots; chunk k is
// copied in on the context's copy-in stream once its slot's previous results
// have left, traced on one of three trace streams (round robin), and copied
// out on the copy-out stream.  The copies of neighbouring chunks overlap the
// traversal, and so do consecutive traversals: a launch ends on its slowest
// ray (a grazing primary ray walks hundreds of nodes), and the next chunk's
// launch fills the SMs the finished warps leave.  The first chunk is small
// (2^18 rays) so the pipeline fills quickly; chunks then double up to what a
// slot holds.
// ---------------------------------------------------------------------------

namespace {

constexpr uint32_t kHostChunk = 1u << 20;  // rays per chunk

// The ring's geometry depends on the scratch size only (never on the call's
// ray count or result size), so slot s covers the same bytes in every call
// that passes the same scratch: its events then order all uses of it.
struct HostSlots {
    uint32_t chunk;  // rays per slot
    uint64_t out_offset, slot_bytes;
};

uint64_t slot_bytes_for(uint32_t chunk) { return align_up((uint64_t)chunk * 32u, 256) + align_up((uint64_t)chunk * 16u, 256); }

HostSlots host_slots(uint64_t scratch_bytes) {
    HostSlots h;
    h.slot_bytes = (scratch_bytes / (uint64_t)rt_context::kHostSlots) & ~255ull;
    uint64_t c = h.slot_bytes / 48u;
    if (c > kHostChunk) c = kHostChunk;
    while (c > 0 && slot_bytes_for((uint32_t)c) > h.slot_bytes) --c;
    h.chunk = (uint32_t)c;
    h.out_offset = align_up(c * 32u, 256);
    return h;
}

int host_setup(rt_context *ctx) {
    if (ctx->host_ready) return RT_OK;
    RT_CUDA_CTX(ctx, cudaStreamCreateWithFlags(&ctx->h2d, cudaStreamNonBlocking));
    RT_CUDA_CTX(ctx, cudaStreamCreateWithFlags(&ctx->d2h, cudaStreamNonBlocking));
    for (int k = 0; k < rt_context::kHostTraceStreams; ++k)
        RT_CUDA_CTX(ctx, cudaStreamCreateWithFlags(&ctx->htr[k], cudaStreamNonBlocking));
    RT_CUDA_CTX(ctx, cudaEventCreateWithFlags(&ctx->ev_start, cudaEventDisableTiming));
    for (int s = 0; s < rt_context::kHostSlots; ++s) {
        RT_CUDA_CTX(ctx, cudaEventCreateWithFlags(&ctx->ev_loaded[s], cudaEventDisableTiming));
        RT_CUDA_CTX(ctx, cudaEventCreateWithFlags(&ctx->ev_traced[s], cudaEventDisableTiming));
        RT_CUDA_CTX(ctx, cudaEventCreateWithFlags(&ctx->ev_free[s], cudaEventDisableTiming));
    }
    ctx->host_ready = true;
    return RT_OK;
}

// Whether every page of the host range [p, p + bytes) is mapped in this
// process.  msync with MS_ASYNC writes nothing back; it only fails with ENOMEM
// where part of the range is unmapped (a gap between two allocations, which a
// kernel reading the range in place would fault on).
bool host_range_mapped(const void *p, uint64_t bytes) {
    const long pg = sysconf(_SC_PAGESIZE);
    const uintptr_t page = pg > 0 ? (uintptr_t)pg : 4096u;
    const uintptr_t lo = reinterpret_cast<uintptr_t>(p) & ~(page - 1u);
    const uintptr_t hi = (reinterpret_cast<uintptr_t>(p) + bytes + page - 1u) & ~(page - 1u);
    return msync(reinterpret_cast<void *>(lo), hi - lo, MS_ASYNC) == 0;
}

// Whether [p, p + bytes) lies inside one CUDA allocation (device, managed or
// pinned host memory), from the driver's pointer attributes; false where the
// driver cannot say.
bool one_cuda_allocation(const void *p, uint64_t bytes) {
    static decltype(&cuPointerGetAttribute) get_attr = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            (void)cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<decltype(&cuPointerGetAttribute)>(f);
    }();
    if (!get_attr) return false;
    CUdeviceptr base = 0;
    size_t size = 0;
    const CUdeviceptr q = (CUdeviceptr)reinterpret_cast<uintptr_t>(p);
    if (get_attr(&base, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, q) != CUDA_SUCCESS ||
        get_attr(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, q) != CUDA_SUCCESS)
        return false;
    return q >= base && q - base + bytes <= size;
}

// True when kernels reach [p, p + bytes) at the same address: pinned or
// registered host memory under unified addressing (cudaHostAlloc,
// cudaHostRegister), device or managed memory, and -- where the device
// accesses pageable memory through the host's page tables (a Grace system's
// NVLink-C2C; `pageable` from the device attributes) -- plain pageable
// memory.  Both ends are checked, and so is what lies between them: a host
// range must be mapped throughout (and, without pageable access, be one
// pinned allocation), a device range must be one allocation.  Anything else
// goes through the staged copies.
bool reachable_in_place(const void *p, uint64_t bytes, bool pageable) {
    if (bytes == 0) return true;
    const uint8_t *b = static_cast<const uint8_t *>(p);
    bool host_side = true, device_side = true;
    for (const uint8_t *q : {b, b + (bytes - 1u)}) {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
            (void)cudaGetLastError();
            return false;
        }
        if (at.type == cudaMemoryTypeHost) {
            if (at.devicePointer != q) return false;
            device_side = false;
        } else if (at.type == cudaMemoryTypeUnregistered) {
            if (!pageable) return false;
            device_side = false;
        } else {
            host_side = false;
        }
    }
    if (host_side) {
        if (!host_range_mapped(p, bytes)) return false;
        return pageable || one_cuda_allocation(p, bytes);
    }
    return device_side && one_cuda_allocation(p, bytes);
}

// Whether the context's device reads and writes pageable host memory
// coherently through the host page tables (queried once).
bool pageable_in_place(rt_context *ctx) {
    if (ctx->pageable_state == 0) {
        int a = 0, b = 0;
        const bool ok = cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, ctx->device) == cudaSuccess &&
                        cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, ctx->device) ==
                            cudaSuccess;
        (void)cudaGetLastError();
        ctx->pageable_state = (ok && a == 1 && b == 1) ? 1 : 2;
    }
    return ctx->pageable_state == 1;
}

int trace_host(rt_context *ctx, cudaStream_t st, uint64_t accel, const rt_ray *hrays, void *hout, uint32_t n,
               bool any, void *scratch, uint64_t scratch_bytes) {
    if (n == 0) return RT_OK;
    const uint32_t out_size = any ? 1u : 16u;
    // Rays and results the kernels reach in place (pinned memory; on a
    // Grace-Blackwell system also pageable memory, through the host page
    // tables): one launch reads the rays and writes the results where they
    // are, over NVLink-C2C.  A ray is read once (32 bytes) and a result
    // written once, so no staging copy, chunk or ring is needed (4.15M rays
    // of the 1M soup: 2.14 ms pinned or pageable, against 2.47 ms staged from
    // pinned, 3.91 ms staged from pageable and 2.07 ms with rays and hits in
    // HBM).
    RT_CUDA_CTX(ctx, cudaSetDevice(ctx->device));
    const bool pageable = pageable_in_place(ctx);
    if (ctx->host_transfer == RT_HOST_TRANSFER_AUTO && (reinterpret_cast<uintptr_t>(hrays) & 15u) == 0 &&
        (any || (reinterpret_cast<uintptr_t>(hout) & 15u) == 0) &&
        reachable_in_place(hrays, (uint64_t)n * 32u, pageable) &&
        reachable_in_place(hout, (uint64_t)n * out_size, pageable))
        return launch_batch(ctx, st, accel, hrays, any ? nullptr : static_cast<rt_hit *>(hout), nullptr,
                            any ? static_cast<uint8_t *>(hout) : nullptr, n, any, nullptr);
    const HostSlots H = host_slots(scratch_bytes);
    if (H.chunk == 0) return set_error(ctx, RT_ERR_OOM, "rt_trace_*_host: scratch smaller than rt_trace_host_scratch_bytes(1)");
    if (reinterpret_cast<uintptr_t>(scratch) & 255u) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_trace_*_host: scratch must be 256-byte aligned");
    int rc = host_setup(ctx);
    if (rc) return rc;
    if (scratch != ctx->host_scratch || scratch_bytes != ctx->host_scratch_bytes) {
        // another ring: copy in nothing before every earlier copy out is done
        for (int k = 0; k < rt_context::kHostSlots; ++k) RT_CUDA_CTX(ctx, cudaStreamWaitEvent(ctx->h2d, ctx->ev_free[k], 0));
        ctx->host_scratch = scratch;
        ctx->host_scratch_bytes = scratch_bytes;
    }
    uint8_t *S = static_cast<uint8_t *>(scratch);
    // everything of the call starts after the work queued on `stream` so far
    RT_CUDA_CTX(ctx, cudaEventRecord(ctx->ev_start, st));
    RT_CUDA_CTX(ctx, cudaStreamWaitEvent(ctx->h2d, ctx->ev_start, 0));
    for (int k = 0; k < rt_context::kHostTraceStreams; ++k)
        RT_CUDA_CTX(ctx, cudaStreamWaitEvent(ctx->htr[k], ctx->ev_start, 0));
    uint32_t chunk = kHostChunk / 4u < H.chunk ? kHostChunk / 4u : H.chunk;
    int s = 0, k = 0;
    for (uint32_t off = 0, m = 0; off < n; off += m, ++k) {
        m = n - off < chunk ? n - off : chunk;
        chunk = chunk * 2u < H.chunk ? chunk * 2u : H.chunk;
        s = (int)(ctx->slot_next++ % (uint32_t)rt_context::kHostSlots);
        cudaStream_t ts = ctx->htr[k % rt_context::kHostTraceStreams];
        uint8_t *rays_d = S + (uint64_t)s * H.slot_bytes;
        uint8_t *out_d = rays_d + H.out_offset;
        RT_CUDA_CTX(ctx, cudaStreamWaitEvent(ctx->h2d, ctx->ev_free[s], 0));
        // cudaMemcpyDefault: the direction follows from the pointers (unified
        // addressing), so a device or managed buffer handed to the host API
        // copies correctly too
        RT_CUDA_CTX(ctx, cudaMemcpyAsync(rays_d, hrays + off, (size_t)m * 32u, cudaMemcpyDefault, ctx->h2d));
        RT_CUDA_CTX(ctx, cudaEventRecord(ctx->ev_loaded[s], ctx->h2d));
        RT_CUDA_CTX(ctx, cudaStreamWaitEvent(ts, ctx->ev_loaded[s], 0));
        rc = launch_batch(ctx, ts, accel, reinterpret_cast<const rt_ray *>(rays_d),
                          any ? nullptr : reinterpret_cast<rt_hit *>(out_d), nullptr, any ? out_d : nullptr, m, any,
                          nullptr);
        if (rc) return rc;
        RT_CUDA_CTX(ctx, cudaEventRecord(ctx->ev_traced[s], ts));
        RT_CUDA_CTX(ctx, cudaStreamWaitEvent(ctx->d2h, ctx->ev_traced[s], 0));
        RT_CUDA_CTX(ctx, cudaMemcpyAsync(static_cast<uint8_t *>(hout) + (size_t)off * out_size, out_d,
                                         (size_t)m * out_size, cudaMemcpyDefault, ctx->d2h));
        RT_CUDA_CTX(ctx, cudaEventRecord(ctx->ev_free[s], ctx->d2h));
    }
    // the caller's stream goes on after the last results have left
    RT_CUDA_CTX(ctx, cudaStreamWaitEvent(st, ctx->ev_free[s], 0));
    return RT_OK;
}

}  // namespace

extern "C" rt_status rt_debug_host_in_place(rt_context *ctx, const void *p, uint64_t bytes, int *in_place) {
    if (!ctx || !in_place || (bytes && !p)) return RT_ERR_INVALID_ARG;
    RT_CUDA_CTX(ctx, cudaSetDevice(ctx->device));
    *in_place = reachable_in_place(p, bytes, pageable_in_place(ctx)) ? 1 : 0;
    return RT_OK;
}

extern "C" rt_status rt_set_host_transfer(rt_context *ctx, uint32_t mode) {
    if (!ctx) return RT_ERR_INVALID_ARG;
    if (mode != RT_HOST_TRANSFER_AUTO && mode != RT_HOST_TRANSFER_STAGED)
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_set_host_transfer: unknown mode");
    ctx->host_transfer = mode;
    return RT_OK;
}

extern "C" rt_status rt_trace_host_scratch_bytes(uint32_t n, int any_hit, uint64_t *bytes) {
    (void)any_hit;  // one ring serves both kinds of call
    if (!bytes) return RT_ERR_INVALID_ARG;
    const uint32_t c = n == 0 ? 1u : (n < kHostChunk ? n : kHostChunk);
    *bytes = slot_bytes_for(c) * (uint64_t)rt_context::kHostSlots;
    return RT_OK;
}

extern "C" rt_status rt_trace_closest_host(rt_context *ctx, rt_stream stream, uint64_t accel, const rt_ray *rays,
                                           rt_hit *hits, uint32_t n, void *scratch, uint64_t scratch_bytes) {
    if (!ctx || !accel || (n && (!rays || !hits || !scratch)))
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_trace_closest_host: null argument");
    return trace_host(ctx, static_cast<cudaStream_t>(stream), accel, rays, hits, n, false, scratch, scratch_bytes);
}

extern "C" rt_status rt_trace_any_host(rt_context *ctx, rt_stream stream, uint64_t accel, const rt_ray *rays,
                                       uint8_t *occluded, uint32_t n, void *scratch, uint64_t scratch_bytes) {
    if (!ctx || !accel || (n && (!rays || !occluded || !scratch)))
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_trace_any_host: null argument");
    return trace_host(ctx, static_cast<cudaStream_t>(stream), accel, rays, occluded, n, true, scratch, scratch_bytes);
}

extern "C" rt_status rt_trace_stats(rt_context *ctx, rt_stream stream, uint64_t accel, const rt_ray *rays,
                                    uint32_t n, int any_hit, unsigned long long *counters) {
    if (!ctx || !accel || !counters || (n && !rays)) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_trace_stats: null argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    RT_CUDA_CTX(ctx, cudaMemsetAsync(counters, 0, 16, st));
    // No hit output: the counters are the result.
    return launch_batch(ctx, st, accel, rays, nullptr, nullptr, nullptr, n, any_hit != 0, counters);
}

extern "C" rt_status rt_trace_rays(rt_context *ctx, rt_stream stream, const rt_pipeline *p, const rt_sbt *sbt,
                                   uint64_t accel, const rt_camera *camera, float *out, uint32_t width,
                                   uint32_t height, uint32_t depth) {
    if (!ctx || !p || !accel || !camera || !out) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_trace_rays: null argument");
    if (depth != 1u) return set_error(ctx, RT_ERR_UNSUPPORTED, "rt_trace_rays: depth must be 1 (2D storage image)");
    if (width == 0 || height == 0) return RT_OK;
    if (p->chit > RT_CHIT_SBT_COLOR) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_trace_rays: unknown closest-hit program");
    if (p->max_recursion > 1u) return set_error(ctx, RT_ERR_UNSUPPORTED, "rt_trace_rays: recursion depth > 1");
    if (p->sbt_record_stride == 0u && p->chit != RT_CHIT_BARYCENTRIC)
        ; /* stride 0 is legal in Vulkan: every geometry uses the same record */
    PipelineArgs a;
    a.accel = reinterpret_cast<const uint8_t *>(accel);
    a.cam[0] = camera->position[0]; a.cam[1] = camera->position[1]; a.cam[2] = camera->position[2];
    camera_aspects(camera, width, height, &a.ay, &a.ax);
    a.width = width;
    a.height = height;
    a.chit = p->chit;
    a.ray_flags = p->ray_flags;
    a.cull_mask = p->cull_mask;
    a.sbt_record_offset = p->sbt_record_offset;
    a.sbt_record_stride = p->sbt_record_stride;
    a.tmin = p->tmin;
    a.tmax = p->tmax;
    a.miss[0] = p->miss_color[0]; a.miss[1] = p->miss_color[1]; a.miss[2] = p->miss_color[2];
    a.sbt = sbt ? sbt->hit_colors : nullptr;
    a.sbt_count = sbt && sbt->hit_colors ? sbt->hit_record_count : 0u;
    a.sbt_stride = sbt ? (sbt->hit_record_stride < 3u ? 3u : sbt->hit_record_stride) : 3u;
    a.out = reinterpret_cast<float4 *>(out);
    a.rays_out = nullptr;
    a.err = ctx->d_err;
    dim3 grid((width + 15u) / 16u, (height + 7u) / 8u);
    k_pipeline<<<grid, 128, 0, static_cast<cudaStream_t>(stream)>>>(a);
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}

extern "C" rt_status rt_generate_primary_rays(rt_context *ctx, rt_stream stream, const rt_camera *camera,
                                              uint32_t width, uint32_t height, float tmin, float tmax,
                                              rt_ray *rays) {
    if (!ctx || !camera || !rays) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_generate_primary_rays: null argument");
    if (width == 0 || height == 0) return RT_OK;
    PipelineArgs a{};
    a.cam[0] = camera->position[0]; a.cam[1] = camera->position[1]; a.cam[2] = camera->position[2];
    camera_aspects(camera, width, height, &a.ay, &a.ax);
    a.width = width;
    a.height = height;
    a.tmin = tmin;
    a.tmax = tmax;
    a.rays_out = rays;
    a.err = ctx->d_err;
    dim3 grid((width + 15u) / 16u, (height + 7u) / 8u);
    k_pipeline<<<grid, 128, 0, static_cast<cudaStream_t>(stream)>>>(a);
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}
