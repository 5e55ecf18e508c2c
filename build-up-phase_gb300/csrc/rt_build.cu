// rt_build.cu -- LBVH -> compressed BVH8 builder (bottom and top level).
//
// Replaces vkCmdBuildAccelerationStructuresKHR (vulkan-raytraced-triangle/
// main.cpp:788-811 for the BLAS, :920-940 for the TLAS) whose work the
// reference leaves to the driver.  The steps the driver hides are explicit
// kernels, all stream-ordered, with no host synchronisation:
//
//   prep      triangle records (geometry transform applied, as Vulkan applies
//             transformData) or instance records + boxes + centroid bounds
//   morton    30- or 63-bit Morton code of each box centre, fused with the
//             digit histograms of the radix sort
//   sort      onesweep LSD radix sort (rt_sort.cu), stable
//   tree      binary radix tree over the sorted keys (Karras, HPG 2012;
//             index-augmented keys for duplicates), built bottom-up as in
//             Apetrei (2014) together with the boxes and SAH leaf decisions
//             (one exchange per node)
//   collapse  one cooperative kernel, breadth-first level by level, eight
//             lanes per wide node: greedy widening to 8 children, octant slot
//             assignment, 8-bit child-box quantisation (Ylitie, Karras,
//             Laine, HPG 2017); then every leaf record gathered into node
//             order by one thread each.  Node and record positions come from
//             grid-wide prefix sums, so the output is deterministic and equal
//             byte for byte to the CPU restatement of the same steps.
#include <cuda_runtime.h>

#include <cstring>

#include "rt_internal.h"


namespace rtc {

namespace {

constexpr int kMaxGeoms = 256;
constexpr int kCollapseThreads = 256;
constexpr int kMaxCoopBlocks = 4096;
constexpr uint32_t kNone = 0xffffffffu;

struct GeomParams {
    uint32_t n_geoms;
    uint32_t table[kMaxGeoms + 1];
    rt_geometry_triangles g[kMaxGeoms];
};

struct BuildLayout {
    uint64_t recs, boxes, keys0, keys1, ids0, ids1, bin, node_box, node_cost, leafable, other, leaf_box,
        wq, slots, desc, counts, blk, misc, sort, total;
};

inline uint32_t node_capacity_for(uint32_t n) { return n < 2 ? 1u : n - 1u; }

// Children per wide node from the build flags (0 = 8); 0 when invalid.
inline uint32_t build_width(uint32_t flags) {
    const uint32_t w = (flags & RT_BUILD_WIDTH_MASK) >> 16;
    if (w == 0u) return 8u;
    return (w >= 4u && w <= 8u) ? w : 0u;
}

BuildLayout build_layout(uint32_t n, uint32_t rec_bytes, int passes) {
    BuildLayout L;
    uint64_t off = 0;
    auto take = [&](uint64_t bytes) {
        uint64_t o = off;
        off += align_up(bytes > 0 ? bytes : 1, 256);
        return o;
    };
    uint64_t ni = n > 0 ? n - 1 : 0;
    uint64_t cap = node_capacity_for(n);
    L.recs = take((uint64_t)n * rec_bytes);
    L.boxes = take((uint64_t)n * 32u);
    L.keys0 = take((uint64_t)n * 8u);
    L.keys1 = take((uint64_t)n * 8u);
    L.ids0 = take((uint64_t)n * 4u);
    L.ids1 = take((uint64_t)n * 4u);
    L.bin = take(ni * 16u);
    L.node_box = take(ni * 32u);
    L.node_cost = take(ni * 4u);
    L.leafable = take(ni);
    L.other = take(ni * 8u);  // k_tree: per internal node, the first child's reference and far end
    L.leaf_box = take((uint64_t)n * 32u);
    L.wq = take(cap * 4u);
    L.slots = take(cap * 32u);
    L.desc = take(cap * 4u);
    L.counts = take(cap * 4u);
    L.blk = take((uint64_t)kMaxCoopBlocks * 8u);
    L.misc = take(256);
    L.sort = take(sort_scratch_bytes(n, passes));
    L.total = off;
    return L;
}

// table_entries: n_geoms + 1 for a BLAS (its geometry table), 0 for a TLAS.
uint64_t accel_bytes_for(uint32_t n, uint32_t rec_bytes, uint32_t table_entries) {
    uint64_t cap = node_capacity_for(n);
    uint64_t b = RT_ACCEL_HEADER_BYTES + cap * 80u + (uint64_t)n * rec_bytes + (uint64_t)table_entries * 4u;
    return align_up(b, 256);
}

// ---------------------------------------------------------------------------
// Device helpers
// ---------------------------------------------------------------------------

// Boxes in scratch: 32 bytes each (lo xyz, 0, hi xyz, 0), one L2 sector,
// moved as two 16-byte accesses; loads go through L2 (other blocks of the
// same launch write them).
__device__ __forceinline__ Box load_box(const float *b, uint32_t i) {
    const float4 *p = reinterpret_cast<const float4 *>(b) + (size_t)i * 2u;
    const float4 lo = __ldcg(p), hi = __ldcg(p + 1);
    Box x;
    x.lo[0] = lo.x; x.lo[1] = lo.y; x.lo[2] = lo.z;
    x.hi[0] = hi.x; x.hi[1] = hi.y; x.hi[2] = hi.z;
    return x;
}
__device__ __forceinline__ void store_box(float *b, uint32_t i, const Box &x) {
    float4 *p = reinterpret_cast<float4 *>(b) + (size_t)i * 2u;
    p[0] = make_float4(x.lo[0], x.lo[1], x.lo[2], 0.0f);
    p[1] = make_float4(x.hi[0], x.hi[1], x.hi[2], 0.0f);
}

__device__ __forceinline__ uint64_t spread3_21(uint32_t x) {
    uint64_t v = x & 0x1fffffu;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// Scene (centroid) bounds: per axis, the minimum and maximum of the
// order-preserving integers of a 256-thread block (redux.sync within each
// warp, shared memory across the eight warps), then one atomic per block and
// value.  Called by every thread of the block.
__device__ __forceinline__ void block_minmax_atomic(int32_t *cbounds, const int32_t (&mn)[3], const int32_t (&mx)[3]) {
    __shared__ int32_t s_mm[8][6];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int32_t wmn = __reduce_min_sync(0xffffffffu, mn[a]);
        const int32_t wmx = __reduce_max_sync(0xffffffffu, mx[a]);
        if (lane == 0) {
            s_mm[warp][a] = wmn;
            s_mm[warp][3 + a] = wmx;
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int v = threadIdx.x;
        int32_t r = s_mm[0][v];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = v < 3 ? min(r, s_mm[w][v]) : max(r, s_mm[w][v]);
        if (v < 3 && r != INT32_MAX) atomicMin(cbounds + v, r);
        if (v >= 3 && r != INT32_MIN) atomicMax(cbounds + v, r);
    }
}

// ---------------------------------------------------------------------------
// Header / init
// ---------------------------------------------------------------------------

__global__ void k_init(rt_accel_header hdr, uint8_t *accel, int32_t *cbounds, uint32_t *root, GeomParams gp,
                       uint32_t write_table) {
    int t = threadIdx.x;
    if (t == 0) *reinterpret_cast<rt_accel_header *>(accel) = hdr;
    if (t == 0) *root = kNone;  // the radix tree's root: none until k_tree completes it
    if (t < 3) { cbounds[t] = INT32_MAX; cbounds[3 + t] = INT32_MIN; }
    if (write_table) {
        uint32_t *tab = reinterpret_cast<uint32_t *>(accel + hdr.geom_offset);
        for (uint32_t g = (uint32_t)t; g <= gp.n_geoms; g += blockDim.x) tab[g] = gp.table[g];
    }
}

__global__ void k_empty_root(uint8_t *accel) {
    rt_accel_header *h = reinterpret_cast<rt_accel_header *>(accel);
    uint4 *node = reinterpret_cast<uint4 *>(accel + h->node_offset);
    node[0] = make_uint4(0, 0, 0, 0);
    node[1] = make_uint4(0, 0, 0, 0);
    node[2] = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
    node[3] = make_uint4(0xffffffffu, 0xffffffffu, 0, 0);
    node[4] = make_uint4(0, 0, 0, 0);
    h->node_count = 1;
    h->depth = 1;
    for (int a = 0; a < 4; ++a) { h->bounds_lo[a] = 0.0f; h->bounds_hi[a] = 0.0f; }
}

// ---------------------------------------------------------------------------
// prep
// ---------------------------------------------------------------------------

// Leaf record and box of triangle p of geometry g (build-input index gi):
// the three vertices (transformed when the geometry has a transform) in .xyz
// and the ids in .w; NaN vertices and the empty box for a triangle that is
// inactive (an index beyond max_vertex, a NaN coordinate).  Shared by the
// build and the refit.
__device__ bool tri_record(const GeomParams &gp, uint32_t g, uint32_t p, uint32_t gi, uint4 *r, Box &b,
                           uint32_t *err, uint32_t *hdr_status) {
    const rt_geometry_triangles &G = gp.g[g];
    float v[3][3];
    bool ok = true;
    for (int k = 0; k < 3; ++k) {
        uint32_t idx = G.index_type == RT_INDEX_UINT32 ? G.indices[3u * p + (uint32_t)k] : 3u * p + (uint32_t)k;
        if (idx > G.max_vertex) {
            ok = false;
            report_error(err, RT_ERR_BOUNDS, gi);
            if (hdr_status) atomicCAS(hdr_status, 0u, (uint32_t)(-RT_ERR_BOUNDS));
            break;
        }
        const float *src = reinterpret_cast<const float *>(reinterpret_cast<const uint8_t *>(G.vertices) +
                                                           (size_t)idx * G.vertex_stride);
        float pt[3] = {src[0], src[1], src[2]};
        if (G.transform) {
            const float *m = &G.transform->m[0][0];
            float mm[12];
#pragma unroll
            for (int q = 0; q < 12; ++q) mm[q] = __ldg(m + q);
            xform_point(mm, pt, v[k]);
        } else {
            v[k][0] = pt[0]; v[k][1] = pt[1]; v[k][2] = pt[2];
        }
    }
    if (ok)
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a)
                if (isnan(v[k][a])) ok = false;
    const float qnan = __int_as_float(0x7fc00000);
    r[0] = make_uint4(__float_as_uint(ok ? v[0][0] : qnan), __float_as_uint(ok ? v[0][1] : qnan),
                      __float_as_uint(ok ? v[0][2] : qnan), gi);
    r[1] = make_uint4(__float_as_uint(ok ? v[1][0] : qnan), __float_as_uint(ok ? v[1][1] : qnan),
                      __float_as_uint(ok ? v[1][2] : qnan), g);
    r[2] = make_uint4(__float_as_uint(ok ? v[2][0] : qnan), __float_as_uint(ok ? v[2][1] : qnan),
                      __float_as_uint(ok ? v[2][2] : qnan), p);
    b = box_empty();
    if (ok)
        for (int a = 0; a < 3; ++a) {
            b.lo[a] = fmn(fmn(v[0][a], v[1][a]), v[2][a]);
            b.hi[a] = fmx(fmx(v[0][a], v[1][a]), v[2][a]);
        }
    return ok;
}

__global__ void __launch_bounds__(256) k_prep_tris(const GeomParams gp, uint32_t n, uint4 *__restrict__ recs,
                                                    float *__restrict__ boxes, int32_t *cbounds, uint32_t *err,
                                                    uint32_t *hdr_status) {
    uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    int32_t cmin[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, cmax[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    if (gi < n) {
        // geometry g with table[g] <= gi < table[g+1]
        uint32_t lo = 0, hi = gp.n_geoms;
        while (hi - lo > 1u) {
            uint32_t mid = (lo + hi) >> 1;
            if (gp.table[mid] <= gi) lo = mid; else hi = mid;
        }
        const uint32_t g = lo;
        const uint32_t p = gi - gp.table[g];
        Box b;
        const bool ok = tri_record(gp, g, p, gi, recs + (size_t)gi * 3u, b, err, hdr_status);
        store_box(boxes, gi, b);
        if (ok)
            for (int a = 0; a < 3; ++a) {
                int32_t o = ford((b.lo[a] + b.hi[a]) * 0.5f);
                cmin[a] = o;
                cmax[a] = o;
            }
    }
    block_minmax_atomic(cbounds, cmin, cmax);
}

__device__ bool invert3x4(const float *m, float out[12]) {
    float a = m[0], b = m[1], c = m[2];
    float d = m[4], e = m[5], f = m[6];
    float g = m[8], h = m[9], i = m[10];
    float c00 = e * i - f * h, c01 = f * g - d * i, c02 = d * h - e * g;
    float det = (a * c00 + b * c01) + c * c02;
    if (!(det != 0.0f) || !isfinite(det)) return false;
    float r = 1.0f / det;
    float inv[9] = {c00 * r, (c * h - b * i) * r, (b * f - c * e) * r,
                    c01 * r, (a * i - c * g) * r, (c * d - a * f) * r,
                    c02 * r, (b * g - a * h) * r, (a * e - b * d) * r};
    for (int row = 0; row < 3; ++row) {
        for (int col = 0; col < 3; ++col) out[4 * row + col] = inv[3 * row + col];
        out[4 * row + 3] = -((inv[3 * row + 0] * m[3] + inv[3 * row + 1] * m[7]) + inv[3 * row + 2] * m[11]);
    }
    return true;
}

// Leaf record (world-to-object 3x4, BLAS address, custom index / mask, SBT
// offset / flags, instance index) and world box of instance i.  Shared by the
// build and the refit.
__device__ void inst_record(const rt_instance &I, uint32_t i, uint4 *r, Box &b) {
    const float *m = &I.transform.m[0][0];
    float w2o[12];
    bool ok = invert3x4(m, w2o);
    if (!ok)
        for (int q = 0; q < 12; ++q) w2o[q] = 0.0f;
    const rt_accel_header *bh = reinterpret_cast<const rt_accel_header *>(I.accel_ref);
    b = box_empty();
    if (ok && bh && bh->prim_count > 0) {
        for (int c = 0; c < 8; ++c) {
            float pt[3] = {(c & 1) ? bh->bounds_hi[0] : bh->bounds_lo[0],
                           (c & 2) ? bh->bounds_hi[1] : bh->bounds_lo[1],
                           (c & 4) ? bh->bounds_hi[2] : bh->bounds_lo[2]};
            float w[3];
            xform_point(m, pt, w);
            for (int a = 0; a < 3; ++a) { b.lo[a] = fmn(b.lo[a], w[a]); b.hi[a] = fmx(b.hi[a], w[a]); }
        }
    }
    r[0] = make_uint4(__float_as_uint(w2o[0]), __float_as_uint(w2o[1]), __float_as_uint(w2o[2]),
                      __float_as_uint(w2o[3]));
    r[1] = make_uint4(__float_as_uint(w2o[4]), __float_as_uint(w2o[5]), __float_as_uint(w2o[6]),
                      __float_as_uint(w2o[7]));
    r[2] = make_uint4(__float_as_uint(w2o[8]), __float_as_uint(w2o[9]), __float_as_uint(w2o[10]),
                      __float_as_uint(w2o[11]));
    r[3] = make_uint4((uint32_t)(I.accel_ref & 0xffffffffu), (uint32_t)(I.accel_ref >> 32), I.custom_index_and_mask,
                      I.sbt_offset_and_flags);
    r[4] = make_uint4(i, 0u, 0u, 0u);
}

__global__ void __launch_bounds__(256) k_prep_inst(const rt_instance *__restrict__ inst, uint32_t n,
                                                    uint4 *__restrict__ recs, float *__restrict__ boxes,
                                                    int32_t *cbounds) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    int32_t cmin[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, cmax[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    if (i < n) {
        const rt_instance I = inst[i];
        Box b;
        inst_record(I, i, recs + (size_t)i * 5u, b);
        store_box(boxes, i, b);
        if (!box_is_empty(b))
            for (int a = 0; a < 3; ++a) {
                int32_t o = ford((b.lo[a] + b.hi[a]) * 0.5f);
                cmin[a] = o;
                cmax[a] = o;
            }
    }
    block_minmax_atomic(cbounds, cmin, cmax);
}

// ---------------------------------------------------------------------------
// morton (+ radix histograms)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_morton(const float *__restrict__ boxes, uint32_t n,
                                                 const int32_t *__restrict__ cbounds, int bpa,
                                                 uint64_t *__restrict__ keys, uint32_t *__restrict__ ids,
                                                 uint32_t *__restrict__ hist, int passes) {
    __shared__ uint32_t sh[8 * 256];
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) sh[i] = 0u;
    __syncthreads();
    float lo[3], scale[3];
    const float maxq = (float)((1u << bpa) - 1u), cells = (float)(1u << bpa);
    const bool any = cbounds[0] != INT32_MAX;
    float cext = 0.0f;  // longest axis of the centroid bounds
    for (int a = 0; a < 3; ++a) {
        float l = any ? ford_inv(cbounds[a]) : 0.0f, h = any ? ford_inv(cbounds[3 + a]) : 0.0f;
        float ext = h - l;
        lo[a] = l;
        scale[a] = ext > 0.0f ? cells / ext : 0.0f;
        if (ext > cext) cext = ext;
    }
    const float large = RT_LARGE_PRIM_FRACTION * cext;
    const uint64_t large_bit = bpa == 21 ? (1ull << 63) : (1ull << 31);
    const uint64_t inactive = bpa == 21 ? ((1ull << 63) - 1ull) : ((1ull << 30) - 1ull);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        Box b = load_box(boxes, i);
        uint64_t key;
        if (box_is_empty(b)) {
            key = inactive;
        } else {
            uint32_t q[3];
            for (int a = 0; a < 3; ++a) {
                float c = (b.lo[a] + b.hi[a]) * 0.5f;
                float f = (c - lo[a]) * scale[a];
                q[a] = !(f > 0.0f) ? 0u : (f >= maxq ? (uint32_t)maxq : (uint32_t)f);
            }
            key = spread3_21(q[0]) | (spread3_21(q[1]) << 1) | (spread3_21(q[2]) << 2);
            float e = 0.0f;  // longest axis of the primitive's box
            for (int a = 0; a < 3; ++a) {
                const float x = b.hi[a] - b.lo[a];
                if (x > e) e = x;
            }
            if (e > large) key |= large_bit;
        }
        keys[i] = key;
        ids[i] = i;
        for (int p = 0; p < passes; ++p) atomicAdd(&sh[p * 256 + ((key >> (8 * p)) & 0xffu)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        uint32_t c = sh[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// ---------------------------------------------------------------------------
// Radix tree + refit + SAH leaf decisions in one pass
// ---------------------------------------------------------------------------
//
// The binary radix tree over the sorted keys (Karras 2012: every internal
// node splits its key range where the keys' common prefix ends, equal keys
// ordered by index) built bottom-up as in Apetrei 2014 ("Fast and Simple
// Agglomerative LBVH Construction"): one thread per leaf climbs; a node
// covering keys [l, r] is the left child of the node split between keys r
// and r + 1, or the right child of the node split between l - 1 and l --
// whichever boundary's keys share the longer prefix (never equal: the keys
// are unique with their indices).  Internal node i is the one split between
// keys i and i + 1.  The first child to reach a node exchanges its reference
// and the far end of its range into the node's 64-bit word; the second child
// gets them back, so it knows its sibling and the node's range, and
// computes the node: box, SAH cost and the leaf decision (the refit), then
// climbs on.  Same tree as a top-down Karras construction, in one launch and
// without its per-node searches.

// Common-prefix length of the keys on either side of boundary b | b + 1, the
// index breaking ties between equal keys.
__device__ __forceinline__ int boundary_delta(uint64_t ka, uint64_t kb, uint32_t b) {
    if (ka == kb) return 64 + __clz((int)(b ^ (b + 1u)));
    return __clzll((long long)(ka ^ kb));
}

struct TreeArgs {
    uint32_t n;
    const uint64_t *keys;  // sorted
    const uint32_t *ids;   // build-input primitive of each sorted key
    const float *boxes;
    uint4 *bin;            // internal node i: left, right, first, last
    float *node_box;
    float *node_cost;
    uint8_t *leafable;
    uint64_t *other;       // per internal node: all ones, then the first child's reference and far end
    float *leaf_box;
    uint32_t *root;        // the root's reference
    uint32_t *err;
};

// Exchange with release (this thread's box and cost stores are visible to
// the thread that reads the value) and acquire (the first child's stores are
// visible to this thread's later loads) at device scope.
__device__ __forceinline__ uint64_t exch_acq_rel(uint64_t *p, uint64_t v) {
    uint64_t old;
    asm volatile("atom.acq_rel.gpu.global.exch.b64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}

// The root k_tree completed: a completed root is reached only through nodes
// completed in this build, every reference in range.  If keys left out of
// order by a sort that gave up kept it from completing one, leaf 0 stands in
// and RT_ERR_BOUNDS is recorded, so the collapse reads nothing out of range.
__global__ void k_tree_root(uint32_t *root, uint32_t n, uint32_t *err) {
    const uint32_t r = *root, i = r & ~kLeafBit;
    if ((r & kLeafBit) ? i < n : i + 1u < n) return;
    report_error(err, RT_ERR_BOUNDS, 0x66000000u | (i & 0xffffffu));
    *root = kLeafBit;
}

// Six blocks per SM (40 registers): more climbs in flight than the five of
// an unbounded register count (1M soup build 0.718 -> 0.715 ms, 2M box 1.336
// -> 1.322 ms).
__global__ void __launch_bounds__(256, 6) k_tree(TreeArgs a) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = a.n;
    if (j >= n) return;
    // the leaf's box and the keys around its range, in one round of loads
    const uint32_t id = __ldg(a.ids + j);
    uint64_t kl = __ldg(a.keys + j), kr = kl;
    uint64_t klm = j > 0 ? __ldg(a.keys + j - 1) : 0ull, krp = j + 1 < n ? __ldg(a.keys + j + 1) : 0ull;
    if (id >= n) report_error(a.err, RT_ERR_BOUNDS, 0x67000000u | (j & 0xffffffu));  // not a sorted id
    const Box lb = id < n ? load_box(a.boxes, id) : box_empty();
    store_box(a.leaf_box, j, lb);
    if (n < 2) return;
    uint32_t me = kLeafBit | j, l = j, r = j;
    Box mb = lb;
    float mcost = RT_SAH_PRIM;
    // A radix tree over 2^30 keys is at most 96 levels deep (63 key bits +
    // 32 index bits); the cap only guards against inconsistent keys.
    for (int climb = 0;; ++climb) {
        if (climb >= 256) {
            report_error(a.err, RT_ERR_BOUNDS, 0x61000000u | j);
            return;
        }
        const bool left = l == 0u ? true : (r == n - 1u ? false : boundary_delta(kr, krp, r) > boundary_delta(klm, kl, l - 1u));
        const uint32_t p = left ? r : l - 1u;
        const uint64_t got = exch_acq_rel(a.other + p, ((uint64_t)me << 32) | (left ? l : r));
        if (got == ~0ull) return;  // first child here: the sibling computes the node
        const uint32_t sib = (uint32_t)(got >> 32), far = (uint32_t)got;
        const uint32_t nl = left ? l : far, nr = left ? far : r;
        if (nl > nr || nr >= n) {
            report_error(a.err, RT_ERR_BOUNDS, 0x61000000u | j);
            return;
        }
        // the sibling's box and cost and the keys around the node's range,
        // in one round of loads
        const uint64_t k_nl = left ? kl : __ldg(a.keys + nl), k_nr = left ? __ldg(a.keys + nr) : kr;
        const uint64_t k_nlm = nl > 0u ? __ldg(a.keys + nl - 1u) : 0ull;
        const uint64_t k_nrp = nr + 1u < n ? __ldg(a.keys + nr + 1u) : 0ull;
        const bool sl = (sib & kLeafBit) != 0u;
        const Box sb = sl ? load_box(a.leaf_box, sib & ~kLeafBit) : load_box(a.node_box, sib);
        const float scost = sl ? RT_SAH_PRIM : __ldcg(a.node_cost + sib);
        const Box &bl = left ? mb : sb, &br = left ? sb : mb;
        const float cl = left ? mcost : scost, cr = left ? scost : mcost;
        const Box b = box_union(bl, br);
        const float an = half_area(b);
        float split;
        if (an > 0.0f) {
            const float sah = half_area(bl) * cl + half_area(br) * cr;
            split = RT_SAH_NODE + sah / an;
        } else {
            split = RT_SAH_NODE + (cl + cr);
        }
        const uint32_t count = nr - nl + 1u;
        const float leaf = (float)count * RT_SAH_PRIM;
        const bool lf = count <= (uint32_t)RT_MAX_LEAF_PRIMS && leaf <= split;
        mcost = lf ? leaf : split;
        store_box(a.node_box, p, b);
        a.node_cost[p] = mcost;
        a.leafable[p] = lf ? 1 : 0;
        a.bin[p] = make_uint4(left ? me : sib, left ? sib : me, nl, nr);
        mb = b;
        me = p;
        l = nl;
        r = nr;
        kl = k_nl;
        kr = k_nr;
        klm = k_nlm;
        krp = k_nrp;
        if (l == 0u && r == n - 1u) {
            *a.root = p;
            return;
        }
    }
}

// ---------------------------------------------------------------------------
// collapse (cooperative, breadth-first)
// ---------------------------------------------------------------------------

struct CollapseArgs {
    uint32_t n;
    uint32_t width;      // children per wide node, 4..8
    uint32_t capacity;
    uint32_t root_ref;
    const uint32_t *root_dev;  // when set: the root's reference, read on the device
    uint32_t *gather;  // per leaf record in node order: its sorted primitive
    const uint4 *bin;
    const float *node_box;
    const uint8_t *leafable;
    const float *leaf_box;
    uint32_t *wq;
    uint32_t *slots;
    uint32_t *desc;
    uint32_t *counts;
    uint32_t *blk;
    uint4 *nodes_out;
    rt_accel_header *hdr;
    uint32_t *bar;  // grid barrier: arrival count, generation (zeroed before the launch)
    uint32_t *err;
};

__device__ __forceinline__ bool ref_is_leaf(uint32_t r) { return (r & kLeafBit) != 0u; }
__device__ __forceinline__ Box ref_box(const CollapseArgs &a, uint32_t r) {
    return load_box(ref_is_leaf(r) ? a.leaf_box : a.node_box, r & ~kLeafBit);
}

// One child reference as the collapse sees it.  The box, the SAH leaf flag
// and the binary node are independent loads (all written by earlier kernels
// of the build, so read through the non-coherent path), issued together: the
// greedy widening costs one round trip per opened node instead of one per
// child and step.
struct RefInfo {
    uint32_t ref;
    uint32_t kid0, kid1;  // binary children of an opened node; kid0 of a leaf child: its first sorted primitive
    uint32_t cnt;         // primitives below; bit 31: internal and not a SAH leaf (gets widened)
    float area;           // half surface area of the box
};
constexpr uint32_t kOpenBit = 0x80000000u;

__device__ __forceinline__ Box load_box_ro(const CollapseArgs &a, uint32_t r) {
    const float4 *p = reinterpret_cast<const float4 *>(ref_is_leaf(r) ? a.leaf_box : a.node_box) +
                      (size_t)(r & ~kLeafBit) * 2u;
    const float4 lo = __ldg(p), hi = __ldg(p + 1);
    Box b;
    b.lo[0] = lo.x; b.lo[1] = lo.y; b.lo[2] = lo.z;
    b.hi[0] = hi.x; b.hi[1] = hi.y; b.hi[2] = hi.z;
    return b;
}

__device__ __forceinline__ RefInfo fetch_ref(const CollapseArgs &a, uint32_t r) {
    const bool leaf = ref_is_leaf(r);
    const uint32_t i = r & ~kLeafBit;
    const Box b = load_box_ro(a, r);
    uint4 nd = make_uint4(0u, 0u, 0u, 0u);
    uint32_t lf = 1u;
    if (!leaf) {
        nd = __ldg(a.bin + i);
        lf = __ldg(a.leafable + i);
    }
    RefInfo x;
    x.ref = r;
    const bool open = !leaf && lf == 0u;
    x.kid0 = leaf ? i : (open ? nd.x : nd.z);
    x.kid1 = nd.y;
    x.cnt = (leaf ? 1u : nd.w - nd.z + 1u) | (open ? kOpenBit : 0u);
    x.area = half_area(b);
    return x;
}
__device__ __forceinline__ bool info_open(const RefInfo &x) { return (x.cnt & kOpenBit) != 0u; }

// RefInfo of lane `src` (every lane of the warp takes part).
__device__ __forceinline__ RefInfo shfl_info(const RefInfo &x, int src) {
    RefInfo y;
    y.ref = __shfl_sync(0xffffffffu, x.ref, src);
    y.kid0 = __shfl_sync(0xffffffffu, x.kid0, src);
    y.kid1 = __shfl_sync(0xffffffffu, x.kid1, src);
    y.cnt = __shfl_sync(0xffffffffu, x.cnt, src);
    y.area = __shfl_sync(0xffffffffu, x.area, src);
    return y;
}

// Quantisation frame of a wide node: the origin (lower corner) and per-axis
// power-of-two scales of its 8-bit child boxes.
struct QFrame {
    float p[3];
    int e[3];
    bool empty;
};

__device__ __forceinline__ QFrame node_frame(const Box &node) {
    QFrame f;
    f.empty = box_is_empty(node);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        f.p[q] = f.empty ? 0.0f : node.lo[q];
        f.e[q] = f.empty ? 0 : qexp_for(__fsub_ru(node.hi[q], f.p[q]));
    }
    return f;
}

// 8-bit bounds of a child box in the frame, rounded outward (lower bounds
// down, upper bounds up) so the quantised box contains the exact one; an
// unused slot, an empty node or an empty child gets the inverted box
// (255, 0).
__device__ __forceinline__ void quantise_child(const QFrame &f, bool used, const Box &b, uint32_t ql[3],
                                               uint32_t qh[3]) {
    const bool inv = !used || f.empty || box_is_empty(b);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        ql[a] = 255u;
        qh[a] = 0u;
        if (inv) continue;
        const float sc = pow2f(-f.e[a]);
        const float dl = __fsub_rd(b.lo[a], f.p[a]) * sc;
        const float dh_raw = __fsub_ru(b.hi[a], f.p[a]);
        const float dh = dh_raw * sc;
        const float fl = floorf(dl), fh = ceilf(dh);
        ql[a] = fl < 0.0f ? 0u : (fl > 255.0f ? 255u : (uint32_t)(int)fl);
        qh[a] = fh < 0.0f ? 0u : (fh > 255.0f ? 255u : (uint32_t)(int)fh);
        if (qh[a] == 0u && dh_raw > 0.0f) qh[a] = 1u;
    }
}

// Word 0 of a wide node: origin, exponents and internal-child mask.
__device__ __forceinline__ uint4 frame_word(const QFrame &f, uint32_t imask) {
    const uint32_t w = ((uint32_t)(uint8_t)(int8_t)f.e[0]) | ((uint32_t)(uint8_t)(int8_t)f.e[1] << 8) |
                       ((uint32_t)(uint8_t)(int8_t)f.e[2] << 16) | (imask << 24);
    return make_uint4(__float_as_uint(f.p[0]), __float_as_uint(f.p[1]), __float_as_uint(f.p[2]), w);
}

// Words 0, 2, 3, 4 of a wide node from its box and its slots' boxes: the
// child boxes as six byte planes (lo x, lo y, lo z, hi x, hi y, hi z), byte s
// of a plane for slot s.  Used by the refit; the build's phase A writes the
// same bytes one slot per lane.
__device__ void encode_node(const Box &node, const Box sbox[8], const bool used[8], uint32_t imask, uint4 *o) {
    const QFrame f = node_frame(node);
    uint32_t q[12] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        uint32_t ql[3], qh[3];
        quantise_child(f, used[s], sbox[s], ql, qh);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            q[2 * a + (s >> 2)] |= ql[a] << (8 * (s & 3));
            q[6 + 2 * a + (s >> 2)] |= qh[a] << (8 * (s & 3));
        }
    }
    o[0] = frame_word(f, imask);
    o[2] = make_uint4(q[0], q[1], q[2], q[3]);
    o[3] = make_uint4(q[4], q[5], q[6], q[7]);
    o[4] = make_uint4(q[8], q[9], q[10], q[11]);
}

// ---------------------------------------------------------------------------
// Phase A, eight lanes per wide node.  Lane j of an aligned group of eight
// holds child j during the widening and the slot assignment, and the group's
// choices are made with shuffles (every lane reaches the same result), so a
// node costs a round trip per level of its treelet's top three binary levels
// (fetched before the widening), one per node opened below them, and a few
// hundred instructions per lane.  Every loop that shuffles is warp-uniform: all 32 lanes run each
// shuffle, groups that are done (or hold no node) take part with `act` off.
// ---------------------------------------------------------------------------

constexpr unsigned kFullMask = 0xffffffffu;

// Lane (0-7) of the largest key among the group's lanes with `ok`, the
// lowest lane on ties; -1 if none.  Keys are > -1 (never NaN) where `ok`.
__device__ __forceinline__ int group_argmax(float key, bool ok) {
    float v = ok ? key : -1.0f;
    int i = ok ? (int)(threadIdx.x & 7u) : 8;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        const float v2 = __shfl_xor_sync(kFullMask, v, o);
        const int i2 = __shfl_xor_sync(kFullMask, i, o);
        if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
    }
    return i < 8 ? i : -1;
}

// Lane of the least key among the lanes with `ok`, the lowest lane on ties;
// -1 if none.  Keys are never NaN where `ok`.
__device__ __forceinline__ int group_argmin(float key, bool ok) {
    float v = ok ? key : kInf;
    int i = ok ? (int)(threadIdx.x & 7u) : 8;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        const float v2 = __shfl_xor_sync(kFullMask, v, o);
        const int i2 = __shfl_xor_sync(kFullMask, i, o);
        if (v2 < v || (v2 == v && i2 < i)) { v = v2; i = i2; }
    }
    return i < 8 ? i : -1;
}

// Phase A of wide node k (the lanes of a group with `valid` false take part
// in the shuffles only):
//  - widening: while fewer than `width` children, open the openable child of
//    largest surface area, the first on ties;
//  - slots: repeatedly the (child, slot) pair of least cost (x + y) + z, the
//    centre offset signed by the slot's octant.  The sequential scan in
//    (child, slot) order keeps its first pair when that pair's cost is NaN
//    (nothing compares below NaN) and otherwise ends on the first least
//    non-NaN pair; each lane finds its own child's first least non-NaN slot
//    and the group takes the least of those, or the first pair when its
//    cost is NaN -- the same choice;
//  - words 0, 2, 3, 4 of the node, the child boxes stored as bytes, one
//    slot per lane.
// Leaves for phase B, per slot, the child node (internal) or the first
// sorted primitive (leaf) in `slots`, and in `desc` the internal-child mask
// (bits 0-7) and each leaf slot's primitive count minus one (two bits per
// slot from bit 8).  Returns the node's internal children and primitives
// (every lane of the group).
__device__ __forceinline__ void collapse_phase_a(const CollapseArgs &a, uint32_t k, bool valid, uint32_t &n_int, uint32_t &n_prim) {
    const int j = (int)(threadIdx.x & 7u);
    const int gb = (int)(threadIdx.x & 24u);
    // wq and the hand-off arrays are written by other blocks of this launch
    // between grid barriers: read through L2 (__ldcg), never a stale L1 line.
    uint32_t sref = 0u;
    RefInfo src = {0u, 0u, 0u, 0u, 0.0f};
    if (valid) {
        sref = __ldcg(a.wq + k);
        src = fetch_ref(a, sref);
    }
    // The treelet's top three binary levels are fetched up front, one round
    // trip per level for the whole group: t1 (lanes 0-1), t2 (lanes 0-3) and
    // t3 (lanes 0-7) hold the nodes at depth 1, 2 and 3 below the wide
    // node's root, node i's children at 2i and 2i + 1 of the next depth
    // (empty where the parent is not opened).  The widening then finds the
    // children of an opened node in these tables by shuffles; only a node
    // opened below depth 3 has its children fetched when it is opened.
    const bool src_open = valid && info_open(src);
    RefInfo t1 = {0u, 0u, 0u, 0u, 0.0f}, t2 = t1, t3 = t1;
    if (src_open && j < 2) t1 = fetch_ref(a, j == 0 ? src.kid0 : src.kid1);
    {
        const RefInfo par = shfl_info(t1, gb | ((j >> 1) & 1));
        if (src_open && j < 4 && info_open(par)) t2 = fetch_ref(a, (j & 1) ? par.kid1 : par.kid0);
    }
    {
        const RefInfo par = shfl_info(t2, gb | ((j >> 1) & 3));
        if (src_open && info_open(par)) t3 = fetch_ref(a, (j & 1) ? par.kid1 : par.kid0);
    }
    // mine: this lane's child, at depth mdepth (4: below the tables) and
    // index midx of its depth
    RefInfo mine = {0u, 0u, 0u, 0u, 0.0f};
    uint32_t mdepth = 0u, midx = 0u;
    int n = 0;
    if (valid) {
        if (!src_open) {
            n = 1;
            if (j == 0) mine = src;
        } else {
            n = 2;
            if (j < 2) {
                mine = t1;
                mdepth = 1u;
                midx = (uint32_t)j;
            }
        }
    }
    bool act = src_open;
    for (;;) {
        act = act && n < (int)a.width;
        if (!__any_sync(kFullMask, act)) break;
        const int best = group_argmax(mine.area, act && j < n && info_open(mine) && mine.area > -1.0f);
        const int from = gb | (best < 0 ? 0 : best);
        if (best < 0) act = false;
        // the opened child's depth and index (the same on every lane of the group)
        const uint32_t bd = __shfl_sync(kFullMask, mdepth, from);
        const uint32_t bi = __shfl_sync(kFullMask, midx, from);
        const bool deep = bd >= 3u;
        RefInfo f0 = {0u, 0u, 0u, 0u, 0.0f}, f1 = f0;
        if (act && deep && j == best) {
            f0 = fetch_ref(a, mine.kid0);
            f1 = fetch_ref(a, mine.kid1);
        }
        const RefInfo tab = bd == 1u ? t2 : t3;
        const RefInfo k0 = shfl_info(deep ? f0 : tab, deep ? from : (gb | (int)((2u * bi) & 7u)));
        const RefInfo k1 = shfl_info(deep ? f1 : tab, deep ? from : (gb | (int)((2u * bi + 1u) & 7u)));
        if (act) {
            if (j == best) {
                mine = k0;
                mdepth = deep ? 4u : bd + 1u;
                midx = 2u * bi;
            } else if (j == n) {
                mine = k1;
                mdepth = deep ? 4u : bd + 1u;
                midx = 2u * bi + 1u;
            }
            ++n;
        }
    }

    // slot costs of this lane's child
    const Box nb = valid ? load_box_ro(a, sref) : box_empty();
    const bool have = valid && j < n;
    const Box cb = have ? load_box_ro(a, mine.ref) : box_empty();
    const bool ne = box_is_empty(nb), ce = box_is_empty(cb);
    float d[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float ncen = (nb.lo[q] + nb.hi[q]) * 0.5f;
        d[q] = (ce || ne) ? 0.0f : (cb.lo[q] + cb.hi[q]) * 0.5f - ncen;
    }
    float cost[8];
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const float x = (s & 1) ? -d[0] : d[0];
        const float y = (s & 2) ? -d[1] : d[1];
        const float z = (s & 4) ? -d[2] : d[2];
        cost[s] = (x + y) + z;
    }
    uint32_t used = 0u;
    int my_slot = -1;
    for (int it = 0; it < 8; ++it) {
        const bool go = valid && it < n;
        if (!__any_sync(kFullMask, go)) break;
        const bool cand = go && j < n && my_slot < 0;
        const int s0 = __ffs((int)(~used & 0xffu)) - 1;
        float c0 = 0.0f, v = kInf;
        int vs = -1;
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            if (s == s0) c0 = cost[s];
            if (((used >> s) & 1u) == 0u && !isnan(cost[s]) && (vs < 0 || cost[s] < v)) {
                v = cost[s];
                vs = s;
            }
        }
        const uint32_t cm = (__ballot_sync(kFullMask, cand) >> gb) & 0xffu;
        const int l0 = __ffs((int)cm) - 1;
        const bool nan0 = __shfl_sync(kFullMask, isnan(c0) ? 1 : 0, gb | (l0 < 0 ? 0 : l0)) != 0;
        int bc = group_argmin(v, cand && vs >= 0);
        int bs = __shfl_sync(kFullMask, vs, gb | (bc < 0 ? 0 : bc));
        if (nan0) {
            bc = l0;
            bs = s0;
        }
        if (go && bc >= 0) {
            if (j == bc) my_slot = bs;
            used |= 1u << bs;
        }
    }

    // phase-B hand-off and the node's counts
    const bool open = have && info_open(mine);
    const uint32_t cnt = mine.cnt & ~kOpenBit;
    uint32_t dbits = 0u, tally = 0u;
    if (have && my_slot >= 0) {
        if (open) {
            dbits = 1u << my_slot;
            tally = 1u;
        } else {
            dbits = (cnt - 1u) << (8 + 2 * my_slot);
            tally = cnt << 16;
        }
    }
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        dbits |= __shfl_xor_sync(kFullMask, dbits, o);
        tally += __shfl_xor_sync(kFullMask, tally, o);
    }
    n_int = tally & 0xffffu;
    n_prim = tally >> 16;
    if (!valid) return;

    const QFrame f = node_frame(nb);
    uint8_t *nbytes = reinterpret_cast<uint8_t *>(a.nodes_out + (size_t)k * 5u);
    if (have && my_slot >= 0) {
        uint32_t ql[3], qh[3];
        quantise_child(f, true, cb, ql, qh);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            nbytes[32 + 8 * q + my_slot] = (uint8_t)ql[q];
            nbytes[56 + 8 * q + my_slot] = (uint8_t)qh[q];
        }
        a.slots[(size_t)k * 8u + my_slot] = open ? mine.ref : mine.kid0;
    }
    if (((used >> j) & 1u) == 0u) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            nbytes[32 + 8 * q + j] = 255;
            nbytes[56 + 8 * q + j] = 0;
        }
        a.slots[(size_t)k * 8u + j] = kNone;
    }
    if (j == 0) {
        a.nodes_out[(size_t)k * 5u] = frame_word(f, dbits & 0xffu);
        a.desc[k] = dbits;
    }
}

// Phase B of wide node k, once its child and record bases are known: word 1
// of the node (bases and slot metadata), its internal children appended to
// the next level's queue, and for each of its leaf records the sorted
// primitive it holds (the gather map; k_gather_records moves the records).
__device__ void collapse_phase_b(const CollapseArgs &a, uint32_t k, uint32_t child_base, uint32_t prim_base) {
    const uint4 *sp = reinterpret_cast<const uint4 *>(a.slots + (size_t)k * 8u);
    const uint4 s0 = __ldcg(sp), s1 = __ldcg(sp + 1);
    const uint32_t desc = __ldcg(a.desc + k);
    const uint32_t slot[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
    uint32_t meta_lo = 0u, meta_hi = 0u, off = 0u, ichild = 0u;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        if (slot[s] == kNone) continue;
        uint32_t m;
        if ((desc >> s) & 1u) {
            m = (1u << 5) | (24u + (uint32_t)s);
            const uint32_t dst = child_base + ichild++;
            if (dst < a.capacity) a.wq[dst] = slot[s];
            else report_error(a.err, RT_ERR_BOUNDS, 0x60000000u | k);
        } else {
            const uint32_t c = ((desc >> (8u + 2u * s)) & 3u) + 1u;
            m = (((1u << c) - 1u) << 5) | off;
            for (uint32_t j = 0; j < c; ++j) {
                const uint32_t d = prim_base + off + j;
                if (d < a.n) a.gather[d] = slot[s] + j;
                else report_error(a.err, RT_ERR_BOUNDS, 0x63000000u | k);
            }
            off += c;
        }
        if (s < 4) meta_lo |= m << (8 * s);
        else meta_hi |= m << (8 * (s - 4));
    }
    a.nodes_out[(size_t)k * 5u + 1u] = make_uint4(child_base, prim_base, meta_lo, meta_hi);
}

template <int N>
__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t *s_red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    uint32_t s = 0;
    for (int i = 0; i < N / 32; ++i) s += s_red[i];
    __syncthreads();
    return s;
}

// Block-wide sums of four values at once (one shared-memory round instead
// of four).
template <int N>
__device__ __forceinline__ uint4 block_sum4(uint4 v, uint4 *s_red4) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
        v.w += __shfl_xor_sync(0xffffffffu, v.w, o);
    }
    if ((threadIdx.x & 31) == 0) s_red4[threadIdx.x >> 5] = v;
    __syncthreads();
    uint4 s = make_uint4(0u, 0u, 0u, 0u);
    for (int i = 0; i < N / 32; ++i) {
        const uint4 c = s_red4[i];
        s.x += c.x; s.y += c.y; s.z += c.z; s.w += c.w;
    }
    __syncthreads();
    return s;
}

template <int N>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *s_red, uint32_t &total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_red[w] = x;
    __syncthreads();
    uint32_t before = 0, tot = 0;
    for (int i = 0; i < N / 32; ++i) {
        uint32_t c = s_red[i];
        if (i < w) before += c;
        tot += c;
    }
    __syncthreads();
    total = tot;
    return before + x - v;
}

// Grid-wide barrier of the cooperative collapse (its blocks are co-resident):
// one arrival per block on a global counter, the last arrival opens the next
// generation.  The wait is bounded: a block that gives up records
// RT_ERR_TIMEOUT and returns false (the collapse then stops).
constexpr uint32_t kCoopSpin = 1u << 22;
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ bool coop_sync(uint32_t *bar, uint32_t nblocks, uint32_t *err, uint32_t code) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const uint32_t gen = ld_acquire_u32(bar + 1);
        __threadfence();
        if (atomicAdd(bar, 1u) + 1u == nblocks) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            uint32_t it = 0;
            while (ld_acquire_u32(bar + 1) == gen && ++it < kCoopSpin) {
            }
            if (it >= kCoopSpin) {
                report_error(err, RT_ERR_TIMEOUT, code);
                ok = 0;
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

__global__ void __launch_bounds__(kCollapseThreads, 4) k_collapse(CollapseArgs a) {
    __shared__ uint32_t s_red[kCollapseThreads / 32];
    __shared__ uint4 s_red4[kCollapseThreads / 32];
    const uint32_t G = gridDim.x, b = blockIdx.x, t = threadIdx.x;
    const uint32_t root_ref = a.root_dev ? __ldcg(a.root_dev) : a.root_ref;
    if (b == 0 && t == 0) a.wq[0] = root_ref;
    if (!coop_sync(a.bar, G, a.err, 0x64000000u)) return;
    uint32_t level_start = 0, level_count = 1, prim_next = 0, depth = 0;
    // Every block evaluates the same level sizes, so all leave together; the
    // level cap (a wide tree is never deeper than its <= 96-level binary
    // tree) only guards against corrupt inputs.
    while (level_count > 0) {
        if (depth >= 256 || level_start + level_count > a.capacity) {
            if (b == 0 && t == 0) report_error(a.err, RT_ERR_BOUNDS, 0x62000000u | depth);
            break;
        }
        ++depth;
        const uint32_t chunk = (level_count + G - 1u) / G;
        const uint32_t c0 = min(b * chunk, level_count), c1 = min(c0 + chunk, level_count);
        uint32_t my_int = 0, my_prim = 0;
        // eight lanes per node (collapse_phase_a); the loop is block-uniform
        for (uint32_t kb = c0; kb < c1; kb += kCollapseThreads / 8u) {
            const uint32_t k = kb + (t >> 3);
            const bool valid = k < c1;
            uint32_t ni, np;
            collapse_phase_a(a, level_start + k, valid, ni, np);
            if (valid && (t & 7u) == 0u) {
                a.counts[level_start + k] = ni | (np << 16);
                my_int += ni;
                my_prim += np;
            }
        }
        {
            const uint4 bs = block_sum4<kCollapseThreads>(make_uint4(my_int, my_prim, 0u, 0u), s_red4);
            my_int = bs.x;
            my_prim = bs.y;
        }
        if (t == 0) { a.blk[2 * b] = my_int; a.blk[2 * b + 1] = my_prim; }
        if (!coop_sync(a.bar, G, a.err, 0x64000000u | depth)) return;
        uint32_t pre_i = 0, pre_p = 0, tot_i = 0, tot_p = 0;
        for (uint32_t q = t; q < G; q += kCollapseThreads) {
            uint32_t vi = __ldcg(a.blk + 2 * q), vp = __ldcg(a.blk + 2 * q + 1);
            tot_i += vi;
            tot_p += vp;
            if (q < b) { pre_i += vi; pre_p += vp; }
        }
        {
            const uint4 bs = block_sum4<kCollapseThreads>(make_uint4(pre_i, pre_p, tot_i, tot_p), s_red4);
            pre_i = bs.x;
            pre_p = bs.y;
            tot_i = bs.z;
            tot_p = bs.w;
        }
        const uint32_t next_start = level_start + level_count;
        uint32_t run_i = pre_i, run_p = pre_p;
        for (uint32_t kb = c0; kb < c1; kb += kCollapseThreads) {
            const uint32_t k = kb + t;
            const bool valid = k < c1;
            const uint32_t packed = valid ? __ldcg(a.counts + level_start + k) : 0u;
            uint32_t total;
            const uint32_t ex = block_excl_scan<kCollapseThreads>(packed, s_red, total);
            if (valid)
                collapse_phase_b(a, level_start + k, next_start + run_i + (ex & 0xffffu),
                                 prim_next + run_p + (ex >> 16));
            run_i += total & 0xffffu;
            run_p += total >> 16;
        }
        level_start = next_start;
        level_count = tot_i;
        prim_next += tot_p;
        if (!coop_sync(a.bar, G, a.err, 0x65000000u | depth)) return;
    }
    if (b == 0 && t == 0) {
        Box rb = ref_box(a, root_ref);
        a.hdr->node_count = level_start;
        a.hdr->depth = depth;
        for (int q = 0; q < 3; ++q) { a.hdr->bounds_lo[q] = rb.lo[q]; a.hdr->bounds_hi[q] = rb.hi[q]; }
        a.hdr->bounds_lo[3] = 0.0f;
        a.hdr->bounds_hi[3] = 0.0f;
    }
}

// Leaf records in node order: record d is the input record of sorted
// primitive gather[d] (written by the collapse's phase B).  One thread per
// record; the grid covers every record.  An index out of range (only an
// incomplete tree leaves one) records RT_ERR_BOUNDS and a zero record.
template <int RW>
__global__ void __launch_bounds__(256) k_gather_records(const uint4 *__restrict__ recs_in, uint4 *__restrict__ recs_out,
                                                        const uint32_t *__restrict__ ids,
                                                        const uint32_t *__restrict__ gather, uint32_t n, uint32_t *err) {
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    const uint32_t gi = __ldg(gather + d);
    const uint32_t id = gi < n ? __ldg(ids + gi) : n;
    uint4 *dst = recs_out + (size_t)d * RW;
    uint4 r[RW];
    if (id >= n) {
        report_error(err, RT_ERR_BOUNDS, 0x68000000u | (d & 0xffffffu));
#pragma unroll
        for (int w = 0; w < RW; ++w) dst[w] = make_uint4(0u, 0u, 0u, 0u);
        return;
    }
    const uint4 *src = recs_in + (size_t)id * RW;
#pragma unroll
    for (int w = 0; w < RW; ++w) r[w] = __ldg(src + w);
#pragma unroll
    for (int w = 0; w < RW; ++w) dst[w] = r[w];
}

// ---------------------------------------------------------------------------
// Host driver shared by BLAS and TLAS
// ---------------------------------------------------------------------------

int coop_grid(rt_context *ctx) {
    static int cached_dev = -1, cached = 0;
    if (cached_dev == ctx->device) return cached;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_collapse, kCollapseThreads, 0) != cudaSuccess)
        return 0;
    int g = per_sm * ctx->sm_count;
    if (g > kMaxCoopBlocks) g = kMaxCoopBlocks;
    cached = g;
    cached_dev = ctx->device;
    return g;
}

struct BuildCall {
    uint32_t kind;
    uint32_t n;
    uint32_t rec_bytes;
    uint32_t n_geoms;
    uint32_t flags;
};

int run_build(rt_context *ctx, cudaStream_t st, const BuildCall &bc, const GeomParams *gp,
              const rt_instance *instances, void *accel, uint64_t accel_bytes, void *scratch,
              uint64_t scratch_bytes, BuildLayout *out_layout) {
    const int bpa = (bc.flags & RT_BUILD_MORTON30) ? 10 : 21;
    const int passes = bpa == 10 ? 4 : 8;
    const uint32_t n = bc.n;
    if (build_width(bc.flags) == 0u) return set_error(ctx, RT_ERR_INVALID_ARG, "RT_BUILD_WIDTH must be 4..8");
    BuildLayout L = build_layout(n, bc.rec_bytes, passes);
    if (out_layout) *out_layout = L;
    const uint64_t need_accel =
        accel_bytes_for(n, bc.rec_bytes, bc.kind == RT_ACCEL_KIND_BLAS ? bc.n_geoms + 1u : 0u);
    if (accel_bytes < need_accel) return set_error(ctx, RT_ERR_OOM, "accel buffer smaller than rt_get_*_build_sizes");
    if (scratch_bytes < L.total) return set_error(ctx, RT_ERR_OOM, "scratch buffer smaller than rt_get_*_build_sizes");
    if (reinterpret_cast<uintptr_t>(accel) & 255u) return set_error(ctx, RT_ERR_INVALID_ARG, "accel must be 256-byte aligned");
    if (reinterpret_cast<uintptr_t>(scratch) & 255u) return set_error(ctx, RT_ERR_INVALID_ARG, "scratch must be 256-byte aligned");
    if (n > (1u << 30) - 1u) return set_error(ctx, RT_ERR_UNSUPPORTED, "more than 2^30-1 primitives");

    uint8_t *A = static_cast<uint8_t *>(accel);
    uint8_t *S = static_cast<uint8_t *>(scratch);
    const uint32_t cap = node_capacity_for(n);

    rt_accel_header h;
    std::memset(&h, 0, sizeof(h));
    h.magic = RT_ACCEL_MAGIC;
    h.version = RT_ACCEL_VERSION;
    h.kind = bc.kind;
    h.prim_count = n;
    h.geom_count = bc.kind == RT_ACCEL_KIND_BLAS ? bc.n_geoms : 0u;
    h.build_flags = bc.flags;
    h.morton_bits = (uint32_t)bpa * 3u;
    h.node_capacity = cap;
    h.node_offset = RT_ACCEL_HEADER_BYTES;
    h.prim_offset = h.node_offset + (uint64_t)cap * 80u;
    h.geom_offset = h.prim_offset + (uint64_t)n * bc.rec_bytes;
    h.total_bytes = need_accel;

    int32_t *cb = reinterpret_cast<int32_t *>(S + L.misc);
    static GeomParams empty_gp;  // zero-initialised; used by TLAS builds
    uint32_t *root_word = reinterpret_cast<uint32_t *>(S + L.misc + 64u);
    k_init<<<1, 256, 0, st>>>(h, A, cb, root_word, gp ? *gp : empty_gp, gp ? 1u : 0u);
    RT_CUDA_CTX(ctx, cudaGetLastError());
    uint32_t *hdr_status = reinterpret_cast<uint32_t *>(A) + 7;  // rt_accel_header::status
    if (n == 0) {
        k_empty_root<<<1, 1, 0, st>>>(A);
        RT_CUDA_CTX(ctx, cudaGetLastError());
        return RT_OK;
    }
    uint4 *recs = reinterpret_cast<uint4 *>(S + L.recs);
    float *boxes = reinterpret_cast<float *>(S + L.boxes);
    const unsigned nb = (n + 255u) / 256u;
    if (bc.kind == RT_ACCEL_KIND_BLAS) {
        k_prep_tris<<<nb, 256, 0, st>>>(*gp, n, recs, boxes, cb, ctx->d_err, hdr_status);
    } else {
        k_prep_inst<<<nb, 256, 0, st>>>(instances, n, recs, boxes, cb);
    }
    RT_CUDA_CTX(ctx, cudaGetLastError());

    uint64_t *keys0 = reinterpret_cast<uint64_t *>(S + L.keys0);
    uint64_t *keys1 = reinterpret_cast<uint64_t *>(S + L.keys1);
    uint32_t *ids0 = reinterpret_cast<uint32_t *>(S + L.ids0);
    uint32_t *ids1 = reinterpret_cast<uint32_t *>(S + L.ids1);
    void *sort_s = S + L.sort;
    uint32_t *hist = sort_hist_ptr(sort_s);
    RT_CUDA_CTX(ctx, cudaMemsetAsync(hist, 0, 8u * 256u * 4u, st));
    {
        unsigned g = nb;
        unsigned cap_g = (unsigned)ctx->sm_count * 8u;
        if (g > cap_g) g = cap_g;
        k_morton<<<g, 256, 0, st>>>(boxes, n, cb, bpa, keys0, ids0, hist, passes);
        RT_CUDA_CTX(ctx, cudaGetLastError());
    }
    int sst = sort_pairs(ctx, st, keys0, ids0, keys1, ids1, n, 8 * passes, sort_s, true, ctx->d_err);
    if (sst) return set_error(ctx, sst, "radix sort launch failed");

    uint4 *bin = reinterpret_cast<uint4 *>(S + L.bin);
    if (n >= 2) RT_CUDA_CTX(ctx, cudaMemsetAsync(S + L.other, 0xff, (size_t)(n - 1) * 8u, st));
    TreeArgs ta;
    ta.n = n;
    ta.keys = keys0;
    ta.ids = ids0;
    ta.boxes = boxes;
    ta.bin = bin;
    ta.node_box = reinterpret_cast<float *>(S + L.node_box);
    ta.node_cost = reinterpret_cast<float *>(S + L.node_cost);
    ta.leafable = reinterpret_cast<uint8_t *>(S + L.leafable);
    ta.other = reinterpret_cast<uint64_t *>(S + L.other);
    ta.leaf_box = reinterpret_cast<float *>(S + L.leaf_box);
    ta.root = root_word;
    ta.err = ctx->d_err;
    k_tree<<<nb, 256, 0, st>>>(ta);
    if (n >= 2) k_tree_root<<<1, 1, 0, st>>>(root_word, n, ctx->d_err);
    RT_CUDA_CTX(ctx, cudaGetLastError());

    CollapseArgs ca;
    ca.n = n;
    ca.width = build_width(bc.flags);
    ca.capacity = cap;
    ca.root_ref = kLeafBit | 0u;                    // one primitive: the root is leaf 0
    ca.root_dev = n >= 2 ? root_word : nullptr;   // otherwise the node k_tree found
    ca.gather = ids1;  // free once the sort has left its result in keys0/ids0
    ca.bin = bin;
    ca.node_box = ta.node_box;
    ca.leafable = ta.leafable;
    ca.leaf_box = ta.leaf_box;
    ca.wq = reinterpret_cast<uint32_t *>(S + L.wq);
    ca.slots = reinterpret_cast<uint32_t *>(S + L.slots);
    ca.desc = reinterpret_cast<uint32_t *>(S + L.desc);
    ca.counts = reinterpret_cast<uint32_t *>(S + L.counts);
    ca.blk = reinterpret_cast<uint32_t *>(S + L.blk);
    ca.nodes_out = reinterpret_cast<uint4 *>(A + h.node_offset);
    ca.hdr = reinterpret_cast<rt_accel_header *>(A);
    ca.bar = reinterpret_cast<uint32_t *>(S + L.misc + 128u);
    ca.err = ctx->d_err;
    RT_CUDA_CTX(ctx, cudaMemsetAsync(ca.bar, 0, 2u * sizeof(uint32_t), st));
    int G = coop_grid(ctx);
    if (G <= 0) return set_error(ctx, RT_ERR_CUDA, "cooperative occupancy query failed");
    // Small levels gain nothing from a huge grid; fewer blocks make each
    // grid barrier cheaper.
    unsigned want = (unsigned)((cap + kCollapseThreads * 4u - 1u) / (kCollapseThreads * 4u));
    if (want < 1u) want = 1u;
    if ((int)want < G) G = (int)want;
    void *args[] = {&ca};
    RT_CUDA_CTX(ctx, cudaLaunchCooperativeKernel((const void *)k_collapse, dim3((unsigned)G),
                                                 dim3(kCollapseThreads), args, 0, st));
    uint4 *recs_out = reinterpret_cast<uint4 *>(A + h.prim_offset);
    if (bc.rec_bytes == 48u)
        k_gather_records<3><<<nb, 256, 0, st>>>(recs, recs_out, ids0, ids1, n, ctx->d_err);
    else
        k_gather_records<5><<<nb, 256, 0, st>>>(recs, recs_out, ids0, ids1, n, ctx->d_err);
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}

// ---------------------------------------------------------------------------
// Refit: new leaf records and boxes in the existing topology
// ---------------------------------------------------------------------------
//
// Each leaf record names its primitive (triangle: build-input index,
// geometry, index in the geometry; instance: instance index), so the records
// are recomputed in place from the new inputs.  Wide nodes are stored in
// breadth-first order (every child after its parent); a node's exact box is
// the union of its slots' boxes -- the union of its primitives' boxes, as in
// the build, since min/max in a total order do not depend on grouping -- and
// is quantised by the build's encode_node.  The nodes are walked bottom-up:
// one thread starts at each node without internal children, and the last of
// a parent's children to arrive (an atomic counter per node) goes on to the
// parent.

struct RefitLayout {
    uint64_t flag, leaf_box, node_box, parent, arrive, total;
};

RefitLayout refit_layout(uint32_t n) {
    RefitLayout L;
    uint64_t off = 0;
    auto take = [&](uint64_t bytes) {
        uint64_t o = off;
        off += align_up(bytes > 0 ? bytes : 1, 256);
        return o;
    };
    const uint64_t cap = node_capacity_for(n);
    L.flag = take(16);
    L.leaf_box = take((uint64_t)n * 32u);
    L.node_box = take(cap * 32u);
    L.parent = take(cap * 4u);
    L.arrive = take(cap * 4u);
    L.total = off;
    return L;
}

// The structure must be the one the inputs describe.
__global__ void k_refit_begin(const rt_accel_header *h, uint32_t kind, uint32_t n, uint32_t n_geoms, uint32_t cap,
                              uint32_t *flag, uint32_t *err) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const bool ok = h->magic == RT_ACCEL_MAGIC && h->kind == kind && h->prim_count == n &&
                    (kind != RT_ACCEL_KIND_BLAS || h->geom_count == n_geoms) && h->node_capacity == cap &&
                    h->node_count >= 1u && h->node_count <= cap && h->node_offset == RT_ACCEL_HEADER_BYTES &&
                    h->prim_offset == RT_ACCEL_HEADER_BYTES + (uint64_t)cap * 80u;
    *flag = ok ? 1u : 0u;
    if (!ok) report_error(err, RT_ERR_INVALID_ARG, 0x68000000u);
}

__global__ void __launch_bounds__(256) k_refit_links(const uint4 *nodes, const rt_accel_header *h, uint32_t cap,
                                                      const uint32_t *flag, uint32_t *parent, uint32_t *arrive,
                                                      uint32_t *err) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cap || *flag == 0u) return;
    const uint32_t nc = h->node_count;
    if (k >= nc) return;
    arrive[k] = 0u;
    const uint32_t imask = nodes[(size_t)k * 5u].w >> 24;
    const uint32_t cb = nodes[(size_t)k * 5u + 1u].x;
    const uint32_t ni = (uint32_t)__popc(imask);
    for (uint32_t j = 0; j < ni; ++j) {
        const uint32_t c = cb + j;
        if (c <= k || c >= nc) {  // children follow their parent in breadth-first order
            report_error(err, RT_ERR_BOUNDS, 0x69000000u | (k & 0xffffffu));
            return;
        }
        parent[c] = k;
    }
}

__global__ void __launch_bounds__(256) k_refit_tris(const GeomParams gp, uint32_t n, uint4 *recs, float *leaf_box,
                                                     const uint32_t *flag, uint32_t *err, uint32_t *hdr_status) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n || *flag == 0u) return;
    uint4 *rec = recs + (size_t)r * 3u;
    const uint32_t gi = rec[0].w, g = rec[1].w, p = rec[2].w;
    Box b = box_empty();
    if (g < gp.n_geoms && p < gp.g[g].tri_count && gi == gp.table[g] + p)
        tri_record(gp, g, p, gi, rec, b, err, hdr_status);
    else
        report_error(err, RT_ERR_BOUNDS, 0x6a000000u | (r & 0xffffffu));
    store_box(leaf_box, r, b);
}

__global__ void __launch_bounds__(256) k_refit_inst(const rt_instance *inst, uint32_t n, uint4 *recs,
                                                     float *leaf_box, const uint32_t *flag, uint32_t *err) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n || *flag == 0u) return;
    uint4 *rec = recs + (size_t)r * 5u;
    const uint32_t i = rec[4].x;
    Box b = box_empty();
    if (i < n) {
        const rt_instance I = inst[i];
        inst_record(I, i, rec, b);
    } else {
        report_error(err, RT_ERR_BOUNDS, 0x6b000000u | (r & 0xffffffu));
    }
    store_box(leaf_box, r, b);
}

__global__ void __launch_bounds__(256) k_refit_nodes(uint4 *nodes, rt_accel_header *h, uint32_t cap, uint32_t n,
                                                      const float *leaf_box, float *node_box, const uint32_t *parent,
                                                      uint32_t *arrive, const uint32_t *flag, uint32_t *err) {
    const uint32_t k0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (k0 >= cap || *flag == 0u) return;
    const uint32_t nc = h->node_count;
    if (k0 >= nc || (__ldcg(nodes + (size_t)k0 * 5u).w >> 24) != 0u) return;  // start below every internal child
    uint32_t k = k0;
    for (int step = 0;; ++step) {
        if (step >= 256) {  // deeper than any build makes: a corrupt structure
            report_error(err, RT_ERR_BOUNDS, 0x6c000000u | (k & 0xffffffu));
            return;
        }
        uint4 *o = nodes + (size_t)k * 5u;
        const uint4 w0 = __ldcg(o), w1 = __ldcg(o + 1);
        const uint32_t imask = w0.w >> 24, cb = w1.x, pb = w1.y;
        Box sbox[8];
        bool used[8];
        Box node = box_empty();
        for (int s = 0; s < 8; ++s) {
            const uint32_t meta = ((s < 4 ? w1.z : w1.w) >> (8 * (s & 3))) & 0xffu;
            used[s] = meta != 0u;
            sbox[s] = box_empty();
            if ((imask >> s) & 1u) {
                const uint32_t c = cb + (uint32_t)__popc(imask & ((1u << s) - 1u));
                if (c < nc) sbox[s] = load_box(node_box, c);
                else report_error(err, RT_ERR_BOUNDS, 0x6d000000u | (k & 0xffffffu));
            } else if (meta) {
                const uint32_t cnt = (uint32_t)__popc(meta >> 5), first = pb + (meta & 0x1fu);
                if (first + cnt <= n) {
                    for (uint32_t j = 0; j < cnt; ++j) sbox[s] = box_union(sbox[s], load_box(leaf_box, first + j));
                } else {
                    report_error(err, RT_ERR_BOUNDS, 0x6e000000u | (k & 0xffffffu));
                }
            }
            if (used[s]) node = box_union(node, sbox[s]);
        }
        encode_node(node, sbox, used, imask, o);
        store_box(node_box, k, node);
        if (k == 0u) {
            for (int q = 0; q < 3; ++q) { h->bounds_lo[q] = node.lo[q]; h->bounds_hi[q] = node.hi[q]; }
            return;
        }
        __threadfence();  // the box is visible before the arrival is counted
        const uint32_t p = parent[k];
        if (p >= k) {  // the root, or a node no parent claimed
            report_error(err, RT_ERR_BOUNDS, 0x6f000000u | (k & 0xffffffu));
            return;
        }
        const uint32_t need = (uint32_t)__popc(__ldcg(nodes + (size_t)p * 5u).w >> 24);
        if (atomicAdd(arrive + p, 1u) + 1u != need) return;
        __threadfence();
        k = p;
    }
}

int run_refit(rt_context *ctx, cudaStream_t st, uint32_t kind, uint32_t n, uint32_t n_geoms, const GeomParams *gp,
              const rt_instance *instances, void *accel, uint64_t accel_bytes, void *scratch,
              uint64_t scratch_bytes) {
    const uint32_t rec_bytes = kind == RT_ACCEL_KIND_BLAS ? 48u : 80u;
    const uint64_t need_accel = accel_bytes_for(n, rec_bytes, kind == RT_ACCEL_KIND_BLAS ? n_geoms + 1u : 0u);
    const RefitLayout L = refit_layout(n);
    if (accel_bytes < need_accel) return set_error(ctx, RT_ERR_OOM, "accel buffer smaller than its build size");
    if (scratch_bytes < L.total) return set_error(ctx, RT_ERR_OOM, "scratch smaller than rt_get_refit_scratch_bytes");
    if (reinterpret_cast<uintptr_t>(accel) & 255u) return set_error(ctx, RT_ERR_INVALID_ARG, "accel must be 256-byte aligned");
    if (reinterpret_cast<uintptr_t>(scratch) & 255u) return set_error(ctx, RT_ERR_INVALID_ARG, "scratch must be 256-byte aligned");
    if (n == 0) return RT_OK;  // an empty structure has nothing to refit
    uint8_t *A = static_cast<uint8_t *>(accel);
    uint8_t *S = static_cast<uint8_t *>(scratch);
    const uint32_t cap = node_capacity_for(n);
    rt_accel_header *hdr = reinterpret_cast<rt_accel_header *>(A);
    uint4 *nodes = reinterpret_cast<uint4 *>(A + RT_ACCEL_HEADER_BYTES);
    uint4 *recs = reinterpret_cast<uint4 *>(A + RT_ACCEL_HEADER_BYTES + (uint64_t)cap * 80u);
    uint32_t *flag = reinterpret_cast<uint32_t *>(S + L.flag);
    float *leaf_box = reinterpret_cast<float *>(S + L.leaf_box);
    float *node_box = reinterpret_cast<float *>(S + L.node_box);
    uint32_t *parent = reinterpret_cast<uint32_t *>(S + L.parent);
    uint32_t *arrive = reinterpret_cast<uint32_t *>(S + L.arrive);
    uint32_t *hdr_status = reinterpret_cast<uint32_t *>(A) + 7;  // rt_accel_header::status
    k_refit_begin<<<1, 32, 0, st>>>(hdr, kind, n, n_geoms, cap, flag, ctx->d_err);
    RT_CUDA_CTX(ctx, cudaMemsetAsync(parent, 0xff, (size_t)cap * 4u, st));
    const unsigned nbc = (cap + 255u) / 256u, nbn = (n + 255u) / 256u;
    k_refit_links<<<nbc, 256, 0, st>>>(nodes, hdr, cap, flag, parent, arrive, ctx->d_err);
    if (kind == RT_ACCEL_KIND_BLAS)
        k_refit_tris<<<nbn, 256, 0, st>>>(*gp, n, recs, leaf_box, flag, ctx->d_err, hdr_status);
    else
        k_refit_inst<<<nbn, 256, 0, st>>>(instances, n, recs, leaf_box, flag, ctx->d_err);
    k_refit_nodes<<<nbc, 256, 0, st>>>(nodes, hdr, cap, n, leaf_box, node_box, parent, arrive, flag, ctx->d_err);
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}

// Fills the geometry table of a bottom-level input; RT_OK or an error.
int geom_params(rt_context *ctx, const rt_geometry_triangles *geoms, uint32_t n_geoms, GeomParams &gp,
                uint64_t &total, const char *who) {
    std::memset(&gp, 0, sizeof(gp));
    gp.n_geoms = n_geoms;
    total = 0;
    for (uint32_t g = 0; g < n_geoms; ++g) {
        const rt_geometry_triangles &G = geoms[g];
        if (G.tri_count && (!G.vertices || G.vertex_stride < 12u ||
                            (G.index_type != RT_INDEX_UINT32 && G.index_type != RT_INDEX_NONE) ||
                            (G.index_type == RT_INDEX_UINT32 && !G.indices)))
            return set_error(ctx, RT_ERR_INVALID_ARG, who);
        if (G.index_type == RT_INDEX_NONE && G.tri_count && (uint64_t)G.tri_count * 3u - 1u > G.max_vertex)
            return set_error(ctx, RT_ERR_INVALID_ARG, who);
        gp.table[g] = (uint32_t)total;
        gp.g[g] = G;
        total += G.tri_count;
    }
    if (total > (1u << 30) - 1u) return set_error(ctx, RT_ERR_UNSUPPORTED, "more than 2^30-1 triangles");
    gp.table[n_geoms] = (uint32_t)total;
    return RT_OK;
}

}  // namespace
}  // namespace rtc

using namespace rtc;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" rt_status rt_get_blas_build_sizes(rt_context *ctx, const uint32_t *tri_counts, uint32_t n_geoms,
                                             uint32_t flags, rt_build_sizes *out) {
    if (!ctx || !out || (n_geoms && !tri_counts)) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_get_blas_build_sizes: null argument");
    if (n_geoms > (uint32_t)kMaxGeoms) return set_error(ctx, RT_ERR_UNSUPPORTED, "more than 256 geometries in one BLAS");
    uint64_t n = 0;
    for (uint32_t g = 0; g < n_geoms; ++g) n += tri_counts[g];
    if (n > (1u << 30) - 1u) return set_error(ctx, RT_ERR_UNSUPPORTED, "more than 2^30-1 triangles");
    int passes = (flags & RT_BUILD_MORTON30) ? 4 : 8;
    out->accel_bytes = accel_bytes_for((uint32_t)n, 48u, n_geoms + 1u);
    out->scratch_bytes = build_layout((uint32_t)n, 48u, passes).total;
    return RT_OK;
}

extern "C" rt_status rt_get_tlas_build_sizes(rt_context *ctx, uint32_t n_instances, uint32_t flags,
                                             rt_build_sizes *out) {
    if (!ctx || !out) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_get_tlas_build_sizes: null argument");
    if (n_instances > (1u << 30) - 1u) return set_error(ctx, RT_ERR_UNSUPPORTED, "too many instances");
    int passes = (flags & RT_BUILD_MORTON30) ? 4 : 8;
    out->accel_bytes = accel_bytes_for(n_instances, 80u, 0);
    out->scratch_bytes = build_layout(n_instances, 80u, passes).total;
    return RT_OK;
}

extern "C" rt_status rt_build_blas(rt_context *ctx, rt_stream stream, const rt_geometry_triangles *geoms,
                                   uint32_t n_geoms, uint32_t flags, void *accel, uint64_t accel_bytes,
                                   void *scratch, uint64_t scratch_bytes) {
    if (!ctx || !accel || !scratch || (n_geoms && !geoms))
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_build_blas: null argument");
    if (n_geoms > (uint32_t)kMaxGeoms) return set_error(ctx, RT_ERR_UNSUPPORTED, "more than 256 geometries in one BLAS");
    if ((flags & RT_BUILD_MORTON30) && (flags & RT_BUILD_MORTON63))
        return set_error(ctx, RT_ERR_INVALID_ARG, "RT_BUILD_MORTON30 and RT_BUILD_MORTON63 are exclusive");
    static thread_local GeomParams gp;
    uint64_t total = 0;
    int rc = geom_params(ctx, geoms, n_geoms, gp, total, "rt_build_blas: bad geometry descriptor");
    if (rc) return rc;
    BuildCall bc{RT_ACCEL_KIND_BLAS, (uint32_t)total, 48u, n_geoms, flags};
    return run_build(ctx, static_cast<cudaStream_t>(stream), bc, &gp, nullptr, accel, accel_bytes, scratch,
                     scratch_bytes, nullptr);
}

extern "C" rt_status rt_build_tlas(rt_context *ctx, rt_stream stream, const rt_instance *instances, uint32_t n,
                                   uint32_t flags, void *accel, uint64_t accel_bytes, void *scratch,
                                   uint64_t scratch_bytes) {
    if (!ctx || !accel || !scratch || (n && !instances))
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_build_tlas: null argument");
    if ((flags & RT_BUILD_MORTON30) && (flags & RT_BUILD_MORTON63))
        return set_error(ctx, RT_ERR_INVALID_ARG, "RT_BUILD_MORTON30 and RT_BUILD_MORTON63 are exclusive");
    BuildCall bc{RT_ACCEL_KIND_TLAS, n, 80u, 0u, flags};
    return run_build(ctx, static_cast<cudaStream_t>(stream), bc, nullptr, instances, accel, accel_bytes, scratch,
                     scratch_bytes, nullptr);
}

extern "C" rt_status rt_get_refit_scratch_bytes(uint32_t prim_count, uint64_t *bytes) {
    if (!bytes) return RT_ERR_INVALID_ARG;
    if (prim_count > (1u << 30) - 1u) return RT_ERR_UNSUPPORTED;
    *bytes = refit_layout(prim_count).total;
    return RT_OK;
}

extern "C" rt_status rt_refit_blas(rt_context *ctx, rt_stream stream, const rt_geometry_triangles *geoms,
                                   uint32_t n_geoms, void *accel, uint64_t accel_bytes, void *scratch,
                                   uint64_t scratch_bytes) {
    if (!ctx || !accel || !scratch || (n_geoms && !geoms))
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_refit_blas: null argument");
    if (n_geoms > (uint32_t)kMaxGeoms) return set_error(ctx, RT_ERR_UNSUPPORTED, "more than 256 geometries in one BLAS");
    static thread_local GeomParams gp;
    uint64_t total = 0;
    int rc = geom_params(ctx, geoms, n_geoms, gp, total, "rt_refit_blas: bad geometry descriptor");
    if (rc) return rc;
    return run_refit(ctx, static_cast<cudaStream_t>(stream), RT_ACCEL_KIND_BLAS, (uint32_t)total, n_geoms, &gp,
                     nullptr, accel, accel_bytes, scratch, scratch_bytes);
}

extern "C" rt_status rt_refit_tlas(rt_context *ctx, rt_stream stream, const rt_instance *instances, uint32_t n,
                                   void *accel, uint64_t accel_bytes, void *scratch, uint64_t scratch_bytes) {
    if (!ctx || !accel || !scratch || (n && !instances))
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_refit_tlas: null argument");
    if (n > (1u << 30) - 1u) return set_error(ctx, RT_ERR_UNSUPPORTED, "too many instances");
    return run_refit(ctx, static_cast<cudaStream_t>(stream), RT_ACCEL_KIND_TLAS, n, 0u, nullptr, instances, accel,
                     accel_bytes, scratch, scratch_bytes);
}

extern "C" uint64_t rt_accel_address(const void *accel) { return (uint64_t)(uintptr_t)accel; }

extern "C" rt_status rt_accel_info(rt_context *ctx, rt_stream stream, const void *accel, uint32_t *node_count,
                                   uint32_t *prim_count, uint32_t *tree_depth) {
    if (!ctx || !accel) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_accel_info: null argument");
    rt_accel_header h;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    RT_CUDA_CTX(ctx, cudaMemcpyAsync(&h, accel, sizeof(h), cudaMemcpyDeviceToHost, st));
    RT_CUDA_CTX(ctx, cudaStreamSynchronize(st));
    if (h.magic != RT_ACCEL_MAGIC) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_accel_info: not an acceleration structure");
    if (node_count) *node_count = h.node_count;
    if (prim_count) *prim_count = h.prim_count;
    if (tree_depth) *tree_depth = h.depth;
    if (h.status) return set_error(ctx, -(int)h.status, "acceleration structure build reported an error");
    return RT_OK;
}

// Offsets (bytes from the scratch base) of the sorted Morton keys, the
// sorted primitive ids and the binary nodes after a BLAS build, for
// stage-by-stage comparison with the CPU restatement.
extern "C" rt_status rt_debug_blas_scratch_layout(uint32_t n_tris, uint32_t flags, uint64_t *keys_off,
                                                  uint64_t *ids_off, uint64_t *bin_off) {
    int passes = (flags & RT_BUILD_MORTON30) ? 4 : 8;
    BuildLayout L = build_layout(n_tris, 48u, passes);
    if (keys_off) *keys_off = L.keys0;
    if (ids_off) *ids_off = L.ids0;
    if (bin_off) *bin_off = L.bin;
    return RT_OK;
}

// ---------------------------------------------------------------------------
// Bottom-level build that allocates nothing
// ---------------------------------------------------------------------------
//
// Callers that cannot allocate device memory -- a plugin that only receives
// buffers from the engine that owns all device memory, or a frame loop that
// may not call cudaMalloc/cudaFree because they can synchronise the whole
// device and stall the work other streams have in flight -- still need a
// build scratch area.  This entry point uses a fixed scratch array compiled
// into the library instead of a caller buffer.
//
// The array lives in device memory of every GPU that loads the library, from
// module load until the process exits.  Host code may not use its name as a
// device address (on the host it names a stand-in object), so the device
// address is fetched once per device with cudaGetSymbolAddress, with that
// device current, by the first call on that device; that first call should
// therefore come before any stream capture.  All calls share the one array:
// two calls whose work overlaps on the GPU (different streams, no ordering
// between them) race on it and both results are undefined.  Each build
// clears, on its stream, every part of the scratch that must start at zero
// (centroid bounds, sort histograms, look-back status, refit counters), so
// what an earlier call left there does not matter.

namespace rtc {
namespace {

constexpr uint64_t kStaticScratchBytes = 40ull << 20;  // 40 MiB per device
constexpr int kStaticScratchDevices = 64;

__device__ __align__(256) uint8_t g_static_scratch[kStaticScratchBytes];

void *g_static_scratch_addr[kStaticScratchDevices] = {};

// Device address of g_static_scratch on ctx->device (looked up once).
int static_scratch_address(rt_context *ctx, void **out) {
    if (ctx->device < 0 || ctx->device >= kStaticScratchDevices)
        return set_error(ctx, RT_ERR_UNSUPPORTED, "static scratch: device ordinal beyond 63");
    void *p = __atomic_load_n(&g_static_scratch_addr[ctx->device], __ATOMIC_ACQUIRE);
    if (!p) {
        int cur = -1;
        RT_CUDA_CTX(ctx, cudaGetDevice(&cur));
        if (cur != ctx->device) RT_CUDA_CTX(ctx, cudaSetDevice(ctx->device));
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (cur != ctx->device) cudaSetDevice(cur);
        if (e != cudaSuccess) return set_cuda_error(ctx, e, "cudaGetSymbolAddress(g_static_scratch)");
        __atomic_store_n(&g_static_scratch_addr[ctx->device], p, __ATOMIC_RELEASE);
    }
    *out = p;
    return RT_OK;
}

}  // namespace

void static_scratch_forget(int device) {
    if (device >= 0 && device < kStaticScratchDevices)
        __atomic_store_n(&g_static_scratch_addr[device], (void *)nullptr, __ATOMIC_RELEASE);
}

}  // namespace rtc

extern "C" rt_status rt_build_blas_static_scratch(rt_context *ctx, rt_stream stream,
                                                  const rt_geometry_triangles *geoms, uint32_t n_geoms,
                                                  uint32_t flags, void *accel, uint64_t accel_bytes) {
    if (!ctx || !accel || (n_geoms && !geoms))
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_build_blas_static_scratch: null argument");
    if (n_geoms > (uint32_t)kMaxGeoms)
        return set_error(ctx, RT_ERR_UNSUPPORTED, "more than 256 geometries in one BLAS");
    if ((flags & RT_BUILD_MORTON30) && (flags & RT_BUILD_MORTON63))
        return set_error(ctx, RT_ERR_INVALID_ARG, "RT_BUILD_MORTON30 and RT_BUILD_MORTON63 are exclusive");
    static thread_local GeomParams gp;
    uint64_t total = 0;
    int rc = geom_params(ctx, geoms, n_geoms, gp, total, "rt_build_blas_static_scratch: bad geometry descriptor");
    if (rc) return rc;
    if (total > RT_STATIC_SCRATCH_MAX_TRIS)
        return set_error(ctx, RT_ERR_UNSUPPORTED,
                         "rt_build_blas_static_scratch: more than RT_STATIC_SCRATCH_MAX_TRIS (131072) triangles; "
                         "use rt_build_blas with a caller-allocated scratch buffer");
    const int passes = (flags & RT_BUILD_MORTON30) ? 4 : 8;
    const BuildLayout L = build_layout((uint32_t)total, 48u, passes);
    if (L.total > kStaticScratchBytes)
        return set_error(ctx, RT_ERR_UNSUPPORTED, "rt_build_blas_static_scratch: scratch layout exceeds the static array");
    void *scratch = nullptr;
    rc = static_scratch_address(ctx, &scratch);
    if (rc) return rc;
    BuildCall bc{RT_ACCEL_KIND_BLAS, (uint32_t)total, 48u, n_geoms, flags};
    return run_build(ctx, static_cast<cudaStream_t>(stream), bc, &gp, nullptr, accel, accel_bytes, scratch,
                     kStaticScratchBytes, nullptr);
}
