/*
 * oracle.cpp -- scalar CPU oracle of the ray-tracing core.
 * TEST INFRASTRUCTURE ONLY: called by tests/, by smoke() and by bench.py's
 * CPU-baseline leg, never by the product.
 *
 * Compile with -ffp-contract=off: every float expression below is evaluated
 * operation by operation in round-to-nearest, and std::fma is used exactly
 * where the GPU kernels issue an FMA, so both sides round identically.
 *
 * What each part restates:
 *   raygen            vulkan-raytraced-triangle/main.cpp:1033-1055
 *   miss              main.cpp:1063-1066
 *   closest hit       main.cpp:1080-1091, SBT rule main.cpp:1260-1262,
 *                     records main.cpp:1306-1317
 *   geometry input    main.cpp:726-746 (stride, indices, transformData)
 *   instances         main.cpp:835-858 (VkAccelerationStructureInstanceKHR)
 *   BVH build         driver-internal in the reference (main.cpp:808, 932):
 *                     LBVH (Karras, HPG 2012) + wide collapse + quantisation
 *                     (Ylitie et al., HPG 2017) as this project defines it
 *   traversal         driver/RT-core internal (main.cpp:1047)
 *   triangle test     Woop, Benthin, Wald, "Watertight Ray/Triangle
 *                     Intersection", JCGT 2(1), 2013
 */
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

constexpr float kInf = std::numeric_limits<float>::infinity();
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr float kTfarScale = 1.0f + 0x1p-20f;
constexpr int kMaxStack = 128;

inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

/* Total order on float bits (-0 < +0); min/max under it are independent of
 * evaluation order, which the GPU's parallel reductions rely on. */
inline int32_t ford(float f) {
    int32_t i = (int32_t)fbits(f);
    return i >= 0 ? i : (i ^ 0x7fffffff);
}
inline float ford_inv(int32_t i) { return bitsf((uint32_t)(i >= 0 ? i : (i ^ 0x7fffffff))); }
inline float fmn(float a, float b) { return ford(b) < ford(a) ? b : a; }
inline float fmx(float a, float b) { return ford(b) > ford(a) ? b : a; }
inline float pow2f(int e) { return bitsf((uint32_t)(e + 127) << 23); }

/* a - b rounded toward -inf / +inf, from the exact error of the rounded
 * difference (Knuth's TwoSum). */
inline float sub_dir(float a, float b, int up) {
    float nb = -b;
    float s = a + nb;
    float bb = s - a;
    float err = (a - (s - bb)) + (nb - bb);
    if (up) {
        if (err > 0.0f) s = std::nextafter(s, kInf);
    } else {
        if (err < 0.0f) s = std::nextafter(s, -kInf);
    }
    return s;
}

struct Box {
    float lo[3], hi[3];
};
inline Box box_empty() {
    Box b;
    for (int a = 0; a < 3; ++a) { b.lo[a] = kInf; b.hi[a] = -kInf; }
    return b;
}
inline bool box_is_empty(const Box &b) {
    return !(b.lo[0] <= b.hi[0] && b.lo[1] <= b.hi[1] && b.lo[2] <= b.hi[2]);
}
inline Box box_union(const Box &x, const Box &y) {
    Box b;
    for (int a = 0; a < 3; ++a) { b.lo[a] = fmn(x.lo[a], y.lo[a]); b.hi[a] = fmx(x.hi[a], y.hi[a]); }
    return b;
}
inline float half_area(const Box &b) {
    if (box_is_empty(b)) return 0.0f;
    float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return (dx * dy + dy * dz) + dz * dx;
}

/* Exponent of the per-axis quantisation grid: smallest e with
 * 255 * 2^e >= ext, clamped to [RT_QEXP_MIN, RT_QEXP_MAX]. */
inline int qexp_for(float ext) {
    if (!(ext > 0.0f)) return RT_QEXP_MIN;
    int biased = (int)((fbits(ext) >> 23) & 0xffu);
    int e = (biased == 0 ? -127 : biased - 127) - 8;
    if (e < RT_QEXP_MIN) e = RT_QEXP_MIN;
    while (e < RT_QEXP_MAX && 255.0f * pow2f(e) < ext) ++e;
    return e;
}

inline void xform_point(const rt_transform3x4 &m, const float p[3], float out[3]) {
    for (int r = 0; r < 3; ++r)
        out[r] = ((m.m[r][0] * p[0] + m.m[r][1] * p[1]) + m.m[r][2] * p[2]) + m.m[r][3];
}
inline void xform_vector(const float m[3][4], const float p[3], float out[3]) {
    for (int r = 0; r < 3; ++r) out[r] = (m[r][0] * p[0] + m[r][1] * p[1]) + m[r][2] * p[2];
}

/* Inverse of an affine 3x4 by the adjugate; returns false when singular. */
bool invert3x4(const rt_transform3x4 &m, float out[3][4]) {
    float a = m.m[0][0], b = m.m[0][1], c = m.m[0][2];
    float d = m.m[1][0], e = m.m[1][1], f = m.m[1][2];
    float g = m.m[2][0], h = m.m[2][1], i = m.m[2][2];
    float c00 = e * i - f * h, c01 = f * g - d * i, c02 = d * h - e * g;
    float det = (a * c00 + b * c01) + c * c02;
    if (!(det != 0.0f) || !std::isfinite(det)) return false;
    float r = 1.0f / det;
    float inv[3][3] = {
        {c00 * r, (c * h - b * i) * r, (b * f - c * e) * r},
        {c01 * r, (a * i - c * g) * r, (c * d - a * f) * r},
        {c02 * r, (b * g - a * h) * r, (a * e - b * d) * r},
    };
    for (int row = 0; row < 3; ++row) {
        for (int col = 0; col < 3; ++col) out[row][col] = inv[row][col];
        out[row][3] = -((inv[row][0] * m.m[0][3] + inv[row][1] * m.m[1][3]) + inv[row][2] * m.m[2][3]);
    }
    return true;
}

/* ---------------------------------------------------------------------- */
/* Morton codes                                                           */
/* ---------------------------------------------------------------------- */

inline uint64_t spread3_21(uint32_t x) {
    uint64_t v = x & 0x1fffffu;
    uint64_t r = 0;
    for (int i = 0; i < 21; ++i) r |= ((v >> i) & 1ull) << (3 * i);
    return r;
}

struct MortonGrid {
    float lo[3];
    float scale[3];
    float maxq;
    int bits_per_axis;
};

MortonGrid morton_grid(const int32_t lo_ord[3], const int32_t hi_ord[3], int bits_per_axis) {
    MortonGrid g;
    g.bits_per_axis = bits_per_axis;
    g.maxq = (float)((1u << bits_per_axis) - 1u);
    float cells = (float)(1u << bits_per_axis);
    for (int a = 0; a < 3; ++a) {
        float lo = ford_inv(lo_ord[a]), hi = ford_inv(hi_ord[a]);
        float ext = hi - lo;
        g.lo[a] = lo;
        g.scale[a] = ext > 0.0f ? cells / ext : 0.0f;
    }
    return g;
}

inline uint64_t morton_key(const MortonGrid &g, const float c[3]) {
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
        float f = (c[a] - g.lo[a]) * g.scale[a];
        q[a] = !(f > 0.0f) ? 0u : (f >= g.maxq ? (uint32_t)g.maxq : (uint32_t)f);
    }
    return spread3_21(q[0]) | (spread3_21(q[1]) << 1) | (spread3_21(q[2]) << 2);
}

/* ---------------------------------------------------------------------- */
/* Generic LBVH -> BVH8 builder over primitives with boxes and records     */
/* ---------------------------------------------------------------------- */

struct BinNode {
    uint32_t left, right, first, last;
};

inline int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }
inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

inline int karras_delta(const std::vector<uint64_t> &k, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    uint64_t a = k[(size_t)i], b = k[(size_t)j];
    if (a == b) return 64 + clz32((uint32_t)i ^ (uint32_t)j);
    return clz64(a ^ b);
}

/* Karras 2012, "Maximizing Parallelism in the Construction of BVHs, Octrees,
 * and k-d Trees", Figure 4, with index-augmented keys for duplicates. */
BinNode karras_node(const std::vector<uint64_t> &k, int64_t n, int64_t i) {
    int d = (karras_delta(k, n, i, i + 1) - karras_delta(k, n, i, i - 1)) > 0 ? 1 : -1;
    int dmin = karras_delta(k, n, i, i - d);
    int64_t lmax = 2;
    while (karras_delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int64_t l = 0;
    for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
        if (karras_delta(k, n, i, i + (l + t) * d) > dmin) l += t;
    int64_t j = i + l * d;
    int dnode = karras_delta(k, n, i, j);
    int64_t s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (karras_delta(k, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int64_t gamma = i + s * d + std::min(d, 0);
    int64_t lo = std::min(i, j), hi = std::max(i, j);
    BinNode nd;
    nd.left = (lo == gamma) ? (kLeafBit | (uint32_t)gamma) : (uint32_t)gamma;
    nd.right = (hi == gamma + 1) ? (kLeafBit | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
    nd.first = (uint32_t)lo;
    nd.last = (uint32_t)hi;
    return nd;
}

struct BuildInput {
    uint32_t n = 0;
    std::vector<Box> boxes;           /* input order */
    std::vector<uint8_t> active;      /* input order */
    std::vector<uint8_t> records;     /* input order, rec_bytes each */
    uint32_t rec_bytes = 48;
};

struct BuildResult {
    std::vector<rt_bvh8_node> nodes;
    std::vector<uint8_t> prims; /* leaf order */
    uint32_t depth = 0;
    Box root;
    uint32_t morton_bits = 63;
};

struct Tree {
    uint32_t n;
    std::vector<uint32_t> ids;       /* sorted position -> input index */
    std::vector<BinNode> nodes;      /* n - 1 internal */
    std::vector<Box> node_box;
    std::vector<float> node_cost;
    std::vector<uint8_t> leafable;
    std::vector<Box> leaf_box;       /* sorted position */
    uint32_t root_ref;
};

inline bool ref_is_leaf(uint32_t r) { return (r & kLeafBit) != 0; }

const Box &ref_box(const Tree &t, uint32_t r) {
    return ref_is_leaf(r) ? t.leaf_box[r & ~kLeafBit] : t.node_box[r];
}
inline bool ref_openable(const Tree &t, uint32_t r) { return !ref_is_leaf(r) && !t.leafable[r]; }
inline void ref_range(const Tree &t, uint32_t r, uint32_t &first, uint32_t &last) {
    if (ref_is_leaf(r)) { first = last = r & ~kLeafBit; }
    else { first = t.nodes[r].first; last = t.nodes[r].last; }
}

/* Builds the binary LBVH and its SAH annotations. */
Tree build_tree(const BuildInput &in, uint32_t flags, uint32_t &morton_bits, orc_lbvh_debug *dbg) {
    Tree t;
    uint32_t n = in.n;
    t.n = n;
    int bpa = (flags & RT_BUILD_MORTON30) ? 10 : 21;
    morton_bits = (uint32_t)bpa * 3u;

    /* centroid bounds over active primitives */
    int32_t clo[3], chi[3];
    for (int a = 0; a < 3; ++a) { clo[a] = ford(kInf); chi[a] = ford(-kInf); }
    std::vector<float> cent((size_t)n * 3);
    uint32_t n_active = 0;
    for (uint32_t i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a) cent[(size_t)i * 3 + a] = (in.boxes[i].lo[a] + in.boxes[i].hi[a]) * 0.5f;
        if (!in.active[i]) continue;
        ++n_active;
        for (int a = 0; a < 3; ++a) {
            int32_t o = ford(cent[(size_t)i * 3 + a]);
            clo[a] = std::min(clo[a], o);
            chi[a] = std::max(chi[a], o);
        }
    }
    if (n_active == 0)
        for (int a = 0; a < 3; ++a) { clo[a] = ford(0.0f); chi[a] = ford(0.0f); }
    MortonGrid g = morton_grid(clo, chi, bpa);
    uint64_t inactive_key = (bpa == 21) ? ((1ull << 63) - 1ull) : ((1ull << 30) - 1ull);

    std::vector<uint64_t> keys(n);
    for (uint32_t i = 0; i < n; ++i)
        keys[i] = in.active[i] ? morton_key(g, &cent[(size_t)i * 3]) : inactive_key;
    /* large primitives (RT_LARGE_PRIM_FRACTION): the bit above the Morton code */
    {
        float cext = 0.0f;
        for (int a = 0; a < 3; ++a) {
            float x = ford_inv(chi[a]) - ford_inv(clo[a]);
            if (x > cext) cext = x;
        }
        const float large = RT_LARGE_PRIM_FRACTION * cext;
        const uint64_t large_bit = (bpa == 21) ? (1ull << 63) : (1ull << 31);
        for (uint32_t i = 0; i < n; ++i) {
            if (!in.active[i]) continue;
            float e = 0.0f;
            for (int a = 0; a < 3; ++a) {
                float x = in.boxes[i].hi[a] - in.boxes[i].lo[a];
                if (x > e) e = x;
            }
            if (e > large) keys[i] |= large_bit;
        }
    }
    if (dbg && dbg->keys_unsorted) std::memcpy(dbg->keys_unsorted, keys.data(), n * 8ull);

    /* stable sort by key (what an LSD radix sort produces) */
    t.ids.resize(n);
    for (uint32_t i = 0; i < n; ++i) t.ids[i] = i;
    std::stable_sort(t.ids.begin(), t.ids.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
    std::vector<uint64_t> sk(n);
    for (uint32_t i = 0; i < n; ++i) sk[i] = keys[t.ids[i]];
    if (dbg && dbg->keys_sorted) std::memcpy(dbg->keys_sorted, sk.data(), n * 8ull);
    if (dbg && dbg->ids_sorted) std::memcpy(dbg->ids_sorted, t.ids.data(), n * 4ull);

    t.leaf_box.resize(n);
    for (uint32_t i = 0; i < n; ++i) t.leaf_box[i] = in.boxes[t.ids[i]];

    if (n < 2) {
        t.root_ref = kLeafBit | 0u;
        return t;
    }
    t.nodes.resize(n - 1);
    for (uint32_t i = 0; i + 1 < n; ++i) t.nodes[i] = karras_node(sk, n, i);
    if (dbg && dbg->bin_nodes)
        for (uint32_t i = 0; i + 1 < n; ++i) {
            dbg->bin_nodes[4 * i + 0] = t.nodes[i].left;
            dbg->bin_nodes[4 * i + 1] = t.nodes[i].right;
            dbg->bin_nodes[4 * i + 2] = t.nodes[i].first;
            dbg->bin_nodes[4 * i + 3] = t.nodes[i].last;
        }

    /* refit + SAH, children before parents (iterative post-order) */
    t.node_box.resize(n - 1);
    t.node_cost.resize(n - 1);
    t.leafable.resize(n - 1);
    std::vector<uint32_t> stack;
    std::vector<uint8_t> expanded(n - 1, 0);
    stack.push_back(0);
    while (!stack.empty()) {
        uint32_t x = stack.back();
        const BinNode &nd = t.nodes[x];
        if (!expanded[x]) {
            expanded[x] = 1;
            if (!ref_is_leaf(nd.right)) stack.push_back(nd.right);
            if (!ref_is_leaf(nd.left)) stack.push_back(nd.left);
            continue;
        }
        stack.pop_back();
        const Box &bl = ref_box(t, nd.left);
        const Box &br = ref_box(t, nd.right);
        Box b = box_union(bl, br);
        float cl = ref_is_leaf(nd.left) ? RT_SAH_PRIM : t.node_cost[nd.left];
        float cr = ref_is_leaf(nd.right) ? RT_SAH_PRIM : t.node_cost[nd.right];
        float an = half_area(b);
        float split;
        if (an > 0.0f) {
            float s = half_area(bl) * cl + half_area(br) * cr;
            split = RT_SAH_NODE + s / an;
        } else {
            split = RT_SAH_NODE + (cl + cr);
        }
        uint32_t count = nd.last - nd.first + 1u;
        float leaf = (float)count * RT_SAH_PRIM;
        bool lf = count <= (uint32_t)RT_MAX_LEAF_PRIMS && leaf <= split;
        t.node_box[x] = b;
        t.node_cost[x] = lf ? leaf : split;
        t.leafable[x] = lf ? 1 : 0;
    }
    t.root_ref = 0;
    return t;
}

/* Children of the wide node whose source is binary reference `src`:
 * greedy opening of the largest-area openable child (SAH leaf decisions
 * fixed in the binary tree). */
int collapse_children(const Tree &t, uint32_t src, uint32_t out[8], int width) {
    if (!ref_openable(t, src)) { out[0] = src; return 1; }
    int n = 2;
    out[0] = t.nodes[src].left;
    out[1] = t.nodes[src].right;
    while (n < width) {
        int best = -1;
        float best_a = -1.0f;
        for (int i = 0; i < n; ++i) {
            if (!ref_openable(t, out[i])) continue;
            float a = half_area(ref_box(t, out[i]));
            if (a > best_a) { best_a = a; best = i; }
        }
        if (best < 0) break;
        uint32_t c = out[best];
        out[best] = t.nodes[c].left;
        out[n++] = t.nodes[c].right;
    }
    return n;
}

/* Assigns children to slots: greedy minimum of
 * cost(c, s) = sum_a sign_s(a) * (centre_c - centre_node)_a. */
void assign_slots(const Box &node, const Box *cb, int n, int slot_of[8]) {
    float diff[8][3];
    float ncen[3];
    for (int a = 0; a < 3; ++a) ncen[a] = (node.lo[a] + node.hi[a]) * 0.5f;
    for (int c = 0; c < n; ++c)
        for (int a = 0; a < 3; ++a) {
            if (box_is_empty(cb[c]) || box_is_empty(node)) diff[c][a] = 0.0f;
            else diff[c][a] = (cb[c].lo[a] + cb[c].hi[a]) * 0.5f - ncen[a];
        }
    float cost[8][8];
    for (int c = 0; c < n; ++c)
        for (int s = 0; s < 8; ++s) {
            float x = (s & 1) ? -diff[c][0] : diff[c][0];
            float y = (s & 2) ? -diff[c][1] : diff[c][1];
            float z = (s & 4) ? -diff[c][2] : diff[c][2];
            cost[c][s] = (x + y) + z;
        }
    bool used[8] = {false, false, false, false, false, false, false, false};
    for (int c = 0; c < n; ++c) slot_of[c] = -1;
    for (int it = 0; it < n; ++it) {
        int bc = -1, bs = -1;
        float bv = kInf;
        for (int c = 0; c < n; ++c) {
            if (slot_of[c] >= 0) continue;
            for (int s = 0; s < 8; ++s) {
                if (used[s]) continue;
                if (bc < 0 || cost[c][s] < bv) { bc = c; bs = s; bv = cost[c][s]; }
            }
        }
        slot_of[bc] = bs;
        used[bs] = true;
    }
}

/* Quantises children boxes against the node box and fills the node. */
void write_node(rt_bvh8_node &nd, const Box &node, const Box *slot_box, const bool *slot_used) {
    std::memset(&nd, 0, sizeof(nd));
    int e[3];
    float p[3];
    bool empty = box_is_empty(node);
    for (int a = 0; a < 3; ++a) {
        p[a] = empty ? 0.0f : node.lo[a];
        e[a] = empty ? 0 : qexp_for(sub_dir(node.hi[a], p[a], 1));
        nd.origin[a] = p[a];
        nd.exp[a] = (int8_t)e[a];
    }
    for (int s = 0; s < 8; ++s) {
        bool inv = !slot_used[s] || empty || box_is_empty(slot_box[s]);
        for (int a = 0; a < 3; ++a) {
            if (inv) { nd.qlo[a][s] = 255; nd.qhi[a][s] = 0; continue; }
            float sc = pow2f(-e[a]);
            float dl = sub_dir(slot_box[s].lo[a], p[a], 0) * sc;
            float dh_raw = sub_dir(slot_box[s].hi[a], p[a], 1);
            float dh = dh_raw * sc;
            float fl = std::floor(dl), fh = std::ceil(dh);
            int ql = fl < 0.0f ? 0 : (fl > 255.0f ? 255 : (int)fl);
            int qh = fh < 0.0f ? 0 : (fh > 255.0f ? 255 : (int)fh);
            if (qh == 0 && dh_raw > 0.0f) qh = 1;
            nd.qlo[a][s] = (uint8_t)ql;
            nd.qhi[a][s] = (uint8_t)qh;
        }
    }
}

BuildResult build_wide(const BuildInput &in, uint32_t flags, orc_lbvh_debug *dbg) {
    BuildResult res;
    const uint32_t wf = (flags & RT_BUILD_WIDTH_MASK) >> 16;
    const int width = wf ? (int)wf : 8;
    Tree t = build_tree(in, flags, res.morton_bits, dbg);
    uint32_t n = in.n;
    res.prims.resize((size_t)n * in.rec_bytes);
    if (n == 0) {
        rt_bvh8_node nd;
        Box b = box_empty();
        Box sb[8];
        for (int s = 0; s < 8; ++s) sb[s] = box_empty();
        bool used[8] = {false, false, false, false, false, false, false, false};
        write_node(nd, b, sb, used);
        res.nodes.push_back(nd);
        res.depth = 1;
        for (int a = 0; a < 3; ++a) { res.root.lo[a] = 0.0f; res.root.hi[a] = 0.0f; }
        return res;
    }
    res.root = ref_box(t, t.root_ref);
    std::vector<uint32_t> level{t.root_ref};
    std::vector<uint32_t> next;
    uint32_t prim_next = 0;
    while (!level.empty()) {
        ++res.depth;
        uint32_t base_index = (uint32_t)res.nodes.size();
        uint32_t next_base = base_index + (uint32_t)level.size();
        next.clear();
        res.nodes.resize(next_base);
        for (size_t k = 0; k < level.size(); ++k) {
            uint32_t src = level[k];
            uint32_t ch[8];
            int nc = collapse_children(t, src, ch, width);
            Box cb[8];
            for (int c = 0; c < nc; ++c) cb[c] = ref_box(t, ch[c]);
            Box nbox = ref_box(t, src);
            int slot_of[8];
            assign_slots(nbox, cb, nc, slot_of);
            uint32_t slot_ref[8];
            bool used[8] = {false, false, false, false, false, false, false, false};
            Box sbox[8];
            for (int c = 0; c < nc; ++c) {
                slot_ref[slot_of[c]] = ch[c];
                used[slot_of[c]] = true;
                sbox[slot_of[c]] = cb[c];
            }
            rt_bvh8_node &nd = res.nodes[base_index + k];
            write_node(nd, nbox, sbox, used);
            nd.child_base = next_base + (uint32_t)next.size();
            nd.prim_base = prim_next;
            uint32_t off = 0;
            for (int s = 0; s < 8; ++s) {
                if (!used[s]) continue;
                uint32_t r = slot_ref[s];
                if (ref_openable(t, r)) {
                    nd.imask |= (uint8_t)(1u << s);
                    nd.meta[s] = (uint8_t)((1u << 5) | (24u + (uint32_t)s));
                    next.push_back(r);
                } else {
                    uint32_t first, last;
                    ref_range(t, r, first, last);
                    uint32_t cnt = last - first + 1u;
                    nd.meta[s] = (uint8_t)((((1u << cnt) - 1u) << 5) | off);
                    for (uint32_t j = 0; j < cnt; ++j)
                        std::memcpy(&res.prims[(size_t)(prim_next + off + j) * in.rec_bytes],
                                    &in.records[(size_t)t.ids[first + j] * in.rec_bytes], in.rec_bytes);
                    off += cnt;
                }
            }
            prim_next += off;
        }
        level.swap(next);
    }
    return res;
}

void write_accel(void *accel, uint32_t kind, uint32_t prim_count, uint32_t geom_count, uint32_t flags,
                 uint32_t node_capacity, uint64_t total, const BuildResult &r, uint32_t rec_bytes,
                 const std::vector<uint32_t> &geom_table) {
    uint8_t *base = (uint8_t *)accel;
    rt_accel_header h;
    std::memset(&h, 0, sizeof(h));
    h.magic = RT_ACCEL_MAGIC;
    h.version = RT_ACCEL_VERSION;
    h.kind = kind;
    h.prim_count = prim_count;
    h.node_count = (uint32_t)r.nodes.size();
    h.geom_count = geom_count;
    h.build_flags = flags;
    h.status = 0;
    h.depth = r.depth;
    h.morton_bits = r.morton_bits;
    h.node_capacity = node_capacity;
    for (int a = 0; a < 3; ++a) { h.bounds_lo[a] = r.root.lo[a]; h.bounds_hi[a] = r.root.hi[a]; }
    h.node_offset = RT_ACCEL_HEADER_BYTES;
    h.prim_offset = h.node_offset + (uint64_t)node_capacity * 80u;
    h.geom_offset = h.prim_offset + (uint64_t)prim_count * rec_bytes;
    h.total_bytes = total;
    std::memcpy(base, &h, sizeof(h));
    std::memcpy(base + h.node_offset, r.nodes.data(), r.nodes.size() * 80u);
    std::memcpy(base + h.prim_offset, r.prims.data(), r.prims.size());
    if (!geom_table.empty()) std::memcpy(base + h.geom_offset, geom_table.data(), geom_table.size() * 4u);
}

inline uint32_t node_capacity_for(uint32_t n) { return n < 2 ? 1u : n - 1u; }
inline uint64_t align256(uint64_t x) { return (x + 255u) & ~255ull; }

/* ---------------------------------------------------------------------- */
/* Ray setup, triangle test, traversal                                    */
/* ---------------------------------------------------------------------- */

struct RaySetup {
    float o[3], d[3], invd[3];
    int neg[3];
    uint32_t oct;
    int kx, ky, kz;
    float sx, sy, sz;
};

void ray_setup(RaySetup &r, const float o[3], const float d[3]) {
    for (int a = 0; a < 3; ++a) {
        r.o[a] = o[a];
        r.d[a] = d[a];
        float dd = std::fabs(d[a]) < RT_DIR_EPS ? std::copysign(RT_DIR_EPS, d[a]) : d[a];
        r.invd[a] = 1.0f / dd;
        r.neg[a] = r.invd[a] < 0.0f ? 1 : 0;
    }
    r.oct = (uint32_t)r.neg[0] | ((uint32_t)r.neg[1] << 1) | ((uint32_t)r.neg[2] << 2);
    float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
    r.kz = ax >= ay ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
    r.kx = r.kz == 2 ? 0 : r.kz + 1;
    r.ky = r.kx == 2 ? 0 : r.kx + 1;
    if (d[r.kz] < 0.0f) std::swap(r.kx, r.ky);
    r.sx = d[r.kx] / d[r.kz];
    r.sy = d[r.ky] / d[r.kz];
    r.sz = 1.0f / d[r.kz];
}

inline int isect_tri(const RaySetup &r, const float *v0, const float *v1, const float *v2, float tmin,
                     float tmax, float &t_out, float &u_out, float &v_out) {
    float A[3], B[3], C[3];
    for (int a = 0; a < 3; ++a) { A[a] = v0[a] - r.o[a]; B[a] = v1[a] - r.o[a]; C[a] = v2[a] - r.o[a]; }
    float ax = A[r.kx] - r.sx * A[r.kz], ay = A[r.ky] - r.sy * A[r.kz];
    float bx = B[r.kx] - r.sx * B[r.kz], by = B[r.ky] - r.sy * B[r.kz];
    float cx = C[r.kx] - r.sx * C[r.kz], cy = C[r.ky] - r.sy * C[r.kz];
    float U = cx * by - cy * bx;
    float V = ax * cy - ay * cx;
    float W = bx * ay - by * ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)cx * (double)by - (double)cy * (double)bx);
        V = (float)((double)ax * (double)cy - (double)ay * (double)cx);
        W = (float)((double)bx * (double)ay - (double)by * (double)ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return 0;
    float det = (U + V) + W;
    if (det == 0.0f) return 0;
    float az = r.sz * A[r.kz], bz = r.sz * B[r.kz], cz = r.sz * C[r.kz];
    float T = (U * az + V * bz) + W * cz;
    float rcp = 1.0f / det;
    float t = T * rcp;
    if (!(t >= tmin && t <= tmax)) return 0;
    t_out = t;
    u_out = V * rcp;
    v_out = W * rcp;
    return 1;
}

/* Box test of the 8 children of a node; returns hit bits for internal
 * children (bit slot^oct) and the leaf record mask (24 bits). */
inline void isect_node(const RaySetup &r, const rt_bvh8_node &nd, float tmin, float tcur, uint32_t &node_hits,
                       uint32_t &prim_hits) {
    float sc[3], adj[3];
    for (int a = 0; a < 3; ++a) {
        sc[a] = pow2f(nd.exp[a]) * r.invd[a];
        adj[a] = (nd.origin[a] - r.o[a]) * r.invd[a];
    }
    node_hits = 0;
    prim_hits = 0;
    float tfar_lim = tcur;
    for (int s = 0; s < 8; ++s) {
        float tn = tmin, tf = tfar_lim;
        for (int a = 0; a < 3; ++a) {
            float qn = (float)(r.neg[a] ? nd.qhi[a][s] : nd.qlo[a][s]);
            float qf = (float)(r.neg[a] ? nd.qlo[a][s] : nd.qhi[a][s]);
            float n = std::fma(qn, sc[a], adj[a]);
            float f = std::fma(qf, sc[a], adj[a]);
            tn = std::fmax(tn, n);
            tf = std::fmin(tf, f);
        }
        if (!(tn <= tf * kTfarScale)) continue;
        if (nd.imask & (1u << s)) {
            node_hits |= 1u << ((uint32_t)s ^ r.oct);
        } else {
            uint32_t m = nd.meta[s];
            prim_hits |= (m >> 5) << (m & 31u);
        }
    }
}

struct AccelView {
    const rt_accel_header *h;
    const rt_bvh8_node *nodes;
    const uint8_t *prims;
};
inline AccelView view_of(const void *accel) {
    AccelView v;
    v.h = (const rt_accel_header *)accel;
    v.nodes = (const rt_bvh8_node *)((const uint8_t *)accel + v.h->node_offset);
    v.prims = (const uint8_t *)accel + v.h->prim_offset;
    return v;
}

struct HitState {
    float t;
    uint64_t key;
    float u, v;
    uint32_t tri;       /* build-input triangle index */
    uint32_t rec;       /* leaf-record index (bottom level) */
    uint32_t geom, prim;
    uint32_t inst;      /* instance index or 0 */
    uint32_t custom, sbt_off;
    bool found;
};

struct Group {
    uint32_t base;
    uint32_t hits;  /* node hits in bits 0..7, imask in 8..15 */
};

/* Traversal of one bottom-level BVH8.  Returns true on an accepted hit when
 * any_hit.  Visiting order: a node's leaf records first, then its internal
 * children in increasing (slot ^ octant); remaining siblings are pushed. */
bool traverse_blas(const AccelView &av, const RaySetup &r, float tmin, HitState &hs, bool any_hit,
                   uint32_t inst_id, uint32_t custom, uint32_t sbt_off, uint64_t *stats) {
    if (av.h->prim_count == 0) return false;
    Group stack[kMaxStack];
    int sp = 0;
    uint32_t node = 0;
    for (;;) {
        uint32_t nh, ph;
        const rt_bvh8_node &nd = av.nodes[node];
        isect_node(r, nd, tmin, hs.t, nh, ph);
        if (stats) stats[0]++;
        while (ph) {
            uint32_t i = (uint32_t)__builtin_ctz(ph);
            ph &= ph - 1u;
            const float *rec = (const float *)(av.prims + (size_t)(nd.prim_base + i) * 48u);
            if (stats) stats[1]++;
            float t, u, v;
            if (!isect_tri(r, rec, rec + 4, rec + 8, tmin, hs.t, t, u, v)) continue;
            uint32_t tri = fbits(rec[3]);
            uint64_t key = ((uint64_t)inst_id << 32) | tri;
            if (any_hit) {
                hs.t = t; hs.key = key; hs.u = u; hs.v = v; hs.tri = tri; hs.rec = nd.prim_base + i;
                hs.geom = fbits(rec[7]); hs.prim = fbits(rec[11]);
                hs.inst = inst_id; hs.custom = custom; hs.sbt_off = sbt_off; hs.found = true;
                return true;
            }
            if (t < hs.t || (t == hs.t && key < hs.key)) {
                hs.t = t; hs.key = key; hs.u = u; hs.v = v; hs.tri = tri; hs.rec = nd.prim_base + i;
                hs.geom = fbits(rec[7]); hs.prim = fbits(rec[11]);
                hs.inst = inst_id; hs.custom = custom; hs.sbt_off = sbt_off; hs.found = true;
            }
        }
        Group g{nd.child_base, nh | ((uint32_t)nd.imask << 8)};
        for (;;) {
            if (g.hits & 0xffu) {
                uint32_t k = (uint32_t)__builtin_ctz(g.hits & 0xffu);
                g.hits &= ~(1u << k);
                uint32_t s = k ^ r.oct;
                uint32_t imask = g.hits >> 8;
                node = g.base + (uint32_t)__builtin_popcount(imask & ((1u << s) - 1u));
                if (g.hits & 0xffu) {
                    if (sp == kMaxStack) return false;
                    stack[sp++] = g;
                }
                break;
            }
            if (sp == 0) return false;
            g = stack[--sp];
        }
    }
}

struct InstView {
    float w2o[3][4];
    uint64_t accel_ref;
    uint32_t cim, sof, id;
};

bool traverse(const void *accel, const rt_ray &ray, HitState &hs, bool any_hit, uint32_t cull_mask,
              uint64_t *stats) {
    AccelView av = view_of(accel);
    hs.t = ray.tmax;
    hs.key = ~0ull;
    hs.found = false;
    hs.u = hs.v = 0.0f;
    hs.tri = hs.geom = hs.prim = hs.inst = hs.custom = hs.sbt_off = 0;
    hs.rec = 0xffffffffu;
    RaySetup r;
    ray_setup(r, ray.org, ray.dir);
    if (av.h->kind == RT_ACCEL_KIND_BLAS) return traverse_blas(av, r, ray.tmin, hs, any_hit, 0, 0, 0, stats);
    if (av.h->prim_count == 0) return false;
    /* two-level: same visiting order over instance records */
    Group stack[kMaxStack];
    int sp = 0;
    uint32_t node = 0;
    for (;;) {
        uint32_t nh, ph;
        const rt_bvh8_node &nd = av.nodes[node];
        isect_node(r, nd, ray.tmin, hs.t, nh, ph);
        if (stats) stats[0]++;
        while (ph) {
            uint32_t i = (uint32_t)__builtin_ctz(ph);
            ph &= ph - 1u;
            InstView iv;
            std::memcpy(&iv, av.prims + (size_t)(nd.prim_base + i) * 80u, sizeof(iv));
            uint32_t mask = iv.cim >> 24;
            if ((mask & cull_mask) == 0u) continue;
            float o2[3], d2[3];
            xform_point(*(const rt_transform3x4 *)iv.w2o, ray.org, o2);
            xform_vector(iv.w2o, ray.dir, d2);
            RaySetup r2;
            ray_setup(r2, o2, d2);
            AccelView bv = view_of((const void *)(uintptr_t)iv.accel_ref);
            if (traverse_blas(bv, r2, ray.tmin, hs, any_hit, iv.id, iv.cim & 0xffffffu, iv.sof & 0xffffffu, stats))
                return true;
        }
        Group g{nd.child_base, nh | ((uint32_t)nd.imask << 8)};
        for (;;) {
            if (g.hits & 0xffu) {
                uint32_t k = (uint32_t)__builtin_ctz(g.hits & 0xffu);
                g.hits &= ~(1u << k);
                uint32_t s = k ^ r.oct;
                uint32_t imask = g.hits >> 8;
                node = g.base + (uint32_t)__builtin_popcount(imask & ((1u << s) - 1u));
                if (g.hits & 0xffu) {
                    if (sp == kMaxStack) return hs.found;
                    stack[sp++] = g;
                }
                break;
            }
            if (sp == 0) return hs.found;
            g = stack[--sp];
        }
    }
}

template <class F>
void parallel_for(uint32_t n, uint32_t n_threads, F f, uint32_t chunk = 4096) {
    if (n_threads == 0) n_threads = std::max(1u, std::thread::hardware_concurrency());
    if (n_threads > n) n_threads = n ? n : 1;
    if (n_threads <= 1) { f(0u, n); return; }
    std::vector<std::thread> th;
    std::atomic<uint32_t> next{0};
    for (uint32_t k = 0; k < n_threads; ++k)
        th.emplace_back([&]() {
            for (;;) {
                uint32_t b = next.fetch_add(chunk);
                if (b >= n) break;
                f(b, std::min(n, b + chunk));
            }
        });
    for (auto &x : th) x.join();
}

/* Prepares triangle records and boxes of a bottom-level build input. */
int prep_triangles(const orc_geometry *geoms, uint32_t n_geoms, BuildInput &in, std::vector<uint32_t> &gtab) {
    uint32_t total = 0;
    gtab.assign(n_geoms + 1, 0);
    for (uint32_t g = 0; g < n_geoms; ++g) { gtab[g] = total; total += geoms[g].tri_count; }
    gtab[n_geoms] = total;
    in.n = total;
    in.rec_bytes = 48;
    in.boxes.resize(total);
    in.active.resize(total);
    in.records.resize((size_t)total * 48u);
    int status = 0;
    for (uint32_t g = 0; g < n_geoms; ++g) {
        const orc_geometry &G = geoms[g];
        for (uint32_t p = 0; p < G.tri_count; ++p) {
            uint32_t gi = gtab[g] + p;
            uint32_t idx[3];
            for (int k = 0; k < 3; ++k)
                idx[k] = G.index_type == RT_INDEX_UINT32 ? G.indices[3 * p + k] : 3 * p + (uint32_t)k;
            float v[3][3];
            bool ok = true;
            for (int k = 0; k < 3; ++k) {
                if (idx[k] > G.max_vertex) { ok = false; status = RT_ERR_BOUNDS; break; }
                const float *src = (const float *)((const uint8_t *)G.vertices + (size_t)idx[k] * G.vertex_stride);
                float pt[3] = {src[0], src[1], src[2]};
                if (G.transform) xform_point(*G.transform, pt, v[k]);
                else for (int a = 0; a < 3; ++a) v[k][a] = pt[a];
            }
            if (ok)
                for (int k = 0; k < 3; ++k)
                    for (int a = 0; a < 3; ++a)
                        if (std::isnan(v[k][a])) ok = false;
            float rec[12];
            for (int k = 0; k < 3; ++k)
                for (int a = 0; a < 3; ++a) rec[4 * k + a] = ok ? v[k][a] : std::numeric_limits<float>::quiet_NaN();
            rec[3] = bitsf(gi);
            rec[7] = bitsf(g);
            rec[11] = bitsf(p);
            std::memcpy(&in.records[(size_t)gi * 48u], rec, 48);
            Box b = box_empty();
            if (ok)
                for (int a = 0; a < 3; ++a) {
                    b.lo[a] = fmn(fmn(v[0][a], v[1][a]), v[2][a]);
                    b.hi[a] = fmx(fmx(v[0][a], v[1][a]), v[2][a]);
                }
            in.boxes[gi] = b;
            in.active[gi] = ok ? 1 : 0;
        }
    }
    return status;
}

/* Leaf record and world box of instance i. */
void inst_input(const rt_instance &I, uint32_t i, rt_inst_record &rec, Box &b) {
    std::memset(&rec, 0, sizeof(rec));
    bool ok = invert3x4(I.transform, rec.world_to_object);
    rec.accel_ref = I.accel_ref;
    rec.custom_index_and_mask = I.custom_index_and_mask;
    rec.sbt_offset_and_flags = I.sbt_offset_and_flags;
    rec.instance_id = i;
    const rt_accel_header *bh = (const rt_accel_header *)(uintptr_t)I.accel_ref;
    b = box_empty();
    if (ok && bh && bh->prim_count > 0) {
        for (int c = 0; c < 8; ++c) {
            float pt[3] = {(c & 1) ? bh->bounds_hi[0] : bh->bounds_lo[0],
                           (c & 2) ? bh->bounds_hi[1] : bh->bounds_lo[1],
                           (c & 4) ? bh->bounds_hi[2] : bh->bounds_lo[2]};
            float w[3];
            xform_point(I.transform, pt, w);
            for (int a = 0; a < 3; ++a) { b.lo[a] = fmn(b.lo[a], w[a]); b.hi[a] = fmx(b.hi[a], w[a]); }
        }
    }
}

/* Refit of the nodes of `accel` whose leaf records already hold the new
 * primitives, leaf_box[r] the box of record r: nodes in reverse order (every
 * child follows its parent), each node's box the union of its slots'. */
void refit_nodes(uint8_t *base, const std::vector<Box> &leaf_box) {
    rt_accel_header *h = (rt_accel_header *)base;
    rt_bvh8_node *nodes = (rt_bvh8_node *)(base + h->node_offset);
    std::vector<Box> nb(h->node_count);
    for (int64_t k = (int64_t)h->node_count - 1; k >= 0; --k) {
        rt_bvh8_node &nd = nodes[k];
        Box sbox[8];
        bool used[8];
        Box node = box_empty();
        for (int s = 0; s < 8; ++s) {
            const uint8_t meta = nd.meta[s];
            used[s] = meta != 0;
            sbox[s] = box_empty();
            if ((nd.imask >> s) & 1u) {
                sbox[s] = nb[nd.child_base + (uint32_t)__builtin_popcount(nd.imask & ((1u << s) - 1u))];
            } else if (meta) {
                const uint32_t cnt = (uint32_t)__builtin_popcount(meta >> 5), first = nd.prim_base + (meta & 0x1fu);
                for (uint32_t j = 0; j < cnt; ++j) sbox[s] = box_union(sbox[s], leaf_box[first + j]);
            }
            if (used[s]) node = box_union(node, sbox[s]);
        }
        const uint32_t cb = nd.child_base, pb = nd.prim_base;
        const uint8_t imask = nd.imask;
        uint8_t meta[8];
        std::memcpy(meta, nd.meta, 8);
        write_node(nd, node, sbox, used);
        nd.child_base = cb;
        nd.prim_base = pb;
        nd.imask = imask;
        std::memcpy(nd.meta, meta, 8);
        nb[k] = node;
    }
    for (int a = 0; a < 3; ++a) { h->bounds_lo[a] = nb[0].lo[a]; h->bounds_hi[a] = nb[0].hi[a]; }
}

/* The tree of `accel` is consistent: children after their parent, leaf
 * ranges inside the records. */
bool tree_ok(const uint8_t *base) {
    const rt_accel_header *h = (const rt_accel_header *)base;
    if (h->node_count == 0 || h->node_count > h->node_capacity) return false;
    const rt_bvh8_node *nodes = (const rt_bvh8_node *)(base + h->node_offset);
    for (uint32_t k = 0; k < h->node_count; ++k) {
        const rt_bvh8_node &nd = nodes[k];
        const uint32_t ni = (uint32_t)__builtin_popcount(nd.imask);
        if (ni && (nd.child_base <= k || (uint64_t)nd.child_base + ni > h->node_count)) return false;
        for (int s = 0; s < 8; ++s)
            if (!((nd.imask >> s) & 1u) && nd.meta[s]) {
                const uint32_t cnt = (uint32_t)__builtin_popcount(nd.meta[s] >> 5);
                if ((uint64_t)nd.prim_base + (nd.meta[s] & 0x1fu) + cnt > h->prim_count) return false;
            }
    }
    return true;
}

}  // namespace

/* ====================================================================== */
/* extern "C" API                                                          */
/* ====================================================================== */

extern "C" {

uint32_t orc_hw_threads(void) { return std::max(1u, std::thread::hardware_concurrency()); }

uint64_t orc_blas_accel_bytes(const uint32_t *tri_counts, uint32_t n_geoms) {
    uint64_t n = 0;
    for (uint32_t g = 0; g < n_geoms; ++g) n += tri_counts[g];
    uint64_t cap = node_capacity_for((uint32_t)n);
    return align256(RT_ACCEL_HEADER_BYTES + cap * 80u + n * 48u + (uint64_t)(n_geoms + 1) * 4u);
}

uint64_t orc_tlas_accel_bytes(uint32_t n_instances) {
    uint64_t cap = node_capacity_for(n_instances);
    return align256(RT_ACCEL_HEADER_BYTES + cap * 80u + (uint64_t)n_instances * 80u);
}

inline bool width_ok(uint32_t flags) {
    const uint32_t w = (flags & RT_BUILD_WIDTH_MASK) >> 16;
    return w == 0u || (w >= 4u && w <= 8u);
}

int orc_build_blas(const orc_geometry *geoms, uint32_t n_geoms, uint32_t flags, void *accel, uint64_t accel_bytes,
                   orc_lbvh_debug *dbg) {
    if (!width_ok(flags)) return RT_ERR_INVALID_ARG;
    std::vector<uint32_t> counts(n_geoms);
    for (uint32_t g = 0; g < n_geoms; ++g) counts[g] = geoms[g].tri_count;
    uint64_t need = orc_blas_accel_bytes(counts.data(), n_geoms);
    if (accel_bytes < need) return RT_ERR_OOM;
    BuildInput in;
    std::vector<uint32_t> gtab;
    int st = prep_triangles(geoms, n_geoms, in, gtab);
    BuildResult r = build_wide(in, flags, dbg);
    write_accel(accel, RT_ACCEL_KIND_BLAS, in.n, n_geoms, flags, node_capacity_for(in.n), need, r, 48, gtab);
    if (st) ((rt_accel_header *)accel)->status = (uint32_t)(-st);
    return st;
}

int orc_build_tlas(const rt_instance *instances, uint32_t n, uint32_t flags, void *accel, uint64_t accel_bytes) {
    if (!width_ok(flags)) return RT_ERR_INVALID_ARG;
    uint64_t need = orc_tlas_accel_bytes(n);
    if (accel_bytes < need) return RT_ERR_OOM;
    BuildInput in;
    in.n = n;
    in.rec_bytes = 80;
    in.boxes.resize(n);
    in.active.resize(n);
    in.records.assign((size_t)n * 80u, 0);
    for (uint32_t i = 0; i < n; ++i) {
        rt_inst_record rec;
        Box b;
        inst_input(instances[i], i, rec, b);
        in.boxes[i] = b;
        in.active[i] = box_is_empty(b) ? 0 : 1;
        std::memcpy(&in.records[(size_t)i * 80u], &rec, 80);
    }
    BuildResult r = build_wide(in, flags, nullptr);
    std::vector<uint32_t> none;
    write_accel(accel, RT_ACCEL_KIND_TLAS, n, 0, flags, node_capacity_for(n), need, r, 80, none);
    return 0;
}

int orc_refit_blas(const orc_geometry *geoms, uint32_t n_geoms, void *accel) {
    uint8_t *base = (uint8_t *)accel;
    rt_accel_header *h = (rt_accel_header *)base;
    uint64_t n = 0;
    for (uint32_t g = 0; g < n_geoms; ++g) n += geoms[g].tri_count;
    if (h->magic != RT_ACCEL_MAGIC || h->kind != RT_ACCEL_KIND_BLAS || h->prim_count != n ||
        h->geom_count != n_geoms || h->node_capacity != node_capacity_for((uint32_t)n))
        return RT_ERR_INVALID_ARG;
    if (n == 0) return 0;
    if (!tree_ok(base)) return RT_ERR_INVALID_ARG;
    BuildInput in;
    std::vector<uint32_t> gtab;
    const int st = prep_triangles(geoms, n_geoms, in, gtab);
    std::vector<Box> leaf_box(n);
    uint8_t *recs = base + h->prim_offset;
    for (uint32_t r = 0; r < n; ++r) {
        uint32_t ids[3];
        for (int k = 0; k < 3; ++k) std::memcpy(&ids[k], recs + (size_t)r * 48u + 16u * k + 12u, 4);
        const uint32_t gi = ids[0], g = ids[1], p = ids[2];
        if (g >= n_geoms || p >= geoms[g].tri_count || gi != gtab[g] + p) return RT_ERR_INVALID_ARG;
        std::memcpy(recs + (size_t)r * 48u, &in.records[(size_t)gi * 48u], 48);
        leaf_box[r] = in.boxes[gi];
    }
    refit_nodes(base, leaf_box);
    if (st && h->status == 0) h->status = (uint32_t)(-st);
    return st;
}

int orc_refit_tlas(const rt_instance *instances, uint32_t n, void *accel) {
    uint8_t *base = (uint8_t *)accel;
    rt_accel_header *h = (rt_accel_header *)base;
    if (h->magic != RT_ACCEL_MAGIC || h->kind != RT_ACCEL_KIND_TLAS || h->prim_count != n ||
        h->node_capacity != node_capacity_for(n))
        return RT_ERR_INVALID_ARG;
    if (n == 0) return 0;
    if (!tree_ok(base)) return RT_ERR_INVALID_ARG;
    std::vector<Box> leaf_box(n);
    uint8_t *recs = base + h->prim_offset;
    for (uint32_t r = 0; r < n; ++r) {
        rt_inst_record rec;
        std::memcpy(&rec, recs + (size_t)r * 80u, 80);
        const uint32_t i = rec.instance_id;
        if (i >= n) return RT_ERR_INVALID_ARG;
        inst_input(instances[i], i, rec, leaf_box[r]);
        std::memcpy(recs + (size_t)r * 80u, &rec, 80);
    }
    refit_nodes(base, leaf_box);
    return 0;
}

int orc_intersect_tri(const float org[3], const float dir[3], float tmin, float tmax, const float v0[3],
                      const float v1[3], const float v2[3], float *t, float *u, float *v) {
    RaySetup r;
    ray_setup(r, org, dir);
    return isect_tri(r, v0, v1, v2, tmin, tmax, *t, *u, *v);
}

void orc_trace_closest(const void *accel, const rt_ray *rays, rt_hit *hits, rt_hit_ext *hits_ext, uint32_t n,
                       uint32_t n_threads, uint64_t *stats) {
    std::atomic<uint64_t> s0{0}, s1{0};
    parallel_for(n, n_threads, [&](uint32_t b, uint32_t e) {
        uint64_t st[2] = {0, 0};
        for (uint32_t i = b; i < e; ++i) {
            HitState hs;
            traverse(accel, rays[i], hs, false, 0xffu, stats ? st : nullptr);
            rt_hit h;
            if (hs.found) { h.t = hs.t; h.prim = hs.tri; h.u = hs.u; h.v = hs.v; }
            else { h.t = kInf; h.prim = RT_NO_HIT; h.u = 0.0f; h.v = 0.0f; }
            if (hits) hits[i] = h;
            if (hits_ext) {
                rt_hit_ext x;
                x.t = h.t; x.u = h.u; x.v = h.v;
                x.instance_id = hs.found ? hs.inst : RT_NO_HIT;
                x.custom_index = hs.found ? hs.custom : 0;
                x.geometry_index = hs.found ? hs.geom : 0;
                x.primitive_id = hs.found ? hs.prim : RT_NO_HIT;
                x.sbt_record = hs.found ? hs.sbt_off + hs.geom : 0;
                hits_ext[i] = x;
            }
        }
        s0 += st[0];
        s1 += st[1];
    });
    if (stats) { stats[0] = s0.load(); stats[1] = s1.load(); }
}

void orc_trace_any(const void *accel, const rt_ray *rays, uint8_t *occluded, uint32_t n, uint32_t n_threads,
                   uint64_t *stats) {
    std::atomic<uint64_t> s0{0}, s1{0};
    parallel_for(n, n_threads, [&](uint32_t b, uint32_t e) {
        uint64_t st[2] = {0, 0};
        for (uint32_t i = b; i < e; ++i) {
            HitState hs;
            occluded[i] = traverse(accel, rays[i], hs, true, 0xffu, stats ? st : nullptr) ? 1 : 0;
        }
        s0 += st[0];
        s1 += st[1];
    });
    if (stats) { stats[0] = s0.load(); stats[1] = s1.load(); }
}

void orc_brute_closest(const orc_geometry *geoms, uint32_t n_geoms, const rt_ray *rays, rt_hit *hits, uint32_t n,
                       int precision, uint32_t n_threads) {
    BuildInput in;
    std::vector<uint32_t> gtab;
    prep_triangles(geoms, n_geoms, in, gtab);
    const float *recs = (const float *)in.records.data();
    parallel_for(n, n_threads, [&](uint32_t b, uint32_t e) {
        for (uint32_t i = b; i < e; ++i) {
            const rt_ray &ray = rays[i];
            rt_hit h{kInf, RT_NO_HIT, 0.0f, 0.0f};
            if (precision == 32) {
                RaySetup r;
                ray_setup(r, ray.org, ray.dir);
                float bt = ray.tmax;
                uint32_t bk = RT_NO_HIT;
                for (uint32_t p = 0; p < in.n; ++p) {
                    if (!in.active[p]) continue;
                    const float *rec = recs + (size_t)p * 12u;
                    float t, u, v;
                    if (!isect_tri(r, rec, rec + 4, rec + 8, ray.tmin, bt, t, u, v)) continue;
                    if (t < bt || (t == bt && p < bk)) { bt = t; bk = p; h = rt_hit{t, p, u, v}; }
                }
            } else {
                /* the same watertight algorithm in double precision */
                double o[3] = {ray.org[0], ray.org[1], ray.org[2]}, d[3] = {ray.dir[0], ray.dir[1], ray.dir[2]};
                double adx = std::fabs(d[0]), ady = std::fabs(d[1]), adz = std::fabs(d[2]);
                int kz = adx >= ady ? (adx >= adz ? 0 : 2) : (ady >= adz ? 1 : 2);
                int kx = kz == 2 ? 0 : kz + 1, ky = kx == 2 ? 0 : kx + 1;
                if (d[kz] < 0.0) std::swap(kx, ky);
                double sx = d[kx] / d[kz], sy = d[ky] / d[kz], sz = 1.0 / d[kz];
                double bt = ray.tmax;
                uint32_t bk = RT_NO_HIT;
                for (uint32_t p = 0; p < in.n; ++p) {
                    if (!in.active[p]) continue;
                    const float *rec = recs + (size_t)p * 12u;
                    double A[3], B[3], C[3];
                    for (int a = 0; a < 3; ++a) { A[a] = rec[a] - o[a]; B[a] = rec[4 + a] - o[a]; C[a] = rec[8 + a] - o[a]; }
                    double ax = A[kx] - sx * A[kz], ay = A[ky] - sy * A[kz];
                    double bx = B[kx] - sx * B[kz], by = B[ky] - sy * B[kz];
                    double cx = C[kx] - sx * C[kz], cy = C[ky] - sy * C[kz];
                    double U = cx * by - cy * bx, V = ax * cy - ay * cx, W = bx * ay - by * ax;
                    if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) continue;
                    double det = U + V + W;
                    if (det == 0.0) continue;
                    double T = U * (sz * A[kz]) + V * (sz * B[kz]) + W * (sz * C[kz]);
                    double t = T / det;
                    if (!(t >= ray.tmin && t <= bt)) continue;
                    if (t < bt || (t == bt && p < bk)) {
                        bt = t; bk = p;
                        h = rt_hit{(float)t, p, (float)(V / det), (float)(W / det)};
                    }
                }
            }
            hits[i] = h;
        }
    });
}

void orc_raygen(const rt_camera *cam, uint32_t width, uint32_t height, uint32_t x, uint32_t y, float org[3],
                float dir[3]) {
    /* aspect_y = tan(radians(yFov) * 0.5): radians and the halving in float
     * as GLSL evaluates them, tan evaluated in double and rounded once (the
     * GPU receives this same value from the host). */
    float half = (cam->y_fov_degree * (float)(3.14159265358979323846 / 180.0)) * 0.5f;
    float ay = (float)std::tan((double)half);
    float ax = (ay * (float)width) / (float)height;
    float sx = (float)x + 0.5f, sy = (float)y + 0.5f;
    float ndx = (sx / (float)width) * 2.0f - 1.0f;
    float ndy = (sy / (float)height) * 2.0f - 1.0f;
    float a = ndx * ax, b = ndy * ay;
    /* a*(1,0,0) + b*(0,-1,0) + (0,0,-1), component by component */
    dir[0] = (a * 1.0f + b * 0.0f) + 0.0f;
    dir[1] = (a * 0.0f + b * -1.0f) + 0.0f;
    dir[2] = (a * 0.0f + b * 0.0f) + -1.0f;
    org[0] = cam->position[0];
    org[1] = cam->position[1];
    org[2] = cam->position[2];
}

int orc_trace_rays(const rt_pipeline *p, const float *sbt_colors, uint32_t sbt_count, uint32_t sbt_stride,
                   const void *accel, const rt_camera *cam, float *out, uint32_t width, uint32_t height,
                   uint32_t n_threads) {
    std::atomic<int> status{0};
    parallel_for(width * height, n_threads, [&](uint32_t b, uint32_t e) {
        for (uint32_t i = b; i < e; ++i) {
            uint32_t x = i % width, y = i / width;
            rt_ray ray;
            orc_raygen(cam, width, height, x, y, ray.org, ray.dir);
            ray.tmin = p->tmin;
            ray.tmax = p->tmax;
            HitState hs;
            bool any = (p->ray_flags & RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT) != 0;
            traverse(accel, ray, hs, any, p->cull_mask & 0xffu, nullptr);
            float c[3];
            if (!hs.found) {
                c[0] = p->miss_color[0]; c[1] = p->miss_color[1]; c[2] = p->miss_color[2];
            } else if (p->ray_flags & RT_RAY_FLAG_SKIP_CLOSEST_HIT) {
                c[0] = c[1] = c[2] = 0.0f;  /* payload keeps raygen's vec3(0.0) */
            } else {
                uint32_t rec = hs.sbt_off + hs.geom * p->sbt_record_stride + p->sbt_record_offset;
                bool bary = p->chit == RT_CHIT_BARYCENTRIC ||
                            (p->chit == RT_CHIT_SAMPLE && hs.prim == 1u && hs.inst == 1u && hs.custom == 100u &&
                             hs.geom == 1u);
                if (bary) {
                    c[0] = (1.0f - hs.u) - hs.v; c[1] = hs.u; c[2] = hs.v;
                } else if (rec < sbt_count) {
                    for (int k = 0; k < 3; ++k) c[k] = sbt_colors[(size_t)rec * sbt_stride + k];
                } else {
                    c[0] = c[1] = c[2] = 0.0f;
                    status = RT_ERR_BOUNDS;
                }
            }
            float *px = out + (size_t)i * 4u;
            px[0] = c[0]; px[1] = c[1]; px[2] = c[2]; px[3] = 0.0f;
        }
    });
    return status.load();
}

void orc_sort_pairs(uint64_t *keys, uint32_t *vals, uint32_t n, uint32_t bits) {
    uint64_t mask = bits >= 64 ? ~0ull : ((1ull << bits) - 1ull);
    std::vector<uint32_t> idx(n);
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return (keys[a] & mask) < (keys[b] & mask); });
    std::vector<uint64_t> k2(n);
    std::vector<uint32_t> v2(n);
    for (uint32_t i = 0; i < n; ++i) { k2[i] = keys[idx[i]]; v2[i] = vals[idx[i]]; }
    std::memcpy(keys, k2.data(), n * 8ull);
    std::memcpy(vals, v2.data(), n * 4ull);
}

}  // extern "C"

/* ====================================================================== */
/* Path tracer (restatement of rtcore_pt.h's light transport)             */
/* ====================================================================== */

namespace {

struct Rng {
    uint64_t state, inc;
    uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
    float uni() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
};

uint64_t mix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

Rng rng_for(uint64_t seed, uint32_t sample, uint32_t pixel) {
    Rng g;
    g.inc = ((uint64_t)pixel << 1u) | 1u;
    g.state = 0;
    g.next();
    g.state += mix64(seed + sample);
    g.next();
    return g;
}

/* PCG32 stream `seq` started from `seed` (the workload generators). */
Rng seeded_rng(uint64_t seed, uint64_t seq) {
    Rng g;
    g.inc = (seq << 1u) | 1u;
    g.state = 0;
    g.next();
    g.state += seed;
    g.next();
    return g;
}

float uni_in(Rng &g, float a, float b) { return a + (b - a) * g.uni(); }

/* Uniform direction on the unit sphere: rejection sampling from the cube. */
void sphere_dir(Rng &g, float d[3]) {
    for (;;) {
        float x = 2.0f * g.uni() - 1.0f, y = 2.0f * g.uni() - 1.0f, z = 2.0f * g.uni() - 1.0f;
        float r2 = (x * x + y * y) + z * z;
        if (r2 > 1e-6f && r2 <= 1.0f) {
            float inv = 1.0f / std::sqrt(r2);
            d[0] = x * inv;
            d[1] = y * inv;
            d[2] = z * inv;
            return;
        }
    }
}

/* Taylor polynomials of sin (to x^9) and cos (to x^8), |x| <= pi/4. */
float poly_sin(float x) {
    float x2 = x * x;
    return x * (1.0f + x2 * (-1.0f / 6.0f + x2 * (1.0f / 120.0f + x2 * (-1.0f / 5040.0f + x2 * (1.0f / 362880.0f)))));
}
float poly_cos(float x) {
    float x2 = x * x;
    return 1.0f + x2 * (-0.5f + x2 * (1.0f / 24.0f + x2 * (-1.0f / 720.0f + x2 * (1.0f / 40320.0f))));
}

inline float dot(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
inline void cross(const float a[3], const float b[3], float c[3]) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

struct LightInfo {
    float n[3];
    float area;
};

}  // namespace

extern "C" void orc_sincos_q(float x, float *s, float *c) {
    *s = poly_sin(x);
    *c = poly_cos(x);
}

namespace {

/* Everything a path needs that does not depend on the pixel: the scene, the
 * light table (per-light normal and area, the area CDF in light order) and
 * the camera's aspect factors. */
struct PtSetup {
    const void *accel;
    AccelView av;
    const uint32_t *tri_material;
    const rt_material *materials;
    uint32_t n_materials;
    const rt_pt_light *lights;
    uint32_t n_lights;
    const rt_pt_params *p;
    std::vector<LightInfo> li;
    std::vector<float> cdf;
    float total, ax, ay;
};

int pt_setup(PtSetup &c, const void *accel, const uint32_t *tri_material, const rt_material *materials,
             uint32_t n_materials, const rt_pt_light *lights, uint32_t n_lights, const rt_pt_params *p) {
    c.accel = accel;
    c.av = view_of(accel);
    if (c.av.h->kind != RT_ACCEL_KIND_BLAS) return RT_ERR_INVALID_ARG;
    c.tri_material = tri_material;
    c.materials = materials;
    c.n_materials = n_materials;
    c.lights = lights;
    c.n_lights = n_lights;
    c.p = p;
    c.li.resize(n_lights);
    c.cdf.resize(n_lights + 1);
    float acc = 0.0f;
    for (uint32_t k = 0; k < n_lights; ++k) {
        const rt_pt_light &l = lights[k];
        float e1[3], e2[3], cr[3];
        for (int a = 0; a < 3; ++a) { e1[a] = l.v1[a] - l.v0[a]; e2[a] = l.v2[a] - l.v0[a]; }
        cross(e1, e2, cr);
        float len = std::sqrt(dot(cr, cr));
        float inv = len > 0.0f ? 1.0f / len : 0.0f;
        for (int a = 0; a < 3; ++a) c.li[k].n[a] = cr[a] * inv;
        c.li[k].area = 0.5f * len;
        acc = acc + c.li[k].area;
        c.cdf[k] = acc;
    }
    c.cdf[n_lights] = acc;
    c.total = acc;
    const float half = (p->camera.y_fov_degree * (float)(3.14159265358979323846 / 180.0)) * 0.5f;
    c.ay = (float)std::tan((double)half);
    c.ax = (c.ay * (float)p->width) / (float)p->height;
    return RT_OK;
}

/* Training pixels of a sample in the learned form: (pixel + offset) % stride
 * == 0, the offset drawn per sample from the seed (rt_path_trace_cached). */
uint32_t train_offset(uint64_t seed, uint32_t sample, uint32_t stride) {
    return (uint32_t)(mix64(seed ^ (0x5851f42d4c957f2dull + sample)) % stride);
}

/* One path: sample `sample` of pixel `pix`.  Adds its radiance to L.  With
 * stride > 0 the path follows the learned form (rec receives what the
 * second vertex recorded; a query path stops there, before next-event
 * estimation); otherwise it is the plain path tracer. */
int pt_sample(const PtSetup &c, uint32_t pix, uint32_t sample, uint32_t stride, orc_path_record *rec,
              float L[3]) {
    const float kInvPi = 0.318309886183790671538f, kPi4 = 0.785398163397448309616f;
    const rt_pt_params *p = c.p;
    int status = 0;
    const uint32_t x = pix % p->width, y = pix / p->width;
    Rng g = rng_for(p->seed, sample, pix);
    float jx = g.uni(), jy = g.uni();
    float sx = (float)x + jx, sy = (float)y + jy;
    float ndx = (sx / (float)p->width) * 2.0f - 1.0f, ndy = (sy / (float)p->height) * 2.0f - 1.0f;
    float pp = ndx * c.ax, qq = ndy * c.ay;
    rt_ray ray;
    for (int a = 0; a < 3; ++a) ray.org[a] = p->camera.position[a];
    ray.dir[0] = (pp * 1.0f + qq * 0.0f) + 0.0f;
    ray.dir[1] = (pp * 0.0f + qq * -1.0f) + 0.0f;
    ray.dir[2] = (pp * 0.0f + qq * 0.0f) + -1.0f;
    ray.tmin = 0.0f;
    ray.tmax = 1e30f;
    float T[3] = {1.0f, 1.0f, 1.0f};
    const uint32_t off = stride ? train_offset(p->seed, sample, stride) : 0u;
    for (uint32_t depth = 0; depth < p->max_depth; ++depth) {
        float u[6];
        for (int k = 0; k < 6; ++k) u[k] = g.uni();
        HitState hs;
        traverse(c.accel, ray, hs, false, 0xffu, nullptr);
        if (!hs.found) break;
        const float *r = (const float *)(c.av.prims + (size_t)hs.rec * 48u);
        const float *v0 = r, *v1 = r + 4, *v2 = r + 8;
        float P[3], e1[3], e2[3], ng[3], n[3];
        for (int a = 0; a < 3; ++a) {
            P[a] = ray.org[a] + hs.t * ray.dir[a];
            e1[a] = v1[a] - v0[a];
            e2[a] = v2[a] - v0[a];
        }
        cross(e1, e2, ng);
        float len = std::sqrt(dot(ng, ng));
        if (!(len > 0.0f)) break;
        for (int a = 0; a < 3; ++a) n[a] = ng[a] / len;
        float cosd = dot(n, ray.dir);
        uint32_t mi = c.tri_material[hs.tri];
        if (mi >= c.n_materials) { status = RT_ERR_BOUNDS; mi = 0; }
        const rt_material &m = c.materials[mi];
        if (depth == 0 && cosd < 0.0f)
            for (int a = 0; a < 3; ++a) L[a] = L[a] + T[a] * m.emission[a];
        if (cosd > 0.0f)
            for (int a = 0; a < 3; ++a) n[a] = -n[a];
        if (!(m.albedo[0] > 0.0f || m.albedo[1] > 0.0f || m.albedo[2] > 0.0f)) break;
        if (stride && depth == 1u) {
            for (int a = 0; a < 3; ++a) {
                rec->rec.pos[a] = P[a];
                rec->rec.dir[a] = -ray.dir[a];
                rec->rec.normal[a] = n[a];
                rec->rec.albedo[a] = m.albedo[a];
                rec->t1[a] = T[a];
                rec->L_before[a] = L[a];
            }
            if ((pix + off) % stride != 0u) {
                rec->kind = 1u;  /* ends in a cache query */
                return status;
            }
            rec->kind = 2u;      /* training path: goes on as plain path tracing */
        }
        if (c.n_lights > 0) {
            float target = u[0] * c.total;
            uint32_t lo = 0, hi = c.n_lights - 1u;
            while (lo < hi) {
                uint32_t mid = (lo + hi) >> 1;
                if (c.cdf[mid] > target) hi = mid; else lo = mid + 1u;
            }
            const rt_pt_light &Lt = c.lights[lo];
            float su = std::sqrt(u[1]);
            float b0 = 1.0f - su, b1 = u[2] * su, b2 = (1.0f - b0) - b1;
            float lp[3], wi[3];
            for (int a = 0; a < 3; ++a) {
                lp[a] = (Lt.v0[a] * b0 + Lt.v1[a] * b1) + Lt.v2[a] * b2;
                wi[a] = lp[a] - P[a];
            }
            float dist2 = dot(wi, wi);
            float dist = std::sqrt(dist2);
            if (dist > 0.0f) {
                float wn[3];
                for (int a = 0; a < 3; ++a) wn[a] = wi[a] / dist;
                float cos_s = dot(n, wn), cos_l = -dot(c.li[lo].n, wn);
                if (cos_s > 0.0f && cos_l > 0.0f) {
                    float f = (((cos_s * cos_l) / dist2) * c.total) * kInvPi;
                    rt_ray sr;
                    float contrib[3];
                    for (int a = 0; a < 3; ++a) {
                        contrib[a] = ((T[a] * m.albedo[a]) * Lt.emission[a]) * f;
                        sr.org[a] = P[a] + n[a] * p->ray_eps;
                    }
                    for (int a = 0; a < 3; ++a) sr.dir[a] = lp[a] - sr.org[a];
                    sr.tmin = 0.0f;
                    sr.tmax = 0.9999f;
                    HitState sh;
                    if (!traverse(c.accel, sr, sh, true, 0xffu, nullptr))
                        for (int a = 0; a < 3; ++a) L[a] = L[a] + contrib[a];
                }
            }
        }
        if (depth >= p->rr_depth) {
            float ps = std::fmax(std::fmax(T[0], T[1]), T[2]);
            ps = ps < 0.95f ? ps : 0.95f;
            if (!(u[5] < ps)) break;
            for (int a = 0; a < 3; ++a) T[a] = T[a] / ps;
        }
        if (depth + 1u >= p->max_depth) break;
        /* cosine-weighted direction: concentric disk lifted to the hemisphere */
        float da = 2.0f * u[3] - 1.0f, db = 2.0f * u[4] - 1.0f, dx, dy;
        if (da == 0.0f && db == 0.0f) {
            dx = 0.0f; dy = 0.0f;
        } else if (std::fabs(da) > std::fabs(db)) {
            float phi = kPi4 * (db / da);
            dx = da * poly_cos(phi); dy = da * poly_sin(phi);
        } else {
            float phi = kPi4 * (da / db);
            dx = db * poly_sin(phi); dy = db * poly_cos(phi);
        }
        float zz = (1.0f - dx * dx) - dy * dy;
        float dz = std::sqrt(zz > 0.0f ? zz : 0.0f);
        float sign = std::copysign(1.0f, n[2]);
        float oa = -1.0f / (sign + n[2]);
        float ob = n[0] * n[1] * oa;
        float t1[3] = {1.0f + sign * n[0] * n[0] * oa, sign * ob, -sign * n[0]};
        float t2[3] = {ob, sign + n[1] * n[1] * oa, -n[1]};
        for (int a = 0; a < 3; ++a) {
            ray.dir[a] = (t1[a] * dx + t2[a] * dy) + n[a] * dz;
            ray.org[a] = P[a] + n[a] * p->ray_eps;
            T[a] = T[a] * m.albedo[a];
        }
        ray.tmin = 0.0f;
        ray.tmax = 1e30f;
    }
    return status;
}

}  // namespace

extern "C" int orc_path_trace(const void *accel, const uint32_t *tri_material, const rt_material *materials,
                              uint32_t n_materials, const rt_pt_light *lights, uint32_t n_lights,
                              const rt_pt_params *p, float *accum, uint32_t n_threads) {
    PtSetup c;
    int rc = pt_setup(c, accel, tri_material, materials, n_materials, lights, n_lights, p);
    if (rc) return rc;
    std::atomic<int> status{0};
    const uint32_t npix = p->width * p->height;
    parallel_for(npix, n_threads, [&](uint32_t b, uint32_t e) {
        for (uint32_t pix = b; pix < e; ++pix) {
            for (uint32_t s = 0; s < p->spp; ++s) {
                float L[3] = {0.0f, 0.0f, 0.0f};
                int st = pt_sample(c, pix, p->sample_offset + s, 0u, nullptr, L);
                if (st) status = st;
                float *px = accum + (size_t)pix * 4u;
                for (int a = 0; a < 3; ++a) px[a] = px[a] + L[a];
                px[3] = px[3] + 1.0f;
            }
        }
    });
    return status.load();
}

extern "C" int orc_path_trace_pixels(const void *accel, const uint32_t *tri_material, const rt_material *materials,
                                     uint32_t n_materials, const rt_pt_light *lights, uint32_t n_lights,
                                     const rt_pt_params *p, uint32_t train_stride, const uint32_t *pixels,
                                     uint32_t n_pixels, orc_path_record *out, uint32_t n_threads) {
    PtSetup c;
    int rc = pt_setup(c, accel, tri_material, materials, n_materials, lights, n_lights, p);
    if (rc) return rc;
    const uint32_t npix = p->width * p->height;
    for (uint32_t k = 0; k < n_pixels; ++k)
        if (pixels[k] >= npix) return RT_ERR_INVALID_ARG;
    std::atomic<int> status{0};
    const uint32_t n = n_pixels * p->spp;
    parallel_for(n, n_threads, [&](uint32_t b, uint32_t e) {
        for (uint32_t i = b; i < e; ++i) {
            const uint32_t k = i / p->spp, s = i % p->spp;
            orc_path_record &r = out[i];
            std::memset(&r, 0, sizeof(r));
            int st = pt_sample(c, pixels[k], p->sample_offset + s, train_stride, &r, r.L);
            if (st) status = st;
        }
    }, 8u);
    return status.load();
}

extern "C" int orc_scene_soup(uint64_t seed, uint32_t n_tris, float *v, uint32_t *idx) {
    Rng g = seeded_rng(mix64(seed), 1u);
    for (uint32_t i = 0; i < n_tris; ++i) {
        float c[3] = {g.uni(), g.uni(), g.uni()};
        float d1[3], d2[3];
        sphere_dir(g, d1);
        sphere_dir(g, d2);
        float l1 = uni_in(g, 0.001f, 0.02f), l2 = uni_in(g, 0.001f, 0.02f);
        float *q = v + (size_t)i * 9u;
        for (int a = 0; a < 3; ++a) {
            float e1 = d1[a] * l1, e2 = d2[a] * l2;
            float v0 = c[a] - (e1 + e2) / 3.0f;
            q[a] = v0;
            q[3 + a] = v0 + e1;
            q[6 + a] = v0 + e2;
        }
        for (uint32_t k = 0; k < 3; ++k) idx[3u * i + k] = 3u * i + k;
    }
    return 0;
}

extern "C" int orc_scene_incoherent_rays(uint64_t seed, uint32_t n, const float lo[3], const float hi[3], float tmax,
                                         rt_ray *rays) {
    Rng g = seeded_rng(mix64(seed), 3u);
    for (uint32_t i = 0; i < n; ++i) {
        rt_ray &r = rays[i];
        for (int a = 0; a < 3; ++a) r.org[a] = uni_in(g, lo[a], hi[a]);
        sphere_dir(g, r.dir);
        r.tmin = 0.0f;
        r.tmax = tmax;
    }
    return 0;
}
