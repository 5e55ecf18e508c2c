// rt_pt.cu -- wavefront path tracer (raygen / extend / shade / shadow /
// resolve / accumulate) on the BVH8 traversal kernels.
//
// No counterpart in the reference sample, which shades a single bounce with
// a constant closest-hit colour (vulkan-raytraced-triangle/main.cpp:1080-1091);
// its camera model (main.cpp:1036-1045) is reused with a sub-pixel jitter.
//
// One wave = one sample of every pixel.  Paths live in structure-of-arrays
// state indexed by pixel (throughput, radiance, RNG state); ray queues hold
// 32-byte rays plus the pixel index.  Per path vertex:
//   extend   k_trace_blas over the queue (length read on the device)
//   shade    hit point, normal, material; emission on the first vertex;
//            next-event estimation: one light sample -> a shadow ray with its
//            would-be contribution; Russian roulette; cosine-weighted
//            Lambertian bounce -> next queue.  Both queues are appended with
//            one atomic per warp (ballot + popc), i.e. compacted in place.
//   shadow   k_trace_blas any-hit over the shadow queue
//   resolve  unoccluded contributions added to the path radiance
// The order in which a path's radiance terms are added is fixed (emission,
// then the light sample of each vertex in turn), and every float operation
// has a fixed order, so the image equals the CPU oracle's bit for bit even
// though queue order varies from run to run.
#include <cuda_runtime.h>

#include <cstring>

#include "../../include/rtcore_pt.h"
#include "rt_internal.h"
#include "rt_pt_math.cuh"

namespace rtc {
namespace {

constexpr int kPtThreads = 256;
constexpr uint32_t kMaxPtDepth = 64;
constexpr float kShadowTmax = 0.9999f;  // stop short of the sampled light point
constexpr float kRrMax = 0.95f;

struct PtLayout {
    uint64_t rays0, rays1, pidx0, pidx1, hits, srays, spidx, scontrib, socc, tput, rad, rng, light_aux, light_cdf,
        counters, total;
    // learned form: cache queries at the second vertex and training samples
    uint64_t qin, qout, qt1, qpidx, tin, ttarget, tt1, tlpre, tpidx;
    uint32_t cap, train_cap;
};

// counter words of the scratch counter block
constexpr uint32_t kCntQuery = 257, kCntTrain = 258, kCntPerSample = 259;  // words [0, 259) reset per sample
constexpr uint32_t kCntRays = 260;    // two u64
constexpr uint32_t kCntSample = 270;  // sample index of the running wave

PtLayout pt_layout(const rt_pt_params &p, uint32_t n_lights, uint32_t train_cap = 0) {
    PtLayout L;
    uint64_t cap = (uint64_t)p.width * p.height;
    L.cap = (uint32_t)cap;
    uint64_t off = 0;
    auto take = [&](uint64_t b) {
        uint64_t o = off;
        off += align_up(b ? b : 1, 256);
        return o;
    };
    L.rays0 = take(cap * 32u);
    L.rays1 = take(cap * 32u);
    L.pidx0 = take(cap * 4u);
    L.pidx1 = take(cap * 4u);
    L.hits = take(cap * 16u);
    L.srays = take(cap * 32u);
    L.spidx = take(cap * 4u);
    L.scontrib = take(cap * 16u);
    L.socc = take(cap);
    L.tput = take(cap * 16u);
    L.rad = take(cap * 16u);
    L.rng = take(cap * 8u);
    L.light_aux = take((uint64_t)(n_lights ? n_lights : 1) * 16u);
    L.light_cdf = take((uint64_t)(n_lights ? n_lights : 1) * 4u + 16u);
    // counters: [0, 65) queue lengths per vertex, [65, 129) shadow lengths,
    // [129, 257) traversal work counters, 257 cache queries, 258 training
    // samples, 260.. two u64 ray counts (8-byte aligned), 270 sample index
    L.counters = take(272u * 4u);
    L.train_cap = train_cap;
    const uint64_t qcap = train_cap ? cap : 0;
    L.qin = take(qcap * 48u);
    L.qout = take(qcap * 16u);
    L.qt1 = take(qcap * 16u);
    L.qpidx = take(qcap * 4u);
    L.tin = take((uint64_t)train_cap * 48u);
    L.ttarget = take((uint64_t)train_cap * 16u);
    L.tt1 = take((uint64_t)train_cap * 16u);
    L.tlpre = take((uint64_t)train_cap * 16u);
    L.tpidx = take((uint64_t)train_cap * 4u);
    L.total = off;
    return L;
}

// Training paths: pixel p of a sample is one when (p + offset) % stride == 0,
// offset drawn per sample; exactly ceil(npix / stride) pixels qualify.
inline uint32_t train_stride(uint64_t npix, uint32_t train_paths) {
    if (train_paths == 0) return 0;
    uint64_t s = npix / train_paths;
    return (uint32_t)(s < 1 ? 1 : s);
}
inline uint32_t train_capacity(uint64_t npix, uint32_t train_paths) {
    uint32_t s = train_stride(npix, train_paths);
    return s ? (uint32_t)((npix + s - 1) / s) : 0u;
}

struct PtArgs {
    const uint8_t *accel;      // bottom-level structure (leaf records behind its header)
    const uint32_t *tri_material;
    const rt_material *materials;
    uint32_t n_materials;
    const rt_pt_light *lights;
    const float4 *light_aux;   // (normal xyz, area)
    const float *light_cdf;    // n_lights cumulative areas, then the total
    uint32_t n_lights;
    float4 *tput;
    float4 *rad;
    uint64_t *rng;
    const float4 *rays_in;
    const uint32_t *pidx_in;
    const float4 *hits;
    float4 *rays_out;
    uint32_t *pidx_out;
    const uint32_t *count_in;
    uint32_t *count_out;
    float4 *srays;
    uint32_t *spidx;
    float4 *scontrib;
    uint32_t *scount;
    uint32_t depth, max_depth, rr_depth;
    float eps;
    unsigned long long *ray_counts;
    uint32_t *err;
    // learned form (cache_mode != 0): at the second vertex a path either
    // ends in a cache query or, for training pixels, records a sample and
    // continues
    uint32_t cache_mode;
    uint32_t stride;          // training pixel stride
    uint64_t seed;
    const uint32_t *sample_dev;
    rt_cache_input *qin;
    float4 *qt1;
    uint32_t *qpidx;
    uint32_t *qcount;
    rt_cache_input *tin;
    float4 *tt1;
    float4 *tlpre;
    uint32_t *tpidx;
    uint32_t *tcount;
};

// Per-light normal, area and the area CDF (fixed summation order).
__global__ void k_pt_setup(const rt_pt_light *lights, uint32_t n_lights, float4 *aux, float *cdf, uint32_t *sample_dev,
                           uint32_t sample_offset, unsigned long long *ray_counts) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    float acc = 0.0f;
    for (uint32_t k = 0; k < n_lights; ++k) {
        const rt_pt_light &l = lights[k];
        float e1[3] = {l.v1[0] - l.v0[0], l.v1[1] - l.v0[1], l.v1[2] - l.v0[2]};
        float e2[3] = {l.v2[0] - l.v0[0], l.v2[1] - l.v0[1], l.v2[2] - l.v0[2]};
        float c[3];
        rtpt::cross3(e1, e2, c);
        float len = sqrtf(rtpt::dot3(c, c));
        float area = 0.5f * len;
        float inv = len > 0.0f ? 1.0f / len : 0.0f;
        aux[k] = make_float4(c[0] * inv, c[1] * inv, c[2] * inv, area);
        acc = acc + area;
        cdf[k] = acc;
    }
    cdf[n_lights] = acc;
    *sample_dev = sample_offset;
    ray_counts[0] = 0ull;
    ray_counts[1] = 0ull;
}

__global__ void __launch_bounds__(kPtThreads) k_pt_raygen(float ax, float ay, float cx, float cy, float cz,
                                                           uint32_t w, uint32_t h, uint64_t seed,
                                                           const uint32_t *sample_dev, float4 *rays, uint32_t *pidx,
                                                           float4 *tput, float4 *rad, uint64_t *rng,
                                                           uint32_t *count0, unsigned long long *ray_counts) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = w * h;
    if (p == 0) {
        *count0 = n;
        atomicAdd(ray_counts, (unsigned long long)n);
    }
    if (p >= n) return;
    const uint32_t x = p % w, y = p / w;
    rtpt::Pcg g = rtpt::pcg_seed(seed, *sample_dev, p);
    const float jx = rtpt::pcg_uniform(g), jy = rtpt::pcg_uniform(g);
    float d[3];
    rtpt::camera_dir(ax, ay, w, h, x, y, jx, jy, d);
    rays[2u * p] = make_float4(cx, cy, cz, 0.0f);
    rays[2u * p + 1u] = make_float4(d[0], d[1], d[2], 1e30f);
    pidx[p] = p;
    tput[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    rad[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    rng[p] = g.state;
}

// One slot per voting lane of the warp in the queue behind `count`.
__device__ __forceinline__ uint32_t warp_append(bool want, uint32_t *count, unsigned long long *stat) {
    const uint32_t mask = __ballot_sync(0xffffffffu, want);
    if (mask == 0u) return 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) {
        base = atomicAdd(count, (uint32_t)__popc(mask));
        if (stat) atomicAdd(stat, (unsigned long long)__popc(mask));
    }
    base = __shfl_sync(0xffffffffu, base, leader);
    return want ? base + (uint32_t)__popc(mask & ((1u << lane) - 1u)) : 0xffffffffu;
}

__global__ void __launch_bounds__(kPtThreads) k_pt_shade(const PtArgs a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *a.count_in;
    bool want_shadow = false, want_next = false;
    bool is_train = false, is_query = false;
    rt_cache_input crec;
    float4 t1 = make_float4(0.f, 0.f, 0.f, 0.f), lpre = make_float4(0.f, 0.f, 0.f, 0.f);
    float so[3] = {0, 0, 0}, sd[3] = {0, 0, 0}, contrib[3] = {0, 0, 0};
    float no[3] = {0, 0, 0}, nd[3] = {0, 0, 0};
    uint32_t p = 0;
    if (i < n) {
        p = a.pidx_in[i];
        rtpt::Pcg g;
        g.state = a.rng[p];
        g.inc = ((uint64_t)p << 1u) | 1u;
        float u[6];
        for (int k = 0; k < 6; ++k) u[k] = rtpt::pcg_uniform(g);
        a.rng[p] = g.state;
        const float4 hit = a.hits[i];
        const uint32_t rec = __float_as_uint(hit.y);
        if (rec != 0xffffffffu) {
            const float4 r0 = a.rays_in[2u * i], r1 = a.rays_in[2u * i + 1u];
            const float o[3] = {r0.x, r0.y, r0.z}, d[3] = {r1.x, r1.y, r1.z};
            const rt_accel_header *hd = reinterpret_cast<const rt_accel_header *>(a.accel);
            const uint4 *pr = reinterpret_cast<const uint4 *>(a.accel + hd->prim_offset) + (size_t)rec * 3u;
            const uint4 q0 = __ldg(pr), q1 = __ldg(pr + 1), q2 = __ldg(pr + 2);
            const float v0[3] = {__uint_as_float(q0.x), __uint_as_float(q0.y), __uint_as_float(q0.z)};
            const float v1[3] = {__uint_as_float(q1.x), __uint_as_float(q1.y), __uint_as_float(q1.z)};
            const float v2[3] = {__uint_as_float(q2.x), __uint_as_float(q2.y), __uint_as_float(q2.z)};
            const uint32_t tri = q0.w;
            const float t = hit.x;
            float P[3], e1[3], e2[3], ng[3], nrm[3];
            for (int k = 0; k < 3; ++k) {
                P[k] = o[k] + t * d[k];
                e1[k] = v1[k] - v0[k];
                e2[k] = v2[k] - v0[k];
            }
            rtpt::cross3(e1, e2, ng);
            const float len = sqrtf(rtpt::dot3(ng, ng));
            if (len > 0.0f) {
                for (int k = 0; k < 3; ++k) nrm[k] = ng[k] / len;
                const float cosd = rtpt::dot3(nrm, d);
                uint32_t mi = a.tri_material[tri];
                if (mi >= a.n_materials) {
                    report_error(a.err, RT_ERR_BOUNDS, 0x80000000u | tri);
                    mi = 0;
                }
                const rt_material m = a.materials[mi];
                float4 T = a.tput[p];
                if (a.depth == 0 && cosd < 0.0f) {
                    float4 R = a.rad[p];
                    R.x = R.x + T.x * m.emission[0];
                    R.y = R.y + T.y * m.emission[1];
                    R.z = R.z + T.z * m.emission[2];
                    a.rad[p] = R;
                }
                if (cosd > 0.0f)
                    for (int k = 0; k < 3; ++k) nrm[k] = -nrm[k];
                const bool reflective = m.albedo[0] > 0.0f || m.albedo[1] > 0.0f || m.albedo[2] > 0.0f;
                if (reflective && a.cache_mode && a.depth == 1u) {
                    // second vertex of the learned form: record (x, -d, n,
                    // albedo); training pixels go on as plain path tracing,
                    // the others end here in a cache query
                    const uint32_t off =
                        (uint32_t)(rtpt::splitmix64(a.seed ^ (0x5851f42d4c957f2dull + *a.sample_dev)) % a.stride);
                    for (int k = 0; k < 3; ++k) {
                        crec.pos[k] = P[k];
                        crec.dir[k] = -d[k];
                        crec.normal[k] = nrm[k];
                        crec.albedo[k] = m.albedo[k];
                    }
                    t1 = T;
                    if ((p + off) % a.stride == 0u) {
                        is_train = true;
                        lpre = a.rad[p];
                    } else {
                        is_query = true;
                    }
                }
                if (reflective && !is_query) {
                    // ---- next-event estimation: one point on one light
                    if (a.n_lights > 0) {
                        const float total = a.light_cdf[a.n_lights];
                        const float target = u[0] * total;
                        uint32_t lo = 0, hi = a.n_lights - 1u;
                        while (lo < hi) {  // first k with cdf[k] > target
                            uint32_t mid = (lo + hi) >> 1;
                            if (a.light_cdf[mid] > target) hi = mid; else lo = mid + 1u;
                        }
                        const rt_pt_light L = a.lights[lo];
                        const float4 ln = a.light_aux[lo];
                        const float su = sqrtf(u[1]);
                        const float b0 = 1.0f - su, b1 = u[2] * su;
                        const float b2 = (1.0f - b0) - b1;
                        float lp[3], wi[3];
                        for (int k = 0; k < 3; ++k) {
                            lp[k] = (L.v0[k] * b0 + L.v1[k] * b1) + L.v2[k] * b2;
                            wi[k] = lp[k] - P[k];
                        }
                        const float dist2 = rtpt::dot3(wi, wi);
                        const float dist = sqrtf(dist2);
                        if (dist > 0.0f) {
                            float wn[3];
                            for (int k = 0; k < 3; ++k) wn[k] = wi[k] / dist;
                            const float lnv[3] = {ln.x, ln.y, ln.z};
                            const float cos_s = rtpt::dot3(nrm, wn);
                            const float cos_l = -rtpt::dot3(lnv, wn);
                            if (cos_s > 0.0f && cos_l > 0.0f) {
                                const float f = (((cos_s * cos_l) / dist2) * total) * rtpt::kInvPi;
                                const float Tv[3] = {T.x, T.y, T.z};
                                for (int k = 0; k < 3; ++k) {
                                    contrib[k] = ((Tv[k] * m.albedo[k]) * L.emission[k]) * f;
                                    so[k] = P[k] + nrm[k] * a.eps;
                                }
                                for (int k = 0; k < 3; ++k) sd[k] = lp[k] - so[k];
                                want_shadow = true;
                            }
                        }
                    }
                    // ---- Russian roulette, then the Lambertian bounce
                    bool alive = true;
                    if (a.depth >= a.rr_depth) {
                        float ps = fmaxf(fmaxf(T.x, T.y), T.z);
                        ps = ps < kRrMax ? ps : kRrMax;
                        if (!(u[5] < ps)) alive = false;
                        else { T.x = T.x / ps; T.y = T.y / ps; T.z = T.z / ps; }
                    }
                    if (alive && a.depth + 1u < a.max_depth) {
                        float x, y;
                        rtpt::concentric_disk(u[3], u[4], x, y);
                        float zz = (1.0f - x * x) - y * y;
                        const float z = sqrtf(zz > 0.0f ? zz : 0.0f);
                        float t1[3], t2[3];
                        rtpt::onb(nrm, t1, t2);
                        for (int k = 0; k < 3; ++k) {
                            nd[k] = (t1[k] * x + t2[k] * y) + nrm[k] * z;
                            no[k] = P[k] + nrm[k] * a.eps;
                        }
                        T.x = T.x * m.albedo[0];
                        T.y = T.y * m.albedo[1];
                        T.z = T.z * m.albedo[2];
                        a.tput[p] = T;
                        want_next = true;
                    }
                }
            }
        }
    }
    const uint32_t sslot = warp_append(want_shadow, a.scount, a.ray_counts + 1);
    if (want_shadow) {
        a.srays[2u * sslot] = make_float4(so[0], so[1], so[2], 0.0f);
        a.srays[2u * sslot + 1u] = make_float4(sd[0], sd[1], sd[2], kShadowTmax);
        a.spidx[sslot] = p;
        a.scontrib[sslot] = make_float4(contrib[0], contrib[1], contrib[2], 0.0f);
    }
    const uint32_t nslot = warp_append(want_next, a.count_out, a.ray_counts);
    if (want_next) {
        a.rays_out[2u * nslot] = make_float4(no[0], no[1], no[2], 0.0f);
        a.rays_out[2u * nslot + 1u] = make_float4(nd[0], nd[1], nd[2], 1e30f);
        a.pidx_out[nslot] = p;
    }
    if (a.cache_mode) {
        const uint32_t tslot = warp_append(is_train, a.tcount, nullptr);
        if (is_train) {
            a.tin[tslot] = crec;
            a.tt1[tslot] = t1;
            a.tlpre[tslot] = lpre;
            a.tpidx[tslot] = p;
        }
        const uint32_t qslot = warp_append(is_query, a.qcount, nullptr);
        if (is_query) {
            a.qin[qslot] = crec;
            a.qt1[qslot] = t1;
            a.qpidx[qslot] = p;
        }
    }
}

// Learned form, after the wave: cache-terminated paths add T1 * max(cache, 0);
// training samples get the target (L - L_before) / T1 (the radiance their
// plain tail brought back through the second vertex).
__global__ void __launch_bounds__(kPtThreads) k_pt_cache_apply(const uint32_t *qcount, const uint32_t *qpidx,
                                                                const float4 *qt1, const float4 *qout, float4 *rad,
                                                                const uint32_t *tcount, const uint32_t *tpidx,
                                                                const float4 *tt1, const float4 *tlpre,
                                                                float4 *ttarget) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *qcount) {
        const uint32_t p = qpidx[i];
        const float4 t = qt1[i], c = qout[i];
        float4 R = rad[p];
        R.x = R.x + t.x * fmaxf(c.x, 0.0f);
        R.y = R.y + t.y * fmaxf(c.y, 0.0f);
        R.z = R.z + t.z * fmaxf(c.z, 0.0f);
        rad[p] = R;
    }
    if (i < *tcount) {
        const uint32_t p = tpidx[i];
        const float4 t = tt1[i], l0 = tlpre[i], R = rad[p];
        ttarget[i] = make_float4(t.x > 0.0f ? (R.x - l0.x) / t.x : 0.0f, t.y > 0.0f ? (R.y - l0.y) / t.y : 0.0f,
                                 t.z > 0.0f ? (R.z - l0.z) / t.z : 0.0f, 0.0f);
    }
}

__global__ void __launch_bounds__(kPtThreads) k_pt_resolve(const uint32_t *scount, const uint8_t *socc,
                                                            const uint32_t *spidx, const float4 *scontrib,
                                                            float4 *rad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *scount || socc[i]) return;
    const uint32_t p = spidx[i];
    const float4 c = scontrib[i];
    float4 R = rad[p];
    R.x = R.x + c.x;
    R.y = R.y + c.y;
    R.z = R.z + c.z;
    rad[p] = R;
}

__global__ void __launch_bounds__(kPtThreads) k_pt_accumulate(uint32_t n, const float4 *rad, float4 *accum,
                                                               uint32_t *sample_dev) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) *sample_dev = *sample_dev + 1u;  // raygen of this sample already read it
    if (p >= n) return;
    const float4 r = rad[p];
    float4 acc = accum[p];
    acc.x = acc.x + r.x;
    acc.y = acc.y + r.y;
    acc.z = acc.z + r.z;
    acc.w = acc.w + 1.0f;
    accum[p] = acc;
}

}  // namespace
}  // namespace rtc

using namespace rtc;

namespace {

int path_trace_impl(rt_context *ctx, rt_stream stream, const rt_pt_scene *scene, const rt_pt_params *p,
                    const rt_pt_cache_params *cp, float *accum, void *scratch, uint64_t scratch_bytes) {
    if (!ctx || !scene || !p || !accum || !scratch || !scene->accel)
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_path_trace: null argument");
    if (!scene->tri_material || !scene->materials || scene->n_materials == 0 ||
        (scene->n_lights && !scene->lights))
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_path_trace: incomplete scene");
    if (p->max_depth == 0 || p->max_depth > kMaxPtDepth)
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_path_trace: max_depth must be in 1..64");
    if (scene->n_lights > (1u << 20)) return set_error(ctx, RT_ERR_UNSUPPORTED, "rt_path_trace: more than 2^20 lights");
    if (cp && (!cp->cache || cp->train_paths == 0 || (cp->train_batch % 64u) != 0u))
        return set_error(ctx, RT_ERR_INVALID_ARG,
                         "rt_path_trace_cached: cache, train_paths > 0 and a train_batch multiple of 64 are required");
    const uint64_t npix = (uint64_t)p->width * p->height;
    if (npix == 0 || p->spp == 0) return RT_OK;
    if (npix > (1u << 30)) return set_error(ctx, RT_ERR_UNSUPPORTED, "rt_path_trace: more than 2^30 pixels");
    const uint32_t tcap = cp ? train_capacity(npix, cp->train_paths) : 0u;
    const PtLayout L = pt_layout(*p, scene->n_lights, tcap);
    if (scratch_bytes < L.total) return set_error(ctx, RT_ERR_OOM, "rt_path_trace: scratch smaller than the size query returned");
    if (reinterpret_cast<uintptr_t>(scratch) & 255u) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_path_trace: scratch must be 256-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint8_t *S = static_cast<uint8_t *>(scratch);
    const uint8_t *accel = reinterpret_cast<const uint8_t *>(scene->accel);
    uint32_t *cnt = reinterpret_cast<uint32_t *>(S + L.counters);
    uint32_t *scnt = cnt + 65;
    uint32_t *tcnt = cnt + 129;
    uint32_t *sample_dev = cnt + kCntSample;
    unsigned long long *ray_counts = reinterpret_cast<unsigned long long *>(cnt + kCntRays);
    float4 *aux = reinterpret_cast<float4 *>(S + L.light_aux);
    float *cdf = reinterpret_cast<float *>(S + L.light_cdf);

    k_pt_setup<<<1, 32, 0, st>>>(scene->lights, scene->n_lights, aux, cdf, sample_dev, p->sample_offset, ray_counts);
    RT_CUDA_CTX(ctx, cudaGetLastError());

    float ax, ay;
    camera_aspects(&p->camera, p->width, p->height, &ay, &ax);
    PtArgs a;
    std::memset(&a, 0, sizeof(a));
    a.accel = accel;
    a.tri_material = scene->tri_material;
    a.materials = scene->materials;
    a.n_materials = scene->n_materials;
    a.lights = scene->lights;
    a.light_aux = aux;
    a.light_cdf = cdf;
    a.n_lights = scene->n_lights;
    a.tput = reinterpret_cast<float4 *>(S + L.tput);
    a.rad = reinterpret_cast<float4 *>(S + L.rad);
    a.rng = reinterpret_cast<uint64_t *>(S + L.rng);
    a.hits = reinterpret_cast<const float4 *>(S + L.hits);
    a.srays = reinterpret_cast<float4 *>(S + L.srays);
    a.spidx = reinterpret_cast<uint32_t *>(S + L.spidx);
    a.scontrib = reinterpret_cast<float4 *>(S + L.scontrib);
    a.max_depth = p->max_depth;
    a.rr_depth = p->rr_depth;
    a.eps = p->ray_eps;
    a.ray_counts = ray_counts;
    a.err = ctx->d_err;
    if (cp) {
        a.cache_mode = 1;
        a.stride = train_stride(npix, cp->train_paths);
        a.seed = p->seed;
        a.sample_dev = sample_dev;
        a.qin = reinterpret_cast<rt_cache_input *>(S + L.qin);
        a.qt1 = reinterpret_cast<float4 *>(S + L.qt1);
        a.qpidx = reinterpret_cast<uint32_t *>(S + L.qpidx);
        a.qcount = cnt + kCntQuery;
        a.tin = reinterpret_cast<rt_cache_input *>(S + L.tin);
        a.tt1 = reinterpret_cast<float4 *>(S + L.tt1);
        a.tlpre = reinterpret_cast<float4 *>(S + L.tlpre);
        a.tpidx = reinterpret_cast<uint32_t *>(S + L.tpidx);
        a.tcount = cnt + kCntTrain;
    }
    float4 *rays[2] = {reinterpret_cast<float4 *>(S + L.rays0), reinterpret_cast<float4 *>(S + L.rays1)};
    uint32_t *pidx[2] = {reinterpret_cast<uint32_t *>(S + L.pidx0), reinterpret_cast<uint32_t *>(S + L.pidx1)};
    uint8_t *socc = S + L.socc;
    const unsigned blocks = (unsigned)((npix + kPtThreads - 1) / kPtThreads);

    for (uint32_t s = 0; s < p->spp; ++s) {
        RT_CUDA_CTX(ctx, cudaMemsetAsync(cnt, 0, kCntPerSample * 4u, st));
        k_pt_raygen<<<blocks, kPtThreads, 0, st>>>(ax, ay, p->camera.position[0], p->camera.position[1],
                                                   p->camera.position[2], p->width, p->height, p->seed, sample_dev,
                                                   rays[0], pidx[0], a.tput, a.rad, a.rng, &cnt[0], ray_counts);
        RT_CUDA_CTX(ctx, cudaGetLastError());
        for (uint32_t d = 0; d < p->max_depth; ++d) {
            const uint32_t q = d & 1u;
            int rc = launch_queue_trace(ctx, st, accel, rays[q], S + L.hits, nullptr, &cnt[d], (uint32_t)npix,
                                        &tcnt[2 * d], false);
            if (rc) return rc;
            a.rays_in = rays[q];
            a.pidx_in = pidx[q];
            a.rays_out = rays[q ^ 1u];
            a.pidx_out = pidx[q ^ 1u];
            a.count_in = &cnt[d];
            a.count_out = &cnt[d + 1];
            a.scount = &scnt[d];
            a.depth = d;
            k_pt_shade<<<blocks, kPtThreads, 0, st>>>(a);
            RT_CUDA_CTX(ctx, cudaGetLastError());
            rc = launch_queue_trace(ctx, st, accel, a.srays, nullptr, socc, &scnt[d], (uint32_t)npix,
                                    &tcnt[2 * d + 1], true);
            if (rc) return rc;
            k_pt_resolve<<<blocks, kPtThreads, 0, st>>>(&scnt[d], socc, a.spidx, a.scontrib, a.rad);
            RT_CUDA_CTX(ctx, cudaGetLastError());
        }
        float4 *ttarget = reinterpret_cast<float4 *>(S + L.ttarget);
        if (cp) {
            int rc = cache_query_dev(ctx, st, cp->cache, a.qin, reinterpret_cast<float *>(S + L.qout), a.qcount,
                                     (uint32_t)npix);
            if (rc) return rc;
            k_pt_cache_apply<<<blocks, kPtThreads, 0, st>>>(a.qcount, a.qpidx, a.qt1,
                                                            reinterpret_cast<const float4 *>(S + L.qout), a.rad,
                                                            a.tcount, a.tpidx, a.tt1, a.tlpre, ttarget);
            RT_CUDA_CTX(ctx, cudaGetLastError());
        }
        k_pt_accumulate<<<blocks, kPtThreads, 0, st>>>((uint32_t)npix, a.rad, reinterpret_cast<float4 *>(accum),
                                                       sample_dev);
        RT_CUDA_CTX(ctx, cudaGetLastError());
        if (cp && cp->train_batch) {
            int rc = cache_train_dev(ctx, st, cp->cache, a.tin, reinterpret_cast<const float *>(ttarget), a.tcount,
                                     tcap, cp->train_batch);
            if (rc) return rc;
        }
    }
    return RT_OK;
}

}  // namespace

extern "C" rt_status rt_pt_scratch_bytes(const rt_pt_params *p, uint64_t *bytes) {
    if (!p || !bytes) return RT_ERR_INVALID_ARG;
    // the light tables are sized for up to 2^20 lights; the call checks the
    // size again with the scene's real light count
    *bytes = pt_layout(*p, 1u << 20).total;
    return RT_OK;
}

extern "C" rt_status rt_pt_cached_scratch_bytes(const rt_pt_params *p, const rt_pt_cache_params *cp,
                                                uint64_t *bytes) {
    if (!p || !cp || !bytes) return RT_ERR_INVALID_ARG;
    const uint64_t npix = (uint64_t)p->width * p->height;
    *bytes = pt_layout(*p, 1u << 20, train_capacity(npix, cp->train_paths)).total;
    return RT_OK;
}

extern "C" rt_status rt_path_trace(rt_context *ctx, rt_stream stream, const rt_pt_scene *scene,
                                   const rt_pt_params *p, float *accum, void *scratch, uint64_t scratch_bytes) {
    return path_trace_impl(ctx, stream, scene, p, nullptr, accum, scratch, scratch_bytes);
}

extern "C" rt_status rt_path_trace_cached(rt_context *ctx, rt_stream stream, const rt_pt_scene *scene,
                                          const rt_pt_params *p, const rt_pt_cache_params *cp, float *accum,
                                          void *scratch, uint64_t scratch_bytes) {
    if (!cp) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_path_trace_cached: null cache parameters");
    return path_trace_impl(ctx, stream, scene, p, cp, accum, scratch, scratch_bytes);
}

extern "C" rt_status rt_pt_ray_counts(rt_context *ctx, rt_stream stream, const rt_pt_params *p, uint32_t n_lights,
                                      const void *scratch, uint64_t *extension_rays, uint64_t *shadow_rays) {
    if (!ctx || !p || !scratch) return RT_ERR_INVALID_ARG;
    const PtLayout L = pt_layout(*p, n_lights);
    unsigned long long h[2];
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint8_t *S = static_cast<const uint8_t *>(scratch);
    RT_CUDA_CTX(ctx, cudaMemcpyAsync(h, S + L.counters + kCntRays * 4u, sizeof(h), cudaMemcpyDeviceToHost, st));
    RT_CUDA_CTX(ctx, cudaStreamSynchronize(st));
    if (extension_rays) *extension_rays = h[0];
    if (shadow_rays) *shadow_rays = h[1];
    return RT_OK;
}
