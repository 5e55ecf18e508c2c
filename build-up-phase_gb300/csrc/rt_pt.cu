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
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/rtcore_batch.h"
#include "../../include/rtcore_pt.h"
#include "../../include/rtcore_debug.h"
#include "rt_internal.h"
#include "rt_pt_math.cuh"
#include "rt_traverse.cuh"

namespace rtc {
namespace {

constexpr int kPtThreads = 256;
constexpr uint32_t kMaxPtDepth = 64;
constexpr float kShadowTmax = 0.9999f;  // stop short of the sampled light point
constexpr float kRrMax = 0.95f;

struct PtLayout {
    uint64_t rays0, rays1, pidx0, pidx1, hits, srays, spidx, scontrib, socc, tput, rad, rng, light_aux, light_cdf,
        counters, stage, stage_pidx, stage_rank, total;
    // learned form: cache queries at the second vertex and training samples
    uint64_t qin, qout, qt1, qpidx, tin, ttarget, tt1, tlpre, tpidx;
    uint32_t cap, train_cap;
    uint32_t wave;  // samples of every pixel traced together (cap = pixels x wave)
};

// Samples per pixel traced as one wave: a wave of k samples has k times the
// rays per traversal launch, so each launch's slow-ray tail is shared by k
// samples.  At most 4, and at most 2^23 paths (~1.9 GB of path state and
// queues).  The learned form queries the cache once per wave and trains on
// the wave's training paths after it.
constexpr uint32_t kPtWaveSamples = 4;
constexpr uint64_t kPtWavePaths = 1ull << 23;
inline uint32_t wave_samples(uint64_t npix, uint32_t spp) {
    uint64_t k = spp < kPtWaveSamples ? spp : kPtWaveSamples;
    while (k > 1u && npix * k > kPtWavePaths) --k;
    return (uint32_t)(k ? k : 1u);
}

// counter words of the scratch counter block
// Counter block (32-bit words): [0, 65) extension queue lengths per depth,
// [65, 129) shadow queue lengths, [129, 257) traversal work counters,
// 257 cache queries, 258 training samples, [259, 779) extension rays per
// direction octant per depth -- all reset per sample -- then two u64 ray
// counts and the sample index of the running wave.
constexpr uint32_t kCntQuery = 257, kCntTrain = 258, kCntBins = 259;
constexpr uint32_t kCntPerSample = kCntBins + 8u * 65u;  // 779
constexpr uint32_t kCntRays = 780;    // two u64 (8-byte aligned)
constexpr uint32_t kCntSample = 784;  // sample index of the running wave
constexpr uint32_t kCntWords = 800;

PtLayout pt_layout(const rt_pt_params &p, uint32_t n_lights, uint32_t train_cap = 0) {
    PtLayout L;
    const uint64_t npix = (uint64_t)p.width * p.height;
    L.wave = wave_samples(npix, p.spp);
    const uint64_t cap = npix * L.wave;
    L.cap = (uint32_t)cap;
    uint64_t off = 0;
    auto take = [&](uint64_t b) {
        uint64_t o = off;
        off += align_up(b ? b : 1, 256);
        return o;
    };
    L.counters = take(kCntWords * 4u);  // first: its offset depends on nothing
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
    L.stage = take(cap * 32u);
    L.stage_pidx = take(cap * 4u);
    L.stage_rank = take(cap * 4u);
    // train_cap: training paths of one sample; a wave holds L.wave samples'
    L.train_cap = train_cap * L.wave;
    const uint64_t qcap = train_cap ? cap : 0;
    L.qin = take(qcap * 48u);
    L.qout = take(qcap * 16u);
    L.qt1 = take(qcap * 16u);
    L.qpidx = take(qcap * 4u);
    L.tin = take((uint64_t)L.train_cap * 48u);
    L.ttarget = take((uint64_t)L.train_cap * 16u);
    L.tt1 = take((uint64_t)L.train_cap * 16u);
    L.tlpre = take((uint64_t)L.train_cap * 16u);
    L.tpidx = take((uint64_t)L.train_cap * 4u);
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

// One scene of a batch on the device (96 bytes).  Paths of a sample pass are
// numbered across the scenes: scene s owns global paths [base, base + w*h).
struct BtScene {
    const uint8_t *accel;
    const uint32_t *tri_material;
    const rt_material *materials;
    const rt_pt_light *lights;
    float4 *accum;
    uint32_t n_materials, n_lights;
    uint32_t light_off;  // first entry of the scene's light tables (its CDF starts at light_off + scene)
    uint32_t width, height;
    uint32_t base;
    float ax, ay;
    float cam[3];
    uint32_t pad[3];
};
static_assert(sizeof(BtScene) == 96, "BtScene layout");

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
    // octant binning of the extension rays: shade writes them to the stage
    // arrays with their rank within their octant, the scatter kernel places
    // them octant by octant
    uint32_t binning;
    float4 *stage;
    uint32_t *stage_pidx;
    uint32_t *stage_rsid;
    uint32_t *stage_rank;
    uint32_t *bins_out;   // the 8 octant counters of the next depth
    // batch (multi-scene kernels): each queue entry carries its scene
    const BtScene *bt;
    uint32_t wave_base;        // global path index of slot 0 of the wave
    uint32_t npix;             // single scene: pixels (path q of a wave is pixel q % npix)
    const uint32_t *rsid_in;
    uint32_t *rsid_out;
    uint32_t *ssid;
};

// Per-light normal, area and the area CDF (fixed summation order), one
// thread per scene.
__device__ void light_table(const rt_pt_light *lights, uint32_t n_lights, float4 *aux, float *cdf) {
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
}

__global__ void k_pt_setup(const rt_pt_light *lights, uint32_t n_lights, float4 *aux, float *cdf, uint32_t *sample_dev,
                           uint32_t sample_offset, unsigned long long *ray_counts) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    light_table(lights, n_lights, aux, cdf);
    *sample_dev = sample_offset;
    ray_counts[0] = 0ull;
    ray_counts[1] = 0ull;
}

__global__ void __launch_bounds__(kPtThreads) k_pt_raygen(float ax, float ay, float cx, float cy, float cz,
                                                           uint32_t w, uint32_t h, uint64_t seed,
                                                           const uint32_t *sample_dev, uint32_t k, float4 *rays,
                                                           uint32_t *pidx, float4 *tput, float4 *rad, uint64_t *rng,
                                                           uint32_t *count0, unsigned long long *ray_counts) {
    // path q of the wave: sample (*sample_dev + q / n) of pixel q % n
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = w * h;
    if (q == 0) {
        *count0 = n * k;
        atomicAdd(ray_counts, (unsigned long long)n * k);
    }
    if (q >= n * k) return;
    const uint32_t j = q / n, p = q - j * n;
    const uint32_t x = p % w, y = p / w;
    rtpt::Pcg g = rtpt::pcg_seed(seed, *sample_dev + j, p);
    const float jx = rtpt::pcg_uniform(g), jy = rtpt::pcg_uniform(g);
    float d[3];
    rtpt::camera_dir(ax, ay, w, h, x, y, jx, jy, d);
    rays[2u * q] = make_float4(cx, cy, cz, 0.0f);
    rays[2u * q + 1u] = make_float4(d[0], d[1], d[2], 1e30f);
    pidx[q] = q;
    tput[q] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    rad[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    rng[q] = g.state;
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

// Direction octant: bit k set when component k is negative.
__device__ __forceinline__ uint32_t octant_of(const float d[3]) {
    return (d[0] < 0.0f ? 1u : 0u) | (d[1] < 0.0f ? 2u : 0u) | (d[2] < 0.0f ? 4u : 0u);
}

// Places the staged extension rays octant by octant: ray i goes to the start
// of its octant's range (prefix of the 8 counts) plus its rank in the octant.
template <bool MULTI>
__global__ void __launch_bounds__(512) k_pt_bin_scatter(const uint32_t *count, const uint32_t *bins,
                                                         const float4 *stage, const uint32_t *stage_pidx,
                                                         const uint32_t *stage_rsid, const uint32_t *stage_rank,
                                                         float4 *rays_out, uint32_t *pidx_out, uint32_t *rsid_out,
                                                         uint32_t cap, uint32_t *err) {
    const uint32_t n = *count;
    uint32_t start[8];
    uint32_t acc = 0;
    for (int b = 0; b < 8; ++b) {
        start[b] = acc;
        acc += bins[b];
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 r0 = stage[2u * i], r1 = stage[2u * i + 1u];
        const float d[3] = {r1.x, r1.y, r1.z};
        const uint32_t b = octant_of(d);
        const uint32_t dst = start[b] + stage_rank[i];
        if (dst >= n || dst >= cap) {  // the counts disagree: a broken invariant, never an out-of-range write
            report_error(err, RT_ERR_BOUNDS, 0x79000000u | (i & 0xffffffu));
            continue;
        }
        rays_out[2u * dst] = r0;
        rays_out[2u * dst + 1u] = r1;
        pidx_out[dst] = stage_pidx[i];
        if (MULTI) rsid_out[dst] = stage_rsid[i];
    }
}

// Shades queue entry i (all 32 lanes of the warp call it together: the
// queue appends are warp-wide).  MULTI: the entry's scene comes from the
// queue and the scene table; otherwise from the arguments.
template <bool MULTI>
__device__ __forceinline__ void shade_one(const PtArgs &a, uint32_t i, uint32_t n) {
    bool want_shadow = false, want_next = false;
    bool is_train = false, is_query = false;
    rt_cache_input crec;
    float4 t1 = make_float4(0.f, 0.f, 0.f, 0.f), lpre = make_float4(0.f, 0.f, 0.f, 0.f);
    float so[3] = {0, 0, 0}, sd[3] = {0, 0, 0}, contrib[3] = {0, 0, 0};
    float no[3] = {0, 0, 0}, nd[3] = {0, 0, 0};
    uint32_t p = 0, sid = 0;
    if (i < n) {
        p = __ldg(a.pidx_in + i);
        // independent of the hit: issued before the dependent record loads
        float4 T = a.tput[p];
        const float4 hit = __ldg(a.hits + i);
        const uint8_t *accel = a.accel;
        const uint32_t *tri_material = a.tri_material;
        const rt_material *materials = a.materials;
        uint32_t n_materials = a.n_materials;
        const rt_pt_light *lights = a.lights;
        const float4 *light_aux = a.light_aux;
        const float *light_cdf = a.light_cdf;
        uint32_t n_lights = a.n_lights;
        uint32_t pix = (!MULTI && a.npix) ? p % a.npix : p;  // pixel index within the scene: the random stream
        if (MULTI) {
            sid = a.rsid_in[i];
            const BtScene &sc = a.bt[sid];
            accel = sc.accel;
            tri_material = sc.tri_material;
            materials = sc.materials;
            n_materials = sc.n_materials;
            lights = sc.lights;
            light_aux = a.light_aux + sc.light_off;
            light_cdf = a.light_cdf + sc.light_off + sid;
            n_lights = sc.n_lights;
            pix = a.wave_base + p - sc.base;
        }
        rtpt::Pcg g;
        g.state = a.rng[p];
        g.inc = ((uint64_t)pix << 1u) | 1u;
        float u[6];
        for (int k = 0; k < 6; ++k) u[k] = rtpt::pcg_uniform(g);
        a.rng[p] = g.state;
        const uint32_t rec = __float_as_uint(hit.y);
        if (rec != 0xffffffffu) {
            const float4 r0 = __ldg(a.rays_in + 2u * i), r1 = __ldg(a.rays_in + 2u * i + 1u);
            const float o[3] = {r0.x, r0.y, r0.z}, d[3] = {r1.x, r1.y, r1.z};
            const rt_accel_header *hd = reinterpret_cast<const rt_accel_header *>(accel);
            const uint4 *pr = reinterpret_cast<const uint4 *>(accel + hd->prim_offset) + (size_t)rec * 3u;
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
                uint32_t mi = __ldg(tri_material + tri);
                if (mi >= n_materials) {
                    report_error(a.err, RT_ERR_BOUNDS, 0x80000000u | tri);
                    mi = 0;
                }
                const rt_material m = materials[mi];
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
                if (!MULTI && reflective && a.cache_mode && a.depth == 1u) {
                    // second vertex of the learned form: record (x, -d, n,
                    // albedo); training pixels go on as plain path tracing,
                    // the others end here in a cache query
                    // path p of the wave: sample (*sample_dev + p / npix) of pixel p % npix
                    const uint32_t jw = p / a.npix, pixp = p - jw * a.npix;
                    const uint32_t off = (uint32_t)(
                        rtpt::splitmix64(a.seed ^ (0x5851f42d4c957f2dull + *a.sample_dev + jw)) % a.stride);
                    for (int k = 0; k < 3; ++k) {
                        crec.pos[k] = P[k];
                        crec.dir[k] = -d[k];
                        crec.normal[k] = nrm[k];
                        crec.albedo[k] = m.albedo[k];
                    }
                    t1 = T;
                    if ((pixp + off) % a.stride == 0u) {
                        is_train = true;
                        lpre = a.rad[p];
                    } else {
                        is_query = true;
                    }
                }
                if (reflective && !is_query) {
                    // ---- next-event estimation: one point on one light
                    if (n_lights > 0) {
                        const float total = light_cdf[n_lights];
                        const float target = u[0] * total;
                        uint32_t lo = 0, hi = n_lights - 1u;
                        while (lo < hi) {  // first k with cdf[k] > target
                            uint32_t mid = (lo + hi) >> 1;
                            if (__ldg(light_cdf + mid) > target) hi = mid; else lo = mid + 1u;
                        }
                        const rt_pt_light L = lights[lo];
                        const float4 ln = __ldg(light_aux + lo);
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
        if (MULTI) a.ssid[sslot] = sid;
    }
    const uint32_t nslot = warp_append(want_next, a.count_out, a.ray_counts);
    if (a.binning) {
        // rank within the ray's direction octant: lanes of one octant (match_any)
        // take their slots with one atomic on the octant's counter
        const uint32_t wm = __ballot_sync(0xffffffffu, want_next);
        if (want_next) {
            const uint32_t bin = octant_of(nd);
            const uint32_t peers = __match_any_sync(wm, bin);
            const int lane = threadIdx.x & 31;
            const int leader = __ffs(peers) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(a.bins_out + bin, (uint32_t)__popc(peers));
            base = __shfl_sync(wm, base, leader);
            a.stage[2u * nslot] = make_float4(no[0], no[1], no[2], 0.0f);
            a.stage[2u * nslot + 1u] = make_float4(nd[0], nd[1], nd[2], 1e30f);
            a.stage_pidx[nslot] = p;
            if (MULTI) a.stage_rsid[nslot] = sid;
            a.stage_rank[nslot] = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
        }
    } else if (want_next) {
        a.rays_out[2u * nslot] = make_float4(no[0], no[1], no[2], 0.0f);
        a.rays_out[2u * nslot + 1u] = make_float4(nd[0], nd[1], nd[2], 1e30f);
        a.pidx_out[nslot] = p;
        if (MULTI) a.rsid_out[nslot] = sid;
    }
    if (!MULTI && a.cache_mode) {
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

// Grid-stride over the queue (a grid of resident blocks, not one thread
// per pixel: deep bounces leave short queues).
template <bool MULTI>
__global__ void __launch_bounds__(512) k_pt_shade(const PtArgs a) {
    const uint32_t n = *a.count_in;
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t w = blockIdx.x * blockDim.x + (threadIdx.x - lane); w < n; w += gridDim.x * blockDim.x)
        shade_one<MULTI>(a, w + lane, n);
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

__global__ void __launch_bounds__(512) k_pt_resolve(const uint32_t *scount, const uint8_t *socc,
                                                     const uint32_t *spidx, const float4 *scontrib, float4 *rad) {
    const uint32_t n = *scount;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (socc[i]) continue;
        const uint32_t p = spidx[i];
        const float4 c = scontrib[i];
        float4 R = rad[p];
        R.x = R.x + c.x;
        R.y = R.y + c.y;
        R.z = R.z + c.z;
        rad[p] = R;
    }
}

// Adds the wave's k samples of pixel p in sample order (the order
// consecutive one-sample waves would add them).
__global__ void __launch_bounds__(kPtThreads) k_pt_accumulate(uint32_t n, uint32_t k, const float4 *rad,
                                                               float4 *accum, uint32_t *sample_dev) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) *sample_dev = *sample_dev + k;  // raygen of this wave already read it
    if (p >= n) return;
    float4 acc = accum[p];
    for (uint32_t j = 0; j < k; ++j) {
        const float4 r = rad[(size_t)j * n + p];
        acc.x = acc.x + r.x;
        acc.y = acc.y + r.y;
        acc.z = acc.z + r.z;
        acc.w = acc.w + 1.0f;
    }
    accum[p] = acc;
}


// ---------------------------------------------------------------------------
// Batch: many scenes per launch (rtcore_batch.h).  The paths of one sample
// pass are numbered across the scenes; a wave holds up to `cap` consecutive
// paths, and every queue entry carries the index of its scene.
// ---------------------------------------------------------------------------

// Per launch: each scene's traversal view and light tables; ray counters.
__global__ void k_bt_setup(const BtScene *bt, uint32_t n_scenes, TravScene *views, float4 *aux, float *cdf,
                           unsigned long long *ray_counts, uint32_t *err) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) {
        ray_counts[0] = 0ull;
        ray_counts[1] = 0ull;
    }
    if (s >= n_scenes) return;
    const BtScene &sc = bt[s];
    TravScene v;
    v.nodes = nullptr;
    v.prims = nullptr;
    v.node_count = 0u;
    v.prim_count = 0u;
    v.pad[0] = v.pad[1] = 0u;
    const bool used = sc.width != 0u && sc.height != 0u;  // no path refers to a scene without pixels
    if (used && sc.accel) {
        const rt_accel_header *hd = reinterpret_cast<const rt_accel_header *>(sc.accel);
        if (hd->kind == RT_ACCEL_KIND_BLAS) {
            v.nodes = reinterpret_cast<const uint4 *>(sc.accel + hd->node_offset);
            v.prims = reinterpret_cast<const uint4 *>(sc.accel + hd->prim_offset);
            v.node_count = hd->prim_count ? hd->node_count : 0u;
            v.prim_count = hd->prim_count;
        } else {
            // the path tracer shades bottom-level structures only
            report_error(err, RT_ERR_UNSUPPORTED, 0x78000000u | s);
        }
    }
    views[s] = v;
    if (used) light_table(sc.lights, sc.n_lights, aux + sc.light_off, cdf + sc.light_off + s);
}

__global__ void __launch_bounds__(512) k_bt_raygen(const BtScene *bt, uint32_t n_scenes, uint32_t wave_base,
                                                   uint32_t n, uint64_t seed, const uint32_t *sample_dev,
                                                   uint32_t pass, float4 *rays, uint32_t *pidx, uint32_t *rsid,
                                                   uint32_t *psid, float4 *tput, float4 *rad, uint64_t *rng,
                                                   uint32_t *count0, unsigned long long *ray_counts) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) {
        *count0 = n;
        atomicAdd(ray_counts, (unsigned long long)n);
    }
    if (p >= n) return;
    const uint32_t gp = wave_base + p;
    // the last scene whose first path is <= gp (a scene without pixels shares
    // its base with the next one)
    uint32_t lo = 0, hi = n_scenes - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (bt[mid].base <= gp) lo = mid; else hi = mid - 1u;
    }
    const BtScene &sc = bt[lo];
    const uint32_t pix = gp - sc.base;
    const uint32_t x = pix % sc.width, y = pix / sc.width;
    rtpt::Pcg g = rtpt::pcg_seed(seed, *sample_dev + pass, pix);
    const float jx = rtpt::pcg_uniform(g), jy = rtpt::pcg_uniform(g);
    float d[3];
    rtpt::camera_dir(sc.ax, sc.ay, sc.width, sc.height, x, y, jx, jy, d);
    rays[2u * p] = make_float4(sc.cam[0], sc.cam[1], sc.cam[2], 0.0f);
    rays[2u * p + 1u] = make_float4(d[0], d[1], d[2], 1e30f);
    pidx[p] = p;
    rsid[p] = lo;
    psid[p] = lo;
    tput[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    rad[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    rng[p] = g.state;
}

__global__ void __launch_bounds__(512) k_bt_accumulate(const BtScene *bt, uint32_t wave_base, uint32_t n,
                                                       const uint32_t *psid, const float4 *rad, uint32_t discard) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n || discard) return;
    const BtScene &sc = bt[psid[p]];
    float4 *acc = sc.accum + (wave_base + p - sc.base);
    const float4 r = rad[p];
    float4 v = *acc;
    v.x = v.x + r.x;
    v.y = v.y + r.y;
    v.z = v.z + r.z;
    v.w = v.w + 1.0f;
    *acc = v;
}

__global__ void k_bt_sample(uint32_t *sample_dev, uint32_t value, uint32_t add) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *sample_dev = add ? *sample_dev + value : value;
}

}  // namespace
}  // namespace rtc

using namespace rtc;

namespace {

// Blocks of `threads` resident on the GPU at once for `kernel`, capped by the
// blocks n items need (grid-stride kernels).
unsigned resident_blocks(rt_context *ctx, const void *kernel, int threads, uint64_t n) {
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, int> cache;
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = cache.find({kernel, threads});
        if (it != cache.end()) {
            per_sm = it->second;
        } else {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess ||
                per_sm < 1) {
                (void)cudaGetLastError();
                per_sm = 1;
            }
            cache[{kernel, threads}] = per_sm;
        }
    }
    const uint64_t need = (n + (uint64_t)threads - 1u) / (uint64_t)threads;
    const uint64_t have = (uint64_t)per_sm * (uint64_t)ctx->sm_count;
    const uint64_t b = need < have ? need : have;
    return (unsigned)(b ? b : 1u);
}

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
    if (cp && (reinterpret_cast<uintptr_t>(cp->cache) & 255u))
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_path_trace_cached: cache must be 256-byte aligned");
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
    a.npix = (uint32_t)npix;
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
    const uint64_t cap = L.cap;  // paths of a full wave: pixels x L.wave samples
    const unsigned blocks = (unsigned)((npix + kPtThreads - 1) / kPtThreads);
    const unsigned shade_blocks = resident_blocks(ctx, (const void *)k_pt_shade<false>, kPtThreads, cap);
    const unsigned resolve_blocks = resident_blocks(ctx, (const void *)k_pt_resolve, kPtThreads, cap);
    const unsigned scatter_blocks = resident_blocks(ctx, (const void *)k_pt_bin_scatter<false>, kPtThreads, cap);
    a.binning = (p->flags & RT_PT_OCTANT_BINNING) ? 1u : 0u;
    a.stage = reinterpret_cast<float4 *>(S + L.stage);
    a.stage_pidx = reinterpret_cast<uint32_t *>(S + L.stage_pidx);
    a.stage_rank = reinterpret_cast<uint32_t *>(S + L.stage_rank);

    for (uint32_t s = 0, kw = 0; s < p->spp; s += kw) {
        // one wave: kw samples of every pixel (kw = L.wave but for the last)
        kw = p->spp - s < L.wave ? p->spp - s : L.wave;
        const uint32_t nw = (uint32_t)(npix * kw);  // paths of this wave
        RT_CUDA_CTX(ctx, cudaMemsetAsync(cnt, 0, kCntPerSample * 4u, st));
        k_pt_raygen<<<(unsigned)((nw + kPtThreads - 1u) / kPtThreads), kPtThreads, 0, st>>>(
            ax, ay, p->camera.position[0], p->camera.position[1], p->camera.position[2], p->width, p->height,
            p->seed, sample_dev, kw, rays[0], pidx[0], a.tput, a.rad, a.rng, &cnt[0], ray_counts);
        RT_CUDA_CTX(ctx, cudaGetLastError());
        // depth 0's extension rays alone; afterwards each launch traces a
        // depth's shadow rays together with the next depth's extension rays
        int rc0 = launch_queue_trace(ctx, st, accel, rays[0], S + L.hits, nullptr, &cnt[0], nw, &tcnt[0], false);
        if (rc0) return rc0;
        for (uint32_t d = 0; d < p->max_depth; ++d) {
            const uint32_t q = d & 1u;
            int rc = RT_OK;
            a.rays_in = rays[q];
            a.pidx_in = pidx[q];
            a.rays_out = rays[q ^ 1u];
            a.pidx_out = pidx[q ^ 1u];
            a.count_in = &cnt[d];
            a.count_out = &cnt[d + 1];
            a.scount = &scnt[d];
            a.depth = d;
            a.bins_out = cnt + kCntBins + 8u * (d + 1u);
            k_pt_shade<false><<<shade_blocks, kPtThreads, 0, st>>>(a);
            RT_CUDA_CTX(ctx, cudaGetLastError());
            if (a.binning && d + 1u < p->max_depth) {
                k_pt_bin_scatter<false><<<scatter_blocks, kPtThreads, 0, st>>>(
                    &cnt[d + 1], a.bins_out, a.stage, a.stage_pidx, nullptr, a.stage_rank, rays[q ^ 1u],
                    pidx[q ^ 1u], nullptr, nw, ctx->d_err);
                RT_CUDA_CTX(ctx, cudaGetLastError());
            }
            // cnt[max_depth] stays 0: the last launch traces shadow rays only
            rc = launch_queue_trace_mixed(ctx, st, accel, rays[q ^ 1u], S + L.hits, &cnt[d + 1], a.srays, socc,
                                          &scnt[d], nw, &tcnt[2 * d + 1]);
            if (rc) return rc;
            k_pt_resolve<<<resolve_blocks, kPtThreads, 0, st>>>(&scnt[d], socc, a.spidx, a.scontrib, a.rad);
            RT_CUDA_CTX(ctx, cudaGetLastError());
        }
        float4 *ttarget = reinterpret_cast<float4 *>(S + L.ttarget);
        if (cp) {
            int rc = cache_query_dev(ctx, st, cp->cache, a.qin, reinterpret_cast<float *>(S + L.qout), a.qcount, nw);
            if (rc) return rc;
            k_pt_cache_apply<<<(unsigned)((nw + kPtThreads - 1u) / kPtThreads), kPtThreads, 0, st>>>(
                a.qcount, a.qpidx, a.qt1, reinterpret_cast<const float4 *>(S + L.qout), a.rad, a.tcount, a.tpidx,
                a.tt1, a.tlpre, ttarget);
            RT_CUDA_CTX(ctx, cudaGetLastError());
        }
        k_pt_accumulate<<<blocks, kPtThreads, 0, st>>>((uint32_t)npix, kw, a.rad, reinterpret_cast<float4 *>(accum),
                                                       sample_dev);
        RT_CUDA_CTX(ctx, cudaGetLastError());
        if (cp && cp->train_batch) {
            int rc = cache_train_dev(ctx, st, cp->cache, a.tin, reinterpret_cast<const float *>(ttarget), a.tcount,
                                     tcap * kw, cp->train_batch);
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

extern "C" rt_status rt_debug_pt_cache_layout(const rt_pt_params *p, const rt_pt_cache_params *cp, uint32_t n_lights,
                                              rt_debug_pt_cache_offsets *out) {
    if (!p || !cp || !out) return RT_ERR_INVALID_ARG;
    const uint64_t npix = (uint64_t)p->width * p->height;
    const PtLayout L = pt_layout(*p, n_lights, train_capacity(npix, cp->train_paths));
    out->query_count = L.counters + (uint64_t)kCntQuery * 4u;
    out->query_in = L.qin;
    out->query_t1 = L.qt1;
    out->query_path = L.qpidx;
    out->query_out = L.qout;
    out->train_count = L.counters + (uint64_t)kCntTrain * 4u;
    out->train_in = L.tin;
    out->train_t1 = L.tt1;
    out->train_before = L.tlpre;
    out->train_path = L.tpidx;
    out->train_target = L.ttarget;
    return RT_OK;
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

// ---------------------------------------------------------------------------
// Batch host side (rtcore_batch.h)
// ---------------------------------------------------------------------------

namespace {

struct BtLayout {
    uint64_t table, views, light_aux, light_cdf, counters;
    uint64_t rays0, rays1, pidx0, pidx1, rsid0, rsid1, hits, srays, spidx, ssid, scontrib, socc, tput, rad, rng, psid;
    uint64_t stage, stage_pidx, stage_rsid, stage_rank;
    uint64_t total;
    uint64_t cap;  // paths per wave
};

BtLayout bt_layout(uint32_t n_scenes, uint64_t n_lights, uint64_t cap) {
    BtLayout L;
    L.cap = cap;
    uint64_t off = 0;
    auto take = [&](uint64_t b) {
        uint64_t o = off;
        off += align_up(b ? b : 1, 256);
        return o;
    };
    L.table = take((uint64_t)n_scenes * sizeof(BtScene));
    L.views = take((uint64_t)n_scenes * sizeof(TravScene));
    L.light_aux = take(n_lights * 16u);
    L.light_cdf = take((n_lights + n_scenes) * 4u);
    L.counters = take(kCntWords * 4u);  // word layout of the single-scene path tracer
    L.rays0 = take(cap * 32u);
    L.rays1 = take(cap * 32u);
    L.pidx0 = take(cap * 4u);
    L.pidx1 = take(cap * 4u);
    L.rsid0 = take(cap * 4u);
    L.rsid1 = take(cap * 4u);
    L.hits = take(cap * 16u);
    L.srays = take(cap * 32u);
    L.spidx = take(cap * 4u);
    L.ssid = take(cap * 4u);
    L.scontrib = take(cap * 16u);
    L.socc = take(cap);
    L.tput = take(cap * 16u);
    L.rad = take(cap * 16u);
    L.rng = take(cap * 8u);
    L.psid = take(cap * 4u);
    L.stage = take(cap * 32u);
    L.stage_pidx = take(cap * 4u);
    L.stage_rsid = take(cap * 4u);
    L.stage_rank = take(cap * 4u);
    L.total = off;
    return L;
}

constexpr uint64_t kMaxBatchPaths = (1ull << 31) - 1u;  // paths of one sample pass over all scenes
constexpr uint64_t kMaxBatchLights = 1ull << 26;

// Totals of a scene table; RT_OK or an error message in *why.
int batch_totals(const rt_batch_scene *scenes, uint32_t n, uint64_t *paths, uint64_t *lights, const char **why) {
    uint64_t P = 0, NL = 0;
    for (uint32_t s = 0; s < n; ++s) {
        const rt_batch_scene &b = scenes[s];
        const uint64_t npix = (uint64_t)b.width * b.height;
        if (npix) {
            if (!b.scene.accel || !b.accum || !b.scene.tri_material || !b.scene.materials ||
                b.scene.n_materials == 0 || (b.scene.n_lights && !b.scene.lights)) {
                *why = "rt_batch: a scene with pixels needs accel, accum, tri_material and materials (and lights)";
                return RT_ERR_INVALID_ARG;
            }
            if (b.scene.n_lights > (1u << 20)) {
                *why = "rt_batch: more than 2^20 lights in a scene";
                return RT_ERR_UNSUPPORTED;
            }
        }
        P += npix;
        NL += b.scene.n_lights;
    }
    if (P > kMaxBatchPaths || NL > kMaxBatchLights) {
        *why = "rt_batch: more than 2^31 - 1 pixels or 2^26 lights in one batch";
        return RT_ERR_UNSUPPORTED;
    }
    *paths = P;
    *lights = NL;
    return RT_OK;
}

// Zero fields take the defaults; RT_OK or RT_ERR_INVALID_ARG.
int batch_tuning(const rt_batch_tuning *in, rt_batch_tuning *out) {
    rt_batch_tuning t;
    rt_batch_default_tuning(&t);
    if (in) {
        if (in->trace_threads) t.trace_threads = in->trace_threads;
        if (in->trace_blocks_per_sm) t.trace_blocks_per_sm = in->trace_blocks_per_sm;
        if (in->stack_ring) t.stack_ring = in->stack_ring;
        if (in->refill) t.refill = in->refill;
        if (in->shade_threads) t.shade_threads = in->shade_threads;
        t.wave_paths = in->wave_paths;
        if (in->bvh_width) t.bvh_width = in->bvh_width;
    }
    if ((t.trace_threads != 128u && t.trace_threads != 256u) ||
        (t.stack_ring != 8u && t.stack_ring != 16u && t.stack_ring != 32u) || t.refill > 32u ||
        t.trace_blocks_per_sm > 64u || (t.shade_threads != 128u && t.shade_threads != 256u && t.shade_threads != 512u) ||
        t.bvh_width < 4u || t.bvh_width > 8u)
        return RT_ERR_INVALID_ARG;
    *out = t;
    return RT_OK;
}

}  // namespace

struct rt_batch_plan {
    rt_context *ctx = nullptr;
    uint32_t n_scenes = 0;
    rt_batch_params p{};
    rt_batch_tuning t{};
    uint32_t flags = 0;
    BtLayout L{};
    uint8_t *scratch = nullptr;
    uint64_t paths = 0;       // per sample pass
    uint32_t kernels = 0;     // kernel launches per rt_batch_launch
    cudaGraphExec_t exec = nullptr;
    bool sample_known = false;
    uint32_t next_sample = 0;
};

namespace {

int batch_enqueue(rt_batch_plan *pl, cudaStream_t st, uint32_t *kernels) {
    rt_context *ctx = pl->ctx;
    const BtLayout &L = pl->L;
    uint8_t *S = pl->scratch;
    uint32_t k = 0;
    *kernels = 0;
    if (pl->paths == 0) return RT_OK;
    uint32_t *cnt = reinterpret_cast<uint32_t *>(S + L.counters);
    uint32_t *scnt = cnt + 65;
    uint32_t *tcnt = cnt + 129;
    uint32_t *sample_dev = cnt + kCntSample;
    unsigned long long *ray_counts = reinterpret_cast<unsigned long long *>(cnt + kCntRays);
    const BtScene *bt = reinterpret_cast<const BtScene *>(S + L.table);
    void *views = S + L.views;
    float4 *aux = reinterpret_cast<float4 *>(S + L.light_aux);
    float *cdf = reinterpret_cast<float *>(S + L.light_cdf);
    const unsigned T = pl->t.shade_threads;
    const uint32_t n_sc = pl->n_scenes;

    k_bt_setup<<<(n_sc + 127u) / 128u, 128, 0, st>>>(bt, n_sc, reinterpret_cast<TravScene *>(views), aux, cdf,
                                                      ray_counts, ctx->d_err);
    ++k;
    RT_CUDA_CTX(ctx, cudaGetLastError());

    PtArgs a;
    std::memset(&a, 0, sizeof(a));
    a.light_aux = aux;
    a.light_cdf = cdf;
    a.tput = reinterpret_cast<float4 *>(S + L.tput);
    a.rad = reinterpret_cast<float4 *>(S + L.rad);
    a.rng = reinterpret_cast<uint64_t *>(S + L.rng);
    a.hits = reinterpret_cast<const float4 *>(S + L.hits);
    a.srays = reinterpret_cast<float4 *>(S + L.srays);
    a.spidx = reinterpret_cast<uint32_t *>(S + L.spidx);
    a.ssid = reinterpret_cast<uint32_t *>(S + L.ssid);
    a.scontrib = reinterpret_cast<float4 *>(S + L.scontrib);
    a.max_depth = pl->p.max_depth;
    a.rr_depth = pl->p.rr_depth;
    a.eps = pl->p.ray_eps;
    a.ray_counts = ray_counts;
    a.err = ctx->d_err;
    a.bt = bt;
    float4 *rays[2] = {reinterpret_cast<float4 *>(S + L.rays0), reinterpret_cast<float4 *>(S + L.rays1)};
    uint32_t *pidx[2] = {reinterpret_cast<uint32_t *>(S + L.pidx0), reinterpret_cast<uint32_t *>(S + L.pidx1)};
    uint32_t *rsid[2] = {reinterpret_cast<uint32_t *>(S + L.rsid0), reinterpret_cast<uint32_t *>(S + L.rsid1)};
    uint32_t *psid = reinterpret_cast<uint32_t *>(S + L.psid);
    uint8_t *socc = S + L.socc;
    const TraceShape shape{pl->t.trace_threads, pl->t.trace_blocks_per_sm, pl->t.stack_ring, pl->t.refill};
    const uint64_t W = L.cap;
    const uint64_t waves = (pl->paths + W - 1u) / W;
    const uint32_t discard = (pl->flags & RT_BATCH_DISCARD) ? 1u : 0u;
    a.binning = (pl->p.flags & RT_PT_OCTANT_BINNING) ? 1u : 0u;
    a.stage = reinterpret_cast<float4 *>(S + L.stage);
    a.stage_pidx = reinterpret_cast<uint32_t *>(S + L.stage_pidx);
    a.stage_rsid = reinterpret_cast<uint32_t *>(S + L.stage_rsid);
    a.stage_rank = reinterpret_cast<uint32_t *>(S + L.stage_rank);

    for (uint32_t pass = 0; pass < pl->p.spp; ++pass) {
        for (uint64_t w = 0; w < waves; ++w) {
            const uint32_t base = (uint32_t)(w * W);
            const uint32_t n = (uint32_t)(pl->paths - base < W ? pl->paths - base : W);
            const unsigned full = (n + T - 1u) / T;
            const unsigned shade_blocks = resident_blocks(ctx, (const void *)k_pt_shade<true>, (int)T, n);
            const unsigned resolve_blocks = resident_blocks(ctx, (const void *)k_pt_resolve, (int)T, n);
            const unsigned scatter_blocks = resident_blocks(ctx, (const void *)k_pt_bin_scatter<true>, (int)T, n);
            RT_CUDA_CTX(ctx, cudaMemsetAsync(cnt, 0, kCntPerSample * 4u, st));
            k_bt_raygen<<<full, T, 0, st>>>(bt, n_sc, base, n, pl->p.seed, sample_dev, pass, rays[0], pidx[0],
                                            rsid[0], psid, a.tput, a.rad, a.rng, &cnt[0], ray_counts);
            ++k;
            RT_CUDA_CTX(ctx, cudaGetLastError());
            a.wave_base = base;
            // depth 0's extension rays alone; afterwards each launch traces a
            // depth's shadow rays together with the next depth's extension rays
            int rc0 = launch_queue_trace_multi(ctx, st, views, n_sc, rsid[0], rays[0], S + L.hits, nullptr, &cnt[0], n,
                                               &tcnt[0], false, shape);
            if (rc0) return rc0;
            ++k;
            for (uint32_t d = 0; d < pl->p.max_depth; ++d) {
                const uint32_t q = d & 1u;
                int rc = RT_OK;
                a.rays_in = rays[q];
                a.pidx_in = pidx[q];
                a.rsid_in = rsid[q];
                a.rays_out = rays[q ^ 1u];
                a.pidx_out = pidx[q ^ 1u];
                a.rsid_out = rsid[q ^ 1u];
                a.count_in = &cnt[d];
                a.count_out = &cnt[d + 1];
                a.scount = &scnt[d];
                a.depth = d;
                a.bins_out = cnt + kCntBins + 8u * (d + 1u);
                k_pt_shade<true><<<shade_blocks, T, 0, st>>>(a);
                ++k;
                RT_CUDA_CTX(ctx, cudaGetLastError());
                if (a.binning && d + 1u < pl->p.max_depth) {
                    k_pt_bin_scatter<true><<<scatter_blocks, T, 0, st>>>(
                        &cnt[d + 1], a.bins_out, a.stage, a.stage_pidx, a.stage_rsid, a.stage_rank, rays[q ^ 1u],
                        pidx[q ^ 1u], rsid[q ^ 1u], n, ctx->d_err);
                    ++k;
                    RT_CUDA_CTX(ctx, cudaGetLastError());
                }
                // cnt[max_depth] stays 0: the last launch traces shadow rays only
                rc = launch_queue_trace_multi_mixed(ctx, st, views, n_sc, rsid[q ^ 1u], rays[q ^ 1u], S + L.hits,
                                                    &cnt[d + 1], a.ssid, a.srays, socc, &scnt[d], n, &tcnt[2 * d + 1],
                                                    shape);
                if (rc) return rc;
                ++k;
                k_pt_resolve<<<resolve_blocks, T, 0, st>>>(&scnt[d], socc, a.spidx, a.scontrib, a.rad);
                ++k;
                RT_CUDA_CTX(ctx, cudaGetLastError());
            }
            k_bt_accumulate<<<full, T, 0, st>>>(bt, base, n, psid, a.rad, discard);
            ++k;
            RT_CUDA_CTX(ctx, cudaGetLastError());
        }
    }
    k_bt_sample<<<1, 32, 0, st>>>(sample_dev, pl->p.spp, 1u);
    ++k;
    RT_CUDA_CTX(ctx, cudaGetLastError());
    *kernels = k;
    return RT_OK;
}

}  // namespace

extern "C" rt_status rt_batch_default_tuning(rt_batch_tuning *t) {
    if (!t) return RT_ERR_INVALID_ARG;
    t->trace_threads = 128u;
    t->trace_blocks_per_sm = 8u;
    t->stack_ring = 16u;
    t->refill = 4u;
    t->shade_threads = 256u;
    t->wave_paths = 0u;
    t->bvh_width = 8u;
    t->reserved = 0u;
    return RT_OK;
}

extern "C" rt_status rt_batch_scratch_bytes(const rt_batch_scene *scenes, uint32_t n_scenes, const rt_batch_params *p,
                                            const rt_batch_tuning *t, uint64_t *bytes) {
    if (!bytes || !p || (n_scenes && !scenes)) return RT_ERR_INVALID_ARG;
    uint64_t P = 0, NL = 0;
    const char *why = nullptr;
    int rc = batch_totals(scenes, n_scenes, &P, &NL, &why);
    if (rc) return rc;
    rt_batch_tuning tt;
    if (batch_tuning(t, &tt)) return RT_ERR_INVALID_ARG;
    const uint64_t cap = (tt.wave_paths && tt.wave_paths < P) ? tt.wave_paths : P;
    *bytes = bt_layout(n_scenes, NL, cap).total;
    return RT_OK;
}

extern "C" rt_status rt_batch_plan_create(rt_context *ctx, const rt_batch_scene *scenes, uint32_t n_scenes,
                                          const rt_batch_params *p, const rt_batch_tuning *t, void *scratch,
                                          uint64_t scratch_bytes, uint32_t flags, rt_batch_plan **plan) {
    if (!ctx || !p || !plan || (n_scenes && !scenes) || !scratch)
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_batch_plan_create: null argument");
    *plan = nullptr;
    if (flags & ~(RT_BATCH_GRAPH | RT_BATCH_DISCARD))
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_batch_plan_create: unknown flags");
    if (p->max_depth == 0 || p->max_depth > kMaxPtDepth || p->spp == 0 || (p->flags & ~RT_PT_OCTANT_BINNING) ||
        p->reserved)
        return set_error(ctx, RT_ERR_INVALID_ARG,
                         "rt_batch_plan_create: spp >= 1, max_depth in 1..64, flags 0 or RT_PT_OCTANT_BINNING");
    uint64_t P = 0, NL = 0;
    const char *why = nullptr;
    int rc = batch_totals(scenes, n_scenes, &P, &NL, &why);
    if (rc) return set_error(ctx, rc, why);
    rt_batch_tuning tt;
    if (batch_tuning(t, &tt))
        return set_error(ctx, RT_ERR_INVALID_ARG,
                         "rt_batch_plan_create: tuning needs 128/256 trace threads, ring 8/16/32, refill <= 32, "
                         "128/256/512 shade threads, BVH width 4..8");
    const uint64_t cap = (tt.wave_paths && tt.wave_paths < P) ? tt.wave_paths : P;
    const BtLayout L = bt_layout(n_scenes, NL, cap);
    if (scratch_bytes < L.total)
        return set_error(ctx, RT_ERR_OOM, "rt_batch_plan_create: scratch smaller than rt_batch_scratch_bytes");
    if (reinterpret_cast<uintptr_t>(scratch) & 255u)
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_batch_plan_create: scratch must be 256-byte aligned");

    std::vector<BtScene> table(n_scenes);
    uint64_t base = 0, loff = 0;
    for (uint32_t s = 0; s < n_scenes; ++s) {
        const rt_batch_scene &b = scenes[s];
        BtScene &e = table[s];
        std::memset(&e, 0, sizeof(e));
        e.accel = reinterpret_cast<const uint8_t *>(b.scene.accel);
        e.tri_material = b.scene.tri_material;
        e.materials = b.scene.materials;
        e.lights = b.scene.lights;
        e.accum = reinterpret_cast<float4 *>(b.accum);
        e.n_materials = b.scene.n_materials;
        e.n_lights = b.scene.n_lights;
        e.light_off = (uint32_t)loff;
        e.width = b.width;
        e.height = b.height;
        e.base = (uint32_t)base;
        if ((uint64_t)b.width * b.height) camera_aspects(&b.camera, b.width, b.height, &e.ay, &e.ax);
        e.cam[0] = b.camera.position[0];
        e.cam[1] = b.camera.position[1];
        e.cam[2] = b.camera.position[2];
        base += (uint64_t)b.width * b.height;
        loff += b.scene.n_lights;
    }
    rt_batch_plan *pl = new rt_batch_plan();
    pl->ctx = ctx;
    pl->n_scenes = n_scenes;
    pl->p = *p;
    pl->t = tt;
    pl->flags = flags;
    pl->L = L;
    pl->scratch = static_cast<uint8_t *>(scratch);
    pl->paths = P;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess && n_scenes)
        e = cudaMemcpy(pl->scratch + L.table, table.data(), table.size() * sizeof(BtScene), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        delete pl;
        return set_cuda_error(ctx, e, "rt_batch_plan_create: scene table upload");
    }
    // Load every kernel the launches use (and size the grid-stride grids)
    // before a capture begins, so that nothing is loaded while capturing.
    {
        const void *kernels[] = {(const void *)k_bt_setup,       (const void *)k_bt_raygen,
                                 (const void *)k_bt_accumulate,  (const void *)k_bt_sample,
                                 (const void *)k_pt_shade<true>, (const void *)k_pt_resolve,
                                 (const void *)k_pt_bin_scatter<true>};
        cudaFuncAttributes fa;
        for (const void *k : kernels)
            if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k);
        if (e == cudaSuccess) {
            resident_blocks(ctx, (const void *)k_pt_shade<true>, (int)tt.shade_threads, 1u);
            resident_blocks(ctx, (const void *)k_pt_resolve, (int)tt.shade_threads, 1u);
            resident_blocks(ctx, (const void *)k_pt_bin_scatter<true>, (int)tt.shade_threads, 1u);
            const TraceShape shape{tt.trace_threads, tt.trace_blocks_per_sm, tt.stack_ring, tt.refill};
            rc = prepare_queue_trace_multi(ctx, shape);
            if (rc) {
                delete pl;
                return rc;
            }
        }
        if (e != cudaSuccess) {
            delete pl;
            return set_cuda_error(ctx, e, "rt_batch_plan_create: kernel attributes");
        }
    }
    if ((flags & RT_BATCH_GRAPH) && P) {
        cudaStream_t cs = nullptr;
        cudaGraph_t graph = nullptr;
        e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            rc = batch_enqueue(pl, cs, &pl->kernels);
            cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
            if (rc == RT_OK && e2 != cudaSuccess) e = e2;
        }
        if (e == cudaSuccess && rc == RT_OK) e = cudaGraphInstantiate(&pl->exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (cs) cudaStreamDestroy(cs);
        if (rc != RT_OK || e != cudaSuccess) {
            if (pl->exec) cudaGraphExecDestroy(pl->exec);
            delete pl;
            (void)cudaGetLastError();
            return rc != RT_OK ? rc : set_cuda_error(ctx, e, "rt_batch_plan_create: graph capture");
        }
    } else {
        // count the launches of one direct enqueue without issuing it
        const uint64_t waves = P ? (P + cap - 1u) / cap : 0u;
        const uint64_t per_wave = 3u + 3u * p->max_depth + ((p->flags & RT_PT_OCTANT_BINNING) ? p->max_depth - 1u : 0u);
        pl->kernels = P ? (uint32_t)(2u + (uint64_t)p->spp * waves * per_wave) : 0u;
    }
    *plan = pl;
    return RT_OK;
}

extern "C" rt_status rt_batch_launch(rt_batch_plan *pl, rt_stream stream, uint32_t sample_offset) {
    if (!pl) return RT_ERR_INVALID_ARG;
    rt_context *ctx = pl->ctx;
    if (pl->paths == 0) return RT_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    RT_CUDA_CTX(ctx, cudaSetDevice(ctx->device));
    if (!pl->sample_known || pl->next_sample != sample_offset) {
        uint32_t *cnt = reinterpret_cast<uint32_t *>(pl->scratch + pl->L.counters);
        k_bt_sample<<<1, 32, 0, st>>>(cnt + kCntSample, sample_offset, 0u);
        RT_CUDA_CTX(ctx, cudaGetLastError());
    }
    if (pl->exec) {
        RT_CUDA_CTX(ctx, cudaGraphLaunch(pl->exec, st));
    } else {
        uint32_t k = 0;
        int rc = batch_enqueue(pl, st, &k);
        if (rc) return rc;
    }
    pl->sample_known = true;
    pl->next_sample = sample_offset + pl->p.spp;
    return RT_OK;
}

extern "C" rt_status rt_batch_ray_counts(rt_batch_plan *pl, rt_stream stream, uint64_t *extension_rays,
                                         uint64_t *shadow_rays) {
    if (!pl) return RT_ERR_INVALID_ARG;
    rt_context *ctx = pl->ctx;
    unsigned long long h[2] = {0ull, 0ull};
    if (pl->paths) {
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        RT_CUDA_CTX(ctx, cudaMemcpyAsync(h, pl->scratch + pl->L.counters + kCntRays * 4u, sizeof(h),
                                         cudaMemcpyDeviceToHost, st));
        RT_CUDA_CTX(ctx, cudaStreamSynchronize(st));
    }
    if (extension_rays) *extension_rays = h[0];
    if (shadow_rays) *shadow_rays = h[1];
    return RT_OK;
}

extern "C" rt_status rt_batch_plan_launches(const rt_batch_plan *pl, uint32_t *kernels) {
    if (!pl || !kernels) return RT_ERR_INVALID_ARG;
    *kernels = pl->kernels;
    return RT_OK;
}

extern "C" rt_status rt_batch_plan_destroy(rt_batch_plan *pl) {
    if (!pl) return RT_OK;
    if (pl->exec) cudaGraphExecDestroy(pl->exec);
    delete pl;
    return RT_OK;
}
