// rt_scene.cpp -- seeded synthetic scenes of the ray-tracing core (host).
//
// Only + - * / and sqrt are used on floats (all correctly rounded), and the
// file is compiled with -ffp-contract=off, so every host architecture
// produces the same scene bits from the same seed.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/rtcore.h"
#include "../../include/rtcore_scene.h"

namespace {

// PCG32 (O'Neill 2014, "PCG: A Family of Simple Fast Space-Efficient
// Statistically Good Algorithms for Random Number Generation"), XSH-RR.
struct Pcg32 {
    uint64_t state = 0, inc = 1;
    Pcg32(uint64_t seed, uint64_t seq) {
        inc = (seq << 1u) | 1u;
        next();
        state += seed;
        next();
    }
    uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
    // uniform in [0, 1) with 24 random bits
    float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
    float uniform(float a, float b) { return a + (b - a) * uniform(); }
};

// SplitMix64: decorrelates per-object seeds.
uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// Direction uniform on the unit sphere by rejection from the cube.
void unit_dir(Pcg32 &g, float d[3]) {
    for (;;) {
        float x = 2.0f * g.uniform() - 1.0f, y = 2.0f * g.uniform() - 1.0f, z = 2.0f * g.uniform() - 1.0f;
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

const float kPhi = 1.6180339887498949f;
const float kIcoV[12][3] = {{-1, kPhi, 0}, {1, kPhi, 0}, {-1, -kPhi, 0}, {1, -kPhi, 0},
                            {0, -1, kPhi}, {0, 1, kPhi}, {0, -1, -kPhi}, {0, 1, -kPhi},
                            {kPhi, 0, -1}, {kPhi, 0, 1}, {-kPhi, 0, -1}, {-kPhi, 0, 1}};
const int kIcoF[20][3] = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11},
                          {1, 5, 9},  {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
                          {3, 9, 4},  {3, 4, 2},  {3, 2, 6},   {3, 6, 8},  {3, 8, 9},
                          {4, 9, 5},  {2, 4, 11}, {6, 2, 10},  {8, 6, 7},  {9, 8, 1}};

uint32_t face_grid_vertices(uint32_t f) { return (f + 1u) * (f + 2u) / 2u; }

}  // namespace

extern "C" rt_status rt_scene_soup(uint64_t seed, uint32_t n_tris, float *v, uint32_t *idx) {
    if (n_tris && (!v || !idx)) return RT_ERR_INVALID_ARG;
    Pcg32 g(splitmix64(seed), 1u);
    for (uint32_t i = 0; i < n_tris; ++i) {
        float c[3] = {g.uniform(), g.uniform(), g.uniform()};
        float d1[3], d2[3];
        unit_dir(g, d1);
        unit_dir(g, d2);
        float l1 = g.uniform(0.001f, 0.02f), l2 = g.uniform(0.001f, 0.02f);
        float e1[3] = {d1[0] * l1, d1[1] * l1, d1[2] * l1};
        float e2[3] = {d2[0] * l2, d2[1] * l2, d2[2] * l2};
        float *p = v + (size_t)i * 9u;
        for (int a = 0; a < 3; ++a) {
            float v0 = c[a] - (e1[a] + e2[a]) / 3.0f;
            p[a] = v0;
            p[3 + a] = v0 + e1[a];
            p[6 + a] = v0 + e2[a];
        }
        idx[3 * i + 0] = 3 * i + 0;
        idx[3 * i + 1] = 3 * i + 1;
        idx[3 * i + 2] = 3 * i + 2;
    }
    return RT_OK;
}

extern "C" rt_status rt_scene_box_counts(uint32_t n_spheres, uint32_t freq, uint32_t *n_vertices,
                                         uint32_t *n_tris, uint32_t *n_materials) {
    if (freq == 0 && n_spheres) return RT_ERR_INVALID_ARG;
    uint64_t nv = 8u + 4u + (uint64_t)n_spheres * 20u * face_grid_vertices(freq);
    uint64_t nt = 12u + 2u + (uint64_t)n_spheres * 20u * (uint64_t)freq * freq;
    if (nv > 0xffffffffull || nt > (1u << 30)) return RT_ERR_UNSUPPORTED;
    if (n_vertices) *n_vertices = (uint32_t)nv;
    if (n_tris) *n_tris = (uint32_t)nt;
    if (n_materials) *n_materials = 4u + n_spheres;
    return RT_OK;
}

extern "C" rt_status rt_scene_box(uint64_t seed, uint32_t n_spheres, uint32_t freq, float *v, uint32_t *idx,
                                  uint32_t *tmat, rt_material *mats) {
    uint32_t nv, nt, nm;
    rt_status rc = rt_scene_box_counts(n_spheres, freq, &nv, &nt, &nm);
    if (rc) return rc;
    if (!v || !idx || !tmat || !mats) return RT_ERR_INVALID_ARG;
    // materials: 0 white, 1 red, 2 green, 3 light, 4+k sphere k
    const float white[3] = {0.73f, 0.73f, 0.73f}, red[3] = {0.65f, 0.05f, 0.05f}, green[3] = {0.12f, 0.45f, 0.15f};
    std::memset(mats, 0, sizeof(rt_material) * nm);
    for (int a = 0; a < 3; ++a) {
        mats[0].albedo[a] = white[a];
        mats[1].albedo[a] = red[a];
        mats[2].albedo[a] = green[a];
        mats[3].albedo[a] = 0.0f;
        mats[3].emission[a] = 15.0f;
    }
    // box corners: bit0 x, bit1 y, bit2 z
    for (int c = 0; c < 8; ++c) {
        v[3 * c + 0] = (c & 1) ? 1.0f : -1.0f;
        v[3 * c + 1] = (c & 2) ? 1.0f : -1.0f;
        v[3 * c + 2] = (c & 4) ? 1.0f : -1.0f;
    }
    // faces as quads (a, b, c, d) -> triangles (a, b, c), (a, c, d), wound to face inward
    const uint32_t quads[6][4] = {
        {0, 1, 5, 4},  // floor   y = -1
        {2, 6, 7, 3},  // ceiling y = +1
        {0, 2, 3, 1},  // back    z = -1
        {4, 5, 7, 6},  // front   z = +1
        {0, 4, 6, 2},  // left    x = -1
        {1, 3, 7, 5},  // right   x = +1
    };
    const uint32_t qmat[6] = {0, 0, 0, 0, 1, 2};
    uint32_t t = 0;
    for (int q = 0; q < 6; ++q) {
        const uint32_t *Q = quads[q];
        idx[3 * t + 0] = Q[0]; idx[3 * t + 1] = Q[1]; idx[3 * t + 2] = Q[2]; tmat[t++] = qmat[q];
        idx[3 * t + 0] = Q[0]; idx[3 * t + 1] = Q[2]; idx[3 * t + 2] = Q[3]; tmat[t++] = qmat[q];
    }
    // light quad just below the ceiling
    const float ly = 0.999f, lh = 0.25f;
    const float lv[4][3] = {{-lh, ly, -lh}, {lh, ly, -lh}, {lh, ly, lh}, {-lh, ly, lh}};
    for (int k = 0; k < 4; ++k)
        for (int a = 0; a < 3; ++a) v[3 * (8 + k) + a] = lv[k][a];
    idx[3 * t + 0] = 8; idx[3 * t + 1] = 9; idx[3 * t + 2] = 10; tmat[t++] = 3;
    idx[3 * t + 0] = 8; idx[3 * t + 1] = 10; idx[3 * t + 2] = 11; tmat[t++] = 3;

    uint32_t vbase = 12;
    for (uint32_t s = 0; s < n_spheres; ++s) {
        Pcg32 g(splitmix64(seed ^ splitmix64(0x51000000ull + s)), 2u);
        float radius = g.uniform(0.05f, 0.25f);
        float cen[3] = {g.uniform(-0.75f, 0.75f), g.uniform(-0.75f, 0.75f), g.uniform(-0.75f, 0.75f)};
        for (int a = 0; a < 3; ++a) mats[4 + s].albedo[a] = g.uniform(0.1f, 0.9f);
        for (int f = 0; f < 20; ++f) {
            const float *A = kIcoV[kIcoF[f][0]], *B = kIcoV[kIcoF[f][1]], *Cc = kIcoV[kIcoF[f][2]];
            const uint32_t fbase = vbase;
            // grid point (i, j), i + j <= freq: A + (B - A) i/freq + (C - A) j/freq
            for (uint32_t i = 0; i <= freq; ++i)
                for (uint32_t j = 0; j + i <= freq; ++j) {
                    float fi = (float)i / (float)freq, fj = (float)j / (float)freq;
                    float p[3];
                    for (int a = 0; a < 3; ++a) p[a] = (A[a] + (B[a] - A[a]) * fi) + (Cc[a] - A[a]) * fj;
                    float inv = radius / std::sqrt((p[0] * p[0] + p[1] * p[1]) + p[2] * p[2]);
                    for (int a = 0; a < 3; ++a) v[3 * vbase + a] = cen[a] + p[a] * inv;
                    ++vbase;
                }
            // row-major index of (i, j) within the face grid
            auto at = [&](uint32_t i, uint32_t j) {
                // rows i = 0..freq have (freq + 1 - i) entries
                uint32_t before = i * (freq + 1u) - (i * (i - 1u)) / 2u;
                return fbase + before + j;
            };
            for (uint32_t i = 0; i < freq; ++i)
                for (uint32_t j = 0; j + i < freq; ++j) {
                    idx[3 * t + 0] = at(i, j); idx[3 * t + 1] = at(i + 1, j); idx[3 * t + 2] = at(i, j + 1);
                    tmat[t++] = 4u + s;
                    if (j + i + 1u < freq) {
                        idx[3 * t + 0] = at(i + 1, j); idx[3 * t + 1] = at(i + 1, j + 1); idx[3 * t + 2] = at(i, j + 1);
                        tmat[t++] = 4u + s;
                    }
                }
        }
    }
    return (t == nt && vbase == nv) ? RT_OK : RT_ERR_BOUNDS;
}

extern "C" rt_status rt_scene_incoherent_rays(uint64_t seed, uint32_t n, const float lo[3], const float hi[3],
                                              float tmax, rt_ray *rays) {
    if (n && (!rays || !lo || !hi)) return RT_ERR_INVALID_ARG;
    Pcg32 g(splitmix64(seed), 3u);
    for (uint32_t i = 0; i < n; ++i) {
        rt_ray &r = rays[i];
        for (int a = 0; a < 3; ++a) r.org[a] = g.uniform(lo[a], hi[a]);
        unit_dir(g, r.dir);
        r.tmin = 0.0f;
        r.tmax = tmax;
    }
    return RT_OK;
}
