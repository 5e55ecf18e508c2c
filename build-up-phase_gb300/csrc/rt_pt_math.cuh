// rt_pt_math.cuh -- scalar light-transport helpers of the path tracer,
// written once for host and device (__host__ __device__).
//
// Only + - * / and sqrt appear (all correctly rounded), with a fixed
// operation order; device code is compiled with -fmad=false and host code
// with -ffp-contract=off, so the GPU path tracer and the CPU oracle follow
// bit-identical paths.  sin/cos are Taylor polynomials on [-pi/4, pi/4]
// (truncation error below 3e-8 there), not the CUDA or libm functions.
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define RT_HD __host__ __device__ __forceinline__
#else
#define RT_HD inline
#endif

namespace rtpt {

constexpr float kInvPi = 0.318309886183790671538f;
constexpr float kPi4 = 0.785398163397448309616f;

// PCG32 XSH-RR (O'Neill 2014) with per-(pixel, sample) streams.
struct Pcg {
    uint64_t state;
    uint64_t inc;
};

RT_HD uint32_t pcg_next(Pcg &g) {
    uint64_t old = g.state;
    g.state = old * 6364136223846793005ull + g.inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
}

RT_HD uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// Stream of pixel `pixel`, sample `sample`.
RT_HD Pcg pcg_seed(uint64_t seed, uint32_t sample, uint32_t pixel) {
    Pcg g;
    g.inc = ((uint64_t)pixel << 1u) | 1u;
    g.state = 0;
    pcg_next(g);
    g.state += splitmix64(seed + sample);
    pcg_next(g);
    return g;
}

RT_HD float pcg_uniform(Pcg &g) { return (float)(pcg_next(g) >> 8) * (1.0f / 16777216.0f); }

// sin and cos of x in [-pi/4, pi/4] (Taylor series to x^9 / x^8, Horner).
RT_HD float sin_q(float x) {
    float x2 = x * x;
    return x * (1.0f + x2 * (-1.0f / 6.0f + x2 * (1.0f / 120.0f + x2 * (-1.0f / 5040.0f + x2 * (1.0f / 362880.0f)))));
}
RT_HD float cos_q(float x) {
    float x2 = x * x;
    return 1.0f + x2 * (-0.5f + x2 * (1.0f / 24.0f + x2 * (-1.0f / 720.0f + x2 * (1.0f / 40320.0f))));
}

// Concentric square -> disk map (Shirley & Chiu 1997).
RT_HD void concentric_disk(float u1, float u2, float &x, float &y) {
    float a = 2.0f * u1 - 1.0f, b = 2.0f * u2 - 1.0f;
    if (a == 0.0f && b == 0.0f) { x = 0.0f; y = 0.0f; return; }
    float aa = a < 0.0f ? -a : a, ab = b < 0.0f ? -b : b;
    if (aa > ab) {
        float phi = kPi4 * (b / a);
        x = a * cos_q(phi);
        y = a * sin_q(phi);
    } else {
        float phi = kPi4 * (a / b);  // angle pi/2 - phi
        x = b * sin_q(phi);
        y = b * cos_q(phi);
    }
}

// Orthonormal basis around unit n (Duff et al., "Building an Orthonormal
// Basis, Revisited", JCGT 2017).
RT_HD void onb(const float n[3], float t1[3], float t2[3]) {
    float sign = copysignf(1.0f, n[2]);
    float a = -1.0f / (sign + n[2]);
    float b = n[0] * n[1] * a;
    t1[0] = 1.0f + sign * n[0] * n[0] * a;
    t1[1] = sign * b;
    t1[2] = -sign * n[0];
    t2[0] = b;
    t2[1] = sign + n[1] * n[1] * a;
    t2[2] = -n[1];
}

RT_HD float dot3(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

RT_HD void cross3(const float a[3], const float b[3], float c[3]) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// Camera ray of the sample's raygen basis through (x + jx, y + jy).
RT_HD void camera_dir(float ax, float ay, uint32_t w, uint32_t h, uint32_t x, uint32_t y, float jx, float jy,
                      float d[3]) {
    float sx = (float)x + jx, sy = (float)y + jy;
    float ndx = (sx / (float)w) * 2.0f - 1.0f;
    float ndy = (sy / (float)h) * 2.0f - 1.0f;
    float p = ndx * ax, q = ndy * ay;
    d[0] = (p * 1.0f + q * 0.0f) + 0.0f;
    d[1] = (p * 0.0f + q * -1.0f) + 0.0f;
    d[2] = (p * 0.0f + q * 0.0f) + -1.0f;
}

}  // namespace rtpt
