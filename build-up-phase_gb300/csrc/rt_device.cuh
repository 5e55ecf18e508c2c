// rt_device.cuh -- device-side arithmetic shared by the build and trace
// kernels of the GB300 ray-tracing core.
//
// Every kernel translation unit is compiled with -fmad=false: a float
// expression is evaluated one IEEE round-to-nearest operation at a time, and
// an FMA is issued only where __fmaf_rn is written.  That is what makes the
// build bit-exact, and the hits bit-identical, against the CPU restatement of
// the same steps.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/rtcore.h"
#include "../../include/rtcore_accel.h"

namespace rtc {

constexpr uint32_t kLeafBit = 0x80000000u;
constexpr float kTfarScale = 1.0f + 0x1p-20f;
constexpr float kInf = __builtin_huge_valf();

// ---------------------------------------------------------------------------
// Float helpers
// ---------------------------------------------------------------------------

// Total order on float bits (-0 < +0): min/max under it give the same bits
// whatever the order of a parallel reduction.
__device__ __forceinline__ int32_t ford(float f) {
    int32_t i = __float_as_int(f);
    return i >= 0 ? i : (i ^ 0x7fffffff);
}
__device__ __forceinline__ float ford_inv(int32_t i) {
    return __int_as_float(i >= 0 ? i : (i ^ 0x7fffffff));
}
__device__ __forceinline__ float fmn(float a, float b) { return ford(b) < ford(a) ? b : a; }
__device__ __forceinline__ float fmx(float a, float b) { return ford(b) > ford(a) ? b : a; }
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }

struct Box {
    float lo[3], hi[3];
};

__device__ __forceinline__ Box box_empty() {
    Box b;
#pragma unroll
    for (int a = 0; a < 3; ++a) { b.lo[a] = kInf; b.hi[a] = -kInf; }
    return b;
}
__device__ __forceinline__ bool box_is_empty(const Box &b) {
    return !(b.lo[0] <= b.hi[0] && b.lo[1] <= b.hi[1] && b.lo[2] <= b.hi[2]);
}
__device__ __forceinline__ Box box_union(const Box &x, const Box &y) {
    Box b;
#pragma unroll
    for (int a = 0; a < 3; ++a) { b.lo[a] = fmn(x.lo[a], y.lo[a]); b.hi[a] = fmx(x.hi[a], y.hi[a]); }
    return b;
}
__device__ __forceinline__ float half_area(const Box &b) {
    if (box_is_empty(b)) return 0.0f;
    float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return (dx * dy + dy * dz) + dz * dx;
}

// Smallest e with 255 * 2^e >= ext, clamped to [RT_QEXP_MIN, RT_QEXP_MAX].
__device__ __forceinline__ int qexp_for(float ext) {
    if (!(ext > 0.0f)) return RT_QEXP_MIN;
    int biased = (int)((__float_as_uint(ext) >> 23) & 0xffu);
    int e = (biased == 0 ? -127 : biased - 127) - 8;
    if (e < RT_QEXP_MIN) e = RT_QEXP_MIN;
    while (e < RT_QEXP_MAX && 255.0f * pow2f(e) < ext) ++e;
    return e;
}

__device__ __forceinline__ void xform_point(const float m[12], const float p[3], float out[3]) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
        out[r] = ((m[4 * r + 0] * p[0] + m[4 * r + 1] * p[1]) + m[4 * r + 2] * p[2]) + m[4 * r + 3];
}
__device__ __forceinline__ void xform_vector(const float m[12], const float p[3], float out[3]) {
#pragma unroll
    for (int r = 0; r < 3; ++r) out[r] = (m[4 * r + 0] * p[0] + m[4 * r + 1] * p[1]) + m[4 * r + 2] * p[2];
}

// ---------------------------------------------------------------------------
// Ray setup and the watertight triangle test
// (Woop, Benthin, Wald, JCGT 2013)
// ---------------------------------------------------------------------------

struct Ray {
    float o[3];
    float d[3];
    float invd[3];
    float sx, sy, sz;
    uint32_t oct;   // bit a set: invd[a] < 0
    uint32_t kxyz;  // kx | ky << 2 | kz << 4
};

__device__ __forceinline__ float sel3(uint32_t k, float x, float y, float z) {
    return k == 0 ? x : (k == 1 ? y : z);
}

__device__ __forceinline__ void ray_setup(Ray &r, const float o[3], const float d[3]) {
    uint32_t oct = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        r.o[a] = o[a];
        r.d[a] = d[a];
        float dd = fabsf(d[a]) < RT_DIR_EPS ? copysignf(RT_DIR_EPS, d[a]) : d[a];
        r.invd[a] = 1.0f / dd;
        oct |= (r.invd[a] < 0.0f ? 1u : 0u) << a;
    }
    r.oct = oct;
    float ax = fabsf(d[0]), ay = fabsf(d[1]), az = fabsf(d[2]);
    uint32_t kz = ax >= ay ? (ax >= az ? 0u : 2u) : (ay >= az ? 1u : 2u);
    uint32_t kx = kz == 2u ? 0u : kz + 1u;
    uint32_t ky = kx == 2u ? 0u : kx + 1u;
    float dkz = sel3(kz, d[0], d[1], d[2]);
    if (dkz < 0.0f) { uint32_t t = kx; kx = ky; ky = t; }
    r.kxyz = kx | (ky << 2) | (kz << 4);
    r.sx = sel3(kx, d[0], d[1], d[2]) / dkz;
    r.sy = sel3(ky, d[0], d[1], d[2]) / dkz;
    r.sz = 1.0f / dkz;
}

// Returns true and (t, u, v) when the triangle is hit with t in [tmin, tmax].
__device__ __forceinline__ bool isect_tri(const Ray &r, float4 v0, float4 v1, float4 v2, float tmin, float tmax,
                                          float &t_out, float &u_out, float &v_out) {
    const uint32_t kx = r.kxyz & 3u, ky = (r.kxyz >> 2) & 3u, kz = (r.kxyz >> 4) & 3u;
    float A0 = v0.x - r.o[0], A1 = v0.y - r.o[1], A2 = v0.z - r.o[2];
    float B0 = v1.x - r.o[0], B1 = v1.y - r.o[1], B2 = v1.z - r.o[2];
    float C0 = v2.x - r.o[0], C1 = v2.y - r.o[1], C2 = v2.z - r.o[2];
    float Akz = sel3(kz, A0, A1, A2), Bkz = sel3(kz, B0, B1, B2), Ckz = sel3(kz, C0, C1, C2);
    float ax = sel3(kx, A0, A1, A2) - r.sx * Akz, ay = sel3(ky, A0, A1, A2) - r.sy * Akz;
    float bx = sel3(kx, B0, B1, B2) - r.sx * Bkz, by = sel3(ky, B0, B1, B2) - r.sy * Bkz;
    float cx = sel3(kx, C0, C1, C2) - r.sx * Ckz, cy = sel3(ky, C0, C1, C2) - r.sy * Ckz;
    float U = cx * by - cy * bx;
    float V = ax * cy - ay * cx;
    float W = bx * ay - by * ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)cx * (double)by - (double)cy * (double)bx);
        V = (float)((double)ax * (double)cy - (double)ay * (double)cx);
        W = (float)((double)bx * (double)ay - (double)by * (double)ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = (U + V) + W;
    if (det == 0.0f) return false;
    float T = (U * (r.sz * Akz) + V * (r.sz * Bkz)) + W * (r.sz * Ckz);
    float rcp = 1.0f / det;
    float t = T * rcp;
    if (!(t >= tmin && t <= tmax)) return false;
    t_out = t;
    u_out = V * rcp;
    v_out = W * rcp;
    return true;
}

// ---------------------------------------------------------------------------
// Wide node test
// ---------------------------------------------------------------------------

struct NodeWords {
    uint4 w0, w1, w2, w3, w4;
};

__device__ __forceinline__ NodeWords load_node(const uint4 *nodes, uint32_t idx) {
    const uint4 *p = nodes + (size_t)idx * 5u;
    NodeWords n;
    n.w0 = __ldg(p + 0);
    n.w1 = __ldg(p + 1);
    n.w2 = __ldg(p + 2);
    n.w3 = __ldg(p + 3);
    n.w4 = __ldg(p + 4);
    return n;
}

__device__ __forceinline__ uint32_t byte_of(uint32_t w, int b) { return (w >> (8 * b)) & 0xffu; }

// Byte b of w as an exact float: PRMT assembles 0x4B0000qq (= 2^23 + q) and
// one FADD removes 2^23.  Same value as (float)q without the conversion pipe.
__device__ __forceinline__ float qbyte(uint32_t w, int b) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | (uint32_t)b)) - 8388608.0f;
}

// Three-input min/max (sm_100+ PTX); exact, so equal to two-input chains.
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Two-wide FP32 arithmetic (PTX .f32x2, sm_100 and later): one instruction
// for two lanes' worth of add or fma, each half rounded exactly as the scalar
// instruction, so the pair equals two scalar results bit for bit.
__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
    uint64_t d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
__device__ __forceinline__ void f2_unpack(uint64_t v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
// Byte b of wx and of wy as the pair (2^23 + qx, 2^23 + qy); adding
// (-2^23, -2^23) leaves the exact byte values.
__device__ __forceinline__ uint64_t qpair2_biased(uint32_t wx, uint32_t wy, int b) {
    const uint32_t lo = __byte_perm(wx, 0x4B000000u, 0x7540u | (uint32_t)b);
    const uint32_t hi = __byte_perm(wy, 0x4B000000u, 0x7540u | (uint32_t)b);
    uint64_t d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "r"(lo), "r"(hi));
    return d;
}

// Box test of a node's 8 children against [tmin, tcur].
//   node_hits: bit (slot ^ oct) for every internal child hit
//   prim_hits: leaf-record mask relative to the node's prim_base
// An internal child's meta byte is 0x20 | (24 + slot) and a leaf's offset is
// below 24, so XOR-ing the octant into the internal bytes (four at a time)
// lets one shift-or per hit slot build both masks: internal children land on
// bit 24 + (slot ^ oct), leaf records on their offsets.
template <bool PAIR_Z = false>
__device__ __forceinline__ void isect_node(const Ray &r, const NodeWords &n, float tmin, float tcur,
                                           uint32_t &node_hits, uint32_t &prim_hits) {
    const float px = __uint_as_float(n.w0.x), py = __uint_as_float(n.w0.y), pz = __uint_as_float(n.w0.z);
    const int ex = (int)(int8_t)(n.w0.w & 0xffu);
    const int ey = (int)(int8_t)((n.w0.w >> 8) & 0xffu);
    const int ez = (int)(int8_t)((n.w0.w >> 16) & 0xffu);
    const float scx = pow2f(ex) * r.invd[0], scy = pow2f(ey) * r.invd[1], scz = pow2f(ez) * r.invd[2];
    const float adjx = (px - r.o[0]) * r.invd[0];
    const float adjy = (py - r.o[1]) * r.invd[1];
    const float adjz = (pz - r.o[2]) * r.invd[2];
    // qlo/qhi words for slots 0-3 (lo) and 4-7 (hi), per axis
    const uint32_t lox[2] = {n.w2.x, n.w2.y}, loy[2] = {n.w2.z, n.w2.w}, loz[2] = {n.w3.x, n.w3.y};
    const uint32_t hix[2] = {n.w3.z, n.w3.w}, hiy[2] = {n.w4.x, n.w4.y}, hiz[2] = {n.w4.z, n.w4.w};
    const uint32_t meta[2] = {n.w1.z, n.w1.w};
    const bool nx = r.oct & 1u, ny = r.oct & 2u, nz = r.oct & 4u;
    // a child's x and y plane distances as one .f32x2 add and fma and, with
    // PAIR_Z (kernels with registers to spare), its near and far z distances
    // as another; each half equals the scalar fma(q, scale, adj)
    const uint64_t bias2 = f2_pack(-8388608.0f, -8388608.0f);
    const uint64_t scxy = f2_pack(scx, scy), adjxy = f2_pack(adjx, adjy);
    uint32_t hits = 0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint32_t nearx = nx ? hix[h] : lox[h], farx = nx ? lox[h] : hix[h];
        const uint32_t neary = ny ? hiy[h] : loy[h], fary = ny ? loy[h] : hiy[h];
        const uint32_t nearz = nz ? hiz[h] : loz[h], farz = nz ? loz[h] : hiz[h];
        const uint32_t inner4 = (meta[h] >> 3) & (meta[h] >> 4) & 0x01010101u;
        const uint32_t mx4 = meta[h] ^ (inner4 * r.oct);
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            float nxv, nyv, fxv, fyv, tn, tf;
            f2_unpack(f2_fma(f2_add(qpair2_biased(nearx, neary, b), bias2), scxy, adjxy), nxv, nyv);
            f2_unpack(f2_fma(f2_add(qpair2_biased(farx, fary, b), bias2), scxy, adjxy), fxv, fyv);
            if constexpr (PAIR_Z) {
                float nzv, fzv;
                f2_unpack(f2_fma(f2_add(qpair2_biased(nearz, farz, b), bias2), f2_pack(scz, scz),
                                 f2_pack(adjz, adjz)),
                          nzv, fzv);
                tn = fmaxf(fmax3(tmin, nxv, nyv), nzv);
                tf = fminf(fmin3(tcur, fxv, fyv), fzv);
            } else {
                tn = fmaxf(fmax3(tmin, nxv, nyv), __fmaf_rn(qbyte(nearz, b), scz, adjz));
                tf = fminf(fmin3(tcur, fxv, fyv), __fmaf_rn(qbyte(farz, b), scz, adjz));
            }
            if (tn <= tf * kTfarScale) {
                const uint32_t m = byte_of(mx4, b);
                hits |= (m >> 5) << (m & 31u);
            }
        }
    }
    node_hits = hits >> 24;
    prim_hits = hits & 0x00ffffffu;
}

// Device-side error reporting: the first error code wins.
__device__ __forceinline__ void report_error(uint32_t *err, int code, uint32_t detail) {
    if (err) {
        if (atomicCAS(err, 0u, (uint32_t)(-code)) == 0u) err[1] = detail;
    }
}

}  // namespace rtc
