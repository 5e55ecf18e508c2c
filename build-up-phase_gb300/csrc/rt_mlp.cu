// rt_mlp.cu -- the MLP radiance cache: encoding, fused forward on the tensor
// cores, backward, Adam.
//
// No counterpart in the reference (its sample has no path tracer to cache).
//
// Network (padded layout, FP32 master parameters and a BF16 copy):
//   layer 0: 96 (81 used) -> 64, ReLU
//   layers 1-4: 64 -> 64, ReLU
//   layer 5: 64 -> 8 (3 used), linear
// Inference (queries): tcgen05 MMAs with TMEM accumulators, see
// k_cache_query_tc.
// Training forward: one warp owns 16 rows of a 128-row tile; each layer is
// m16n8k16 BF16 MMAs with FP32 accumulation; the FP32 accumulator fragment of
// one layer is exactly the A-operand fragment layout of the next (after bias,
// ReLU and BF16 packing), so activations never leave registers between
// layers.  Weights sit in shared memory with padded row strides.
// Backward: the same MMAs propagate delta through W (B fragments of W read
// transposed from its forward layout with ldmatrix.trans); the weight
// gradients delta^T A are MMAs too (both operands loaded transposed with
// ldmatrix.trans), added to global FP32 gradients once per weight and tile;
// Adam updates the FP32 master copy and refreshes the BF16 one.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/rtcore_cache.h"
#include "rt_internal.h"

namespace rtc {
namespace {

constexpr int kLayers = 6;
constexpr int kParams = 23368;  // sum of out*in + out

__host__ __device__ constexpr int in_dim(int l) { return l == 0 ? 96 : 64; }
__host__ __device__ constexpr int out_dim(int l) { return l == 5 ? 8 : 64; }
__host__ __device__ constexpr int w_off(int l) {
    int o = 0;
    for (int k = 0; k < l; ++k) o += out_dim(k) * in_dim(k) + out_dim(k);
    return o;
}
__host__ __device__ constexpr int b_off(int l) { return w_off(l) + out_dim(l) * in_dim(l); }
static_assert(w_off(kLayers) == kParams, "parameter count");

// shared-memory strides (elements): +8 bf16 keeps fragment loads conflict free
__host__ __device__ constexpr int w_stride(int l) { return in_dim(l) + 8; }
constexpr int kBiasFloats = 64 * 5 + 8;
constexpr int kInStride = 104;
constexpr int kActStride = 72;

// State buffer layout (bytes)
struct CacheState {
    float params[kParams];
    float grads[kParams];
    float m[kParams];
    float v[kParams];
    __nv_bfloat16 wbf[kParams];
    uint32_t step;
    float lo[3], hi[3];
    float lr, beta1, beta2, eps;
    float loss;
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&h);
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// c[j] = bias + A (16 x 16*KS) * V^T where V is row-major [8*NT][16*KS] in
// shared memory (stride vs).  bias may be null.
template <int KS, int NT>
__device__ __forceinline__ void warp_dense(const uint32_t (&a)[KS][4], const __nv_bfloat16 *V, int vs,
                                           const float *bias, float (&c)[NT][4], int lane) {
    const int g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const float b0 = bias ? bias[8 * j + 2 * q] : 0.0f, b1 = bias ? bias[8 * j + 2 * q + 1] : 0.0f;
        c[j][0] = b0; c[j][1] = b1; c[j][2] = b0; c[j][3] = b1;
    }
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const __nv_bfloat16 *row = V + (8 * j + g) * vs + 16 * ks + 2 * q;
            const uint32_t b0 = *reinterpret_cast<const uint32_t *>(row);
            const uint32_t b1 = *reinterpret_cast<const uint32_t *>(row + 8);
            mma_bf16(c[j], a[ks], b0, b1);
        }
    }
}

// ReLU + BF16 pack of an accumulator (16 x 64) into the next layer's A
// fragments.
__device__ __forceinline__ void relu_to_a(const float (&c)[8][4], uint32_t (&a)[4][4]) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        a[q][0] = pack_bf16(fmaxf(c[2 * q][0], 0.0f), fmaxf(c[2 * q][1], 0.0f));
        a[q][1] = pack_bf16(fmaxf(c[2 * q][2], 0.0f), fmaxf(c[2 * q][3], 0.0f));
        a[q][2] = pack_bf16(fmaxf(c[2 * q + 1][0], 0.0f), fmaxf(c[2 * q + 1][1], 0.0f));
        a[q][3] = pack_bf16(fmaxf(c[2 * q + 1][2], 0.0f), fmaxf(c[2 * q + 1][3], 0.0f));
    }
}

// A fragments of a 16-row slab from a row-major BF16 shared-memory matrix.
template <int KS>
__device__ __forceinline__ void load_a(const __nv_bfloat16 *M, int ms, int r0, int lane, uint32_t (&a)[KS][4]) {
    const int g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
        const __nv_bfloat16 *p0 = M + (r0 + g) * ms + 16 * ks + 2 * q;
        const __nv_bfloat16 *p1 = p0 + 8 * ms;
        a[ks][0] = *reinterpret_cast<const uint32_t *>(p0);
        a[ks][1] = *reinterpret_cast<const uint32_t *>(p1);
        a[ks][2] = *reinterpret_cast<const uint32_t *>(p0 + 8);
        a[ks][3] = *reinterpret_cast<const uint32_t *>(p1 + 8);
    }
}

// Input encoding of one row into 96 BF16 values.
__device__ void encode_row(const rt_cache_input &in, const CacheState *S, __nv_bfloat16 *out) {
    float f[96];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float ext = S->hi[a] - S->lo[a];
        const float pn = ext > 0.0f ? (in.pos[a] - S->lo[a]) / ext : 0.0f;
        // octave k = sin/cos(2^k pi x): one sincospif, then the double-angle
        // recurrence (the error doubles per octave: ~2^11 ulp after 11
        // octaves, far below the BF16 rounding of the features)
        float s, c;
        sincospif(pn, &s, &c);
#pragma unroll
        for (int k = 0; k < 12; ++k) {
            f[24 * a + 2 * k] = s;
            f[24 * a + 2 * k + 1] = c;
            const float s2 = 2.0f * s * c, c2 = (c - s) * (c + s);
            s = s2;
            c = c2;
        }
    }
    for (int a = 0; a < 3; ++a) {
        f[72 + a] = in.dir[a];
        f[75 + a] = in.normal[a];
        f[78 + a] = in.albedo[a];
    }
    for (int k = 81; k < 96; ++k) f[k] = 0.0f;
    for (int k = 0; k < 96; k += 2)
        *reinterpret_cast<uint32_t *>(out + k) = pack_bf16(f[k], f[k + 1]);
}

constexpr int kQueryRows = 128;

// ---------------------------------------------------------------------------
// Training: forward + backward over 128-row tiles, gradients into S->grads
// ---------------------------------------------------------------------------
//
// Eight warps, 16 rows each.  Forward as in the inference form, keeping each
// layer's BF16 post-activations.  Backward, layer L = 5 .. 0: the weight and
// bias gradients dW_L = delta_L^T A_{L-1}, db_L = sum delta_L over the tile's
// 128 rows, on the tensor cores (m16n8k16, BF16 operands loaded transposed
// from shared memory with ldmatrix.trans, FP32 accumulation, one atomic add
// per weight and tile), then delta_{L-1} = (delta_L W_L) * relu'(A_{L-1})
// with W_L read transposed by ldmatrix.trans from its forward layout.

// Programmatic dependent launch between the training kernels (forward +
// backward, Adam, the next batch's forward + backward): each kernel lets the
// next one launch as soon as all of its own blocks run, then waits for the
// kernel before it to complete (its writes visible) before it reads or
// writes anything, so a launch's scheduling overlaps the previous kernel's
// tail.  Launched without the attribute both instructions do nothing.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

constexpr int kTrainRows = 128;
constexpr int kTrainThreads = 256;
__host__ __device__ constexpr int tw_rows(int l) { return l == 5 ? 16 : 64; }  // weight rows kept in shared memory
__host__ __device__ constexpr int tw_off(int l) {
    int o = 0;
    for (int k = 0; k < l; ++k) o += tw_rows(k) * w_stride(k);
    return o;
}
constexpr int kTwElems = tw_off(kLayers);                    // 26240 BF16
constexpr int kDStride = 72;                                 // BF16 delta rows
constexpr size_t kTrainSmem = (size_t)kTwElems * 2 + (size_t)kBiasFloats * 4 + (size_t)kTrainRows * kInStride * 2 +
                              (size_t)5 * kTrainRows * kActStride * 2 + (size_t)kTrainRows * kDStride * 2;
static_assert(kTrainSmem <= 227u * 1024u, "shared memory of the training kernel");

__device__ __forceinline__ void ldsm_x4_t(const void *p, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"((uint32_t)__cvta_generic_to_shared(p)));
}
__device__ __forceinline__ void ldsm_x2_t(const void *p, uint32_t &r0, uint32_t &r1) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];"
                 : "=r"(r0), "=r"(r1)
                 : "r"((uint32_t)__cvta_generic_to_shared(p)));
}

// Weights (BF16, padded rows; the 8-output layer padded to 16 zero rows) and
// FP32 biases into shared memory, 16 bytes at a time.  Every thread issues
// all of its loads before it stores any (the chunks are independent), so the
// copy costs about one memory round trip instead of one per layer and step:
// 5.5 us of a 16,384-sample batch when each layer's loads waited on the
// previous layer's stores.
constexpr int kTrainWChunks = 64 * 12 + 4 * 64 * 8 + 16 * 8;  // 2,944 sixteen-byte chunks
constexpr int kTrainWPerThread = (kTrainWChunks + kTrainThreads - 1) / kTrainThreads;
__device__ __forceinline__ void train_chunk(int e, int &l, int &o, int &c) {
    if (e < 768) { l = 0; o = e / 12; c = e % 12; }
    else if (e < 2816) { l = 1 + (e - 768) / 512; o = ((e - 768) % 512) / 8; c = (e - 768) % 8; }
    else { l = 5; o = (e - 2816) / 8; c = (e - 2816) % 8; }
}
__device__ void load_weights_train(const CacheState *S, __nv_bfloat16 *sW, float *sB) {
    uint4 r[kTrainWPerThread];
#pragma unroll
    for (int k = 0; k < kTrainWPerThread; ++k) {
        const int e = threadIdx.x + k * kTrainThreads;
        r[k] = make_uint4(0u, 0u, 0u, 0u);
        if (e < kTrainWChunks) {
            int l, o, c;
            train_chunk(e, l, o, c);
            if (o < out_dim(l)) r[k] = reinterpret_cast<const uint4 *>(S->wbf + w_off(l))[o * (in_dim(l) / 8) + c];
        }
    }
    float b[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int e = threadIdx.x + k * kTrainThreads, l = e < 320 ? e / 64 : 5, o = e < 320 ? e % 64 : e - 320;
        b[k] = (e < kBiasFloats && o < out_dim(l)) ? S->params[b_off(l) + o] : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < kTrainWPerThread; ++k) {
        const int e = threadIdx.x + k * kTrainThreads;
        if (e >= kTrainWChunks) continue;
        int l, o, c;
        train_chunk(e, l, o, c);
        *reinterpret_cast<uint4 *>(sW + tw_off(l) + o * w_stride(l) + 8 * c) = r[k];
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int e = threadIdx.x + k * kTrainThreads;
        if (e < kBiasFloats) sB[e] = b[k];  // layer l's bias at 64 l, the output layer's at 320
    }
}

// c[j] = A (16 x 16*KS, registers) * W (row-major [16*KS][*], shared memory,
// read transposed): the backward product delta * W over NT n-tiles of 8.
template <int KS, int NT>
__device__ __forceinline__ void warp_dense_wt(const uint32_t (&a)[KS][4], const __nv_bfloat16 *W, int ws,
                                              float (&c)[NT][4], int lane) {
    static_assert(NT % 2 == 0, "n-tiles in pairs");
    const int row = lane & 7, mat = lane >> 3;
#pragma unroll
    for (int j = 0; j < NT; ++j) c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.0f;
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
#pragma unroll
        for (int jp = 0; jp < NT / 2; ++jp) {
            // matrices: (k 0-7, n 0-7), (k 8-15, n 0-7), (k 0-7, n 8-15), (k 8-15, n 8-15)
            const __nv_bfloat16 *p = W + (16 * ks + 8 * (mat & 1) + row) * ws + 16 * jp + 8 * (mat >> 1);
            uint32_t b0, b1, b2, b3;
            ldsm_x4_t(p, b0, b1, b2, b3);
            mma_bf16(c[2 * jp], a[ks], b0, b1);
            mma_bf16(c[2 * jp + 1], a[ks], b2, b3);
        }
    }
}

// dW[o][i] += sum_r delta[r][o] * A[r][i] over the tile's 128 rows for the
// outputs [o0, o0 + 16) and NT n-tiles of inputs from i0, on the tensor
// cores; rows o >= OUT (padding) are dropped.
template <int IN, int OUT, int NT>
__device__ __forceinline__ void warp_grad_w(const __nv_bfloat16 *sD, const __nv_bfloat16 *sA, int as, int o0, int i0,
                                            float *gW, float *gb, int lane) {
    const int row = lane & 7, mat = lane >> 3, g = lane >> 2, q = lane & 3;
    float c[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.0f;
#pragma unroll 2
    for (int ks = 0; ks < kTrainRows / 16; ++ks) {
        const int r = 16 * ks;
        // A = delta^T (m = output, k = row): matrices (rows r..r+7 | r+8..r+15) x (o0.. | o0+8..)
        uint32_t a[4];
        ldsm_x4_t(sD + (r + 8 * (mat >> 1) + row) * kDStride + o0 + 8 * (mat & 1), a[0], a[1], a[2], a[3]);
        if constexpr (NT == 1) {
            uint32_t b0, b1;
            ldsm_x2_t(sA + (r + 8 * (mat & 1) + row) * as + i0, b0, b1);
            mma_bf16(c[0], a, b0, b1);
        } else {
#pragma unroll
            for (int jp = 0; jp < NT / 2; ++jp) {
                // B = A (k = row, n = input): matrices (r.., i) (r+8.., i) (r.., i+8) (r+8.., i+8)
                uint32_t b0, b1, b2, b3;
                ldsm_x4_t(sA + (r + 8 * (mat & 1) + row) * as + i0 + 16 * jp + 8 * (mat >> 1), b0, b1, b2, b3);
                mma_bf16(c[2 * jp], a, b0, b1);
                mma_bf16(c[2 * jp + 1], a, b2, b3);
            }
        }
    }
    // input IN is the tile's column of ones: its sums are the bias gradient;
    // columns past it are discarded
#pragma unroll
    // (each lane holds two adjacent inputs of a row: one 8-byte vector add)
    for (int j = 0; j < NT; ++j) {
        const int i = i0 + 8 * j + 2 * q;  // even; IN is even
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int o = o0 + g + 8 * h;
            const float x = c[j][2 * h], y = c[j][2 * h + 1];
            if (o >= OUT || (x == 0.0f && y == 0.0f)) continue;
            if (i < IN)
                asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(gW + o * IN + i), "f"(x), "f"(y) : "memory");
            else if (i == IN && x != 0.0f)
                atomicAdd(gb + o, x);
        }
    }
}

// The weight and bias gradients of layer L, split over the eight warps.  The
// input tiles carry a column of ones right after their last input (column 96
// of the encoded inputs, 64 of the activations, in the row padding), so the
// warps whose input range reaches it take one more n-tile and the MMAs leave
// the bias gradient sum_r delta[r][o] there: no separate row loop (it held two
// warps for ~2 us per layer while the block waited at its barrier).
__device__ __forceinline__ void grads_of_layer(int L, const __nv_bfloat16 *sD, const __nv_bfloat16 *ain, int as,
                                               float *grads, int warp, int lane) {
    if (L == 0) {
        if (warp >> 2)
            warp_grad_w<96, 64, 8>(sD, ain, as, 16 * (warp & 3), 48, grads + w_off(0), grads + b_off(0), lane);
        else
            warp_grad_w<96, 64, 6>(sD, ain, as, 16 * (warp & 3), 0, grads + w_off(0), grads + b_off(0), lane);
    } else if (L == 5) {
        if (warp == 7)
            warp_grad_w<64, 8, 2>(sD, ain, as, 0, 56, grads + w_off(5), grads + b_off(5), lane);
        else
            warp_grad_w<64, 8, 1>(sD, ain, as, 0, 8 * warp, grads + w_off(5), grads + b_off(5), lane);
    } else {
        if (warp >> 2)
            warp_grad_w<64, 64, 6>(sD, ain, as, 16 * (warp & 3), 32, grads + w_off(L), grads + b_off(L), lane);
        else
            warp_grad_w<64, 64, 4>(sD, ain, as, 16 * (warp & 3), 0, grads + w_off(L), grads + b_off(L), lane);
    }
}

// bump_step: this launch is followed by an Adam step (k_cache_adam), whose
// step count it advances first (block 0), so no launch of its own is needed.
__global__ void __launch_bounds__(kTrainThreads, 1) k_cache_fwd_bwd(CacheState *S, const rt_cache_input *in,
                                                                    const float4 *targets, uint32_t n,
                                                                    float inv_count, const uint32_t *n_dev,
                                                                    uint32_t row0, uint32_t bump_step) {
    pdl_enter();
    if (bump_step && blockIdx.x == 0 && threadIdx.x == 0) S->step += 1u;
    if (n_dev) {
        // rows [row0, row0 + n) of a set whose size is produced on the device
        const uint32_t total = *n_dev;
        n = total > row0 ? min(n, total - row0) : 0u;
        if (n == 0) return;
        in += row0;
        targets += row0;
        inv_count = 1.0f / (3.0f * (float)n);
    }
    extern __shared__ __align__(16) uint8_t smem[];
    __nv_bfloat16 *sW = reinterpret_cast<__nv_bfloat16 *>(smem);
    float *sB = reinterpret_cast<float *>(sW + kTwElems);
    __nv_bfloat16 *sIn = reinterpret_cast<__nv_bfloat16 *>(sB + kBiasFloats);
    __nv_bfloat16 *sAct = sIn + kTrainRows * kInStride;
    __nv_bfloat16 *sD = sAct + 5 * kTrainRows * kActStride;
    load_weights_train(S, sW, sB);
    {
        // the ones columns of the bias gradients (row padding, never written otherwise)
        const uint4 ones = make_uint4(0x3f803f80u, 0x3f803f80u, 0x3f803f80u, 0x3f803f80u);
        for (int e = threadIdx.x; e < 6 * kTrainRows; e += kTrainThreads) {
            const int t = e / kTrainRows, r = e % kTrainRows;
            if (t == 0) *reinterpret_cast<uint4 *>(sIn + r * kInStride + 96) = ones;
            else *reinterpret_cast<uint4 *>(sAct + (t - 1) * kTrainRows * kActStride + r * kActStride + 64) = ones;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, q = lane & 3;
    const int r0 = warp * 16;
    const uint32_t tiles = (n + kTrainRows - 1) / kTrainRows;
    float loss = 0.0f;
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        __syncthreads();
        if (threadIdx.x < kTrainRows) {
            const uint32_t row = tile * kTrainRows + threadIdx.x;
            __nv_bfloat16 *dst = sIn + threadIdx.x * kInStride;
            if (row < n) encode_row(in[row], S, dst);
            else
                for (int k = 0; k < 96; k += 2) *reinterpret_cast<uint32_t *>(dst + k) = 0u;
        }
        __syncthreads();
        // ---- forward, keeping post-activations for the backward pass
        uint32_t a0[6][4];
        load_a<6>(sIn, kInStride, r0, lane, a0);
        float c[8][4];
        warp_dense<6, 8>(a0, sW + tw_off(0), w_stride(0), sB, c, lane);
        uint32_t a[4][4];
        relu_to_a(c, a);
#pragma unroll 1
        for (int l = 1; l <= 5; ++l) {
            // store layer l-1 output (the input of layer l) as BF16
            __nv_bfloat16 *act = sAct + (l - 1) * kTrainRows * kActStride;
#pragma unroll
            for (int qq = 0; qq < 4; ++qq) {
                *reinterpret_cast<uint32_t *>(act + (r0 + g) * kActStride + 16 * qq + 2 * q) = a[qq][0];
                *reinterpret_cast<uint32_t *>(act + (r0 + g + 8) * kActStride + 16 * qq + 2 * q) = a[qq][1];
                *reinterpret_cast<uint32_t *>(act + (r0 + g) * kActStride + 16 * qq + 8 + 2 * q) = a[qq][2];
                *reinterpret_cast<uint32_t *>(act + (r0 + g + 8) * kActStride + 16 * qq + 8 + 2 * q) = a[qq][3];
            }
            if (l <= 4) {
                warp_dense<4, 8>(a, sW + tw_off(l), w_stride(l), sB + 64 * l, c, lane);
                relu_to_a(c, a);
            }
        }
        float y[1][4];
        warp_dense<4, 1>(a, sW + tw_off(5), w_stride(5), sB + 320, y, lane);
        // ---- loss gradient at the outputs (cols 0..2 of each row); delta_5
        // as BF16 (cols 0..15, 3..15 zero)
        float dy[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int rr = r0 + g + (e >= 2 ? 8 : 0), col = 2 * q + (e & 1);
            const uint32_t row = tile * kTrainRows + rr;
            dy[e] = 0.0f;
            if (col < 3 && row < n) {
                const float4 tg = targets[row];
                const float yt = col == 0 ? tg.x : (col == 1 ? tg.y : tg.z);
                const float diff = y[0][e] - yt, den = y[0][e] * y[0][e] + 0.01f;
                dy[e] = 2.0f * diff / den * inv_count;
                loss += diff * diff / den;
            }
        }
        uint32_t ad[4][4];
        ad[0][0] = pack_bf16(dy[0], dy[1]);
        ad[0][1] = pack_bf16(dy[2], dy[3]);
        ad[0][2] = 0u;
        ad[0][3] = 0u;
        *reinterpret_cast<uint32_t *>(sD + (r0 + g) * kDStride + 2 * q) = ad[0][0];
        *reinterpret_cast<uint32_t *>(sD + (r0 + g + 8) * kDStride + 2 * q) = ad[0][1];
        *reinterpret_cast<uint32_t *>(sD + (r0 + g) * kDStride + 8 + 2 * q) = 0u;
        *reinterpret_cast<uint32_t *>(sD + (r0 + g + 8) * kDStride + 8 + 2 * q) = 0u;
        // ---- backward, layers 5 .. 0
#pragma unroll 1
        for (int L = 5; L >= 0; --L) {
            __syncthreads();  // delta_L and every activation complete
            const __nv_bfloat16 *ain = L == 0 ? sIn : sAct + (L - 1) * kTrainRows * kActStride;
            const int as = L == 0 ? kInStride : kActStride;
            grads_of_layer(L, sD, ain, as, S->grads, warp, lane);
            if (L == 0) break;
            // delta_{L-1} = (delta_L W_L) * relu'(act_{L-1})
            float dc[8][4];
            if (L == 5) {
                uint32_t a1[1][4] = {{ad[0][0], ad[0][1], ad[0][2], ad[0][3]}};
                warp_dense_wt<1, 8>(a1, sW + tw_off(5), w_stride(5), dc, lane);
            } else {
                warp_dense_wt<4, 8>(ad, sW + tw_off(L), w_stride(L), dc, lane);
            }
            const __nv_bfloat16 *act = sAct + (L - 1) * kTrainRows * kActStride;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const __nv_bfloat162 m0 =
                    *reinterpret_cast<const __nv_bfloat162 *>(act + (r0 + g) * kActStride + 8 * j + 2 * q);
                const __nv_bfloat162 m1 =
                    *reinterpret_cast<const __nv_bfloat162 *>(act + (r0 + g + 8) * kActStride + 8 * j + 2 * q);
                if (!(__bfloat162float(m0.x) > 0.0f)) dc[j][0] = 0.0f;
                if (!(__bfloat162float(m0.y) > 0.0f)) dc[j][1] = 0.0f;
                if (!(__bfloat162float(m1.x) > 0.0f)) dc[j][2] = 0.0f;
                if (!(__bfloat162float(m1.y) > 0.0f)) dc[j][3] = 0.0f;
            }
#pragma unroll
            for (int qq = 0; qq < 4; ++qq) {
                ad[qq][0] = pack_bf16(dc[2 * qq][0], dc[2 * qq][1]);
                ad[qq][1] = pack_bf16(dc[2 * qq][2], dc[2 * qq][3]);
                ad[qq][2] = pack_bf16(dc[2 * qq + 1][0], dc[2 * qq + 1][1]);
                ad[qq][3] = pack_bf16(dc[2 * qq + 1][2], dc[2 * qq + 1][3]);
            }
            __syncthreads();  // every warp is done reading delta_L
#pragma unroll
            for (int qq = 0; qq < 4; ++qq) {
                *reinterpret_cast<uint32_t *>(sD + (r0 + g) * kDStride + 16 * qq + 2 * q) = ad[qq][0];
                *reinterpret_cast<uint32_t *>(sD + (r0 + g + 8) * kDStride + 16 * qq + 2 * q) = ad[qq][1];
                *reinterpret_cast<uint32_t *>(sD + (r0 + g) * kDStride + 16 * qq + 8 + 2 * q) = ad[qq][2];
                *reinterpret_cast<uint32_t *>(sD + (r0 + g + 8) * kDStride + 16 * qq + 8 + 2 * q) = ad[qq][3];
            }
        }
    }
    // block loss -> state (mean over samples and channels)
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if (lane == 0) atomicAdd(&S->loss, loss * inv_count);
}

// ---------------------------------------------------------------------------
// Inference on the 5th-generation tensor cores (tcgen05 + TMEM)
// ---------------------------------------------------------------------------
//
// One CTA = 4 warps = 128 threads, one query row per thread, 128-row tiles.
// Operands live in shared memory in the canonical K-major layout without
// swizzle: 8-row x 16-byte core matrices; element (r, k) of a tile with K
// columns sits at (r/8)*16K + (k/8)*128 + (r%8)*16 + (k%8)*2 bytes, so one
// MMA step of K = 16 is described by LBO = 128 (next core matrix along K) and
// SBO = 16K (next 8-row group).  Thread 0 issues tcgen05.mma.kind::f16 with
// M = 128, N = 64 (N = 16 for the output layer), K = 16 per instruction,
// BF16 x BF16 -> FP32 accumulators in TMEM (row r = TMEM lane r), and commits
// to an mbarrier.  The accumulators start from the layer's bias (written with
// tcgen05.st), so the MMAs add the bias.  The epilogue of every thread reads
// its row's 64 accumulators with tcgen05.ld (each warp its own 32-lane
// quarter), applies ReLU and packs BF16 in one cvt.rn.relu.bf16x2.f32 per
// pair, writes the row into the next layer's A tile and the next layer's bias
// into the columns it has read; fence.proxy.async makes the generic-proxy
// stores visible to the next MMA.  Every mbarrier wait is bounded: on expiry the kernel records
// RT_ERR_TIMEOUT, waits once more (bounded) for its MMAs, frees its TMEM and
// returns.

constexpr int kTcRows = 128;
constexpr int kTcGroups = 4;                      // independent 128-row tile groups per CTA
constexpr int kTcThreads = 128 * kTcGroups;
constexpr uint32_t kTcTmemCols = 64u * kTcGroups;  // one 64-column accumulator per group
// tile byte sizes / offsets
__host__ __device__ constexpr uint32_t tc_tile_bytes(int rows, int k) { return (uint32_t)(rows / 8) * 16u * k; }
__host__ __device__ constexpr uint32_t tc_w_off(int l) {
    uint32_t o = 0;
    for (int i = 0; i < l; ++i) o += tc_tile_bytes(i == 5 ? 16 : 64, in_dim(i));
    return o;
}
constexpr uint32_t kTcWBytes = tc_w_off(6);                        // 47104: all weights, shared by the groups
constexpr uint32_t kTcBias = kTcWBytes;                            // 336 floats
constexpr uint32_t kTcBar = kTcBias + 336u * 4u;                   // one mbarrier per group + the TMEM address
constexpr uint32_t kTcGroupBase = (kTcBar + 64u + 127u) & ~127u;
// per group: the K = 96 input tile (reused as the second hidden tile once
// layer 0 has read it) and the first hidden tile (K = 64)
constexpr uint32_t kTcA0 = 0;
constexpr uint32_t kTcH0 = tc_tile_bytes(kTcRows, 96);
constexpr uint32_t kTcH1 = kTcA0;
constexpr uint32_t kTcGroupBytes = kTcH0 + tc_tile_bytes(kTcRows, 64);  // 40960
constexpr uint32_t kTcSmem = kTcGroupBase + kTcGroups * kTcGroupBytes;
static_assert(kTcSmem <= 227u * 1024u, "shared memory of the inference kernel");
constexpr int kTcSpinLimit = 1 << 20;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint32_t tc_off(int r, int k, int kdim) {
    return (uint32_t)(r >> 3) * 16u * (uint32_t)kdim + (uint32_t)(k >> 3) * 128u + (uint32_t)(r & 7) * 16u +
           (uint32_t)(k & 7) * 2u;
}
// Shared-memory matrix descriptor: start >> 4, LBO >> 4, SBO >> 4,
// descriptor version 1 (bits 46-47), no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3fffu) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: FP32 accumulate (bits 4-5 = 1), BF16
// A and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22,
// M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    for (int it = 0; it < kTcSpinLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// 16 consecutive accumulator columns of this thread's TMEM lane from a
// 16-byte aligned shared-memory array (four 16-byte loads)
__device__ __forceinline__ void tc_st16_smem(uint32_t taddr, const float *src) {
    const float4 *p = reinterpret_cast<const float4 *>(src);
    const float4 a = p[0], b = p[1], c = p[2], d = p[3];
    const float v[16] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w, d.x, d.y, d.z, d.w};
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
            taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
        "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
        "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])),
        "r"(__float_as_uint(v[11])), "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])),
        "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
        : "memory");
}
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// max(lo, 0) and max(hi, 0) rounded to BF16 and packed (lo in the low half):
// one cvt.rn.relu.bf16x2.f32
__device__ __forceinline__ uint32_t relu_pack_bf16(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void group_sync(int group) {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + group), "r"(kTcRows) : "memory");
}

__global__ void __launch_bounds__(kTcThreads, 1) k_cache_query_tc(const CacheState *S, const rt_cache_input *in,
                                                                  float4 *out, uint32_t n, const uint32_t *n_dev,
                                                                  uint32_t *err) {
    if (n_dev) n = min(n, *n_dev);
    extern __shared__ __align__(16) uint8_t smem[];
    uint8_t *sW = smem;
    float *sB = reinterpret_cast<float *>(smem + kTcBias);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kTcBar);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + kTcBar + 8u * kTcGroups);
    // per group: set by a thread whose barrier wait ran out, before the
    // group's barrier, read by all the group's threads after it (so the whole
    // group leaves its loop together)
    __shared__ int s_gfail[kTcGroups];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int group = tid / kTcRows, gtid = tid % kTcRows;
    uint8_t *gsm = smem + kTcGroupBase + (uint32_t)group * kTcGroupBytes;

    // ---- weights (canonical K-major) and biases into shared memory, once
    for (int l = 0; l < kLayers; ++l) {
        const int kin = in_dim(l), nout = l == 5 ? 16 : 64, nreal = out_dim(l);
        const __nv_bfloat16 *gw = S->wbf + w_off(l);
        __nv_bfloat16 *dst = reinterpret_cast<__nv_bfloat16 *>(sW + tc_w_off(l));
        for (int e = tid; e < nout * kin; e += kTcThreads) {
            const int o = e / kin, i = e % kin;
            dst[tc_off(o, i, kin) / 2] = o < nreal ? gw[o * kin + i] : __float2bfloat16(0.0f);
        }
    }
    for (int e = tid; e < 336; e += kTcThreads) {
        const int l = e < 320 ? e / 64 : 5, o = e < 320 ? e % 64 : e - 320;
        sB[e] = o < out_dim(l) ? S->params[b_off(l) + o] : 0.0f;
    }
    if (tid < kTcGroups) s_gfail[tid] = 0;
    if (tid == 0) {
        for (int g = 0; g < kTcGroups; ++g)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bars + g)) : "memory");
        // make the initialised barriers visible to the tensor core's arrivals
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // this group's accumulator columns; warp w of the group reads TMEM lanes
    // [32 (w % 4), 32 (w % 4) + 32)
    const uint32_t tmem = *tmem_slot + 64u * (uint32_t)group;
    const uint32_t bar_a = smem_u32(bars + group);
    const uint32_t w_base = smem_u32(sW);
    uint32_t phase = 0;
    volatile int *gfail = s_gfail + group;
    const uint32_t tiles = (n + kTcRows - 1) / kTcRows;
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;

    // The groups run independently (own tiles, buffers, barrier, phase): the
    // tensor core works on one group's layer while the others encode or run
    // their epilogues.
    // this thread's input row of the group's next tile, loaded one tile ahead
    const uint32_t tile_stride = gridDim.x * kTcGroups;
    uint32_t tile = blockIdx.x * kTcGroups + (uint32_t)group;
    rt_cache_input cur;
    if (tile < tiles && tile * kTcRows + (uint32_t)gtid < n) cur = in[tile * kTcRows + (uint32_t)gtid];
    for (; tile < tiles; tile += tile_stride) {
        // ---- encode this thread's row into the K = 96 input tile
        const uint32_t row = tile * kTcRows + (uint32_t)gtid;
        {
            __align__(16) __nv_bfloat16 feat[96];
            if (row < n) {
                encode_row(cur, S, feat);
            } else {
                for (int k = 0; k < 96; ++k) feat[k] = __float2bfloat16(0.0f);
            }
            for (int kc = 0; kc < 12; ++kc)
                *reinterpret_cast<uint4 *>(gsm + kTcA0 + tc_off(gtid, 8 * kc, 96)) =
                    *reinterpret_cast<const uint4 *>(feat + 8 * kc);
        }
        // layer 0's bias into this row's accumulators: the MMAs add onto it
        for (int c16 = 0; c16 < 4; ++c16) tc_st16_smem(tmem + lane_base + 16u * c16, sB + 16 * c16);
        tc_wait_st();
        {
            const uint32_t nrow = (tile + tile_stride) * kTcRows + (uint32_t)gtid;
            if (tile + tile_stride < tiles && nrow < n) cur = in[nrow];  // in flight during the layers
        }
        fence_async_smem();
        tc_fence_before();
        group_sync(group);
        tc_fence_after();
#pragma unroll 1
        for (int l = 0; l < kLayers; ++l) {
            const int kin = in_dim(l);
            const uint32_t a_base = smem_u32(gsm + (l == 0 ? kTcA0 : ((l & 1) ? kTcH0 : kTcH1)));
            const uint32_t b_base = w_base + tc_w_off(l);
            // the issuing thread alone waits for the MMAs; the rest of the
            // group sleeps in the group barrier instead of polling
            if (gtid == 0) {
                const uint32_t idesc = tc_idesc(kTcRows, l == 5 ? 16 : 64);
                for (int ks = 0; ks < kin / 16; ++ks) {
                    const uint64_t da = tc_desc(a_base + 256u * ks, 128u, 16u * kin);
                    const uint64_t db = tc_desc(b_base + 256u * ks, 128u, 16u * kin);
                    tc_mma(tmem, da, db, idesc, 1u);  // onto the bias
                }
                tc_commit(bar_a);
                if (!mbar_wait_bounded(bar_a, phase)) {
                    report_error(err, RT_ERR_TIMEOUT, 0x90000000u | (uint32_t)l);
                    mbar_wait_bounded(bar_a, phase);  // once more: no MMA may outlive the TMEM
                    *gfail = 1;
                }
                tc_fence_before();
            }
            phase ^= 1u;
            group_sync(group);
            tc_fence_after();
            if (*gfail) break;  // read after the barrier: the same for the whole group
            if (l < 5) {
                // hidden layer: ReLU -> BF16 row of the next A tile; the
                // next layer's bias replaces each column group once read
                uint8_t *next = gsm + ((l & 1) ? kTcH1 : kTcH0);
                const float *nbias = sB + 64 * (l + 1);
#pragma unroll
                for (int c32 = 0; c32 < 2; ++c32) {
                    // two 16-column loads in flight per wait
                    float v[2][16];
                    tc_ld16(tmem + lane_base + 32u * c32, v[0]);
                    tc_ld16(tmem + lane_base + 32u * c32 + 16u, v[1]);
                    tc_wait_ld();
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int c16 = 2 * c32 + h;
                        if (l < 4 || c16 == 0) tc_st16_smem(tmem + lane_base + 16u * c16, nbias + 16 * c16);
                        uint32_t packed[8];
#pragma unroll
                        for (int k = 0; k < 8; ++k) packed[k] = relu_pack_bf16(v[h][2 * k], v[h][2 * k + 1]);
                        *reinterpret_cast<uint4 *>(next + tc_off(gtid, 16 * c16, 64)) =
                            make_uint4(packed[0], packed[1], packed[2], packed[3]);
                        *reinterpret_cast<uint4 *>(next + tc_off(gtid, 16 * c16 + 8, 64)) =
                            make_uint4(packed[4], packed[5], packed[6], packed[7]);
                    }
                }
                tc_wait_st();
            } else {
                float v[16];
                tc_ld16(tmem + lane_base, v);
                tc_wait_ld();
                if (row < n) out[row] = make_float4(v[0], v[1], v[2], 0.0f);
            }
            fence_async_smem();
            tc_fence_before();
            group_sync(group);
            tc_fence_after();
            if (*gfail) break;
        }
        if (*gfail) break;
    }
    // ---- teardown: every MMA has been waited for (a group that gave up
    // waited once more); free the TMEM
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*tmem_slot), "r"(kTcTmemCols)
                     : "memory");
}

// One Adam step on every parameter; S->step already counts it (advanced by
// the k_cache_fwd_bwd launch before).  Thread 0 also hands the batch's mean
// loss to loss_out and clears it for the next batch.
__global__ void k_cache_adam(CacheState *S, float *loss_out) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        if (loss_out) *loss_out = S->loss;
        S->loss = 0.0f;
    }
    if (i >= kParams) return;
    const uint32_t t = S->step;
    const float g = S->grads[i];
    const float m = S->beta1 * S->m[i] + (1.0f - S->beta1) * g;
    const float v = S->beta2 * S->v[i] + (1.0f - S->beta2) * g * g;
    S->m[i] = m;
    S->v[i] = v;
    const float mh = m / (1.0f - powf(S->beta1, (float)t));
    const float vh = v / (1.0f - powf(S->beta2, (float)t));
    const float p = S->params[i] - S->lr * mh / (sqrtf(vh) + S->eps);
    S->params[i] = p;
    S->wbf[i] = __float2bfloat16(p);
    S->grads[i] = 0.0f;
}

__global__ void k_cache_refresh_bf16(CacheState *S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kParams) S->wbf[i] = __float2bfloat16(S->params[i]);
}

// Launch with programmatic stream serialization (see pdl_enter).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned threads, size_t smem, cudaStream_t st,
                       Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

int set_smem(rt_context *ctx) {
    RT_CUDA_CTX(ctx, cudaFuncSetAttribute(k_cache_query_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
    RT_CUDA_CTX(ctx, cudaFuncSetAttribute(k_cache_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem));
    return RT_OK;
}

int launch_fwd_bwd(rt_context *ctx, cudaStream_t st, CacheState *S, const rt_cache_input *in, const float *tg,
                   uint32_t n, uint32_t bump_step) {
    const uint32_t tiles = (n + kTrainRows - 1) / kTrainRows;
    uint32_t grid = (uint32_t)ctx->sm_count;
    if (grid > tiles) grid = tiles;
    if (grid == 0) return RT_OK;
    RT_CUDA_CTX(ctx, launch_pdl(k_cache_fwd_bwd, grid, kTrainThreads, kTrainSmem, st, S, in,
                                reinterpret_cast<const float4 *>(tg), n, 1.0f / (3.0f * (float)n),
                                static_cast<const uint32_t *>(nullptr), 0u, bump_step));
    return RT_OK;
}

// He-uniform initial weights of the padded layout, host side (PCG32).
std::vector<float> initial_params(uint32_t seed) {
    std::vector<float> p(kParams, 0.0f);
    uint64_t state = 0, inc = ((uint64_t)seed << 1u) | 1u;
    auto next = [&]() {
        uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u), rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    };
    next();
    state += 0x853c49e6748fea9bull;
    next();
    const int used_in[kLayers] = {RT_CACHE_INPUTS, 64, 64, 64, 64, 64};
    const int used_out[kLayers] = {64, 64, 64, 64, 64, RT_CACHE_OUTPUTS};
    for (int l = 0; l < kLayers; ++l) {
        const float s = std::sqrt(6.0f / (float)used_in[l]);
        for (int o = 0; o < used_out[l]; ++o)
            for (int i = 0; i < used_in[l]; ++i) {
                float u = (float)(next() >> 8) * (1.0f / 16777216.0f);
                p[w_off(l) + o * in_dim(l) + i] = (2.0f * u - 1.0f) * s;
            }
    }
    return p;
}

}  // namespace
}  // namespace rtc

using namespace rtc;

extern "C" rt_status rt_cache_bytes(uint64_t *bytes) {
    if (!bytes) return RT_ERR_INVALID_ARG;
    *bytes = align_up(sizeof(CacheState), 256);
    return RT_OK;
}

extern "C" uint32_t rt_cache_param_count(void) { return (uint32_t)kParams; }

extern "C" rt_status rt_cache_init(rt_context *ctx, rt_stream stream, void *cache, const rt_cache_config *cfg) {
    if (!ctx || !cache || !cfg) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_init: null argument");
    if (reinterpret_cast<uintptr_t>(cache) & 255u) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_init: cache must be 256-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = set_smem(ctx);
    if (rc) return rc;
    std::vector<uint8_t> h(sizeof(CacheState), 0);
    CacheState *hs = reinterpret_cast<CacheState *>(h.data());
    std::vector<float> p = initial_params(cfg->seed);
    std::memcpy(hs->params, p.data(), sizeof(float) * kParams);
    for (int i = 0; i < kParams; ++i) {
        __nv_bfloat16 b = __float2bfloat16(p[i]);
        hs->wbf[i] = b;
    }
    for (int a = 0; a < 3; ++a) { hs->lo[a] = cfg->scene_lo[a]; hs->hi[a] = cfg->scene_hi[a]; }
    hs->lr = cfg->lr;
    hs->beta1 = cfg->beta1;
    hs->beta2 = cfg->beta2;
    hs->eps = cfg->eps;
    RT_CUDA_CTX(ctx, cudaMemcpyAsync(cache, h.data(), h.size(), cudaMemcpyHostToDevice, st));
    RT_CUDA_CTX(ctx, cudaStreamSynchronize(st));
    return RT_OK;
}

extern "C" rt_status rt_cache_query(rt_context *ctx, rt_stream stream, const void *cache, const rt_cache_input *in,
                                    float *out, uint32_t n) {
    if (!ctx || !cache || (n && (!in || !out))) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_query: null argument");
    if (reinterpret_cast<uintptr_t>(cache) & 255u) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_query: cache must be 256-byte aligned");
    if (n == 0) return RT_OK;
    int rc = set_smem(ctx);
    if (rc) return rc;
    const uint32_t groups = (n + kQueryRows * kTcGroups - 1) / (kQueryRows * kTcGroups);
    uint32_t grid = (uint32_t)ctx->sm_count;
    if (grid > groups) grid = groups;
    k_cache_query_tc<<<grid, kTcThreads, kTcSmem, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const CacheState *>(cache), in, reinterpret_cast<float4 *>(out), n, nullptr, ctx->d_err);
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}

extern "C" rt_status rt_cache_train(rt_context *ctx, rt_stream stream, void *cache, const rt_cache_input *in,
                                    const float *targets, uint32_t n, uint32_t batch, float *loss_out) {
    if (!ctx || !cache || (n && (!in || !targets))) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_train: null argument");
    if (reinterpret_cast<uintptr_t>(cache) & 255u) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_train: cache must be 256-byte aligned");
    if (batch == 0 || batch % 64u) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_train: batch must be a positive multiple of 64");
    int rc = set_smem(ctx);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CacheState *S = static_cast<CacheState *>(cache);
    for (uint32_t b = 0; b < n; b += batch) {
        const uint32_t m = (n - b) < batch ? (n - b) : batch;
        rc = launch_fwd_bwd(ctx, st, S, in + b, targets + 4u * (size_t)b, m, 1u);
        if (rc) return rc;
        RT_CUDA_CTX(ctx, launch_pdl(k_cache_adam, (kParams + 255) / 256, 256, 0, st, S, loss_out));
    }
    return RT_OK;
}

extern "C" rt_status rt_cache_gradient(rt_context *ctx, rt_stream stream, void *cache, const rt_cache_input *in,
                                       const float *targets, uint32_t n, float *grad_out) {
    if (!ctx || !cache || !grad_out || (n && (!in || !targets)))
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_gradient: null argument");
    if (reinterpret_cast<uintptr_t>(cache) & 255u) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_gradient: cache must be 256-byte aligned");
    int rc = set_smem(ctx);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CacheState *S = static_cast<CacheState *>(cache);
    RT_CUDA_CTX(ctx, cudaMemsetAsync(S->grads, 0, sizeof(float) * kParams, st));
    rc = launch_fwd_bwd(ctx, st, S, in, targets, n, 0u);
    if (rc) return rc;
    RT_CUDA_CTX(ctx, cudaMemcpyAsync(grad_out, S->grads, sizeof(float) * kParams, cudaMemcpyDeviceToDevice, st));
    RT_CUDA_CTX(ctx, cudaMemsetAsync(S->grads, 0, sizeof(float) * kParams, st));
    RT_CUDA_CTX(ctx, cudaMemsetAsync(&S->loss, 0, sizeof(float), st));
    return RT_OK;
}

extern "C" rt_status rt_cache_get_params(rt_context *ctx, rt_stream stream, const void *cache, float *params) {
    if (!ctx || !cache || !params) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_get_params: null argument");
    const CacheState *S = static_cast<const CacheState *>(cache);
    RT_CUDA_CTX(ctx, cudaMemcpyAsync(params, S->params, sizeof(float) * kParams, cudaMemcpyDeviceToDevice,
                                     static_cast<cudaStream_t>(stream)));
    return RT_OK;
}

extern "C" rt_status rt_cache_set_params(rt_context *ctx, rt_stream stream, void *cache, const float *params) {
    if (!ctx || !cache || !params) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_set_params: null argument");
    if (reinterpret_cast<uintptr_t>(cache) & 255u) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_set_params: cache must be 256-byte aligned");
    CacheState *S = static_cast<CacheState *>(cache);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    RT_CUDA_CTX(ctx, cudaMemcpyAsync(S->params, params, sizeof(float) * kParams, cudaMemcpyDeviceToDevice, st));
    k_cache_refresh_bf16<<<(kParams + 255) / 256, 256, 0, st>>>(S);
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}

// ---------------------------------------------------------------------------
// Checkpoints
// ---------------------------------------------------------------------------

namespace {

struct CheckpointHeader {
    char magic[4];         // "RTMC"
    uint32_t version;      // 1
    uint32_t params;       // kParams
    uint32_t reserved0;
    uint64_t state_bytes;  // sizeof(CacheState)
    uint64_t checksum;     // FNV-1a 64 of the state bytes
    uint8_t reserved[32];
};
static_assert(sizeof(CheckpointHeader) == 64, "checkpoint header");

uint64_t fnv1a64(const uint8_t *p, size_t n) {
    uint64_t h = 0xcbf29ce484222325ull;
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

}  // namespace

extern "C" rt_status rt_cache_save(rt_context *ctx, rt_stream stream, const void *cache, const char *path) {
    if (!ctx || !cache || !path) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_save: null argument");
    std::vector<uint8_t> state(sizeof(CacheState));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    RT_CUDA_CTX(ctx, cudaMemcpyAsync(state.data(), cache, state.size(), cudaMemcpyDeviceToHost, st));
    RT_CUDA_CTX(ctx, cudaStreamSynchronize(st));
    CheckpointHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, "RTMC", 4);
    h.version = 1u;
    h.params = (uint32_t)kParams;
    h.state_bytes = state.size();
    h.checksum = fnv1a64(state.data(), state.size());
    const std::string tmp = std::string(path) + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_save: cannot open the file for writing");
    bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 && std::fwrite(state.data(), 1, state.size(), f) == state.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_save: write failed");
    }
    return RT_OK;
}

extern "C" rt_status rt_cache_load(rt_context *ctx, rt_stream stream, void *cache, const char *path) {
    if (!ctx || !cache || !path) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_load: null argument");
    FILE *f = std::fopen(path, "rb");
    if (!f) return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_load: cannot open the file");
    CheckpointHeader h;
    std::vector<uint8_t> state(sizeof(CacheState));
    const bool got = std::fread(&h, sizeof(h), 1, f) == 1 &&
                     std::memcmp(h.magic, "RTMC", 4) == 0 && h.version == 1u && h.params == (uint32_t)kParams &&
                     h.state_bytes == state.size() && std::fread(state.data(), 1, state.size(), f) == state.size();
    const bool at_end = got && std::fgetc(f) == EOF;
    std::fclose(f);
    if (!got || !at_end)
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_load: not a cache checkpoint of this network");
    if (fnv1a64(state.data(), state.size()) != h.checksum)
        return set_error(ctx, RT_ERR_INVALID_ARG, "rt_cache_load: checksum mismatch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    RT_CUDA_CTX(ctx, cudaMemcpyAsync(cache, state.data(), state.size(), cudaMemcpyHostToDevice, st));
    RT_CUDA_CTX(ctx, cudaStreamSynchronize(st));
    return RT_OK;
}

// ---------------------------------------------------------------------------
// Device-count launchers for the path tracer's learned form (no host reads,
// no allocation): the number of query / training rows is produced on the
// device by the shading kernels.
// ---------------------------------------------------------------------------
namespace rtc {

int cache_query_dev(rt_context *ctx, cudaStream_t st, const void *cache, const rt_cache_input *in, float *out,
                    const uint32_t *n_dev, uint32_t max_n) {
    if (max_n == 0) return RT_OK;
    int rc = set_smem(ctx);
    if (rc) return rc;
    const uint32_t groups = (max_n + kQueryRows * kTcGroups - 1) / (kQueryRows * kTcGroups);
    uint32_t grid = (uint32_t)ctx->sm_count;
    if (grid > groups) grid = groups;
    k_cache_query_tc<<<grid, kTcThreads, kTcSmem, st>>>(static_cast<const CacheState *>(cache), in,
                                                 reinterpret_cast<float4 *>(out), max_n, n_dev, ctx->d_err);
    RT_CUDA_CTX(ctx, cudaGetLastError());
    return RT_OK;
}

// Adam steps over the first *n_dev samples in batches of `batch` (at most
// max_n samples in total).
int cache_train_dev(rt_context *ctx, cudaStream_t st, void *cache, const rt_cache_input *in, const float *targets,
                    const uint32_t *n_dev, uint32_t max_n, uint32_t batch) {
    if (max_n == 0 || batch == 0) return RT_OK;
    int rc = set_smem(ctx);
    if (rc) return rc;
    CacheState *S = static_cast<CacheState *>(cache);
    for (uint32_t b = 0; b < max_n; b += batch) {
        const uint32_t m = (max_n - b) < batch ? (max_n - b) : batch;
        const uint32_t tiles = (m + kTrainRows - 1) / kTrainRows;
        uint32_t grid = (uint32_t)ctx->sm_count;
        if (grid > tiles) grid = tiles;
        RT_CUDA_CTX(ctx, launch_pdl(k_cache_fwd_bwd, grid, kTrainThreads, kTrainSmem, st, S, in,
                                    reinterpret_cast<const float4 *>(targets), m, 0.0f, n_dev, b, 1u));
        RT_CUDA_CTX(ctx, launch_pdl(k_cache_adam, (kParams + 255) / 256, 256, 0, st, S,
                                    static_cast<float *>(nullptr)));
    }
    return RT_OK;
}

}  // namespace rtc
