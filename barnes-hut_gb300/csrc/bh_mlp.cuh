// The acceptance network: 8 -> 64 -> 64 -> 1, ReLU, BF16 weights with FP32
// accumulation, predicting log10 of the relative force error of accepting a
// node unopened for a group of bodies.  No reference counterpart.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>
#include <cstring>

namespace bh {

constexpr int kFeat = 8;
constexpr int kHid = 64;
// Parameter layout (float32 master copy): W1[64][8] b1[64] W2[64][64] b2[64] W3[64] b3
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kHid * kFeat;
constexpr int kOffW2 = kOffB1 + kHid;
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;
constexpr int kOffB3 = kOffW3 + kHid;
constexpr int kParams = kOffB3 + 1;  // 4801

// Round to bfloat16 (nearest even) and back: the value a BF16 weight or
// activation carries into the FP32 accumulation.
__host__ __device__ inline float bf16r(float x)
{
#ifdef __CUDA_ARCH__
    return __bfloat162float(__float2bfloat16_rn(x));
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;  // inf / nan unchanged
    const uint32_t lsb = (u >> 16) & 1u;
    u += 0x7fffu + lsb;
    u &= 0xffff0000u;
    float r;
    memcpy(&r, &u, 4);
    return r;
#endif
}

// Feature scaling of a trained model: standardised input z = (f - mean)/std,
// accepted range [lo, hi] of z per feature (the training set's extent), and
// the label's scale: log10 error = y * lstd + lmean.
struct MlpScale {
    float mean[kFeat];
    float inv_std[kFeat];
    float lo[kFeat];
    float hi[kFeat];
    float lmean;
    float lstd;
};

constexpr int kScaleFloats = (int)(sizeof(MlpScale) / sizeof(float));  // 34

// A trained model laid out for the traversal's fused inference: the weights
// as mma.sync m16n8k16 B fragments (BF16 pairs, one per lane), biases and the
// last layer in FP32, the feature scaling and the acceptance threshold.
struct MlpDev {
    uint32_t w1f[8][32];    // layer 1: n-tile j, lane -> {W1[8j+g][2t], W1[8j+g][2t+1]}
    uint2 w2f[8][4][32];    // layer 2: n-tile j, k-tile kk, lane -> two pairs
    float b1[kHid];
    float b2[kHid];
    float w3[kHid];         // BF16-rounded
    float b3;
    MlpScale sc;
    float log_thresh;       // accept when the predicted log10 error is below
    float theta_max2;       // candidates: side^2 < theta_max^2 d_min^2
};

__device__ inline uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat16 a = __float2bfloat16_rn(lo), b = __float2bfloat16_rn(hi);
    return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// D = A B + C for one 16x8x16 tile, BF16 inputs, FP32 accumulation.
__device__ inline void mma_bf16_16816(float& c0, float& c1, float& c2, float& c3, uint32_t a0, uint32_t a1,
                                      uint32_t a2, uint32_t a3, uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c0), "+f"(c1), "+f"(c2), "+f"(c3)
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Warp-wide inference on standardised feature rows F[r][0..7] (shared
// memory, row stride 9), r < rows: lane r receives row r's network output
// (standardised log10 error).  All 32 lanes must call it with the same rows.  Two 16-row tiles; layer 1 is
// 8 mma (K = 8 padded to 16), layer 2 is 32 mma; the layer-1 accumulator
// fragments are reused in registers as layer-2 A fragments; layer 3 is a
// per-thread dot product reduced over the four lanes of a row group.
__device__ inline float mlp_predict_warp(const MlpDev* __restrict__ M, const float (*F)[9], int lane, int rows = 32)
{
    const int g = lane >> 2, t = lane & 3;
    float out[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    const int ntiles = rows > 16 ? 2 : 1;  // warp-uniform: skip the second tile when unused
#pragma unroll 1
    for (int mt = 0; mt < ntiles; ++mt) {
        const int r0 = 16 * mt + g, r1 = r0 + 8;
        const uint32_t a0 = pack_bf16(F[r0][2 * t], F[r0][2 * t + 1]);
        const uint32_t a1 = pack_bf16(F[r1][2 * t], F[r1][2 * t + 1]);
        uint32_t A2[4][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            float c0 = M->b1[8 * j + 2 * t], c1 = M->b1[8 * j + 2 * t + 1], c2 = c0, c3 = c1;
            mma_bf16_16816(c0, c1, c2, c3, a0, a1, 0u, 0u, __ldg(&M->w1f[j][lane]), 0u);
            const uint32_t lo = pack_bf16(fmaxf(c0, 0.f), fmaxf(c1, 0.f));
            const uint32_t hi = pack_bf16(fmaxf(c2, 0.f), fmaxf(c3, 0.f));
            A2[j >> 1][(j & 1) * 2] = lo;
            A2[j >> 1][(j & 1) * 2 + 1] = hi;
        }
        float pg = 0.f, pg8 = 0.f;
#pragma unroll 2
        for (int j = 0; j < 8; ++j) {
            float c0 = M->b2[8 * j + 2 * t], c1 = M->b2[8 * j + 2 * t + 1], c2 = c0, c3 = c1;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const uint2 bb = __ldg(&M->w2f[j][kk][lane]);
                mma_bf16_16816(c0, c1, c2, c3, A2[kk][0], A2[kk][1], A2[kk][2], A2[kk][3], bb.x, bb.y);
            }
            const float w0 = M->w3[8 * j + 2 * t], w1 = M->w3[8 * j + 2 * t + 1];
            pg = fmaf(w0, bf16r(fmaxf(c0, 0.f)), pg);
            pg = fmaf(w1, bf16r(fmaxf(c1, 0.f)), pg);
            pg8 = fmaf(w0, bf16r(fmaxf(c2, 0.f)), pg8);
            pg8 = fmaf(w1, bf16r(fmaxf(c3, 0.f)), pg8);
        }
        pg += __shfl_xor_sync(0xffffffffu, pg, 1);
        pg += __shfl_xor_sync(0xffffffffu, pg, 2);
        pg8 += __shfl_xor_sync(0xffffffffu, pg8, 1);
        pg8 += __shfl_xor_sync(0xffffffffu, pg8, 2);
        if (mt == 0) { out[0][0] = pg + M->b3; out[0][1] = pg8 + M->b3; }
        else { out[1][0] = pg + M->b3; out[1][1] = pg8 + M->b3; }
    }
    const int src = 4 * (lane & 7);
    const float v00 = __shfl_sync(0xffffffffu, out[0][0], src);
    const float v01 = __shfl_sync(0xffffffffu, out[0][1], src);
    const float v10 = __shfl_sync(0xffffffffu, out[1][0], src);
    const float v11 = __shfl_sync(0xffffffffu, out[1][1], src);
    const int mt = lane >> 4, h = (lane >> 3) & 1;
    return mt ? (h ? v11 : v10) : (h ? v01 : v00);
}

}  // namespace bh
