// nbg_mlp.cuh -- the learned monopole correction's MLP on BF16 tensor cores.
//
// Network: 16 -> 64 -> 64 -> 3, GELU (tanh form, Hendrycks & Gimpel 2016)
// after the two hidden layers, BF16 weights and activations, FP32 accumulate.
// A warp evaluates 32 samples at once with mma.sync.m16n8k16 (two 16-row
// tiles): a lane stages its sample's 16 features, the accumulator fragments
// of one layer are re-packed in registers as the A fragments of the next
// (the m16n8 C layout and the m16n8k16 A layout share rows and columns), so
// activations never leave registers between layers.
//
// Parameters (FP32 master copy, k-major): W1[16][64], b1[64], W2[64][64],
// b2[64], W3[64][3], b3[3].
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace nbg {
namespace mlp {

constexpr int kIn = 16, kH = 64, kOut = 3;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kIn * kH;   // 1024
constexpr int kOffW2 = kOffB1 + kH;         // 1088
constexpr int kOffB2 = kOffW2 + kH * kH;    // 5184
constexpr int kOffW3 = kOffB2 + kH;         // 5248
constexpr int kOffB3 = kOffW3 + kH * kOut;  // 5440
constexpr int kParams = kOffB3 + kOut;      // 5443

// Fragment-ordered BF16 weights: one uint2 (the two B registers) per lane per
// 16x8 tile.  Tiles: W1 (kt 0, nt 0..7), W2 (kt 0..3, nt 0..7),
// W3 (kt 0..3, nt 0, columns >= 3 zero), W3^T (kt 0, nt 0..7; rows >= 3 zero),
// W2^T (kt 0..3, nt 0..7).  The transposes serve the backward pass.
constexpr int kTileW1 = 0;
constexpr int kTileW2 = 8;
constexpr int kTileW3 = 40;
constexpr int kTileW3T = 44;
constexpr int kTileW2T = 52;
constexpr int kTiles = 84;
constexpr int kFragWords = kTiles * 32;  // uint2 entries
// biases, FP32, padded: b1[64], b2[64], b3[8]
constexpr int kBias = 136;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint2 b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))).
__device__ __forceinline__ float tanh_mufu(float x) {
    float r;
    asm("tanh.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
constexpr float kGeluC = 0.7978845608028654f;  // sqrt(2/pi)
constexpr float kGeluA = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
    const float u = kGeluC * fmaf(kGeluA * x, x * x, x);
    return 0.5f * x * (1.f + tanh_mufu(u));
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float u = kGeluC * fmaf(kGeluA * x, x * x, x);
    const float t = tanh_mufu(u);
    const float du = kGeluC * fmaf(3.f * kGeluA * x, x, 1.f);
    return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * du;
}

// A fragments of the 32 x 16 input block staged row-per-sample in shared
// memory as BF16 (8 words per row).
__device__ __forceinline__ void load_input_frags(const uint32_t* xs, int lane, uint32_t a[2][4]) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int r0 = 16 * m + g, r1 = r0 + 8;
        a[m][0] = xs[r0 * 8 + t];
        a[m][1] = xs[r1 * 8 + t];
        a[m][2] = xs[r0 * 8 + 4 + t];
        a[m][3] = xs[r1 * 8 + 4 + t];
    }
}

// Hidden layer: acc[m][nt] = bias + A x W (K = 16 * KT), N = 64.
template <int KT>
__device__ __forceinline__ void layer64(const uint32_t (*a)[KT][4], const uint2* frag, int tile0,
                                        const float* bias, int lane, float acc[2][8][4]) {
    const int t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float b0 = bias[8 * nt + 2 * t], b1 = bias[8 * nt + 2 * t + 1];
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            acc[m][nt][0] = b0;
            acc[m][nt][1] = b1;
            acc[m][nt][2] = b0;
            acc[m][nt][3] = b1;
        }
    }
#pragma unroll
    for (int kt = 0; kt < KT; ++kt)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const uint2 b = frag[(tile0 + kt * 8 + nt) * 32 + lane];
#pragma unroll
            for (int m = 0; m < 2; ++m) mma_bf16(acc[m][nt], a[m][kt], b);
        }
}

// GELU on a 32 x 64 accumulator block, re-packed as the A fragments of the
// next layer (K = 64: 4 k-tiles).
__device__ __forceinline__ void gelu_to_frags(const float acc[2][8][4], uint32_t a[2][4][4]) {
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const float* lo = acc[m][2 * kt];
            const float* hi = acc[m][2 * kt + 1];
            a[m][kt][0] = pack_bf16(gelu(lo[0]), gelu(lo[1]));
            a[m][kt][1] = pack_bf16(gelu(lo[2]), gelu(lo[3]));
            a[m][kt][2] = pack_bf16(gelu(hi[0]), gelu(hi[1]));
            a[m][kt][3] = pack_bf16(gelu(hi[2]), gelu(hi[3]));
        }
}

// Output layer: out[m][4] = b3 + A x W3 (columns 0..2 meaningful).
__device__ __forceinline__ void layer_out(const uint32_t a[2][4][4], const uint2* frag,
                                          const float* bias, int lane, float out[2][4]) {
    const int t = lane & 3;
    const float b0 = bias[128 + 2 * t], b1 = bias[128 + 2 * t + 1];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        out[m][0] = b0;
        out[m][1] = b1;
        out[m][2] = b0;
        out[m][3] = b1;
    }
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        const uint2 b = frag[(kTileW3 + kt) * 32 + lane];
#pragma unroll
        for (int m = 0; m < 2; ++m) mma_bf16(out[m], a[m][kt], b);
    }
}

// Full inference for the warp: each lane supplies one sample's features and
// receives that sample's 3 outputs.  xs: 32 x 8 words of per-warp staging,
// os: 32 x 4 floats of per-warp staging (both shared memory).
__device__ __forceinline__ void infer_warp(const float feat[kIn], float g[3], const uint2* frag,
                                           const float* bias, uint32_t* xs, float* os, int lane) {
#pragma unroll
    for (int k = 0; k < 8; ++k) xs[lane * 8 + k] = pack_bf16(feat[2 * k], feat[2 * k + 1]);
    __syncwarp();
    uint32_t a0[2][1][4];
    {
        uint32_t tmp[2][4];
        load_input_frags(xs, lane, tmp);
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int q = 0; q < 4; ++q) a0[m][0][q] = tmp[m][q];
    }
    float acc[2][8][4];
    uint32_t a1[2][4][4];
    layer64<1>(a0, frag, kTileW1, bias, lane, acc);
    gelu_to_frags(acc, a1);
    layer64<4>(a1, frag, kTileW2, bias + 64, lane, acc);
    gelu_to_frags(acc, a1);
    float out[2][4];
    layer_out(a1, frag, bias, lane, out);
    // route outputs: sample 16m + g (+8) sits in lanes 4g (+1) of tile m
    const int gq = lane >> 2, t = lane & 3;
    if (t < 2) {
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            const int s0 = 16 * m + gq, s1 = s0 + 8;
            os[s0 * 4 + 2 * t] = out[m][0];
            os[s1 * 4 + 2 * t] = out[m][2];
            if (t == 0) {
                os[s0 * 4 + 1] = out[m][1];
                os[s1 * 4 + 1] = out[m][3];
            }
        }
    }
    __syncwarp();
    g[0] = os[lane * 4 + 0];
    g[1] = os[lane * 4 + 1];
    g[2] = os[lane * 4 + 2];
    __syncwarp();
}

}  // namespace mlp
}  // namespace nbg
