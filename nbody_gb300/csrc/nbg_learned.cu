// nbg_learned.cu -- learned correction of the Barnes-Hut monopole.
//
// No reference counterpart.  For an interaction between a body and a cell
// that the walk accepts at the loose ratio (lambda_l = 1/theta_l) but that
// the tight ratio (lambda_t, default 2 = 1/0.5) would open, a small MLP
// predicts the residual between the cell's exact subtree force and its
// monopole:
//     a_exact - a_mono = (m / s^2) * g(features),
// with s the cell's geometric radius (the reference's critical radius at
// ratio 1: half bounding-box diagonal + |box centre - mass centre|,
// nbody/nbody_space_heap.cpp:129-132) and 16 dimensionless features:
//     u = (x - c) / s (3)            body offset from the mass centre
//     Q_ab / (m s^2) (6)             second central mass moments
//     (bmax - bmin) / (2 s) (3)      box half extents (mass spread)
//     1 / |u| (1)
//     (c - box centre) / s (3)       mass-centre offset inside the box
// The network's three outputs are coefficients of the vectors u/|u|,
// Q u/|u| and the mass-centre offset (apply_head), so its correction turns
// with the cell.  The engine generates training samples from its own trees
// (exact subtree sums over contiguous leaf ranges), trains the network with BF16
// tensor-core forward/backward kernels and Adam -- both in a fixed order,
// so equal seeds give equal samples and equal weights -- and applies it to
// the FP32 walk.  Inference (learned.walk):
//   1 (default): the default group walk records the band cells and
//     nbg_learned_tc.cu evaluates the band rows on tcgen05 tensor cores;
//   0: the warp-coherent walk in this file, with the network fused in as
//     mma.sync batches, per body (learned.group = 0: one MLP sample per
//     (body, cell) pair) or per warp (learned.group = 1: one sample per
//     (warp, cell) at the warp's centroid, shared by its 32 bodies).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "nbg_learned.cuh"
#include "nbg_mlp.cuh"
#include "nbg_ptx.cuh"
#include "nbg_stats.cuh"
#include "nbg_tree.cuh"

namespace nbg {

namespace {

using namespace mlp;

// ---------------------------------------------------------------------------
// node moments and features
// ---------------------------------------------------------------------------
__global__ void moments_leaf_kernel(double* mom, size_t sz, int n) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        for (int q = 0; q < 6; ++q) mom[q * sz + n + p] = 0.0;
}

// Parallel-axis combination: Q = Q_l + Q_r + m_l d_l d_l^T + m_r d_r d_r^T,
// d = child centre - parent centre.  Order (xx, yy, zz, xy, xz, yz).
__global__ void moments_level_kernel(int first, int count, TreeState t, double* mom) {
    const size_t sz = t.size;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const size_t idx = (size_t)first + k;
        double q[6] = {0, 0, 0, 0, 0, 0};
        for (int side = 0; side < 2; ++side) {
            const size_t c = 2 * idx + side;
            const double mc = t.mass[c];
            const double dx = t.com[c] - t.com[idx];
            const double dy = t.com[sz + c] - t.com[sz + idx];
            const double dz = t.com[2 * sz + c] - t.com[2 * sz + idx];
            q[0] += mom[0 * sz + c] + mc * dx * dx;
            q[1] += mom[1 * sz + c] + mc * dy * dy;
            q[2] += mom[2 * sz + c] + mc * dz * dz;
            q[3] += mom[3 * sz + c] + mc * dx * dy;
            q[4] += mom[4 * sz + c] + mc * dx * dz;
            q[5] += mom[5 * sz + c] + mc * dy * dz;
        }
        for (int j = 0; j < 6; ++j) mom[j * sz + idx] = q[j];
    }
}

// feat[3 * idx + 0..2] = (Qxx, Qyy, Qzz, Qxy)/(m s^2), (Qxz, Qyz)/(m s^2), ex, ey,
//                        ez, ox, oy, oz
__global__ void features_kernel(TreeState t, const double* mom, double lambda) {
    const size_t sz = t.size;
    for (size_t idx = 1 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < sz;
         idx += (size_t)gridDim.x * blockDim.x) {
        const double m = t.mass[idx];
        const double s = sqrt(t.crit2[idx]) / lambda;
        float4 f0 = make_float4(0, 0, 0, 0), f1 = f0, f2 = f0;
        if (s > 0.0 && m > 0.0) {
            const double k = 1.0 / (m * s * s);
            double e[3], o[3];
            for (int d = 0; d < 3; ++d) {
                const double mn = t.bmin[d * sz + idx], mx = t.bmax[d * sz + idx];
                e[d] = (mx - mn) / (2.0 * s);
                o[d] = (t.com[d * sz + idx] - 0.5 * (mx + mn)) / s;
            }
            f0 = make_float4((float)(mom[0 * sz + idx] * k), (float)(mom[1 * sz + idx] * k),
                             (float)(mom[2 * sz + idx] * k), (float)(mom[3 * sz + idx] * k));
            f1 = make_float4((float)(mom[4 * sz + idx] * k), (float)(mom[5 * sz + idx] * k),
                             (float)e[0], (float)e[1]);
            f2 = make_float4((float)e[2], (float)o[0], (float)o[1], (float)o[2]);
        }
        t.feat[3 * idx + 0] = f0;
        t.feat[3 * idx + 1] = f1;
        t.feat[3 * idx + 2] = f2;
    }
}

// ---------------------------------------------------------------------------
// fragment-ordered BF16 weights from the FP32 master copy
// ---------------------------------------------------------------------------
__device__ __forceinline__ float wat(const float* w, int layer, int k, int n) {
    // layer 1: W1[k][n] (16x64); 2: W2 (64x64); 3: W3 (64x3, n<3);
    // 4: W3^T (k<3, 64 cols): W3[n][k]; 5: W2^T: W2[n][k]
    switch (layer) {
        case 1: return w[kOffW1 + k * kH + n];
        case 2: return w[kOffW2 + k * kH + n];
        case 3: return n < kOut ? w[kOffW3 + k * kOut + n] : 0.f;
        case 4: return k < kOut ? w[kOffW3 + n * kOut + k] : 0.f;
        default: return w[kOffW2 + n * kH + k];
    }
}

__global__ void make_frags_kernel(const float* __restrict__ w, uint2* __restrict__ frag,
                                  float* __restrict__ bias) {
    const int tile = blockIdx.x;  // 0 .. kTiles-1
    const int lane = threadIdx.x;
    int layer, kt, nt;
    if (tile < kTileW2) { layer = 1; kt = 0; nt = tile; }
    else if (tile < kTileW3) { layer = 2; kt = (tile - kTileW2) / 8; nt = (tile - kTileW2) % 8; }
    else if (tile < kTileW3T) { layer = 3; kt = tile - kTileW3; nt = 0; }
    else if (tile < kTileW2T) { layer = 4; kt = 0; nt = tile - kTileW3T; }
    else { layer = 5; kt = (tile - kTileW2T) / 8; nt = (tile - kTileW2T) % 8; }
    const int g = lane >> 2, t = lane & 3;
    const int k0 = 16 * kt + 2 * t, n = 8 * nt + g;
    uint2 v;
    v.x = pack_bf16(wat(w, layer, k0, n), wat(w, layer, k0 + 1, n));
    v.y = pack_bf16(wat(w, layer, k0 + 8, n), wat(w, layer, k0 + 9, n));
    frag[tile * 32 + lane] = v;
    if (tile == 0) {
        for (int i = lane; i < kBias; i += 32) {
            float b = 0.f;
            if (i < 64) b = w[kOffB1 + i];
            else if (i < 128) b = w[kOffB2 + i - 64];
            else if (i - 128 < kOut) b = w[kOffB3 + i - 128];
            bias[i] = b;
        }
    }
}

// ---------------------------------------------------------------------------
// training: forward + backward for a batch, gradients accumulated in FP32
// ---------------------------------------------------------------------------
constexpr int kTrainWarps = 4;

struct WarpStage {               // per-warp staging, BF16 pairs packed in u32
    uint32_t xs[32 * 8];         // X rows (sample-major) for the input fragments
    uint32_t xT[16 * 16];        // X^T  [16 features][32 samples]
    uint32_t a1T[64 * 16];       // A1^T [64][32]
    uint32_t a2T[64 * 16];       // A2^T [64][32]
    uint32_t d3T[8 * 16];        // dY^T [8][32]
    uint32_t d2T[64 * 16];       // dZ2^T [64][32]
    uint32_t d1T[64 * 16];       // dZ1^T [64][32]
};

// Each warp sums its samples' gradients into its own slice (wacc[warp]), so
// no two warps add to one word; the block adds the slices in warp order at
// the end.
struct TrainSmem {
    uint2 frag[kFragWords];
    float bias[kBias];
    float wacc[kTrainWarps][kParams + 5];
    double lsum[kTrainWarps];
    WarpStage ws[kTrainWarps];
};

__device__ __forceinline__ void store_T(uint32_t* T, int row, int col, float v) {
    // element (row, col) of a [rows][32] BF16 matrix stored as u32 pairs
    __nv_bfloat16* p = reinterpret_cast<__nv_bfloat16*>(T);
    p[row * 32 + col] = __float2bfloat16_rn(v);
}

// C-layout block [2 m][NT][4] (rows = samples) -> transposed BF16 [cols][32].
template <int NT>
__device__ __forceinline__ void stage_T(uint32_t* T, const float c[2][NT][4], int lane) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const int s0 = 16 * m + g, col = 8 * nt + 2 * t;
            store_T(T, col, s0, c[m][nt][0]);
            store_T(T, col + 1, s0, c[m][nt][1]);
            store_T(T, col, s0 + 8, c[m][nt][2]);
            store_T(T, col + 1, s0 + 8, c[m][nt][3]);
        }
}

// A fragment (16 rows from row0, 16 K-columns from k0) of a [rows][32] matrix.
__device__ __forceinline__ void frag_A_T(const uint32_t* T, int row0, int k0, int lane,
                                         uint32_t a[4]) {
    const int g = lane >> 2, t = lane & 3;
    a[0] = T[(row0 + g) * 16 + (k0 >> 1) + t];
    a[1] = T[(row0 + g + 8) * 16 + (k0 >> 1) + t];
    a[2] = T[(row0 + g) * 16 + (k0 >> 1) + 4 + t];
    a[3] = T[(row0 + g + 8) * 16 + (k0 >> 1) + 4 + t];
}

// B fragment (K = 16 samples from k0, N = 8 columns from n0) of a [cols][32] matrix.
__device__ __forceinline__ uint2 frag_B_T(const uint32_t* T, int n0, int k0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    uint2 b;
    b.x = T[(n0 + g) * 16 + (k0 >> 1) + t];
    b.y = T[(n0 + g) * 16 + (k0 >> 1) + 4 + t];
    return b;
}

// gacc[off + r * ld + c] += C-tile (16 x 8 at r0, c0); gacc is the warp's
// own slice and the lanes' words are distinct, so plain adds
__device__ __forceinline__ void acc_tile(float* gacc, int off, int ld, int r0, int c0, int cmax,
                                         const float c[4], int lane) {
    const int g = lane >> 2, t = lane & 3;
    const int cc = c0 + 2 * t;
    if (cc < cmax) {
        gacc[off + (r0 + g) * ld + cc] += c[0];
        gacc[off + (r0 + g + 8) * ld + cc] += c[2];
    }
    if (cc + 1 < cmax) {
        gacc[off + (r0 + g) * ld + cc + 1] += c[1];
        gacc[off + (r0 + g + 8) * ld + cc + 1] += c[3];
    }
}

// column sums over the 32 samples of a C-layout block -> gacc[off + col]
template <int NT>
__device__ __forceinline__ void acc_colsum(float* gacc, int off, int cmax, const float c[2][NT][4],
                                           int lane) {
    const int t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        float s0 = c[0][nt][0] + c[0][nt][2] + c[1][nt][0] + c[1][nt][2];
        float s1 = c[0][nt][1] + c[0][nt][3] + c[1][nt][1] + c[1][nt][3];
        for (int o = 4; o < 32; o <<= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        }
        if (lane < 4) {
            const int col = 8 * nt + 2 * t;
            if (col < cmax) gacc[off + col] += s0;
            if (col + 1 < cmax) gacc[off + col + 1] += s1;
        }
    }
}

__global__ void __launch_bounds__(kTrainWarps * 32)
train_kernel(const float* __restrict__ x, const float* __restrict__ tg, const int* __restrict__ order,
             size_t b0, size_t bsize, const uint2* __restrict__ frag_g,
             const float* __restrict__ bias_g, float* __restrict__ grad_part,
             double* __restrict__ loss_part, float wnorm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    for (int i = threadIdx.x; i < kFragWords; i += blockDim.x) S.frag[i] = frag_g[i];
    for (int i = threadIdx.x; i < kBias; i += blockDim.x) S.bias[i] = bias_g[i];
    for (int i = threadIdx.x; i < kTrainWarps * (kParams + 5); i += blockDim.x)
        (&S.wacc[0][0])[i] = 0.f;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    WarpStage& W = S.ws[warp];
    float* gacc = S.wacc[warp];  // this warp's gradient sums
    const float inv_b = 1.f / (float)bsize;
    double sq = 0.0;
    const size_t chunks = (bsize + 31) / 32;
    for (size_t ch = (size_t)blockIdx.x * kTrainWarps + warp; ch < chunks;
         ch += (size_t)gridDim.x * kTrainWarps) {
        // ---- stage inputs ----
        const size_t si = ch * 32 + lane;
        const bool live = si < bsize;
        const size_t src = live ? (size_t)order[b0 + si] : 0;
        float feat[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) feat[k] = live ? x[src * 16 + k] : 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) W.xs[lane * 8 + k] = pack_bf16(feat[2 * k], feat[2 * k + 1]);
#pragma unroll
        for (int k = 0; k < 16; ++k) store_T(W.xT, k, lane, feat[k]);
        __syncwarp();
        // ---- forward ----
        uint32_t a0[2][1][4];
        {
            uint32_t tmp[2][4];
            load_input_frags(W.xs, lane, tmp);
            for (int m = 0; m < 2; ++m)
                for (int q = 0; q < 4; ++q) a0[m][0][q] = tmp[m][q];
        }
        float z1[2][8][4], z2[2][8][4];
        uint32_t a1[2][4][4], a2[2][4][4];
        layer64<1>(a0, S.frag, kTileW1, S.bias, lane, z1);
        gelu_to_frags(z1, a1);
        {
            float act[2][8][4];
            for (int m = 0; m < 2; ++m)
                for (int nt = 0; nt < 8; ++nt)
                    for (int q = 0; q < 4; ++q) act[m][nt][q] = gelu(z1[m][nt][q]);
            stage_T<8>(W.a1T, act, lane);
        }
        layer64<4>(a1, S.frag, kTileW2, S.bias + 64, lane, z2);
        gelu_to_frags(z2, a2);
        {
            float act[2][8][4];
            for (int m = 0; m < 2; ++m)
                for (int nt = 0; nt < 8; ++nt)
                    for (int q = 0; q < 4; ++q) act[m][nt][q] = gelu(z2[m][nt][q]);
            stage_T<8>(W.a2T, act, lane);
        }
        float out[2][4];
        layer_out(a2, S.frag, S.bias, lane, out);
        // ---- loss gradient through the head, rows = samples ----
        // g = sum_i c_i b_i, loss = |g - T|^2, dL/dc_i = 2 (g - T) . b_i / B.
        // Lane (g, t) of a row quad holds output columns 2t, 2t+1 of rows g
        // and g + 8: c0, c1 on t = 0 and c2 on t = 1; every lane of the quad
        // gathers the three, evaluates the head and keeps its own columns.
        float d3[2][1][4];
        for (int m = 0; m < 2; ++m)
            for (int h = 0; h < 2; ++h) {  // h: row g or g + 8
                const size_t s = ch * 32 + 16 * m + g + 8 * h;
                const bool sl = s < bsize;
                const size_t srow = sl ? (size_t)order[b0 + s] : 0;
                float c[3];
                c[0] = __shfl_sync(0xffffffffu, out[m][2 * h], lane & ~3);
                c[1] = __shfl_sync(0xffffffffu, out[m][2 * h + 1], lane & ~3);
                c[2] = __shfl_sync(0xffffffffu, out[m][2 * h], (lane & ~3) | 1);
                float dc[4] = {0.f, 0.f, 0.f, 0.f};
                if (sl) {
                    float fe[16];
#pragma unroll
                    for (int k = 0; k < 16; ++k) fe[k] = x[srow * 16 + k];
                    float b[3][3], gp[3];
                    head_basis(fe, b);
                    apply_head(fe, c, gp);
                    float e[3];
#pragma unroll
                    for (int k = 0; k < 3; ++k) e[k] = gp[k] - tg[srow * 4 + k];
                    // weighted loss: the squared error in force units, (m / s^2)^2
                    // |g - T|^2, normalised to a mean weight of 1 (wnorm > 0)
                    const float ws = tg[srow * 4 + 3];
                    const float fac = wnorm > 0.f ? ws * ws * wnorm : 1.f;
                    if (t == 0)
                        sq += (double)fac * ((double)e[0] * e[0] + (double)e[1] * e[1] +
                                             (double)e[2] * e[2]);
#pragma unroll
                    for (int i = 0; i < 3; ++i)
                        dc[i] = 2.f * inv_b * fac *
                                fmaf(e[0], b[i][0], fmaf(e[1], b[i][1], e[2] * b[i][2]));
                }
                const int col = 2 * t;
                d3[m][0][2 * h] = col < kOut ? dc[col] : 0.f;
                d3[m][0][2 * h + 1] = col + 1 < kOut ? dc[col + 1] : 0.f;
            }
        stage_T<1>(W.d3T, d3, lane);
        __syncwarp();
        // ---- dA2 = dY W3^T ; dZ2 = dA2 * gelu'(Z2) ----
        uint32_t ad3[2][1][4];
        for (int m = 0; m < 2; ++m) {
            ad3[m][0][0] = pack_bf16(d3[m][0][0], d3[m][0][1]);
            ad3[m][0][1] = pack_bf16(d3[m][0][2], d3[m][0][3]);
            ad3[m][0][2] = 0u;
            ad3[m][0][3] = 0u;
        }
        float dz[2][8][4];
        for (int m = 0; m < 2; ++m)
            for (int nt = 0; nt < 8; ++nt)
                for (int q = 0; q < 4; ++q) dz[m][nt][q] = 0.f;
        for (int nt = 0; nt < 8; ++nt) {
            const uint2 b = S.frag[(kTileW3T + nt) * 32 + lane];
            for (int m = 0; m < 2; ++m) mma_bf16(dz[m][nt], ad3[m][0], b);
        }
        for (int m = 0; m < 2; ++m)
            for (int nt = 0; nt < 8; ++nt)
                for (int q = 0; q < 4; ++q) dz[m][nt][q] *= gelu_grad(z2[m][nt][q]);
        stage_T<8>(W.d2T, dz, lane);
        acc_colsum<8>(gacc, kOffB2, kH, dz, lane);
        acc_colsum<1>(gacc, kOffB3, kOut, d3, lane);
        // ---- dA1 = dZ2 W2^T ; dZ1 = dA1 * gelu'(Z1) ----
        uint32_t adz[2][4][4];
        for (int m = 0; m < 2; ++m)
            for (int kt = 0; kt < 4; ++kt) {
                adz[m][kt][0] = pack_bf16(dz[m][2 * kt][0], dz[m][2 * kt][1]);
                adz[m][kt][1] = pack_bf16(dz[m][2 * kt][2], dz[m][2 * kt][3]);
                adz[m][kt][2] = pack_bf16(dz[m][2 * kt + 1][0], dz[m][2 * kt + 1][1]);
                adz[m][kt][3] = pack_bf16(dz[m][2 * kt + 1][2], dz[m][2 * kt + 1][3]);
            }
        float d1[2][8][4];
        for (int m = 0; m < 2; ++m)
            for (int nt = 0; nt < 8; ++nt)
                for (int q = 0; q < 4; ++q) d1[m][nt][q] = 0.f;
        for (int kt = 0; kt < 4; ++kt)
            for (int nt = 0; nt < 8; ++nt) {
                const uint2 b = S.frag[(kTileW2T + kt * 8 + nt) * 32 + lane];
                for (int m = 0; m < 2; ++m) mma_bf16(d1[m][nt], adz[m][kt], b);
            }
        for (int m = 0; m < 2; ++m)
            for (int nt = 0; nt < 8; ++nt)
                for (int q = 0; q < 4; ++q) d1[m][nt][q] *= gelu_grad(z1[m][nt][q]);
        stage_T<8>(W.d1T, d1, lane);
        acc_colsum<8>(gacc, kOffB1, kH, d1, lane);
        __syncwarp();
        // ---- weight gradients: K = the 32 samples ----
        // dW3[h][c] = A2^T dY : M = 64 (4 tiles), N = 8, K = 32
        for (int mt = 0; mt < 4; ++mt) {
            float c[4] = {0, 0, 0, 0};
            for (int kt = 0; kt < 2; ++kt) {
                uint32_t a[4];
                frag_A_T(W.a2T, 16 * mt, 16 * kt, lane, a);
                mma_bf16(c, a, frag_B_T(W.d3T, 0, 16 * kt, lane));
            }
            acc_tile(gacc, kOffW3, kOut, 16 * mt, 0, kOut, c, lane);
        }
        // dW2[h][h'] = A1^T dZ2 : M = 64, N = 64, K = 32
        for (int mt = 0; mt < 4; ++mt)
            for (int nt = 0; nt < 8; ++nt) {
                float c[4] = {0, 0, 0, 0};
                for (int kt = 0; kt < 2; ++kt) {
                    uint32_t a[4];
                    frag_A_T(W.a1T, 16 * mt, 16 * kt, lane, a);
                    mma_bf16(c, a, frag_B_T(W.d2T, 8 * nt, 16 * kt, lane));
                }
                acc_tile(gacc, kOffW2, kH, 16 * mt, 8 * nt, kH, c, lane);
            }
        // dW1[f][h] = X^T dZ1 : M = 16, N = 64, K = 32
        for (int nt = 0; nt < 8; ++nt) {
            float c[4] = {0, 0, 0, 0};
            for (int kt = 0; kt < 2; ++kt) {
                uint32_t a[4];
                frag_A_T(W.xT, 0, 16 * kt, lane, a);
                mma_bf16(c, a, frag_B_T(W.d1T, 8 * nt, 16 * kt, lane));
            }
            acc_tile(gacc, kOffW1, kH, 0, 8 * nt, kH, c, lane);
        }
        __syncwarp();
    }
    // the block's loss and gradient: the warps' sums in warp order
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if (lane == 0) S.lsum[warp] = sq;
    __syncthreads();
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) {
        float v = S.wacc[0][i];
#pragma unroll
        for (int w = 1; w < kTrainWarps; ++w) v += S.wacc[w][i];
        grad_part[(size_t)blockIdx.x * kParams + i] = v;
    }
    if (threadIdx.x == 0) {
        double l = S.lsum[0];
        for (int w = 1; w < kTrainWarps; ++w) l += S.lsum[w];
        loss_part[blockIdx.x] = l;
    }
}

// grad = the pass's gradient (the blocks' partials in block order); the
// pass's loss is added to loss[0].
__global__ void grad_reduce_kernel(const float* __restrict__ grad_part, int blocks,
                                   float* __restrict__ grad, const double* __restrict__ loss_part,
                                   double* __restrict__ loss) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x) {
        float v = grad_part[i];
        for (int b = 1; b < blocks; ++b) v += grad_part[(size_t)b * kParams + i];
        grad[i] = v;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double l = 0.0;
        for (int b = 0; b < blocks; ++b) l += loss_part[b];
        loss[0] += l;
    }
}

__global__ void adam_kernel(float* w, float* grad, float* m1, float* m2, float lr, float b1,
                            float b2, float eps, float c1, float c2, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gr = grad[i];
        const float a = b1 * m1[i] + (1.f - b1) * gr;
        const float b = b2 * m2[i] + (1.f - b2) * gr * gr;
        m1[i] = a;
        m2[i] = b;
        w[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
        grad[i] = 0.f;
    }
}

// ---------------------------------------------------------------------------
// sample generation
// ---------------------------------------------------------------------------
__device__ __forceinline__ int next_down_i(int idx) { return (idx >> (__ffs(~idx) - 1)) + 1; }

// One thread per sampled leaf k (index in [n, 2n)): walk at the loose ratio
// and find every accepted internal node inside the band whose subtree holds
// at most 2^max_level_leaves_log2 bodies.  The first pass (WRITE false)
// counts them into counts[k]; the second writes leaf k's pairs, in walk
// order, from slot first[k] (the counts' exclusive prefix sum), those below
// cap.  So the sample store's order and content follow the sampled leaves'
// order, whatever the schedule.
template <bool WRITE>
__global__ void sample_pairs_kernel(const int* __restrict__ leaves, int nb, TreeState t, int n,
                                    float band2, int max_level_leaves_log2, int levels,
                                    int* __restrict__ pairs, unsigned* __restrict__ counts,
                                    const unsigned long long* __restrict__ first,
                                    unsigned long long cap) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nb) return;
    const int leaf = leaves[k];
    const float4 me = t.node4[leaf];
    int curr = 1;
    const int sz = (int)t.size;
    int steps = 0;
    unsigned found = 0;
    const unsigned long long slot0 = WRITE ? first[k] : 0ull;
    do {
        const float4 nd = t.node4[curr];
        const float dx = nd.x - me.x, dy = nd.y - me.y, dz = nd.z - me.z;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if (d2 > nd.w) {
            if (curr < n && d2 <= nd.w * band2) {
                const int lv = 31 - __clz(curr);
                if (levels - lv <= max_level_leaves_log2) {
                    if (WRITE) {
                        const unsigned long long slot = slot0 + found;
                        if (slot < cap) {
                            pairs[2 * slot] = leaf;
                            pairs[2 * slot + 1] = curr;
                        }
                    }
                    ++found;
                }
            }
            curr = next_down_i(curr);
        } else {
            curr = (2 * curr < sz) ? 2 * curr : next_down_i(curr);
        }
    } while (curr != 1 && ++steps <= sz);
    if (!WRITE) counts[k] = found;
}

// One warp per pair: exact subtree acceleration (FP64) minus the monopole,
// scaled by s^2 / m; features from the FP32 records the walk uses.
__global__ void sample_targets_kernel(const int* __restrict__ pairs, size_t npairs,
                                      const double* __restrict__ y, const double* __restrict__ mass,
                                      TreeState t, int n, int levels, double lambda, double eps2,
                                      float* __restrict__ xo, float* __restrict__ to,
                                      int* __restrict__ meta) {
    const int lane = threadIdx.x & 31;
    const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= npairs) return;
    const int leaf = pairs[2 * w], node = pairs[2 * w + 1];
    const size_t sz = t.size;
    const int b = t.body_n[leaf];
    const double bx = y[b], by = y[n + b], bz = y[2 * n + b];
    const int lv = 31 - __clz(node);
    const int span = 1 << (levels - lv);
    const int first = node << (levels - lv);
    double ex = 0.0, ey = 0.0, ez = 0.0;
    for (int k = lane; k < span; k += 32) {
        const int j = t.body_n[first + k];
        const double dx = y[j] - bx, dy = y[n + j] - by, dz = y[2 * n + j] - bz;
        const double r2 = dx * dx + dy * dy + dz * dz + eps2;
        const double s = mass[j] / (r2 * sqrt(r2));
        ex += dx * s;
        ey += dy * s;
        ez += dz * s;
    }
    for (int o = 16; o > 0; o >>= 1) {
        ex += __shfl_xor_sync(0xffffffffu, ex, o);
        ey += __shfl_xor_sync(0xffffffffu, ey, o);
        ez += __shfl_xor_sync(0xffffffffu, ez, o);
    }
    if (lane != 0) return;
    const double m = t.mass[node];
    const double cx = t.com[node] - bx, cy = t.com[sz + node] - by, cz = t.com[2 * sz + node] - bz;
    const double r2 = cx * cx + cy * cy + cz * cz + eps2;
    const double sm = m / (r2 * sqrt(r2));
    const double s = sqrt(t.crit2[node]) / lambda;
    const double scale = s * s / m;
    to[4 * w + 0] = (float)((ex - cx * sm) * scale);
    to[4 * w + 1] = (float)((ey - cy * sm) * scale);
    to[4 * w + 2] = (float)((ez - cz * sm) * scale);
    to[4 * w + 3] = (float)(m / (s * s));  // force scale of the cell (training weight)
    const float4 nd = t.node4[node];
    const float4 me = t.node4[leaf];
    float feat[16];
    make_features(nd.x - me.x, nd.y - me.y, nd.z - me.z, (float)(1.0 / s), t.feat[3 * node],
                  t.feat[3 * node + 1], t.feat[3 * node + 2], feat);
    for (int k = 0; k < 16; ++k) xo[16 * w + k] = feat[k];
    meta[2 * w] = b;
    meta[2 * w + 1] = node;
}

// ---------------------------------------------------------------------------
// the learned walk
// ---------------------------------------------------------------------------
constexpr int kWalkThreads = 128;
constexpr int kWalkWarps = kWalkThreads / 32;

struct WalkSmem {
    uint2 frag[kFragWords];
    float bias[kBias];
    uint32_t xs[kWalkWarps][32 * 8];
    float os[kWalkWarps][32 * 4];
    int queue[kWalkWarps][32];
};

template <bool GROUP>
__global__ void __launch_bounds__(kWalkThreads)
learned_walk_kernel(const double* __restrict__ y, double* __restrict__ f, int n, float eps2,
                    float band2, float inv_lambda, TreeState t, const uint2* __restrict__ frag_g,
                    const float* __restrict__ bias_g, unsigned* err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WalkSmem& S = *reinterpret_cast<WalkSmem*>(smem_raw);
    for (int i = threadIdx.x; i < kFragWords; i += blockDim.x) S.frag[i] = frag_g[i];
    for (int i = threadIdx.x; i < kBias; i += blockDim.x) S.bias[i] = bias_g[i];
    __syncthreads();
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if ((tid & ~31) >= n) return;
    const bool live = tid < n;
    const int leaf = n + (live ? tid : n - 1);
    const float4 me = __ldg(&t.node4[leaf]);
    const float xi = me.x, yi = me.y, zi = me.z;
    // warp centroid (group mode)
    float cx = xi, cy = yi, cz = zi;
    if (GROUP) {
        for (int o = 16; o > 0; o >>= 1) {
            cx += __shfl_xor_sync(0xffffffffu, cx, o);
            cy += __shfl_xor_sync(0xffffffffu, cy, o);
            cz += __shfl_xor_sync(0xffffffffu, cz, o);
        }
        cx *= (1.f / 32.f);
        cy *= (1.f / 32.f);
        cz *= (1.f / 32.f);
    }
    float ax = 0.f, ay = 0.f, az = 0.f;
    float gx = 0.f, gy = 0.f, gz = 0.f;  // group correction (same on every lane)
    int qn = 0;
    unsigned visits = 0, inter = 0, rows = 0;
    int curr = 1;
    const int sz = (int)t.size;

    auto flush_group = [&]() {
        // lane l evaluates queued cell l at the centroid
        float feat[16];
        float corr[3] = {0.f, 0.f, 0.f};
        const bool have = lane < qn;
        const int node = have ? S.queue[warp][lane] : 1;
        const float4 nd = __ldg(&t.node4[node]);
        const float s = sqrtf(nd.w) * inv_lambda;
        const float inv_s = 1.f / s;
        make_features(nd.x - cx, nd.y - cy, nd.z - cz, inv_s, __ldg(&t.feat[3 * node]),
                      __ldg(&t.feat[3 * node + 1]), __ldg(&t.feat[3 * node + 2]), feat);
        float cg[3], g[3];
        mlp::infer_warp(feat, cg, S.frag, S.bias, S.xs[warp], S.os[warp], lane);
        apply_head(feat, cg, g);
        if (have) {
            const float k = __ldg(&t.nodem[node]) * inv_s * inv_s;
            corr[0] = k * g[0];
            corr[1] = k * g[1];
            corr[2] = k * g[2];
        }
        for (int o = 16; o > 0; o >>= 1) {
            corr[0] += __shfl_xor_sync(0xffffffffu, corr[0], o);
            corr[1] += __shfl_xor_sync(0xffffffffu, corr[1], o);
            corr[2] += __shfl_xor_sync(0xffffffffu, corr[2], o);
        }
        gx += corr[0];
        gy += corr[1];
        gz += corr[2];
        if (lane == 0) rows += (unsigned)qn;  // one network row per queued cell
        qn = 0;
    };

    do {
        const float4 nd = __ldg(&t.node4[curr]);
        const float dx = nd.x - xi, dy = nd.y - yi, dz = nd.z - zi;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const bool is_leaf = curr >= n;
        const bool open = !(d2 > nd.w);
        if (is_leaf || !__any_sync(0xffffffffu, open)) {
            if (!open) {
                const float m = __ldg(&t.nodem[curr]);
                const float inv = rsqrt_mufu(d2 + eps2);
                const float s3 = m * inv * (inv * inv);
                ax = fmaf(dx, s3, ax);
                ay = fmaf(dy, s3, ay);
                az = fmaf(dz, s3, az);
                ++inter;
            }
            if (!is_leaf) {
                if (GROUP) {
                    const float ex = nd.x - cx, ey = nd.y - cy, ez = nd.z - cz;
                    const float dc2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
                    if (dc2 <= nd.w * band2) {  // uniform across the warp
                        if (lane == 0) S.queue[warp][qn] = curr;
                        __syncwarp();
                        if (++qn == 32) flush_group();
                    }
                } else {
                    const bool band = d2 <= nd.w * band2;
                    if (__any_sync(0xffffffffu, band)) {
                        const float s = sqrtf(nd.w) * inv_lambda;
                        const float inv_s = 1.f / s;
                        float feat[16];
                        make_features(dx, dy, dz, inv_s, __ldg(&t.feat[3 * curr]),
                                      __ldg(&t.feat[3 * curr + 1]), __ldg(&t.feat[3 * curr + 2]),
                                      feat);
                        float cg[3], g[3];
                        mlp::infer_warp(feat, cg, S.frag, S.bias, S.xs[warp], S.os[warp], lane);
                        apply_head(feat, cg, g);
                        if (band) {
                            ++rows;
                            const float k = __ldg(&t.nodem[curr]) * inv_s * inv_s;
                            ax = fmaf(k, g[0], ax);
                            ay = fmaf(k, g[1], ay);
                            az = fmaf(k, g[2], az);
                        }
                    }
                }
            }
            curr = next_down_i(curr);
        } else {
            curr = 2 * curr;
        }
        if (++visits > (unsigned)sz) {
            if (lane == 0) atomicOr(err, kDevErrWalkOverflow);
            break;
        }
    } while (curr != 1);
    if (GROUP && qn > 0) flush_group();
    if (live) {
        const int b = t.body_n[leaf];
        f[b] = y[3 * n + b];
        f[n + b] = y[4 * n + b];
        f[2 * n + b] = y[5 * n + b];
        f[3 * n + b] = (double)(ax + gx);
        f[4 * n + b] = (double)(ay + gy);
        f[5 * n + b] = (double)(az + gz);
    }
    if (!live) inter = rows = 0;
    for (int o = 16; o > 0; o >>= 1) {
        inter += __shfl_xor_sync(0xffffffffu, inter, o);
        rows += __shfl_xor_sync(0xffffffffu, rows, o);
    }
    if (lane == 0) {
        atomicAdd(&t.counters[0], (unsigned long long)visits);
        atomicAdd(&t.counters[1], (unsigned long long)inter);
        atomicAdd(&t.counters[4], (unsigned long long)rows);
    }
}

// Inference on given feature rows (the walk's routine, one warp per 32 rows).
__global__ void __launch_bounds__(128)
predict_kernel(const float* __restrict__ x, size_t count, float* __restrict__ out,
               const uint2* __restrict__ frag_g, const float* __restrict__ bias_g) {
    __shared__ uint2 frag[kFragWords];
    __shared__ float bias[kBias];
    __shared__ uint32_t xs[4][32 * 8];
    __shared__ float os[4][32 * 4];
    for (int i = threadIdx.x; i < kFragWords; i += blockDim.x) frag[i] = frag_g[i];
    for (int i = threadIdx.x; i < kBias; i += blockDim.x) bias[i] = bias_g[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t row = ((size_t)blockIdx.x * 4 + warp) * 32 + lane;
    if (((size_t)blockIdx.x * 4 + warp) * 32 >= count) return;
    float feat[16];
    for (int k = 0; k < 16; ++k) feat[k] = row < count ? x[row * 16 + k] : 0.f;
    float g[3];
    mlp::infer_warp(feat, g, frag, bias, xs[warp], os[warp], lane);
    if (row < count)
        for (int c = 0; c < 3; ++c) out[row * 4 + c] = g[c];
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
nbg_status learn_alloc(nbg_engine* e) {
    if (e->learn != nullptr) return NBG_OK;
    LearnState* L = new LearnState();
    e->learn = L;
    NBG_CUDA(e, cudaMalloc(&L->w, kParams * sizeof(float)));
    NBG_CUDA(e, cudaMalloc(&L->grad, kParams * sizeof(float)));
    NBG_CUDA(e, cudaMalloc(&L->m1, kParams * sizeof(float)));
    NBG_CUDA(e, cudaMalloc(&L->m2, kParams * sizeof(float)));
    NBG_CUDA(e, cudaMalloc(&L->frag, kFragWords * sizeof(uint2)));
    NBG_CUDA(e, cudaMalloc(&L->bias, kBias * sizeof(float)));
    NBG_CUDA(e, cudaMalloc(&L->loss, 2 * sizeof(double)));
    NBG_CUDA(e, cudaMemsetAsync(L->grad, 0, kParams * sizeof(float), e->stream));
    NBG_CUDA(e, cudaMemsetAsync(L->m1, 0, kParams * sizeof(float), e->stream));
    NBG_CUDA(e, cudaMemsetAsync(L->m2, 0, kParams * sizeof(float), e->stream));
    return NBG_OK;
}

nbg_status rebuild_frags(nbg_engine* e) {
    LearnState* L = e->learn;
    make_frags_kernel<<<kTiles, 32, 0, e->stream>>>(L->w, L->frag, L->bias);
    NBG_LAUNCHED(e, "make_frags_kernel");
    return tc_rebuild_weights(e);
}

}  // namespace

// node features of the current tree (after tree_build / tree_refit)
nbg_status tree_features(nbg_engine* e) {
    TreeState* t = e->tree;
    LearnState* L = e->learn;
    const size_t sz = t->size;
    if (t->feat == nullptr) NBG_CUDA(e, cudaMalloc(&t->feat, 3 * sz * sizeof(float4)));
    if (L->mom_size < sz) {
        cudaFree(L->mom);
        L->mom = nullptr;
        NBG_CUDA(e, cudaMalloc(&L->mom, 6 * sz * sizeof(double)));
        L->mom_size = sz;
    }
    const int n = (int)t->n;
    const unsigned g = grid_for(n, 256, (unsigned)e->sm_count * 8u);
    moments_leaf_kernel<<<g, 256, 0, e->stream>>>(L->mom, sz, n);
    NBG_LAUNCHED(e, "moments_leaf_kernel");
    for (int lv = t->levels - 1; lv >= 0; --lv) {
        const int first = 1 << lv;
        moments_level_kernel<<<grid_for(first, 256, (unsigned)e->sm_count * 8u), 256, 0,
                               e->stream>>>(first, first, *t, L->mom);
        NBG_LAUNCHED(e, "moments_level_kernel");
    }
    features_kernel<<<grid_for(sz, 256, (unsigned)e->sm_count * 8u), 256, 0, e->stream>>>(
        *t, L->mom, t->lambda);
    NBG_LAUNCHED(e, "features_kernel");
    return NBG_OK;
}

namespace {

size_t train_smem() { return sizeof(TrainSmem); }
size_t walk_smem() { return sizeof(WalkSmem); }

}  // namespace

bool learned_ready(const nbg_engine* e) { return e->learn != nullptr && e->learn->has_weights; }

void learn_destroy(nbg_engine* e) {
    LearnState* L = e->learn;
    if (L == nullptr) return;
    void* ptrs[] = {L->w, L->grad, L->m1, L->m2, L->frag, L->bias, L->loss, L->grad_part,
                    L->loss_part, L->x, L->t, L->meta, L->pairs, L->mom};
    for (void* p : ptrs) cudaFree(p);
    learned_tc_free(L);
    delete L;
    e->learn = nullptr;
}

nbg_status learned_walk(nbg_engine* e, const double* y, double* f) {
    if (!learned_ready(e))
        return set_error(e, NBG_ERR_NOT_INITIALIZED,
                         "learned correction enabled but no weights are loaded");
    nbg_status s = tree_features(e);
    if (s != NBG_OK) return s;
    TreeState* t = e->tree;
    const int n = (int)e->count;
    // "learned.walk": 1 (default) the group walk with the network on the
    // tcgen05 tensor cores (nbg_learned_tc.cu), which runs on the default
    // group walk only (64-body groups, monopole cells, acceptance not frozen);
    // 0, or any other walk setting: the warp-coherent per-body walk below,
    // one mma.sync batch per band cell
    if (e->tune_get("learned.walk", 1) == 1 && e->tune_get("learned.group", 0) == 0 &&
        e->tune_get("bh.walk", 1) == 1 && e->tune_get("bh.group", 64) == 64 &&
        e->tune_get("bh.order", 1) == 1 && e->tune_get("bh.freeze_within_step", 0) == 0 &&
        e->tune_get("bh.acc_smem", 1) != 0 && n >= 64)
        return learned_tc_walk(e, y, f);
    const double lam_l = e->params.distance_to_node_radius_ratio;
    const double lam_t = e->params.learned_tight_ratio;
    const float band2 = (float)((lam_t / lam_l) * (lam_t / lam_l));
    const float eps2 = (float)(e->params.softening * e->params.softening);
    const bool group = e->tune_get("learned.group", 0) != 0;
    const size_t smem = walk_smem();
    auto kern = group ? learned_walk_kernel<true> : learned_walk_kernel<false>;
    NBG_CUDA(e, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int threads = ((n + 31) / 32) * 32;
    kern<<<(threads + kWalkThreads - 1) / kWalkThreads, kWalkThreads, smem, e->stream>>>(
        y, f, n, eps2, band2, (float)(1.0 / lam_l), *t, e->learn->frag, e->learn->bias, e->d_err);
    NBG_LAUNCHED(e, "learned_walk_kernel");
    return NBG_OK;
}

// The learned path's fcompute.  The tree is built (or refit) at the loose
// ratio lambda_l with FP64 nodes (the features need them) and the learned
// walk writes f.  At the first fcompute of every engine step the judge
// ("learned.judge" = 1, the default) compares the learned forces and the
// plain walk's at the tight ratio lambda_t on a sampled direct sum; when the
// learned p99 is the larger, the tree is rebuilt at lambda_t and the plain
// mixed walk (the engine's non-learned Barnes-Hut path) rewrites f, and every
// further fcompute of that step takes the plain path as well, so that one
// solver step sees one force field.
nbg_status learned_fcompute(nbg_engine* e, uint64_t step, const double* y, double* f) {
    if (!learned_ready(e))
        return set_error(e, NBG_ERR_NOT_INITIALIZED,
                         "learned correction enabled but no weights are loaded");
    LearnState* L = e->learn;
    const double lam_l = e->params.distance_to_node_radius_ratio;
    const double lam_t = e->params.learned_tight_ratio;
    const bool judge = e->tune_get("learned.judge", 1) != 0;
    if (judge && L->plain_valid && L->plain_step == step) {
        nbg_status s = bh_tree(e, step, y, true, lam_t);
        if (s != NBG_OK) return s;
        return mixed_walk(e, y, f);
    }
    nbg_status s = bh_tree(e, step, y, true, lam_l);
    if (s != NBG_OK) return s;
    {
        ProfScope ps(e, NBG_K_BH_WALK);
        s = learned_walk(e, y, f);
    }
    if (s != NBG_OK || !judge || (L->judged_valid && L->judged_step == step)) return s;
    JudgeResult r;
    s = judge_learned(e, step, f, lam_l, lam_t, &r);
    if (s != NBG_OK) return s;
    L->judged_valid = true;
    L->judged_step = step;
    L->judged++;
    L->last = r;
    if (!r.use_plain) return NBG_OK;
    L->fallbacks++;
    L->plain_valid = true;
    L->plain_step = step;
    s = tree_build(e, y, true, lam_t);
    if (s != NBG_OK) return s;
    e->tree->built_step = step;
    return mixed_walk(e, y, f);
}

}  // namespace nbg

using namespace nbg;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

nbg_status nbg_learn_set_weights(nbg_engine* e, const float* w, size_t count) {
    if (e == nullptr || w == nullptr) return NBG_ERR_INVALID_ARG;
    if (count != (size_t)kParams)
        return set_error(e, NBG_ERR_SIZE_MISMATCH, "expected %d parameters", kParams);
    nbg_status s = learn_alloc(e);
    if (s != NBG_OK) return s;
    NBG_CUDA(e, cudaMemcpyAsync(e->learn->w, w, kParams * sizeof(float), cudaMemcpyHostToDevice,
                                e->stream));
    s = rebuild_frags(e);
    if (s != NBG_OK) return s;
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    e->learn->has_weights = true;
    return NBG_OK;
}

nbg_status nbg_learn_get_weights(nbg_engine* e, float* w, size_t count) {
    if (e == nullptr || w == nullptr) return NBG_ERR_INVALID_ARG;
    if (count != (size_t)kParams)
        return set_error(e, NBG_ERR_SIZE_MISMATCH, "expected %d parameters", kParams);
    if (!learned_ready(e)) return set_error(e, NBG_ERR_NOT_INITIALIZED, "no weights");
    NBG_CUDA(e, cudaMemcpyAsync(w, e->learn->w, kParams * sizeof(float), cudaMemcpyDeviceToHost,
                                e->stream));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    return NBG_OK;
}

size_t nbg_learn_param_count(void) { return (size_t)kParams; }

nbg_status nbg_learn_generate(nbg_engine* e, size_t max_samples, uint64_t seed,
                              int max_subtree_log2, size_t* produced) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    if (e->params.algo != NBG_ALGO_BH || e->count == 0)
        return set_error(e, NBG_ERR_INVALID_ARG, "sample generation needs an initialised BH engine");
    nbg_status s = learn_alloc(e);
    if (s != NBG_OK) return s;
    LearnState* L = e->learn;
    const double* y = static_cast<const double*>(e->y->dptr);
    s = tree_build(e, y, true, e->params.distance_to_node_radius_ratio);
    if (s != NBG_OK) return s;
    s = tree_features(e);
    if (s != NBG_OK) return s;
    TreeState* t = e->tree;
    const int n = (int)e->count;
    // grow the sample store
    const size_t need = L->count + max_samples;
    if (need > L->cap) {
        size_t cap = std::max(need, L->cap * 2);
        float *nx = nullptr, *nt = nullptr;
        int* nm = nullptr;
        NBG_CUDA(e, cudaMalloc(&nx, cap * 16 * sizeof(float)));
        NBG_CUDA(e, cudaMalloc(&nt, cap * 4 * sizeof(float)));
        NBG_CUDA(e, cudaMalloc(&nm, cap * 2 * sizeof(int)));
        if (L->count) {
            NBG_CUDA(e, cudaMemcpyAsync(nx, L->x, L->count * 16 * sizeof(float),
                                        cudaMemcpyDeviceToDevice, e->stream));
            NBG_CUDA(e, cudaMemcpyAsync(nt, L->t, L->count * 4 * sizeof(float),
                                        cudaMemcpyDeviceToDevice, e->stream));
            NBG_CUDA(e, cudaMemcpyAsync(nm, L->meta, L->count * 2 * sizeof(int),
                                        cudaMemcpyDeviceToDevice, e->stream));
        }
        NBG_CUDA(e, cudaStreamSynchronize(e->stream));
        cudaFree(L->x);
        cudaFree(L->t);
        cudaFree(L->meta);
        L->x = nx;
        L->t = nt;
        L->meta = nm;
        L->cap = cap;
    }
    cudaFree(L->pairs);
    L->pairs = nullptr;
    NBG_CUDA(e, cudaMalloc(&L->pairs, max_samples * 2 * sizeof(int)));
    // sampled bodies: a seeded random permutation of leaves, enough to fill
    std::vector<int> leaves(n);
    for (int i = 0; i < n; ++i) leaves[i] = n + i;
    uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
    for (int i = n - 1; i > 0; --i) {  // Fisher-Yates with a 64-bit LCG
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        const int j = (int)((st >> 33) % (uint64_t)(i + 1));
        std::swap(leaves[i], leaves[j]);
    }
    const int nb = std::min(n, (int)std::max<size_t>(256, max_samples / 64));
    DevScratch s_bodies;  // freed on every return
    NBG_CUDA(e, cudaMalloc(&s_bodies.p, nb * sizeof(int)));
    int* d_bodies = s_bodies.as<int>();
    NBG_CUDA(e, cudaMemcpyAsync(d_bodies, leaves.data(), nb * sizeof(int), cudaMemcpyHostToDevice,
                                e->stream));
    const double lam_l = e->params.distance_to_node_radius_ratio;
    const double lam_t = e->params.learned_tight_ratio;
    const float band2 = (float)((lam_t / lam_l) * (lam_t / lam_l));
    // pairs per sampled leaf, their exclusive prefix sum (on the host), then
    // the pairs at those slots
    DevScratch s_counts, s_first;
    NBG_CUDA(e, cudaMalloc(&s_counts.p, nb * sizeof(unsigned)));
    NBG_CUDA(e, cudaMalloc(&s_first.p, nb * sizeof(unsigned long long)));
    sample_pairs_kernel<false><<<(nb + 127) / 128, 128, 0, e->stream>>>(
        d_bodies, nb, *t, n, band2, max_subtree_log2, t->levels, nullptr, s_counts.as<unsigned>(),
        nullptr, 0ull);
    NBG_LAUNCHED(e, "sample_pairs_kernel");
    std::vector<unsigned> counts(nb);
    NBG_CUDA(e, cudaMemcpyAsync(counts.data(), s_counts.p, nb * sizeof(unsigned),
                                cudaMemcpyDeviceToHost, e->stream));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    std::vector<unsigned long long> first(nb);
    unsigned long long got = 0;
    for (int k = 0; k < nb; ++k) {
        first[k] = got;
        got += counts[k];
    }
    NBG_CUDA(e, cudaMemcpyAsync(s_first.p, first.data(), nb * sizeof(unsigned long long),
                                cudaMemcpyHostToDevice, e->stream));
    sample_pairs_kernel<true><<<(nb + 127) / 128, 128, 0, e->stream>>>(
        d_bodies, nb, *t, n, band2, max_subtree_log2, t->levels, L->pairs, nullptr,
        s_first.as<unsigned long long>(), (unsigned long long)max_samples);
    NBG_LAUNCHED(e, "sample_pairs_kernel");
    const size_t np = std::min((size_t)got, max_samples);
    if (np > 0) {
        const double eps2 = e->params.softening * e->params.softening;
        const size_t threads = np * 32;
        sample_targets_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, e->stream>>>(
            L->pairs, np, y, e->d_mass, *t, n, t->levels, lam_l, eps2, L->x + L->count * 16,
            L->t + L->count * 4, L->meta + L->count * 2);
        NBG_LAUNCHED(e, "sample_targets_kernel");
        NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    }
    L->count += np;
    if (produced) *produced = np;
    return NBG_OK;
}

size_t nbg_learn_sample_count(const nbg_engine* e) {
    return (e == nullptr || e->learn == nullptr) ? 0 : e->learn->count;
}

nbg_status nbg_learn_read_samples(nbg_engine* e, size_t offset, size_t count, float* x, float* t,
                                  int* meta) {
    if (e == nullptr || e->learn == nullptr) return NBG_ERR_INVALID_ARG;
    LearnState* L = e->learn;
    if (offset + count > L->count) return set_error(e, NBG_ERR_SIZE_MISMATCH, "past the end");
    if (x) NBG_CUDA(e, cudaMemcpy(x, L->x + offset * 16, count * 16 * sizeof(float), cudaMemcpyDeviceToHost));
    if (t) NBG_CUDA(e, cudaMemcpy(t, L->t + offset * 4, count * 4 * sizeof(float), cudaMemcpyDeviceToHost));
    if (meta) NBG_CUDA(e, cudaMemcpy(meta, L->meta + offset * 2, count * 2 * sizeof(int), cudaMemcpyDeviceToHost));
    return NBG_OK;
}

nbg_status nbg_learn_clear_samples(nbg_engine* e) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    if (e->learn) e->learn->count = 0;
    return NBG_OK;
}

// One pass of forward + backward over `order[b0 .. b0 + bsize)` of (x, t):
// grad = the pass's gradient, loss[0] += its squared error, both summed in
// a fixed order (equal inputs give equal results).
static nbg_status run_train_pass(nbg_engine* e, const float* x, const float* t, const int* order,
                                 size_t b0, size_t bsize, float wnorm = 0.f) {
    LearnState* L = e->learn;
    const size_t smem = train_smem();
    NBG_CUDA(e, cudaFuncSetAttribute(train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    const size_t chunks = (bsize + 31) / 32;
    unsigned grid = (unsigned)std::min<size_t>((chunks + kTrainWarps - 1) / kTrainWarps,
                                               (size_t)e->sm_count);
    if (grid < 1) grid = 1;
    if ((int)grid > L->part_blocks) {
        cudaFree(L->grad_part);
        cudaFree(L->loss_part);
        L->grad_part = nullptr;
        L->loss_part = nullptr;
        L->part_blocks = 0;
        NBG_CUDA(e, cudaMalloc(&L->grad_part, (size_t)grid * kParams * sizeof(float)));
        NBG_CUDA(e, cudaMalloc(&L->loss_part, (size_t)grid * sizeof(double)));
        L->part_blocks = (int)grid;
    }
    train_kernel<<<grid, kTrainWarps * 32, smem, e->stream>>>(
        x, t, order, b0, bsize, L->frag, L->bias, L->grad_part, L->loss_part, wnorm);
    NBG_LAUNCHED(e, "train_kernel");
    grad_reduce_kernel<<<(kParams + 255) / 256, 256, 0, e->stream>>>(L->grad_part, (int)grid,
                                                                       L->grad, L->loss_part,
                                                                       L->loss);
    NBG_LAUNCHED(e, "grad_reduce_kernel");
    return NBG_OK;
}

nbg_status nbg_learn_init_weights(nbg_engine* e, uint64_t seed) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status s = learn_alloc(e);
    if (s != NBG_OK) return s;
    // Glorot-uniform weights, zero biases, from a 64-bit LCG
    std::vector<float> w(kParams, 0.f);
    uint64_t st = seed * 2862933555777941757ull + 3037000493ull;
    auto uni = [&]() {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        return (double)(st >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    };
    auto fill = [&](int off, int fan_in, int fan_out) {
        const double a = std::sqrt(6.0 / (fan_in + fan_out));
        for (int i = 0; i < fan_in * fan_out; ++i) w[off + i] = (float)(a * uni());
    };
    fill(kOffW1, kIn, kH);
    fill(kOffW2, kH, kH);
    fill(kOffW3, kH, kOut);
    e->learn->adam_step = 0;
    NBG_CUDA(e, cudaMemsetAsync(e->learn->m1, 0, kParams * sizeof(float), e->stream));
    NBG_CUDA(e, cudaMemsetAsync(e->learn->m2, 0, kParams * sizeof(float), e->stream));
    return nbg_learn_set_weights(e, w.data(), w.size());
}

nbg_status nbg_learn_train(nbg_engine* e, int epochs, size_t batch, double lr, uint64_t seed,
                           double val_fraction, double* train_mse, double* val_mse) {
    if (e == nullptr || epochs < 0 || batch == 0) return NBG_ERR_INVALID_ARG;
    LearnState* L = e->learn;
    if (L == nullptr || L->count < 64) return set_error(e, NBG_ERR_NOT_INITIALIZED, "no samples");
    if (!L->has_weights) {
        nbg_status s = nbg_learn_init_weights(e, seed);
        if (s != NBG_OK) return s;
    }
    const size_t total = L->count;
    size_t nval = (size_t)(val_fraction * (double)total);
    if (nval >= total) nval = total / 10;
    const size_t ntrain = total - nval;
    // seeded permutation of the sample store: [train | validation]
    std::vector<int> perm(total);
    for (size_t i = 0; i < total; ++i) perm[i] = (int)i;
    uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
    for (size_t i = total - 1; i > 0; --i) {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        const size_t j = (size_t)((st >> 33) % (uint64_t)(i + 1));
        std::swap(perm[i], perm[j]);
    }
    // "learned.weighted": weight each sample's squared error by its cell's
    // force scale (m / s^2)^2, normalised over the training set
    float wnorm = 0.f;
    if (e->tune_get("learned.weighted", 0) != 0) {
        std::vector<float> ht(4 * total);
        NBG_CUDA(e, cudaMemcpy(ht.data(), L->t, 4 * total * sizeof(float), cudaMemcpyDeviceToHost));
        double sw = 0.0;
        for (size_t i = 0; i < ntrain; ++i) {
            const double w = ht[4 * (size_t)perm[i] + 3];
            sw += w * w;
        }
        wnorm = sw > 0.0 ? (float)((double)ntrain / sw) : 0.f;
    }
    DevScratch s_perm;  // freed on every return
    NBG_CUDA(e, cudaMalloc(&s_perm.p, total * sizeof(int)));
    int* d_perm = s_perm.as<int>();
    NBG_CUDA(e, cudaMemcpyAsync(d_perm, perm.data(), total * sizeof(int), cudaMemcpyHostToDevice,
                                e->stream));
    const int adam_threads = 256;
    const size_t steps_per_epoch = (ntrain + batch - 1) / batch;
    const size_t total_steps = steps_per_epoch * (size_t)epochs;
    double last_train = 0.0;
    size_t step = 0;
    for (int ep = 0; ep < epochs; ++ep) {
        NBG_CUDA(e, cudaMemsetAsync(L->loss, 0, 2 * sizeof(double), e->stream));
        for (size_t b0 = 0; b0 < ntrain; b0 += batch, ++step) {
            const size_t bs = std::min(batch, ntrain - b0);
            nbg_status s = run_train_pass(e, L->x, L->t, d_perm, b0, bs, wnorm);
            if (s != NBG_OK) return s;
            // cosine-decayed learning rate
            const double frac = total_steps > 1 ? (double)step / (double)(total_steps - 1) : 0.0;
            const double lr_t = lr * 0.5 * (1.0 + std::cos(3.141592653589793 * frac)) + 1e-2 * lr;
            L->adam_step++;
            const double c1 = 1.0 - std::pow(0.9, (double)L->adam_step);
            const double c2 = 1.0 - std::pow(0.999, (double)L->adam_step);
            adam_kernel<<<(kParams + adam_threads - 1) / adam_threads, adam_threads, 0, e->stream>>>(
                L->w, L->grad, L->m1, L->m2, (float)lr_t, 0.9f, 0.999f, 1e-8f, (float)c1,
                (float)c2, kParams);
            NBG_LAUNCHED(e, "adam_kernel");
            s = rebuild_frags(e);
            if (s != NBG_OK) return s;
        }
        double h[2] = {0, 0};
        NBG_CUDA(e, cudaMemcpyAsync(h, L->loss, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
        NBG_CUDA(e, cudaStreamSynchronize(e->stream));
        last_train = h[0] / (double)(ntrain * kOut);
    }
    // validation MSE: a forward/backward pass with the gradient discarded
    double val = 0.0;
    if (nval > 0) {
        NBG_CUDA(e, cudaMemsetAsync(L->loss, 0, 2 * sizeof(double), e->stream));
        nbg_status s = run_train_pass(e, L->x, L->t, d_perm, ntrain, nval, wnorm);
        if (s != NBG_OK) return s;
        NBG_CUDA(e, cudaMemsetAsync(L->grad, 0, kParams * sizeof(float), e->stream));
        double h[2] = {0, 0};
        NBG_CUDA(e, cudaMemcpyAsync(h, L->loss, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
        NBG_CUDA(e, cudaStreamSynchronize(e->stream));
        val = h[0] / (double)(nval * kOut);
    }
    if (train_mse) *train_mse = last_train;
    if (val_mse) *val_mse = val;
    return NBG_OK;
}

nbg_status nbg_learn_loss_grad(nbg_engine* e, const float* x, const float* t, size_t count,
                               double* loss_sum, float* grad) {
    if (e == nullptr || x == nullptr || t == nullptr || count == 0) return NBG_ERR_INVALID_ARG;
    LearnState* L = e->learn;
    if (L == nullptr || !L->has_weights) return set_error(e, NBG_ERR_NOT_INITIALIZED, "no weights");
    DevScratch sx, st, sord;  // freed on every return
    NBG_CUDA(e, cudaMalloc(&sx.p, count * 16 * sizeof(float)));
    NBG_CUDA(e, cudaMalloc(&st.p, count * 4 * sizeof(float)));
    NBG_CUDA(e, cudaMalloc(&sord.p, count * sizeof(int)));
    float* dx = sx.as<float>();
    float* dt = st.as<float>();
    int* dord = sord.as<int>();
    std::vector<int> ord(count);
    for (size_t i = 0; i < count; ++i) ord[i] = (int)i;
    NBG_CUDA(e, cudaMemcpyAsync(dx, x, count * 16 * sizeof(float), cudaMemcpyHostToDevice, e->stream));
    NBG_CUDA(e, cudaMemcpyAsync(dt, t, count * 4 * sizeof(float), cudaMemcpyHostToDevice, e->stream));
    NBG_CUDA(e, cudaMemcpyAsync(dord, ord.data(), count * sizeof(int), cudaMemcpyHostToDevice,
                                e->stream));
    NBG_CUDA(e, cudaMemsetAsync(L->grad, 0, kParams * sizeof(float), e->stream));
    NBG_CUDA(e, cudaMemsetAsync(L->loss, 0, 2 * sizeof(double), e->stream));
    nbg_status s = run_train_pass(e, dx, dt, dord, 0, count);
    if (s != NBG_OK) return s;
    double h[2] = {0, 0};
    NBG_CUDA(e, cudaMemcpyAsync(h, L->loss, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
    if (grad)
        NBG_CUDA(e, cudaMemcpyAsync(grad, L->grad, kParams * sizeof(float), cudaMemcpyDeviceToHost,
                                    e->stream));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    NBG_CUDA(e, cudaMemsetAsync(L->grad, 0, kParams * sizeof(float), e->stream));
    if (loss_sum) *loss_sum = h[0];
    return NBG_OK;
}

nbg_status nbg_learn_predict(nbg_engine* e, const float* x, size_t count, float* out) {
    if (e == nullptr || x == nullptr || out == nullptr || count == 0) return NBG_ERR_INVALID_ARG;
    if (!learned_ready(e)) return set_error(e, NBG_ERR_NOT_INITIALIZED, "no weights");
    DevScratch sx, sout;  // freed on every return
    NBG_CUDA(e, cudaMalloc(&sx.p, count * 16 * sizeof(float)));
    NBG_CUDA(e, cudaMalloc(&sout.p, count * 4 * sizeof(float)));
    float* dx = sx.as<float>();
    float* dout = sout.as<float>();
    NBG_CUDA(e, cudaMemcpyAsync(dx, x, count * 16 * sizeof(float), cudaMemcpyHostToDevice, e->stream));
    const size_t warps = (count + 31) / 32;
    predict_kernel<<<(unsigned)((warps + 3) / 4), 128, 0, e->stream>>>(dx, count, dout, e->learn->frag,
                                                                    e->learn->bias);
    NBG_LAUNCHED(e, "predict_kernel");
    std::vector<float> tmp(count * 4);
    NBG_CUDA(e, cudaMemcpyAsync(tmp.data(), dout, count * 4 * sizeof(float), cudaMemcpyDeviceToHost,
                                e->stream));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    for (size_t i = 0; i < count; ++i)
        for (int c = 0; c < 3; ++c) out[i * 3 + c] = tmp[i * 4 + c];
    return NBG_OK;
}

nbg_status nbg_learn_judge_stats(nbg_engine* e, double* out, size_t count) {
    if (e == nullptr || out == nullptr || count < NBG_JUDGE_STATS) return NBG_ERR_INVALID_ARG;
    for (size_t k = 0; k < NBG_JUDGE_STATS; ++k) out[k] = 0.0;
    const LearnState* L = e->learn;
    if (L == nullptr || !L->judged_valid) return NBG_OK;
    const JudgeResult& r = L->last;
    const double v[NBG_JUDGE_STATS] = {
        (double)L->judged_step, r.p50_learned, r.p99_learned, r.p50_plain, r.p99_plain,
        r.rms_learned, r.rms_plain, r.use_plain ? 1.0 : 0.0, (double)r.samples,
        (double)L->judged, (double)L->fallbacks};
    for (size_t k = 0; k < NBG_JUDGE_STATS; ++k) out[k] = v[k];
    return NBG_OK;
}

nbg_status nbg_learn_band_rows(nbg_engine* e, uint64_t* rows) {
    if (e == nullptr || rows == nullptr) return NBG_ERR_INVALID_ARG;
    if (e->tree == nullptr) return set_error(e, NBG_ERR_NOT_INITIALIZED, "no tree built yet");
    unsigned long long h = 0;
    NBG_CUDA(e, cudaMemcpyAsync(&h, e->tree->counters + 4, sizeof(h), cudaMemcpyDeviceToHost,
                                e->stream));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    *rows = h;
    return NBG_OK;
}

nbg_status nbg_tree_leaves(nbg_engine* e, int* body_of_leaf) {
    if (e == nullptr || body_of_leaf == nullptr) return NBG_ERR_INVALID_ARG;
    if (e->tree == nullptr || !e->tree->built) return set_error(e, NBG_ERR_NOT_INITIALIZED, "no tree");
    NBG_CUDA(e, cudaMemcpyAsync(body_of_leaf, e->tree->body_n + e->tree->n, e->tree->n * sizeof(int),
                                cudaMemcpyDeviceToHost, e->stream));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    return NBG_OK;
}

}  // extern "C"
