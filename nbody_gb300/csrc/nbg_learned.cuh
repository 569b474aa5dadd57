// nbg_learned.cuh -- state and device helpers shared by the learned
// monopole correction's files: nbg_learned.cu (samples, training, the
// per-body learned walk, the C ABI), nbg_learned_tc.cu (inference on the
// group walk with tcgen05 tensor cores).  No reference counterpart.
#pragma once

#include <stdint.h>

#include "nbg_internal.cuh"
#include "nbg_mlp.cuh"

namespace nbg {

// Band cells a 64-body group may record for the tensor-core path; a group
// with more is walked body by body instead.
constexpr int kCandCap = 2048;
// tcgen05 operand block: W1^T (64 x 16), W2^T / 2 (64 x 64), W3^T / 2
// (16 x 64, rows past 3 zero) as K-major BF16 core matrices, then the bias
// operands B1 (64 x 16), B2 (64 x 16), B3 (16 x 16): row n holds the bias
// of output n split into three BF16 terms (columns 0-2, the rest zero),
// which a K = 16 MMA against a block of ones adds to the accumulator.
constexpr int kTcwW1 = 0;                  // words
constexpr int kTcwW2 = kTcwW1 + 64 * 16 / 2;
constexpr int kTcwW3 = kTcwW2 + 64 * 64 / 2;
constexpr int kTcwB1 = kTcwW3 + 16 * 64 / 2;
constexpr int kTcwB2 = kTcwB1 + 64 * 16 / 2;
constexpr int kTcwB3 = kTcwB2 + 64 * 16 / 2;
constexpr int kTcwWords = kTcwB3 + 16 * 16 / 2;

struct LearnState {
    // model
    float* w = nullptr;      // FP32 master parameters [kParams]
    float* grad = nullptr;   // [kParams]
    float* m1 = nullptr;     // Adam first moment
    float* m2 = nullptr;     // Adam second moment
    uint2* frag = nullptr;   // fragment-ordered BF16 weights [kFragWords]
    float* bias = nullptr;   // padded biases [kBias]
    double* loss = nullptr;  // [2] sum of squared error, sample count
    // per-block gradient and loss partials of one training pass, added in
    // block order (no atomics: a pass's gradient does not depend on the schedule)
    float* grad_part = nullptr;   // [part_blocks][kParams]
    double* loss_part = nullptr;  // [part_blocks]
    int part_blocks = 0;
    int64_t adam_step = 0;
    bool has_weights = false;
    // training samples
    float* x = nullptr;      // [cap][16]
    float* t = nullptr;      // [cap][4]
    int* meta = nullptr;     // [cap][2] (body, node) of the snapshot that made it
    size_t count = 0, cap = 0;
    // sample-generation scratch
    int* pairs = nullptr;    // [cap][2]
    double* mom = nullptr;   // [6][size] FP64 second moments of the current tree
    size_t mom_size = 0;
    // per-step judge (nbg_judge.cu): the step judged last, the step sent to
    // the plain walk, counts, the last figures
    bool judged_valid = false, plain_valid = false;
    uint64_t judged_step = 0, plain_step = 0;
    uint64_t judged = 0, fallbacks = 0;
    JudgeResult last;
    // tensor-core (tcgen05) inference on the group walk (nbg_learned_tc.cu):
    // the weights and biases as K-major BF16 operands, kTcwWords
    // words; each group's band cells; the kernel's next group
    uint32_t* tcw = nullptr;
    int* cand = nullptr;         // [groups][kCandCap] band cells of each group
    unsigned* cand_n = nullptr;  // [groups] their count (0: group walked per body)
    size_t cand_groups = 0;      // groups the arrays hold
    unsigned* tc_next = nullptr; // [1] the tensor-core kernel's next group
};

// The 16 features of (body at x, cell); dx = c - x (FP32, as the walk has it).
__device__ __forceinline__ void make_features(float dx, float dy, float dz, float inv_s,
                                              float4 f0, float4 f1, float4 f2, float feat[16]) {
    const float ux = -dx * inv_s, uy = -dy * inv_s, uz = -dz * inv_s;
    feat[0] = ux;
    feat[1] = uy;
    feat[2] = uz;
    feat[3] = f0.x;
    feat[4] = f0.y;
    feat[5] = f0.z;
    feat[6] = f0.w;
    feat[7] = f1.x;
    feat[8] = f1.y;
    feat[9] = f1.z;
    feat[10] = f1.w;
    feat[11] = f2.x;
    feat[12] = rsqrtf(fmaf(ux, ux, fmaf(uy, uy, uz * uz)));
    feat[13] = f2.y;
    feat[14] = f2.z;
    feat[15] = f2.w;
}

// Equivariant output head: the network's three outputs are coefficients of
// vectors that turn with the cell and the body -- the body direction u/|u|,
// the quadrupole applied to it Q u/|u|, and the mass-centre offset o:
//     g = c0 u/|u| + c1 Q u/|u| + c2 o.
// The exact quadrupole correction has this form, and a bias of the network
// can no longer point the same way for every cell around a body (where it
// would add up instead of cancelling).  basis[i] is the i-th vector.
__device__ __forceinline__ void head_basis(const float feat[16], float basis[3][3]) {
    const float iu = feat[12];
    const float ux = feat[0] * iu, uy = feat[1] * iu, uz = feat[2] * iu;
    // Q = [[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]], feat[3..8] = xx, yy, zz, xy, xz, yz
    basis[0][0] = ux;
    basis[0][1] = uy;
    basis[0][2] = uz;
    basis[1][0] = fmaf(feat[3], ux, fmaf(feat[6], uy, feat[7] * uz));
    basis[1][1] = fmaf(feat[6], ux, fmaf(feat[4], uy, feat[8] * uz));
    basis[1][2] = fmaf(feat[7], ux, fmaf(feat[8], uy, feat[5] * uz));
    basis[2][0] = feat[13];
    basis[2][1] = feat[14];
    basis[2][2] = feat[15];
}

__device__ __forceinline__ void apply_head(const float feat[16], const float c[3], float g[3]) {
    float b[3][3];
    head_basis(feat, b);
#pragma unroll
    for (int k = 0; k < 3; ++k) g[k] = fmaf(c[0], b[0][k], fmaf(c[1], b[1][k], c[2] * b[2][k]));
}


// learned-path host steps shared across files
bool learned_ready(const nbg_engine* e);        // weights loaded
nbg_status tree_features(nbg_engine* e);       // node features of the current tree
nbg_status tc_rebuild_weights(nbg_engine* e);   // tcgen05 operands from the FP32 weights
nbg_status learned_tc_walk(nbg_engine* e, const double* y, double* f);  // group walk + tcgen05
void learned_tc_free(LearnState* L);

}  // namespace nbg
