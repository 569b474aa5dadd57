// nbg_tree.cuh -- Barnes-Hut tree state shared by the build (nbg_tree.cu) and
// the traversals (nbg_bh.cu).
//
// Layout: the reference's binary heap (nbody/nbody_space_heap.h:8-49):
// root 1, children 2i and 2i+1, leaves at [N, 2N) for N = 2^K bodies,
// heap size 2N (index 0 unused).
#pragma once

#include "nbg_internal.cuh"

namespace nbg {

struct TreeState {
    size_t n = 0;     // bodies (power of two)
    size_t size = 0;  // heap size = 2n
    int levels = 0;   // K = log2(n)
    bool built = false;
    double lambda = 0.0;

    // build scratch
    uint64_t* keys[2] = {nullptr, nullptr};  // radix keys (ping-pong)
    int* vals[2] = {nullptr, nullptr};       // radix values (ping-pong)
    int* lists[3] = {nullptr, nullptr, nullptr};  // bodies sorted by x / y / z per segment
    int* spare[2] = {nullptr, nullptr};      // partition outputs
    unsigned char* flag = nullptr;           // [n] 1 = goes to the left child
    int* tile_count = nullptr;               // [2][n / kPartTile + 1]
    unsigned* hist = nullptr;                // radix per-block digit counts
    unsigned* totals = nullptr;              // radix per-digit totals

    // heap arrays, FP64 SoA (the reference's node fields)
    double* com = nullptr;    // [3][size] mass centre
    double* mass = nullptr;   // [size]
    double* bmin = nullptr;   // [3][size]
    double* bmax = nullptr;   // [3][size]
    double* crit2 = nullptr;  // [size] (lambda * r)^2, 0 for leaves
    int* body_n = nullptr;    // [size] body of a leaf

    // FP32 node records for the mixed-precision walk: (com.xyz, crit2), mass
    float4* node4 = nullptr;  // [size]
    float* nodem = nullptr;   // [size]

    // learned-correction node features (quadrupole, spread), see nbg_learned.cu
    float4* feat = nullptr;   // [3][size] or null

    // quadrupole walk records (nbg_bh.cu): second central mass moments,
    // quad[2 idx] = (Mxx, Myy, Mzz, tr M / 2), quad[2 idx + 1] = (Mxy, Mxz, Myz, 0)
    float4* quad = nullptr;   // [2][size] or null

    // walk counters: node visits and accepted interactions (mixed walk)
    unsigned long long* counters = nullptr;  // [4]
};

constexpr int kPartTile = 2048;  // elements per partition tile (256 threads x 8)

nbg_status tree_build(nbg_engine* e, const double* y);  // full kd-median build
nbg_status tree_refit(nbg_engine* e, const double* y);  // fixed topology, new positions

}  // namespace nbg
