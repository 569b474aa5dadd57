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
    int curve = 0;    // leaf order of the last build: 0 kd-median, 1 Morton, 2 Hilbert
    double lambda = 0.0;  // opening ratio the node records' crit2 were formed with
    uint64_t built_step = 0;  // engine step of the last full build

    // build scratch
    uint64_t* keys[2] = {nullptr, nullptr};  // radix keys (ping-pong)
    int* vals[2] = {nullptr, nullptr};       // radix values (ping-pong)
    int* lists[3] = {nullptr, nullptr, nullptr};  // bodies sorted by x / y / z per segment
    int* spare[2] = {nullptr, nullptr};      // partition outputs
    unsigned char* flag = nullptr;           // [n] 1 = goes to the left child
    int* tile_count = nullptr;               // [2][n / kPartTile + 1]
    unsigned* hist = nullptr;                // radix per-block digit counts
    unsigned* totals = nullptr;              // radix per-digit totals
    unsigned long long* box = nullptr;       // [6] order keys of the bounding box (curve builds)

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
    // f32: the last build formed only the FP32 records, from FP32 boxes
    // (box4[node] = min corner, box4[size + node] = max corner); the FP64
    // arrays above are then not current
    bool f32 = false;
    float4* box4 = nullptr;   // [2][size]

    // frozen acceptance ("bh.freeze_within_step"): the FP32 records of the
    // step's full build, which the walks test acceptance (and form group
    // boxes) against while the refit records of the step's later stages
    // give the forces; null when not in use
    float4* node4_acc = nullptr;  // [size]
    uint64_t acc_step = 0;        // built_step of the records in node4_acc
    // with frozen acceptance, each leaf's FP32 rounding residual (x - hi,
    // y - hi, z - hi, 0) of the position in node4, so that the walks form
    // pair differences as (x_j - x_i) + (lo_j - lo_i): the FP32 rounding of
    // absolute positions would otherwise change a close pair's force in
    // steps as the bodies move within a step
    float4* leaf_lo = nullptr;    // [n]

    // learned-correction node features (quadrupole, spread), see nbg_learned.cu
    float4* feat = nullptr;   // [3][size] or null
    // the group walk's band cells for the learned correction on tensor cores
    // (set only while the learned path runs it): every cell a 64-body group
    // accepts at lambda_l whose mass centre is within the tight ratio of the
    // group's box (d_min^2 <= crit2 band2, band2 = (lambda_t / lambda_l)^2)
    int* cand = nullptr;          // [groups][cand_cap]
    unsigned* cand_n = nullptr;   // [groups]
    int cand_cap = 0;
    float band2 = 0.f;

    // quadrupole walk records (nbg_bh.cu): second central mass moments M
    // stored as S = -3 M, quad[2 idx] = (Sxx, Syy, Szz, tr S / 2),
    // quad[2 idx + 1] = (Sxy, Sxz, Syz, 0)
    float4* quad = nullptr;   // [2][size] or null

    // walk counters: node tests, interactions, deepest group-walk stack,
    // groups handed to the per-body fallback walk, learned-walk band rows
    // (body-cell pairs the network corrected)
    unsigned long long* counters = nullptr;  // [5]

    // group walks that exceed a node-test cap give up; their group ids go
    // to fb_list and a per-body walk computes those bodies (nbg_bh.cu).
    // The cap is test_cap when that is set, else cap_state[0], set from the
    // test counts of sampled groups by bh_test_cap_kernel.
    int* fb_list = nullptr;                  // [n / 32]
    unsigned* fb_count = nullptr;            // [2]: queued groups, the walk's next group
    unsigned long long* cap_state = nullptr; // [1]
    unsigned long long test_cap = 0;
};

// Stack entries per warp of the group and per-body walks: 48 per tree level
// plus 32 (a step pops 16 entries and pushes at most 32), set per launch
// from the tree depth; the deepest group-walk stack of every launch is
// recorded in counters[2].
constexpr int kGWStackPerLevel = 48;
inline int group_stack_cap(int levels) { return kGWStackPerLevel * (levels + 1) + 32; }

constexpr int kPartTile = 2048;  // elements per partition tile (256 threads x 8)

// Full build.  FP64 precision: the reference's kd-median tree.  Mixed
// precision: leaves in Hilbert order ("bh.build" = 2, the default), Morton
// order (1) or the kd-median tree (0); a curve tree halves the ordered list
// at every level (one sort, no partitions; a different tree).
// fp64_nodes: form the FP64 node arrays (the FP64 walk, the learned
// correction's features); otherwise only the FP32 records.  lambda: the
// opening ratio of the nodes' critical radii.
nbg_status tree_build(nbg_engine* e, const double* y, bool fp64_nodes, double lambda);
// fixed topology, new positions (and critical radii at lambda)
nbg_status tree_refit(nbg_engine* e, const double* y, double lambda);

// nbg_bh.cu.  The tree for one fcompute: a full build or a refit of the last
// topology.  The reference's rule (nbody/nbody_engine_cuda_bh_tex.cpp:46-163)
// builds when tree_build_rate is 0 or step % rate == 0 and refits otherwise.
// With "bh.refit_within_step" = 1 the engine builds only at the first
// fcompute of each engine step (the step number changes) and refits for the
// other stages of that step (the solver advances the step once per advise).
// "bh.freeze_within_step" = 1 does the same and also keeps the step build's
// records for the acceptance tests, so every body interacts with the same
// cells at every stage of the step and its force is a smooth function of
// the positions (the refit moves the cells' mass centres); without it an
// acceptance test that flips between stages puts a jump in the force.  A
// caller that needs the FP64 node arrays (fp64_nodes) gets a build when the
// last one formed only the FP32 records.
nbg_status bh_tree(nbg_engine* e, uint64_t step, const double* y, bool fp64_nodes, double lambda);
// The plain mixed-precision walk over the current tree (group walk by
// default, "bh.walk" = 0 the warp-coherent walk), writing all of f.
// emit: the default group walk also records each group's band cells (the
// fields cand, cand_n, cand_cap, band2 set) and the per-body fallback walk is
// left to the caller (f of the groups in fb_list is not written).
nbg_status mixed_walk(nbg_engine* e, const double* y, double* f, bool emit = false);

}  // namespace nbg
