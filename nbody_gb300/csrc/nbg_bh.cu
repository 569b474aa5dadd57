// nbg_bh.cu -- Barnes-Hut force walks over the heap built by nbg_tree.cu.
//
// Index algebra of the heap (nbody/nbody_space_heap_func_priv.h:4-73):
//   left = 2i, right = 2i + 1, next_down(i) = (i >> ctz(~i)) + 1,
//   skip_idx = next_down, next_up(i) = 2i if 2i < size else next_down(i).
// A walk starts at the root (1), accepts a node when d^2 > crit2 (then skips
// its subtree) and otherwise descends; it ends when it returns to the root
// (nbody/nbody_space_heap_stackless.cpp:3-28).  Leaves have crit2 = 0, so a
// body skips itself (d^2 = 0).  The stack walk of the 'heap' layout
// (nbody/nbody_space_heap.cpp:64-97) visits the same nodes in the same order,
// so both layouts use the stackless form here.
//
//  * FP64 walk (precision fp64): one thread per body, the reference's
//    arithmetic in its order (nbody_data::force, then / m_i) -- the parity
//    path, equal to the reference's simple_bh results.
//  * mixed walk (precision mixed): FP32 node records, one warp walks one
//    node sequence for its 32 bodies (leaf order, so a warp holds 32
//    neighbouring bodies): a node is opened when any lane needs it opened,
//    so every load is a warp-wide broadcast and the walk never diverges.
//    Each lane's accepted set refines its own per-body set, so the result is
//    at least as accurate as the per-body walk at the same opening ratio.
#include "nbg_ptx.cuh"
#include "nbg_tree.cuh"

namespace nbg {

nbg_status learned_walk(nbg_engine* e, const double* y, double* f);  // nbg_learned.cu
bool learned_ready(const nbg_engine* e);

namespace {

__device__ __forceinline__ int next_down(int idx) { return (idx >> (__ffs(~idx) - 1)) + 1; }

// Walk step cap: a stackless walk visits each node at most once, so more
// than `size` visits means a corrupt tree; the walk stops and flags it.

__global__ void bh_walk_fp64_kernel(const double* __restrict__ y, const double* __restrict__ mass,
                                    double* __restrict__ f, int n, int nested, TreeState t,
                                    unsigned* err) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= n) return;
    const size_t sz = t.size;
    int b;
    double v1[3];
    if (nested) {  // nested_tree: threads follow the leaves
        const size_t leaf = (size_t)n + tid;
        b = t.body_n[leaf];
        v1[0] = t.com[leaf];
        v1[1] = t.com[sz + leaf];
        v1[2] = t.com[2 * sz + leaf];
    } else {  // cycle: threads follow the bodies
        b = tid;
        v1[0] = y[b];
        v1[1] = y[n + b];
        v1[2] = y[2 * n + b];
    }
    const double m1 = mass[b];
    const double mneg = __dmul_rn(-1.0, m1);
    double fx = 0.0, fy = 0.0, fz = 0.0;
    int curr = 1;
    long long steps = 0;
    do {
        const double dx = __dsub_rn(v1[0], t.com[curr]);
        const double dy = __dsub_rn(v1[1], t.com[sz + curr]);
        const double dz = __dsub_rn(v1[2], t.com[2 * sz + curr]);
        double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
        if (r2 > t.crit2[curr]) {
            if (r2 < kMinDistance) r2 = kMinDistance;
            const double c = __ddiv_rn(__dmul_rn(mneg, t.mass[curr]), __dmul_rn(r2, __dsqrt_rn(r2)));
            fx = __dadd_rn(fx, __dmul_rn(dx, c));
            fy = __dadd_rn(fy, __dmul_rn(dy, c));
            fz = __dadd_rn(fz, __dmul_rn(dz, c));
            curr = next_down(curr);
        } else {
            curr = (2 * (size_t)curr < sz) ? 2 * curr : next_down(curr);
        }
        if (++steps > (long long)sz) {
            atomicOr(err, kDevErrWalkOverflow);
            break;
        }
    } while (curr != 1);
    f[b] = y[3 * n + b];
    f[n + b] = y[4 * n + b];
    f[2 * n + b] = y[5 * n + b];
    f[3 * n + b] = __ddiv_rn(fx, m1);
    f[4 * n + b] = __ddiv_rn(fy, m1);
    f[5 * n + b] = __ddiv_rn(fz, m1);
}

// Warp-coherent FP32 walk; acceleration a_i = sum m (c - x_i) (d^2 + eps^2)^-3/2.
template <bool CLAMP>
__global__ void __launch_bounds__(256)
bh_walk_mixed_kernel(const double* __restrict__ y, double* __restrict__ f, int n, float eps2,
                     TreeState t, unsigned* err) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    if ((tid & ~31) >= n) return;  // whole warps past the last body
    const bool live = tid < n;
    const int leaf = n + (live ? tid : n - 1);
    const float4 me = __ldg(&t.node4[leaf]);
    const float xi = me.x, yi = me.y, zi = me.z;
    const int nn = n;
    float ax = 0.f, ay = 0.f, az = 0.f;
    unsigned visits = 0, inter = 0;
    int curr = 1;
    const int sz = (int)t.size;
    do {
        const float4 nd = __ldg(&t.node4[curr]);
        const float dx = nd.x - xi, dy = nd.y - yi, dz = nd.z - zi;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const bool is_leaf = curr >= nn;
        const bool open = !(d2 > nd.w);
        if (is_leaf || !__any_sync(0xffffffffu, open)) {
            if (!open) {  // leaves: every lane but the body itself
                const float m = __ldg(&t.nodem[curr]);
                float r2 = d2 + eps2;
                if (CLAMP) r2 = fmaxf(r2, 1e-8f);
                const float inv = rsqrt_mufu(r2);
                const float s = m * inv * (inv * inv);
                ax = fmaf(dx, s, ax);
                ay = fmaf(dy, s, ay);
                az = fmaf(dz, s, az);
                ++inter;
            }
            curr = next_down(curr);
        } else {
            curr = 2 * curr;
        }
        if (++visits > (unsigned)sz) {
            if (lane == 0) atomicOr(err, kDevErrWalkOverflow);
            break;
        }
    } while (curr != 1);
    if (live) {
        const int b = t.body_n[leaf];
        f[b] = y[3 * n + b];
        f[n + b] = y[4 * n + b];
        f[2 * n + b] = y[5 * n + b];
        f[3 * n + b] = (double)ax;
        f[4 * n + b] = (double)ay;
        f[5 * n + b] = (double)az;
    }
    // node visits are per warp (broadcast loads); interactions per body
    if (!live) inter = 0;
    for (int o = 16; o > 0; o >>= 1) inter += __shfl_xor_sync(0xffffffffu, inter, o);
    if (lane == 0) {
        atomicAdd(&t.counters[0], (unsigned long long)visits);
        atomicAdd(&t.counters[1], (unsigned long long)inter);
    }
}

}  // namespace

nbg_status bh_fcompute(nbg_engine* e, uint64_t step, const double* y, double* f) {
    const int n = (int)e->count;
    const uint64_t rate = e->params.tree_build_rate;
    const bool build = e->tree == nullptr || !e->tree->built || rate == 0 || step % rate == 0;
    nbg_status s = build ? tree_build(e, y) : tree_refit(e, y);
    if (s != NBG_OK) return s;
    TreeState* t = e->tree;
    ProfScope ps(e, NBG_K_BH_WALK);
    if (e->params.precision == NBG_PREC_FP64) {
        bh_walk_fp64_kernel<<<(n + 127) / 128, 128, 0, e->stream>>>(
            y, e->d_mass, f, n, e->params.traverse_type == NBG_TRAVERSE_NESTED_TREE ? 1 : 0, *t,
            e->d_err);
        NBG_LAUNCHED(e, "bh_walk_fp64_kernel");
        return NBG_OK;
    }
    if (e->params.learned) return learned_walk(e, y, f);
    const float eps2 = (float)(e->params.softening * e->params.softening);
    const bool clamp = !(e->params.softening > 0.0);
    // warps past n still walk (their lanes mirror the last body) so that
    // every warp is full; n is a power of two, so only n < 32 has such lanes
    const int threads = ((n + 31) / 32) * 32;
    if (clamp)
        bh_walk_mixed_kernel<true><<<(threads + 255) / 256, 256, 0, e->stream>>>(y, f, n, eps2, *t,
                                                                               e->d_err);
    else
        bh_walk_mixed_kernel<false><<<(threads + 255) / 256, 256, 0, e->stream>>>(y, f, n, eps2, *t,
                                                                                e->d_err);
    NBG_LAUNCHED(e, "bh_walk_mixed_kernel");
    return NBG_OK;
}

}  // namespace nbg

extern "C" nbg_status nbg_bh_counters(nbg_engine* e, uint64_t* visits, uint64_t* interactions) {
    using namespace nbg;
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    if (e->tree == nullptr) return set_error(e, NBG_ERR_NOT_INITIALIZED, "no tree built yet");
    unsigned long long h[2] = {0, 0};
    NBG_CUDA(e, cudaMemcpyAsync(h, e->tree->counters, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    NBG_CUDA(e, cudaMemsetAsync(e->tree->counters, 0, 4 * sizeof(unsigned long long), e->stream));
    if (visits) *visits = h[0];
    if (interactions) *interactions = h[1];
    return NBG_OK;
}
