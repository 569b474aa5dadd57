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
//    This walk is the one the learned correction extends (bh.walk = 0).
//  * group walk (precision mixed, the default, bh.walk = 1): a warp tests 32
//    nodes at a time against the bounding box of its 64 (or 32) bodies and
//    evaluates the accepted nodes from an interaction list in shared memory
//    with packed FP32x2 pair math (details at bh_group_walk_kernel).  Warps
//    are persistent; a group that exceeds a node-test cap (bh_test_cap_kernel,
//    from sampled groups' tests) is queued, and bh_body_walk_kernel walks its
//    bodies one warp per body.
//  * the quadrupole term (bh.order = 2) uses per-node second moments
//    (quad_levels_kernel) in both the group walk and the per-body walk.
#include <algorithm>

#include "nbg_ptx.cuh"
#include "nbg_tree.cuh"

namespace nbg {

// nbg_learned.cu: the learned path's fcompute (learned walk, judge, fallback)
nbg_status learned_fcompute(nbg_engine* e, uint64_t step, const double* y, double* f);

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
    unsigned inter = 0;
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
            ++inter;
        } else {
            curr = (2 * (size_t)curr < sz) ? 2 * curr : next_down(curr);
        }
        if (++steps > (long long)sz) {
            atomicOr(err, kDevErrWalkOverflow);
            break;
        }
    } while (curr != 1);
    // node visits and interactions of this thread's body, one atomic per
    // group of converged threads
    const unsigned mask = __activemask();
    const unsigned vis = __reduce_add_sync(mask, (unsigned)steps);
    const unsigned itr = __reduce_add_sync(mask, inter);
    if ((threadIdx.x & 31) == __ffs(mask) - 1) {
        atomicAdd(&t.counters[0], (unsigned long long)vis);
        atomicAdd(&t.counters[1], (unsigned long long)itr);
    }
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

// ---------------------------------------------------------------------------
// group walk: 32 nodes tested per warp step, interactions evaluated in batches
// ---------------------------------------------------------------------------
// A warp owns 32 consecutive leaves (a compact kd subtree).  Its stack holds
// opened nodes; an entry c stands for the two children 2c and 2c + 1.  Each
// step pops up to 16 entries, so each lane tests one node, against the
// bounding box of the warp's 32 bodies: a node is accepted when the box's
// nearest point is outside the node's critical radius (then every body of
// the group accepts it); leaves are always accepted (a body meets itself at
// distance 0, which contributes nothing); other nodes are opened and pushed.
// The walk starts from entry 0, whose children are the unused heap slot 0
// (skipped) and the root.  Accepted nodes go to an interaction list kept as
// four float arrays (x, y, z, m): the stores of one step are consecutive,
// and one LDS.128 of an array returns two aligned FP32x2 operand pairs.
// When the list fills, every lane evaluates it for its own body with the
// direct-sum pair term and folds the result into two-sum accumulators; the
// node loads of the step that finds the list full are issued before that
// evaluation, which covers their latency.
// Each body's accepted set refines its per-body set (box distance <= body
// distance), so the result is at least as accurate as the reference's
// per-body walk at the same ratio.
constexpr int kGWWarps = 4;
constexpr int kGWThreads = kGWWarps * 32;
constexpr int kGWList = 256;    // interaction entries per warp

struct GroupSmem {  // followed by the stacks, kGWWarps x stack_cap ints
    float lx[kGWWarps][kGWList];
    float ly[kGWWarps][kGWList];
    float lz[kGWWarps][kGWList];
    float lm[kGWWarps][kGWList];
};

// groups whose node tests set the group walk's test cap (one warp each, one block)
constexpr int kCapSamples = 32;

// Second list of the quadrupole walk (bh.order = 2): accepted cells with their
// second moments; leaves stay in the monopole list.  Arrays in the order
// x, y, z, m, Sxx, Syy, Szz, tr S / 2, Sxy, Sxz, Syz, S = -3 M (the moments
// as stored, scaled so that the walk's term needs no constant factor).
constexpr int kGWQList = 128;
constexpr int kGWQFields = 11;
struct QuadLists {
    float v[kGWWarps][kGWQFields][kGWQList];
};

// Monopole plus quadrupole term of a cell (mass centre c, mass m, second
// central moments M) on a body at x, for two cells at once; d = c - x:
//   a = d (m / r^3 - 3 k / r^5) - (3 / r^5) M d,  k = tr M / 2 - (5/2) (d.M.d) / r^2,
// from the expansion of 1 / |r - s| about the mass centre to second order
// (the first-order term vanishes there).  With the stored S = -3 M:
//   a = d (m / r^3 + k' / r^5) + (S d) / r^5,  k' = tr S / 2 - (5/2) (d.S.d) / r^2
// (31 packed operations for two cells).
template <bool CLAMP>
__device__ __forceinline__ void quad_pair(const f2_t* q, f2_t xi, f2_t yi, f2_t zi, f2_t eps2,
                                          f2_t& ax, f2_t& ay, f2_t& az) {
    const f2_t dx = f2_sub(q[0], xi);
    const f2_t dy = f2_sub(q[1], yi);
    const f2_t dz = f2_sub(q[2], zi);
    f2_t r2 = f2_fma(dz, dz, eps2);
    r2 = f2_fma(dy, dy, r2);
    r2 = f2_fma(dx, dx, r2);
    float r2a, r2b;
    f2_unpack(r2, r2a, r2b);
    if (CLAMP) {
        r2a = fmaxf(r2a, 1e-8f);
        r2b = fmaxf(r2b, 1e-8f);
    }
    const f2_t inv = f2_pack(rsqrt_mufu(r2a), rsqrt_mufu(r2b));
    const f2_t inv2 = f2_mul(inv, inv);
    const f2_t inv3 = f2_mul(inv2, inv);
    const f2_t inv5 = f2_mul(inv3, inv2);
    // S d with S = [[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]]
    const f2_t sdx = f2_fma(q[9], dz, f2_fma(q[8], dy, f2_mul(q[4], dx)));
    const f2_t sdy = f2_fma(q[10], dz, f2_fma(q[5], dy, f2_mul(q[8], dx)));
    const f2_t sdz = f2_fma(q[6], dz, f2_fma(q[10], dy, f2_mul(q[9], dx)));
    const f2_t dsd = f2_fma(dz, sdz, f2_fma(dy, sdy, f2_mul(dx, sdx)));
    const f2_t k = f2_fma(f2_mul(dsd, inv2), f2_pack(-2.5f, -2.5f), q[7]);
    const f2_t cd = f2_fma(inv5, k, f2_mul(q[3], inv3));
    ax = f2_fma(inv5, sdx, f2_fma(cd, dx, ax));
    ay = f2_fma(inv5, sdy, f2_fma(cd, dy, ay));
    az = f2_fma(inv5, sdz, f2_fma(cd, dz, az));
}

template <bool CLAMP>
__device__ __forceinline__ void group_pair(f2_t xj, f2_t yj, f2_t zj, f2_t mj, f2_t xi, f2_t yi,
                                           f2_t zi, f2_t eps2, f2_t& ax, f2_t& ay, f2_t& az) {
    const f2_t dx = f2_sub(xj, xi);
    const f2_t dy = f2_sub(yj, yi);
    const f2_t dz = f2_sub(zj, zi);
    f2_t r2 = f2_fma(dz, dz, eps2);
    r2 = f2_fma(dy, dy, r2);
    r2 = f2_fma(dx, dx, r2);
    float r2a, r2b;
    f2_unpack(r2, r2a, r2b);
    if (CLAMP) {
        r2a = fmaxf(r2a, 1e-8f);
        r2b = fmaxf(r2b, 1e-8f);
    }
    const f2_t inv = f2_pack(rsqrt_mufu(r2a), rsqrt_mufu(r2b));
    const f2_t s3 = f2_mul(f2_mul(mj, inv), f2_mul(inv, inv));
    ax = f2_fma(dx, s3, ax);
    ay = f2_fma(dy, s3, ay);
    az = f2_fma(dz, s3, az);
}

// The pair term with positions split as FP32 hi + lo (frozen acceptance):
// d = (x_j - x_i) + (lo_j - lo_i), so a close pair's difference keeps the
// bits the FP32 rounding of its absolute positions drops.
template <bool CLAMP>
__device__ __forceinline__ void group_pair_lo(f2_t xj, f2_t yj, f2_t zj, f2_t mj, f2_t lxj,
                                              f2_t lyj, f2_t lzj, f2_t xi, f2_t yi, f2_t zi,
                                              f2_t lxi, f2_t lyi, f2_t lzi, f2_t eps2, f2_t& ax,
                                              f2_t& ay, f2_t& az) {
    const f2_t dx = f2_add(f2_sub(xj, xi), f2_sub(lxj, lxi));
    const f2_t dy = f2_add(f2_sub(yj, yi), f2_sub(lyj, lyi));
    const f2_t dz = f2_add(f2_sub(zj, zi), f2_sub(lzj, lzi));
    f2_t r2 = f2_fma(dz, dz, eps2);
    r2 = f2_fma(dy, dy, r2);
    r2 = f2_fma(dx, dx, r2);
    float r2a, r2b;
    f2_unpack(r2, r2a, r2b);
    if (CLAMP) {
        r2a = fmaxf(r2a, 1e-8f);
        r2b = fmaxf(r2b, 1e-8f);
    }
    const f2_t inv = f2_pack(rsqrt_mufu(r2a), rsqrt_mufu(r2b));
    const f2_t s3 = f2_mul(f2_mul(mj, inv), f2_mul(inv, inv));
    ax = f2_fma(dx, s3, ax);
    ay = f2_fma(dy, s3, ay);
    az = f2_fma(dz, s3, az);
}

// BPL bodies per lane: a group of 32 BPL consecutive leaves per warp (lane l
// holds leaves l, l + 32, ...); every list entry is evaluated for all of them.
// SMACC: the per-body two-sum accumulators (6 BPL packed values per lane)
// live in shared memory instead of registers; they are touched once per list
// evaluation, and the registers they free allow more resident warps.
// EMIT: cells accepted with the group box's nearest point inside the tight
// ratio (the learned correction's band) are recorded in t.cand; a group
// with more than t.cand_cap of them is handed to the per-body walk.
template <bool CLAMP, int BPL, int ORDER, int EUNR, bool SMACC, bool FROZEN = false,
          bool EMIT = false, int NPL = 1>
__device__ __forceinline__ void group_walk_one(const double* __restrict__ y, double* __restrict__ f,
                                               int n, float eps2v, const TreeState& t,
                                               int stack_cap, unsigned* err,
                                               unsigned char* smem_raw, const int gw) {
    GroupSmem& S = *reinterpret_cast<GroupSmem*>(smem_raw);
    QuadLists& Q = *reinterpret_cast<QuadLists*>(smem_raw + sizeof(GroupSmem));
    int* stacks = reinterpret_cast<int*>(smem_raw + sizeof(GroupSmem) +
                                         (ORDER == 2 ? sizeof(QuadLists) : 0));
    f2_t* acc_sm = reinterpret_cast<f2_t*>(stacks + kGWWarps * stack_cap) + threadIdx.x;
    f2_t acc_reg[SMACC ? 1 : 6 * BPL];
    // slot (3 b + component) * 2 + {0: high part, 1: low part}
    auto slot = [&](int q) -> f2_t& {
        if constexpr (SMACC) return acc_sm[q * kGWThreads];
        else return acc_reg[q];
    };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // me: the bodies' positions for the forces; mb: for the group's box (with
    // FROZEN, the positions of the step's build, as every acceptance test)
    float4 me[BPL], mb[BPL];
#pragma unroll
    for (int b = 0; b < BPL; ++b) {
        me[b] = __ldg(&t.node4[n + gw * 32 * BPL + b * 32 + lane]);
        mb[b] = FROZEN ? __ldg(&t.node4_acc[n + gw * 32 * BPL + b * 32 + lane]) : me[b];
    }
    // bounding box of the group
    float lo[3] = {mb[0].x, mb[0].y, mb[0].z}, hi[3] = {mb[0].x, mb[0].y, mb[0].z};
#pragma unroll
    for (int b = 1; b < BPL; ++b) {
        lo[0] = fminf(lo[0], mb[b].x);
        lo[1] = fminf(lo[1], mb[b].y);
        lo[2] = fminf(lo[2], mb[b].z);
        hi[0] = fmaxf(hi[0], mb[b].x);
        hi[1] = fmaxf(hi[1], mb[b].y);
        hi[2] = fmaxf(hi[2], mb[b].z);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    // the box as centre and half extent: the nearest point's offset on an
    // axis is max(|x - centre| - half, 0)
    float cb[3], hb[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        cb[a] = 0.5f * (lo[a] + hi[a]);
        hb[a] = 0.5f * (hi[a] - lo[a]);
    }
    int* stack = stacks + warp * stack_cap;
    float* lx = S.lx[warp];
    float* ly = S.ly[warp];
    float* lz = S.lz[warp];
    float* lm = S.lm[warp];
    const uint32_t ax_addr = smem_addr(lx), ay_addr = smem_addr(ly);
    const uint32_t az_addr = smem_addr(lz), am_addr = smem_addr(lm);
    const f2_t eps2 = f2_pack(eps2v, eps2v);
    const f2_t zero = f2_pack(0.f, 0.f);
    f2_t xi[BPL], yi[BPL], zi[BPL];
    // FROZEN: the bodies' FP32 residuals, and per-warp residual lists beside
    // the interaction list (after the shared-memory accumulators; zero for
    // cells)
    f2_t xil[FROZEN ? BPL : 1], yil[FROZEN ? BPL : 1], zil[FROZEN ? BPL : 1];
    float* llx = reinterpret_cast<float*>(reinterpret_cast<f2_t*>(stacks + kGWWarps * stack_cap) +
                                          (SMACC ? kGWThreads * 6 * BPL : 0)) + warp * kGWList;
    float* lly = llx + kGWWarps * kGWList;
    float* llz = lly + kGWWarps * kGWList;
#pragma unroll
    for (int b = 0; b < BPL; ++b) {
        xi[b] = f2_pack(me[b].x, me[b].x);
        yi[b] = f2_pack(me[b].y, me[b].y);
        zi[b] = f2_pack(me[b].z, me[b].z);
        if constexpr (FROZEN) {
            const float4 lo = __ldg(&t.leaf_lo[gw * 32 * BPL + b * 32 + lane]);
            xil[b] = f2_pack(lo.x, lo.x);
            yil[b] = f2_pack(lo.y, lo.y);
            zil[b] = f2_pack(lo.z, lo.z);
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) slot(6 * b + q) = zero;
    }
    const unsigned lt = (1u << lane) - 1u;
    unsigned long long tests = 0, inter = 0;
    if (lane == 0) stack[0] = 0;
    __syncwarp();
    int sp = 1, lc = 0, peak = 1, ec = 0;
    bool overflow = false, abandoned = false;
    const unsigned long long test_cap = t.test_cap != 0 ? t.test_cap : t.cap_state[0];

    auto evaluate = [&]() {
        // pad to a whole quad with massless entries
        const int pad = (4 - (lc & 3)) & 3;
        if (lane < pad) {
            lx[lc + lane] = 0.f;
            ly[lc + lane] = 0.f;
            lz[lc + lane] = 0.f;
            lm[lc + lane] = 0.f;
            if constexpr (FROZEN) {
                llx[lc + lane] = 0.f;
                lly[lc + lane] = 0.f;
                llz[lc + lane] = 0.f;
            }
        }
        __syncwarp();
        f2_t ax[BPL], ay[BPL], az[BPL], bx[BPL], by[BPL], bz[BPL];
#pragma unroll
        for (int b = 0; b < BPL; ++b) ax[b] = ay[b] = az[b] = bx[b] = by[b] = bz[b] = zero;
        const int quads = (lc + 3) >> 2;
        if constexpr (FROZEN) {
            const uint32_t lx_addr = smem_addr(llx), ly_addr = smem_addr(lly);
            const uint32_t lz_addr = smem_addr(llz);
#pragma unroll 1
            for (int r = 0; r < quads; ++r) {
                const float4 X = lds128(ax_addr + 16u * r);
                const float4 Y = lds128(ay_addr + 16u * r);
                const float4 Z = lds128(az_addr + 16u * r);
                const float4 M = lds128(am_addr + 16u * r);
                const float4 LX = lds128(lx_addr + 16u * r);
                const float4 LY = lds128(ly_addr + 16u * r);
                const float4 LZ = lds128(lz_addr + 16u * r);
#pragma unroll
                for (int b = 0; b < BPL; ++b) {
                    group_pair_lo<CLAMP>(f2_pack(X.x, X.y), f2_pack(Y.x, Y.y), f2_pack(Z.x, Z.y),
                                         f2_pack(M.x, M.y), f2_pack(LX.x, LX.y),
                                         f2_pack(LY.x, LY.y), f2_pack(LZ.x, LZ.y), xi[b], yi[b],
                                         zi[b], xil[b], yil[b], zil[b], eps2, ax[b], ay[b], az[b]);
                    group_pair_lo<CLAMP>(f2_pack(X.z, X.w), f2_pack(Y.z, Y.w), f2_pack(Z.z, Z.w),
                                         f2_pack(M.z, M.w), f2_pack(LX.z, LX.w),
                                         f2_pack(LY.z, LY.w), f2_pack(LZ.z, LZ.w), xi[b], yi[b],
                                         zi[b], xil[b], yil[b], zil[b], eps2, bx[b], by[b], bz[b]);
                }
            }
        } else {
#pragma unroll EUNR
        for (int r = 0; r < quads; ++r) {
            const float4 X = lds128(ax_addr + 16u * r);
            const float4 Y = lds128(ay_addr + 16u * r);
            const float4 Z = lds128(az_addr + 16u * r);
            const float4 M = lds128(am_addr + 16u * r);
#pragma unroll
            for (int b = 0; b < BPL; ++b) {
                group_pair<CLAMP>(f2_pack(X.x, X.y), f2_pack(Y.x, Y.y), f2_pack(Z.x, Z.y),
                                  f2_pack(M.x, M.y), xi[b], yi[b], zi[b], eps2, ax[b], ay[b],
                                  az[b]);
                group_pair<CLAMP>(f2_pack(X.z, X.w), f2_pack(Y.z, Y.w), f2_pack(Z.z, Z.w),
                                  f2_pack(M.z, M.w), xi[b], yi[b], zi[b], eps2, bx[b], by[b],
                                  bz[b]);
            }
        }
        }
#pragma unroll
        for (int b = 0; b < BPL; ++b) {
            f2_two_sum(slot(6 * b + 0), slot(6 * b + 1), f2_add(ax[b], bx[b]));
            f2_two_sum(slot(6 * b + 2), slot(6 * b + 3), f2_add(ay[b], by[b]));
            f2_two_sum(slot(6 * b + 4), slot(6 * b + 5), f2_add(az[b], bz[b]));
        }
        inter += (unsigned long long)lc;
        lc = 0;
        __syncwarp();
    };

    int qc = 0;  // entries in the quadrupole list
    auto evaluate_quad = [&]() {
        float(*v)[kGWQList] = Q.v[warp];
        const int pad = (4 - (qc & 3)) & 3;
        if (lane < pad) {  // massless, momentless padding
#pragma unroll
            for (int fld = 0; fld < kGWQFields; ++fld) v[fld][qc + lane] = 0.f;
        }
        __syncwarp();
        const uint32_t base = smem_addr(&v[0][0]);
        const int quads = (qc + 3) >> 2;
        f2_t ax[BPL], ay[BPL], az[BPL];
#pragma unroll
        for (int b = 0; b < BPL; ++b) ax[b] = ay[b] = az[b] = zero;
#pragma unroll 1
        for (int r = 0; r < quads; ++r) {
            f2_t lo2[kGWQFields], hi2[kGWQFields];
#pragma unroll
            for (int fld = 0; fld < kGWQFields; ++fld) {
                const float4 w = lds128(base + 4u * (uint32_t)(fld * kGWQList) + 16u * r);
                lo2[fld] = f2_pack(w.x, w.y);
                hi2[fld] = f2_pack(w.z, w.w);
            }
#pragma unroll
            for (int b = 0; b < BPL; ++b) {
                quad_pair<CLAMP>(lo2, xi[b], yi[b], zi[b], eps2, ax[b], ay[b], az[b]);
                quad_pair<CLAMP>(hi2, xi[b], yi[b], zi[b], eps2, ax[b], ay[b], az[b]);
            }
        }
#pragma unroll
        for (int b = 0; b < BPL; ++b) {
            f2_two_sum(slot(6 * b + 0), slot(6 * b + 1), ax[b]);
            f2_two_sum(slot(6 * b + 2), slot(6 * b + 3), ay[b]);
            f2_two_sum(slot(6 * b + 4), slot(6 * b + 5), az[b]);
        }
        inter += (unsigned long long)qc;
        qc = 0;
        __syncwarp();
    };

    // NPL nodes per lane and step: 16 NPL popped entries, 32 NPL children
    // tested, NPL independent node loads in flight per lane
    while (sp > 0) {
        const int k = min(sp, 16 * NPL);
        int c[NPL];
#pragma unroll
        for (int w = 0; w < NPL; ++w) {
            const int slot = lane + 32 * w;
            c[w] = slot < 2 * k ? 2 * stack[sp - 1 - (slot >> 1)] + (slot & 1) : 0;
        }
        __syncwarp();
        sp -= k;
        // issued before a full list is evaluated, which covers their latency;
        // lanes past the popped entries read record 0 (unused, zeroed), and
        // leaves' second moments are zero
        float4 nd[NPL], nda[NPL], nq0[NPL], nq1[NPL];
        float ndm[NPL];
#pragma unroll
        for (int w = 0; w < NPL; ++w) {
            nd[w] = __ldg(&t.node4[c[w]]);
            nda[w] = FROZEN ? __ldg(&t.node4_acc[c[w]]) : nd[w];  // acceptance record
            ndm[w] = __ldg(&t.nodem[c[w]]);
            if (ORDER == 2) {
                nq0[w] = __ldg(&t.quad[2 * c[w]]);
                nq1[w] = __ldg(&t.quad[2 * c[w] + 1]);
            }
        }
        if (lc > kGWList - 32 * NPL) evaluate();  // room for this step's entries
        if (ORDER == 2 && qc > kGWQList - 32 * NPL) evaluate_quad();
        bool accept[NPL], open[NPL], band[NPL];
#pragma unroll
        for (int w = 0; w < NPL; ++w) {
            accept[w] = open[w] = band[w] = false;
            if (c[w] != 0) {  // slots past the popped entries hold 0
                if (c[w] >= n) {
                    accept[w] = true;
                } else {
                    const float ex = fmaxf(fabsf(nda[w].x - cb[0]) - hb[0], 0.f);
                    const float ey = fmaxf(fabsf(nda[w].y - cb[1]) - hb[1], 0.f);
                    const float ez = fmaxf(fabsf(nda[w].z - cb[2]) - hb[2], 0.f);
                    const float dmin2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
                    accept[w] = dmin2 > nda[w].w;
                    open[w] = !accept[w];
                    if constexpr (EMIT) band[w] = accept[w] && dmin2 <= nda[w].w * t.band2;
                }
            }
        }
        // every popped entry stands for two tested children, except the root's
        // stand-in entry 0 at the first step (its child 0 is not a node)
        tests += (unsigned long long)(2 * k);
        if (tests > test_cap) {  // a group spread over much of the system:
            abandoned = true;      // its bodies are walked one by one instead
            break;
        }
        if constexpr (EMIT) {
            unsigned bm[NPL];
            int nb = 0;
#pragma unroll
            for (int w = 0; w < NPL; ++w) {
                bm[w] = __ballot_sync(0xffffffffu, band[w]);
                nb += __popc(bm[w]);
            }
            if (ec + nb > t.cand_cap) {  // walked body by body instead
                abandoned = true;
                break;
            }
#pragma unroll
            for (int w = 0; w < NPL; ++w) {
                if (band[w]) t.cand[(size_t)gw * t.cand_cap + ec + __popc(bm[w] & lt)] = c[w];
                ec += __popc(bm[w]);
            }
        }
        // cells with moments go to the quadrupole list (ORDER 2), the rest
        // (leaves, or every node for ORDER 1) to the monopole list
#pragma unroll
        for (int w = 0; w < NPL; ++w) {
            const bool to_quad = ORDER == 2 && accept[w] && c[w] < n;
            const bool to_mono = accept[w] && !to_quad;
            const unsigned am = __ballot_sync(0xffffffffu, to_mono);
            if (to_mono) {
                const int q = lc + __popc(am & lt);
                lx[q] = nd[w].x;
                ly[q] = nd[w].y;
                lz[q] = nd[w].z;
                lm[q] = ndm[w];
                if constexpr (FROZEN) {  // leaves carry their residuals, cells none
                    const float4 lo = c[w] >= n ? __ldg(&t.leaf_lo[c[w] - n])
                                                : make_float4(0.f, 0.f, 0.f, 0.f);
                    llx[q] = lo.x;
                    lly[q] = lo.y;
                    llz[q] = lo.z;
                }
            }
            lc += __popc(am);
            if (ORDER == 2) {
                const unsigned aq = __ballot_sync(0xffffffffu, to_quad);
                if (to_quad) {
                    float(*v)[kGWQList] = Q.v[warp];
                    const int q = qc + __popc(aq & lt);
                    const float4 q0 = nq0[w], q1 = nq1[w];
                    v[0][q] = nd[w].x;
                    v[1][q] = nd[w].y;
                    v[2][q] = nd[w].z;
                    v[3][q] = ndm[w];
                    v[4][q] = q0.x;
                    v[5][q] = q0.y;
                    v[6][q] = q0.z;
                    v[7][q] = q0.w;
                    v[8][q] = q1.x;
                    v[9][q] = q1.y;
                    v[10][q] = q1.z;
                }
                qc += __popc(aq);
            }
        }
        unsigned om[NPL];
        int npush = 0;
#pragma unroll
        for (int w = 0; w < NPL; ++w) {
            om[w] = __ballot_sync(0xffffffffu, open[w]);
            npush += __popc(om[w]);
        }
        if (sp + npush > stack_cap) {  // beyond 48 entries per level: reported, never written
            overflow = true;
            break;
        }
        int base = sp;
#pragma unroll
        for (int w = 0; w < NPL; ++w) {
            if (open[w]) stack[base + __popc(om[w] & lt)] = c[w];
            base += __popc(om[w]);
        }
        sp += npush;
        peak = max(peak, sp);
        __syncwarp();
    }
    if (overflow) {
        if (lane == 0) atomicOr(err, kDevErrWalkOverflow);
    }
    tests -= 1;  // child 0 of the first step
    if (lane == 0) {
        atomicAdd(&t.counters[0], tests);
        atomicMax(&t.counters[2], (unsigned long long)peak);
    }
    if constexpr (EMIT) {
        if (lane == 0) t.cand_n[gw] = abandoned ? 0u : (unsigned)ec;
    }
    if (abandoned) {
        if (lane == 0) {
            t.fb_list[atomicAdd(t.fb_count, 1u)] = gw;
            atomicAdd(&t.counters[3], 1ull);
        }
        return;
    }
    if (lc > 0) evaluate();
    if (ORDER == 2 && qc > 0) evaluate_quad();
#pragma unroll
    for (int bb = 0; bb < BPL; ++bb) {
        float h0, h1, l0, l1;
        const int b = t.body_n[n + gw * 32 * BPL + bb * 32 + lane];
        f[b] = y[3 * n + b];
        f[n + b] = y[4 * n + b];
        f[2 * n + b] = y[5 * n + b];
        f2_unpack(slot(6 * bb + 0), h0, h1);
        f2_unpack(slot(6 * bb + 1), l0, l1);
        f[3 * n + b] = ((double)h0 + (double)h1) + ((double)l0 + (double)l1);
        f2_unpack(slot(6 * bb + 2), h0, h1);
        f2_unpack(slot(6 * bb + 3), l0, l1);
        f[4 * n + b] = ((double)h0 + (double)h1) + ((double)l0 + (double)l1);
        f2_unpack(slot(6 * bb + 4), h0, h1);
        f2_unpack(slot(6 * bb + 5), l0, l1);
        f[5 * n + b] = ((double)h0 + (double)h1) + ((double)l0 + (double)l1);
    }
    if (lane == 0) atomicAdd(&t.counters[1], inter * 32ull * BPL);
}

// Persistent over the groups (n is a power of two >= 32 BPL, so groups are
// full): each warp starts at its own group and then takes the next untaken
// one from a counter, so the last groups spread over all warps instead of
// leaving a partial wave.  A group's forces do not depend on which warp
// computes it.
template <bool CLAMP, int MINB, int BPL, int ORDER, int EUNR = 2, bool SMACC = false,
          bool FROZEN = false, bool EMIT = false, int NPL = 1>
__global__ void __launch_bounds__(kGWThreads, MINB)
bh_group_walk_kernel(const double* __restrict__ y, double* __restrict__ f, int n, float eps2v,
                     TreeState t, int stack_cap, unsigned* err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int groups = n / (32 * BPL);
    int gw = blockIdx.x * kGWWarps + (threadIdx.x >> 5);
    while (gw < groups) {
        group_walk_one<CLAMP, BPL, ORDER, EUNR, SMACC, FROZEN, EMIT, NPL>(y, f, n, eps2v, t,
                                                                         stack_cap, err, smem_raw,
                                                                         gw);
        int next = 0;
        if (lane == 0) next = (int)atomicAdd(&t.fb_count[1], 1u);
        gw = gridDim.x * kGWWarps + __shfl_sync(0xffffffffu, next, 0);
    }
}

// The group walk's test cap: ratio x the median node tests of kCapSamples
// groups spread over the leaves (every stride-th), a function of the tree
// alone, so that equal trees give equal forces.  One block, one warp per
// sample, each running the group walk's traversal without its force
// evaluation.  The samples walk in rounds of doubling test limits (4096,
// 8192, ...) and stop once more than half have finished: the median is then
// known without walking the samples above it, which are the slow ones.
template <int BPL>
__global__ void __launch_bounds__(kCapSamples * 32, 1)
bh_test_cap_kernel(int n, int stride, int samples, TreeState t, int stack_cap, unsigned ratio) {
    extern __shared__ int cap_stacks[];
    __shared__ unsigned long long counts[kCapSamples];
    __shared__ int finished[kCapSamples];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool active = warp < samples;
    const int gw = warp * stride;
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    if (active) {
#pragma unroll
        for (int b = 0; b < BPL; ++b) {
            const float4 me = __ldg(&t.node4[n + gw * 32 * BPL + b * 32 + lane]);
            lo[0] = fminf(lo[0], me.x);
            lo[1] = fminf(lo[1], me.y);
            lo[2] = fminf(lo[2], me.z);
            hi[0] = fmaxf(hi[0], me.x);
            hi[1] = fmaxf(hi[1], me.y);
            hi[2] = fmaxf(hi[2], me.z);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    float cb[3], hb[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        cb[a] = 0.5f * (lo[a] + hi[a]);
        hb[a] = 0.5f * (hi[a] - lo[a]);
    }
    int* stack = cap_stacks + warp * stack_cap;
    const unsigned lt = (1u << lane) - 1u;
    if (lane == 0) stack[0] = 0;
    __syncwarp();
    int sp = active ? 1 : 0;
    unsigned long long tests = 0, limit = 4096;
    for (int round = 0; round < 40; ++round, limit *= 2) {
        // two node tests per lane and step (32 entries popped): the same
        // tests as the walk in another order, with two loads in flight
        while (sp > 0 && tests <= limit) {
            const int k = min(sp, 32);
            int c[2];
            bool open[2];
#pragma unroll
            for (int w = 0; w < 2; ++w) {
                const int slot = lane + 32 * w;
                c[w] = slot < 2 * k ? 2 * stack[sp - 1 - (slot >> 1)] + (slot & 1) : 0;
            }
            __syncwarp();
            sp -= k;
            int nvalid = 0;
#pragma unroll
            for (int w = 0; w < 2; ++w) {
                open[w] = false;
                if (c[w] != 0 && c[w] < n) {
                    const float4 nd = __ldg(&t.node4[c[w]]);
                    const float ex = fmaxf(fabsf(nd.x - cb[0]) - hb[0], 0.f);
                    const float ey = fmaxf(fabsf(nd.y - cb[1]) - hb[1], 0.f);
                    const float ez = fmaxf(fabsf(nd.z - cb[2]) - hb[2], 0.f);
                    open[w] = !(fmaf(ex, ex, fmaf(ey, ey, ez * ez)) > nd.w);
                }
                nvalid += __popc(__ballot_sync(0xffffffffu, c[w] != 0));
            }
            tests += (unsigned long long)nvalid;
            const unsigned om0 = __ballot_sync(0xffffffffu, open[0]);
            const unsigned om1 = __ballot_sync(0xffffffffu, open[1]);
            const int npush = __popc(om0) + __popc(om1);
            if (sp + npush > stack_cap) {  // the walk itself reports the overflow
                sp = 0;
                break;
            }
            if (open[0]) stack[sp + __popc(om0 & lt)] = c[0];
            if (open[1]) stack[sp + __popc(om0) + __popc(om1 & lt)] = c[1];
            sp += npush;
            __syncwarp();
        }
        if (lane == 0 && active) {
            counts[warp] = tests;
            finished[warp] = sp == 0;
        }
        __syncthreads();
        int fin = 0;
        for (int j = 0; j < samples; ++j) fin += finished[j];
        if (2 * fin > samples) break;  // the same decision in every thread
        __syncthreads();
    }
    // finished samples hold their counts, the others a count above the last
    // limit: the value of rank samples / 2 is the median
    if (threadIdx.x < samples) {
        const unsigned long long v = counts[threadIdx.x];
        int rank = 0;
        for (int j = 0; j < samples; ++j)
            rank += (counts[j] < v || (counts[j] == v && j < (int)threadIdx.x)) ? 1 : 0;
        if (rank == samples / 2) t.cap_state[0] = max((unsigned long long)ratio * v, 4096ull);
    }
}

// The bodies of the groups the group walk gave up on, one warp per body: the
// group walk's traversal with the body's own point as the group's box, so
// a node is accepted when d^2 > crit^2 from the body (the reference's
// per-body rule; leaves always, the body's own leaf adding zero), 32 node
// tests per step.  Each lane evaluates the nodes it accepted (with the
// quadrupole term for cells with ORDER 2) into two-sum accumulators; the
// warp's sum is formed in FP64.
template <bool CLAMP, int BPL, int ORDER, bool FROZEN = false>
__global__ void __launch_bounds__(kGWThreads)
bh_body_walk_kernel(const double* __restrict__ y, double* __restrict__ f, int n, float eps2,
                    TreeState t, int stack_cap, unsigned* err) {
    extern __shared__ int body_stacks[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    int* stack = body_stacks + warp * stack_cap;
    const unsigned bodies = *t.fb_count * 32u * BPL;
    const unsigned warps = gridDim.x * kGWWarps;
    for (unsigned w = blockIdx.x * kGWWarps + warp; w < bodies; w += warps) {
        const int gw = t.fb_list[w / (32 * BPL)];
        const int leaf = n + gw * 32 * BPL + (int)(w % (32 * BPL));
        const float4 me = __ldg(&t.node4[leaf]);
        // with FROZEN the acceptance tests use the step build's records, and
        // pair differences add the leaves' FP32 residuals
        const float4 mea = FROZEN ? __ldg(&t.node4_acc[leaf]) : me;
        const float4 mel = FROZEN ? __ldg(&t.leaf_lo[leaf - n]) : make_float4(0.f, 0.f, 0.f, 0.f);
        float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
        // (h, l) += p with the rounding error of h + p kept in l
        auto add = [](float& h, float& l, float p) {
            const float s = h + p, bp = s - h;
            l += (h - (s - bp)) + (p - bp);
            h = s;
        };
        unsigned long long inter = 0;
        __syncwarp();
        if (lane == 0) stack[0] = 0;
        __syncwarp();
        int sp = 1;
        while (sp > 0) {
            const int k = min(sp, 16);
            int c = 0;
            if (lane < 2 * k) c = 2 * stack[sp - 1 - (lane >> 1)] + (lane & 1);
            __syncwarp();
            sp -= k;
            const bool valid = lane < 2 * k && c != 0;
            bool accept = false, open = false;
            float dx = 0.f, dy = 0.f, dz = 0.f;
            if (valid) {
                const float4 nd = __ldg(&t.node4[c]);
                dx = nd.x - me.x;
                dy = nd.y - me.y;
                dz = nd.z - me.z;
                if (FROZEN) {
                    const float4 lo =
                        c >= n ? __ldg(&t.leaf_lo[c - n]) : make_float4(0.f, 0.f, 0.f, 0.f);
                    dx += lo.x - mel.x;
                    dy += lo.y - mel.y;
                    dz += lo.z - mel.z;
                    const float4 nda = __ldg(&t.node4_acc[c]);
                    const float ax = nda.x - mea.x, ay = nda.y - mea.y, az = nda.z - mea.z;
                    accept = c >= n || fmaf(ax, ax, fmaf(ay, ay, az * az)) > nda.w;
                } else {
                    accept = c >= n || fmaf(dx, dx, fmaf(dy, dy, dz * dz)) > nd.w;
                }
                open = !accept;
            }
            if (accept) {
                float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
                if (CLAMP) r2 = fmaxf(r2, 1e-8f);
                const float inv = rsqrt_mufu(r2);
                const float inv2 = inv * inv, inv3 = inv2 * inv;
                const float s3 = __ldg(&t.nodem[c]) * inv3;
                float ax = dx * s3, ay = dy * s3, az = dz * s3;
                if (ORDER == 2 && c < n) {
                    // a += d k' / r^5 + (S d) / r^5, k' = tr S / 2 - 2.5 dSd / r^2,
                    // with the stored S = -3 M
                    const float4 q0 = __ldg(&t.quad[2 * c]), q1 = __ldg(&t.quad[2 * c + 1]);
                    const float inv5 = inv3 * inv2;
                    const float sx = fmaf(q1.y, dz, fmaf(q1.x, dy, q0.x * dx));
                    const float sy = fmaf(q1.z, dz, fmaf(q0.y, dy, q1.x * dx));
                    const float sz = fmaf(q0.z, dz, fmaf(q1.z, dy, q1.y * dx));
                    const float dsd = fmaf(dz, sz, fmaf(dy, sy, dx * sx));
                    const float ck = inv5 * fmaf(-2.5f * dsd, inv2, q0.w);
                    ax += fmaf(ck, dx, inv5 * sx);
                    ay += fmaf(ck, dy, inv5 * sy);
                    az += fmaf(ck, dz, inv5 * sz);
                }
                add(hx, lx, ax);
                add(hy, ly, ay);
                add(hz, lz, az);
            }
            inter += (unsigned long long)__popc(__ballot_sync(0xffffffffu, accept));
            const unsigned om = __ballot_sync(0xffffffffu, open);
            const int npush = __popc(om);
            if (sp + npush > stack_cap) {  // beyond 48 entries per level: reported, never written
                if (lane == 0) atomicOr(err, kDevErrWalkOverflow);
                break;
            }
            if (open) stack[sp + __popc(om & lt)] = c;
            sp += npush;
            __syncwarp();
        }
        double ax = (double)hx + (double)lx, ay = (double)hy + (double)ly;
        double az = (double)hz + (double)lz;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            ax += __shfl_xor_sync(0xffffffffu, ax, o);
            ay += __shfl_xor_sync(0xffffffffu, ay, o);
            az += __shfl_xor_sync(0xffffffffu, az, o);
        }
        if (lane == 0) {
            const int b = t.body_n[leaf];
            f[b] = y[3 * n + b];
            f[n + b] = y[4 * n + b];
            f[2 * n + b] = y[5 * n + b];
            f[3 * n + b] = ax;
            f[4 * n + b] = ay;
            f[5 * n + b] = az;
            atomicAdd(&t.counters[1], inter);
        }
    }
}

// Second central mass moments per node, bottom-up in FP32 (parallel axis:
// M = sum over children of M_c + m_c d d^T, d = child centre - node centre);
// leaves have none.
__global__ void quad_leaf_kernel(float4* quad, int n) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        quad[2 * (size_t)(n + p)] = make_float4(0.f, 0.f, 0.f, 0.f);
        quad[2 * (size_t)(n + p) + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

__device__ __forceinline__ void quad_node(size_t idx, TreeState& t) {
    const float4 pc = t.node4[idx];
    float xx = 0.f, yy = 0.f, zz = 0.f, xy = 0.f, xz = 0.f, yz = 0.f;
    for (int side = 0; side < 2; ++side) {
        const size_t c = 2 * idx + side;
        const float4 cc = t.node4[c];
        const float mc = t.nodem[c];
        const float4 q0 = t.quad[2 * c], q1 = t.quad[2 * c + 1];
        // parallel-axis shift of the child's moments, in the stored scale
        // S = -3 M
        const float dx = cc.x - pc.x, dy = cc.y - pc.y, dz = cc.z - pc.z;
        const float w = -3.f * mc;
        xx += q0.x + w * dx * dx;
        yy += q0.y + w * dy * dy;
        zz += q0.z + w * dz * dz;
        xy += q1.x + w * dx * dy;
        xz += q1.y + w * dx * dz;
        yz += q1.z + w * dy * dz;
    }
    t.quad[2 * idx] = make_float4(xx, yy, zz, 0.5f * (xx + yy + zz));
    t.quad[2 * idx + 1] = make_float4(xy, xz, yz, 0.f);
}

// Levels [lv_lo, lv_hi) of the moments, bottom-up, in one launch: block b
// owns the subtree under node 2^lv_lo + b (at most 9 levels, 256 nodes at
// its bottom), a block barrier between levels.
__global__ void __launch_bounds__(256) quad_levels_kernel(int lv_lo, int lv_hi, TreeState t) {
    const size_t root = ((size_t)1 << lv_lo) + blockIdx.x;
    for (int lv = lv_hi - 1; lv >= lv_lo; --lv) {
        const int span = 1 << (lv - lv_lo);
        const size_t first = root << (lv - lv_lo);
        for (int k = threadIdx.x; k < span; k += blockDim.x) quad_node(first + k, t);
        __syncthreads();
    }
}

nbg_status tree_quadrupoles(nbg_engine* e) {
    TreeState* t = e->tree;
    const int n = (int)t->n;
    if (t->quad == nullptr) {
        NBG_CUDA(e, cudaMalloc(&t->quad, 2 * t->size * sizeof(float4)));
        // leaves have no moments; only inner nodes are written afterwards
        quad_leaf_kernel<<<grid_for(n, 256, (unsigned)e->sm_count * 8u), 256, 0, e->stream>>>(t->quad, n);
        NBG_LAUNCHED(e, "quad_leaf_kernel");
    }
    for (int hi = t->levels; hi > 0;) {
        const int lo = std::max(0, hi - 9);
        quad_levels_kernel<<<1u << lo, 256, 0, e->stream>>>(lo, hi, *t);
        NBG_LAUNCHED(e, "quad_levels_kernel");
        hi = lo;
    }
    return NBG_OK;
}

}  // namespace

namespace {
// Residual of each leaf's FP32 position (frozen acceptance): lo = y - hi.
__global__ void leaf_lo_kernel(const double* __restrict__ y, int n, TreeState t) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int b = t.body_n[n + p];
        const float4 hi = t.node4[n + p];
        t.leaf_lo[p] = make_float4((float)(y[b] - (double)hi.x), (float)(y[n + b] - (double)hi.y),
                                   (float)(y[2 * n + b] - (double)hi.z), 0.f);
    }
}
}  // namespace

nbg_status bh_tree(nbg_engine* e, uint64_t step, const double* y, bool fp64_nodes, double lambda) {
    const TreeState* t = e->tree;
    const bool freeze = e->tune_get("bh.freeze_within_step", 0) != 0;
    bool build;
    if (t == nullptr || !t->built || (fp64_nodes && t->f32))
        build = true;
    else if (freeze && (t->node4_acc == nullptr || t->acc_step != t->built_step))
        build = true;  // no acceptance records of this step's build
    else if (freeze || e->tune_get("bh.refit_within_step", 0) != 0)
        build = step != t->built_step;
    else {
        const uint64_t rate = e->params.tree_build_rate;
        build = rate == 0 || step % rate == 0;
    }
    nbg_status s = build ? tree_build(e, y, fp64_nodes, lambda) : tree_refit(e, y, lambda);
    if (s != NBG_OK) return s;
    TreeState* tt = e->tree;
    if (build) {
        tt->built_step = step;
        if (freeze) {  // the acceptance records of this step
            if (tt->node4_acc == nullptr)
                NBG_CUDA(e, cudaMalloc(&tt->node4_acc, tt->size * sizeof(float4)));
            NBG_CUDA(e, cudaMemcpyAsync(tt->node4_acc, tt->node4, tt->size * sizeof(float4),
                                        cudaMemcpyDeviceToDevice, e->stream));
            tt->acc_step = step;
        }
    }
    if (freeze) {  // the leaves' residuals, at every build and refit
        if (tt->leaf_lo == nullptr)
            NBG_CUDA(e, cudaMalloc(&tt->leaf_lo, tt->n * sizeof(float4)));
        const int n = (int)tt->n;
        leaf_lo_kernel<<<grid_for(n, 256, (unsigned)e->sm_count * 8u), 256, 0, e->stream>>>(
            y, n, *tt);
        NBG_LAUNCHED(e, "leaf_lo_kernel");
    }
    return NBG_OK;
}

nbg_status bh_fcompute(nbg_engine* e, uint64_t step, const double* y, double* f) {
    const int n = (int)e->count;
    const double lambda = e->params.distance_to_node_radius_ratio;
    if (e->params.precision == NBG_PREC_FP64) {
        nbg_status s = bh_tree(e, step, y, true, lambda);
        if (s != NBG_OK) return s;
        ProfScope ps(e, NBG_K_BH_WALK);
        bh_walk_fp64_kernel<<<(n + 127) / 128, 128, 0, e->stream>>>(
            y, e->d_mass, f, n, e->params.traverse_type == NBG_TRAVERSE_NESTED_TREE ? 1 : 0,
            *e->tree, e->d_err);
        NBG_LAUNCHED(e, "bh_walk_fp64_kernel");
        return NBG_OK;
    }
    if (e->params.learned) return learned_fcompute(e, step, y, f);
    nbg_status s = bh_tree(e, step, y, false, lambda);
    if (s != NBG_OK) return s;
    return mixed_walk(e, y, f);
}

namespace {
nbg_status mixed_walk_impl(nbg_engine* e, const double* y, double* f, bool emit);
}  // namespace

// the emitting walk is one part of the learned walk, whose caller times it
nbg_status mixed_walk(nbg_engine* e, const double* y, double* f, bool emit) {
    if (emit) return mixed_walk_impl(e, y, f, true);
    ProfScope ps(e, NBG_K_BH_WALK);
    return mixed_walk_impl(e, y, f, false);
}

namespace {
nbg_status mixed_walk_impl(nbg_engine* e, const double* y, double* f, bool emit) {
    const int n = (int)e->count;
    TreeState* t = e->tree;
    const float eps2 = (float)(e->params.softening * e->params.softening);
    const bool clamp = !(e->params.softening > 0.0);
    if (e->tune_get("bh.walk", 1) == 1 && n >= 32) {
        // "bh.group": bodies per warp group (32 or 64); "bh.walk_blocks":
        // CTAs per SM the kernel's register budget is set for (3, 4, 5, 6 or
        // 8: 168, 128, 102, 80 or 64 registers; 3 for quadrupole cells only)
        // "bh.order": 1 monopole cells, 2 monopole + quadrupole cells
        const int order = e->tune_get("bh.order", 1) >= 2 ? 2 : 1;
        if (order == 2) {
            nbg_status qs = tree_quadrupoles(e);
            if (qs != NBG_OK) return qs;
        }
        const int stack_cap = group_stack_cap(t->levels);
        size_t smem = sizeof(GroupSmem) + (order == 2 ? sizeof(QuadLists) : 0) +
                      (size_t)kGWWarps * stack_cap * sizeof(int);
        // "bh.group": 32, 64 (default) or 128 bodies per warp group (128:
        // monopole cells only, accumulators in shared memory, 4 CTAs per SM)
        const bool frozen_req = e->tune_get("bh.freeze_within_step", 0) != 0;
        const int64_t gsz = e->tune_get("bh.group", 64);
        const int bpl = (gsz >= 128 && n >= 128 && order == 1 && !frozen_req) ? 4
                        : (gsz >= 64 && n >= 64) ? 2 : 1;
        // 64-body groups keep their accumulators in shared memory by default
        // and run 5 CTAs per SM ("bh.acc_smem" = 0: registers, 4 CTAs)
        const bool acc_smem = bpl == 2 && order == 1 && e->tune_get("bh.acc_smem", 1) != 0;
        // the quadrupole walk of 64-body groups runs 3 CTAs per SM by default
        // (164 registers, no spill; at 4 CTAs it spills and is 5 % slower)
        const int64_t wb = e->tune_get("bh.walk_blocks",
                                       bpl == 2 ? (order == 2 ? 3 : acc_smem ? 5 : 4) : 6);
        using WalkKernel = void (*)(const double*, double*, int, float, TreeState, int, unsigned*);
        WalkKernel kern;
        // frozen acceptance runs its own build of the default walk (64-body
        // groups, monopole cells, shared-memory accumulators, residual
        // lists; a 4-CTA register budget)
        const bool frozen = e->tune_get("bh.freeze_within_step", 0) != 0 &&
                            t->node4_acc != nullptr && t->acc_step == t->built_step &&
                            t->leaf_lo != nullptr;
        if (frozen && !(bpl == 2 && order == 1 && acc_smem))
            return set_error(e, NBG_ERR_UNSUPPORTED,
                             "bh.freeze_within_step runs the default group walk only "
                             "(64-body groups, monopole cells)");
        if (emit && (frozen || !(bpl == 2 && order == 1 && acc_smem)))
            return set_error(e, NBG_ERR_UNSUPPORTED,
                             "the learned correction on tensor cores runs on the default group "
                             "walk only (64-body groups, monopole cells, no frozen acceptance)");
#define NBG_GW(C, B) (wb >= 8 ? bh_group_walk_kernel<C, 8, B, 1> : wb >= 6 ? bh_group_walk_kernel<C, 6, B, 1> \
                      : wb >= 5 ? bh_group_walk_kernel<C, 5, B, 1> : bh_group_walk_kernel<C, 4, B, 1>)
        if (emit) {
            // the default monopole build (two node tests per lane and step),
            // recording the band cells
            smem += (size_t)kGWThreads * 6 * 2 * sizeof(f2_t);
            kern = clamp ? bh_group_walk_kernel<true, 5, 2, 1, 2, true, false, true, 2>
                         : bh_group_walk_kernel<false, 5, 2, 1, 2, true, false, true, 2>;
        } else if (bpl == 4) {
            smem += (size_t)kGWThreads * 6 * 4 * sizeof(f2_t);
            kern = clamp ? bh_group_walk_kernel<true, 4, 4, 1, 2, true>
                         : bh_group_walk_kernel<false, 4, 4, 1, 2, true>;
        } else if (frozen) {
            // the default build keeps its accumulators in shared memory, and
            // the frozen walk three residual lists per warp after them
            smem += (size_t)kGWThreads * 6 * 2 * sizeof(f2_t) +
                    (size_t)3 * kGWWarps * kGWList * sizeof(float);
            kern = clamp ? bh_group_walk_kernel<true, 4, 2, 1, 2, true, true>
                         : bh_group_walk_kernel<false, 4, 2, 1, 2, true, true>;
        }
        // quadrupole cells: one node test per lane and step by default (two
        // fill the quadrupole list twice as fast and gain nothing)
        else if (order == 2 && bpl == 2 && wb <= 3 && e->tune_get("bh.walk_npl", 1) >= 2)
            kern = clamp ? bh_group_walk_kernel<true, 3, 2, 2, 2, false, false, false, 2>
                         : bh_group_walk_kernel<false, 3, 2, 2, 2, false, false, false, 2>;
        else if (order == 2 && bpl == 2 && wb <= 3)
            kern = clamp ? bh_group_walk_kernel<true, 3, 2, 2> : bh_group_walk_kernel<false, 3, 2, 2>;
        else if (order == 2)
            kern = bpl == 2 ? (clamp ? bh_group_walk_kernel<true, 4, 2, 2> : bh_group_walk_kernel<false, 4, 2, 2>)
                            : (clamp ? bh_group_walk_kernel<true, 5, 1, 2> : bh_group_walk_kernel<false, 5, 1, 2>);
        else if (acc_smem) {
            // accumulators in shared memory (4 or 5 CTAs per SM); at 5 CTAs
            // "bh.eval_unroll" 1, 2 (default) or 4 quads per list step
            smem += (size_t)kGWThreads * 6 * 2 * sizeof(f2_t);
            const int64_t eu = e->tune_get("bh.eval_unroll", 2);
            if (wb >= 5 && eu >= 4)
                kern = clamp ? bh_group_walk_kernel<true, 5, 2, 1, 4, true>
                             : bh_group_walk_kernel<false, 5, 2, 1, 4, true>;
            else if (wb >= 5 && eu <= 1)
                kern = clamp ? bh_group_walk_kernel<true, 5, 2, 1, 1, true>
                             : bh_group_walk_kernel<false, 5, 2, 1, 1, true>;
            else if (wb >= 5 && e->tune_get("bh.walk_npl", 2) >= 2)
                // two node tests per lane and step (the default): half the
                // dependent traversal steps, two loads in flight
                kern = clamp ? bh_group_walk_kernel<true, 5, 2, 1, 2, true, false, false, 2>
                             : bh_group_walk_kernel<false, 5, 2, 1, 2, true, false, false, 2>;
            else
                kern = clamp ? (wb >= 5 ? bh_group_walk_kernel<true, 5, 2, 1, 2, true>
                                        : bh_group_walk_kernel<true, 4, 2, 1, 2, true>)
                             : (wb >= 5 ? bh_group_walk_kernel<false, 5, 2, 1, 2, true>
                                        : bh_group_walk_kernel<false, 4, 2, 1, 2, true>);
        } else if (bpl == 2 && wb <= 4 && e->tune_get("bh.eval_unroll", 2) != 2) {
            // list-evaluation unroll of the default 64-body build
            const bool u4 = e->tune_get("bh.eval_unroll", 2) >= 4;
            kern = clamp ? (u4 ? bh_group_walk_kernel<true, 4, 2, 1, 4> : bh_group_walk_kernel<true, 4, 2, 1, 1>)
                         : (u4 ? bh_group_walk_kernel<false, 4, 2, 1, 4> : bh_group_walk_kernel<false, 4, 2, 1, 1>);
        } else if (bpl == 2)
            kern = clamp ? NBG_GW(true, 2) : NBG_GW(false, 2);
        else
            kern = clamp ? NBG_GW(true, 1) : NBG_GW(false, 1);
#undef NBG_GW
        NBG_CUDA(e, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
        const int warps = n / (32 * bpl);
        // "bh.test_cap": node tests after which a group walk gives up and
        // its bodies are walked one by one; 0 (the default) sets it to
        // "bh.test_cap_ratio" (default 2) times the median tests of
        // kCapSamples groups spread over the leaves.  Groups of one part of
        // the system have tests within a few tens of percent of each other;
        // only groups that mix a dense region with a sparse one (bodies far
        // apart in the group) reach the cap.  Such groups come from the jumps
        // of a curve order; a kd-median tree's groups are subtrees, whose
        // tests stay within a few tens of percent of each other, so there
        // the walk is not capped and the pre-pass is skipped.
        t->test_cap = (unsigned long long)std::max<int64_t>(e->tune_get("bh.test_cap", 0), 0);
        if (t->test_cap == 0 && t->curve == 0) t->test_cap = ~0ull;
        if (t->test_cap == 0) {
            const unsigned ratio = (unsigned)std::max<int64_t>(e->tune_get("bh.test_cap_ratio", 2), 1);
            const int samples = std::min(warps, kCapSamples);  // both powers of two
            const size_t csmem = (size_t)kCapSamples * stack_cap * sizeof(int);
            auto capk = bpl == 4 ? bh_test_cap_kernel<4>
                        : bpl == 2 ? bh_test_cap_kernel<2> : bh_test_cap_kernel<1>;
            NBG_CUDA(e, cudaFuncSetAttribute(capk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)csmem));
            // the cap counts acceptance tests: against the step build's
            // records when those decide acceptance
            TreeState tc = *t;
            if (frozen) tc.node4 = t->node4_acc;
            capk<<<1, kCapSamples * 32, csmem, e->stream>>>(n, warps / samples, samples, tc,
                                                            stack_cap, ratio);
            NBG_LAUNCHED(e, "bh_test_cap_kernel");
        }
        // fb_count[0]: groups handed to the fallback, [1]: the walk's next group
        NBG_CUDA(e, cudaMemsetAsync(t->fb_count, 0, 2 * sizeof(unsigned), e->stream));
        // "bh.persistent" (default 1): as many CTAs as fit at once; 0: one
        // CTA per kGWWarps groups
        unsigned blocks = (unsigned)((warps + kGWWarps - 1) / kGWWarps);
        if (e->tune_get("bh.persistent", 1) != 0) {
            int per_sm = 0;
            NBG_CUDA(e, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kGWThreads, smem));
            blocks = std::min(blocks, (unsigned)std::max(per_sm, 1) * (unsigned)e->sm_count);
        }
        kern<<<blocks, kGWThreads, smem, e->stream>>>(y, f, n, eps2, *t, stack_cap, e->d_err);
        NBG_LAUNCHED(e, "bh_group_walk_kernel");
        if (emit) return NBG_OK;
        auto fb = frozen
            ? (clamp ? bh_body_walk_kernel<true, 2, 1, true> : bh_body_walk_kernel<false, 2, 1, true>)
            : bpl == 4
            ? (clamp ? bh_body_walk_kernel<true, 4, 1> : bh_body_walk_kernel<false, 4, 1>)
            : order == 2
            ? (clamp ? (bpl == 2 ? bh_body_walk_kernel<true, 2, 2> : bh_body_walk_kernel<true, 1, 2>)
                     : (bpl == 2 ? bh_body_walk_kernel<false, 2, 2> : bh_body_walk_kernel<false, 1, 2>))
            : (clamp ? (bpl == 2 ? bh_body_walk_kernel<true, 2, 1> : bh_body_walk_kernel<true, 1, 1>)
                     : (bpl == 2 ? bh_body_walk_kernel<false, 2, 1> : bh_body_walk_kernel<false, 1, 1>));
        const size_t fsmem = (size_t)kGWWarps * stack_cap * sizeof(int);
        NBG_CUDA(e, cudaFuncSetAttribute(fb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem));
        fb<<<(unsigned)e->sm_count * 8u, kGWThreads, fsmem, e->stream>>>(y, f, n, eps2, *t, stack_cap,
                                                                     e->d_err);
        NBG_LAUNCHED(e, "bh_body_walk_kernel");
        return NBG_OK;
    }
    if (e->tune_get("bh.freeze_within_step", 0) != 0)
        return set_error(e, NBG_ERR_UNSUPPORTED,
                         "bh.freeze_within_step runs the default group walk only");
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
}  // namespace

}  // namespace nbg

extern "C" nbg_status nbg_bh_counters(nbg_engine* e, uint64_t* visits, uint64_t* interactions) {
    using namespace nbg;
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    if (e->tree == nullptr) return set_error(e, NBG_ERR_NOT_INITIALIZED, "no tree built yet");
    unsigned long long h[2] = {0, 0};
    NBG_CUDA(e, cudaMemcpyAsync(h, e->tree->counters, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    NBG_CUDA(e, cudaMemsetAsync(e->tree->counters, 0, 5 * sizeof(unsigned long long), e->stream));
    if (visits) *visits = h[0];
    if (interactions) *interactions = h[1];
    return NBG_OK;
}

extern "C" nbg_status nbg_bh_fallback_groups(nbg_engine* e, uint64_t* groups) {
    using namespace nbg;
    if (e == nullptr || groups == nullptr) return NBG_ERR_INVALID_ARG;
    if (e->tree == nullptr) return set_error(e, NBG_ERR_NOT_INITIALIZED, "no tree built yet");
    unsigned long long h = 0;
    NBG_CUDA(e, cudaMemcpyAsync(&h, e->tree->counters + 3, sizeof(h), cudaMemcpyDeviceToHost,
                                e->stream));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    *groups = h;
    return NBG_OK;
}

extern "C" nbg_status nbg_bh_stack_peak(nbg_engine* e, uint64_t* peak, uint64_t* capacity) {
    using namespace nbg;
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    if (e->tree == nullptr) return set_error(e, NBG_ERR_NOT_INITIALIZED, "no tree built yet");
    unsigned long long h = 0;
    NBG_CUDA(e, cudaMemcpyAsync(&h, e->tree->counters + 2, sizeof(h), cudaMemcpyDeviceToHost,
                                e->stream));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    if (peak) *peak = h;
    if (capacity) *capacity = (uint64_t)group_stack_cap(e->tree->levels);
    return NBG_OK;
}
