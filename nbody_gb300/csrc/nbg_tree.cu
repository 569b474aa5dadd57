// nbg_tree.cu -- GPU builds of the Barnes-Hut heap: the reference's
// kd-median tree (always for FP64) and, for mixed precision, a tree whose
// leaves follow a space-filling curve (Hilbert by default, or Morton).
//
// The reference builds the tree on the host (nbody/nbody_space_heap.cpp:13-37,
// 136-190): recursive median split with std::nth_element along x, y, z in
// turn; the left child takes the count/2 smallest bodies; then a bottom-up
// update of mass, mass centre, bounding box and the critical radius
// (nbody/nbody_space_heap.cpp:119-134).
//
// GPU form (N = 2^K bodies):
//  1. Three stable LSD radix sorts of the bodies by x, y and z with exact
//     FP64 keys (ties broken by body index) give three lists.
//  2. Level by level (segment size S = N >> level, split axis = level mod 3)
//     the list of the split axis is already ordered inside every segment, so
//     its first S/2 entries are exactly the left child.  A flag per body marks
//     them; the two other lists are stably partitioned by that flag, which
//     keeps every child segment ordered along all three axes.  After K levels
//     the lists give the leaf order: leaf N + p holds body list[p].
//  3. Bottom-up, nine levels per launch, the reference's node update in FP64
//     with explicit roundings (no contraction), so nodes match a
//     non-contracting build of the reference bit for bit.
// With distinct coordinates the subsets equal nth_element's; the whole tree,
// and therefore every acceptance decision of the walk, matches the reference.
//
// Curve form: the bounding box, one 63-bit key per body (Morton, or the
// Hilbert index by Skilling's transform), one stable radix sort of the key
// bits from 16 up, leaf p = the p-th body along the curve, every node the
// union of its two halves; mixed precision updates the nodes in FP32 from
// FP32 boxes when no FP64 node arrays are needed.
#include <algorithm>
#include <cstring>

#include "nbg_tree.cuh"

namespace nbg {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;  // 2048 keys per block
constexpr int kDigits = 256;

__device__ __forceinline__ uint64_t order_key(double v) {
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void init_keys_kernel(const double* __restrict__ coord, int n,
                                 uint64_t* __restrict__ keys, int* __restrict__ vals) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        keys[i] = order_key(coord[i]);
        vals[i] = i;
    }
}

// ---- Morton-order build (mixed precision option) ----
__device__ __forceinline__ double order_key_inverse(uint64_t k) {
    const uint64_t b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    return __longlong_as_double((long long)b);
}

// box[0..2] = min order keys, box[3..5] = max order keys of x, y, z.
__global__ void bbox_kernel(const double* __restrict__ y, int n, unsigned long long* box) {
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int d = 0; d < 3; ++d) {
            const unsigned long long k = order_key(y[(size_t)d * n + i]);
            lo[d] = min(lo[d], k);
            hi[d] = max(hi[d], k);
        }
    for (int d = 0; d < 3; ++d)
        for (int o = 16; o > 0; o >>= 1) {
            lo[d] = min(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = max(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
    // one atomic per CTA and bound: the six addresses are shared by all CTAs
    __shared__ unsigned long long part[6][32];
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int d = 0; d < 3; ++d) {
            part[d][w] = lo[d];
            part[3 + d][w] = hi[d];
        }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int d = threadIdx.x;
        unsigned long long v = part[d][0];
        for (int k = 1; k < nw; ++k) v = d < 3 ? min(v, part[d][k]) : max(v, part[d][k]);
        if (d < 3) atomicMin(&box[d], v);
        else atomicMax(&box[d], v);
    }
}

// 21 bits per axis, x in the lowest bit of every triple
__device__ __forceinline__ uint64_t spread3(uint32_t v) {
    uint64_t x = v & 0x1FFFFFu;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// Hilbert index of a cell of the 2^21-per-axis grid: Skilling's transform of
// the axes to the "transposed" index (J. Skilling, "Programming the Hilbert
// curve", AIP Conf. Proc. 707, 2004), then the bits interleaved from the most
// significant, axis 0 first.  Consecutive indices are adjacent cells.
__device__ __forceinline__ uint64_t hilbert_key(uint32_t x0, uint32_t x1, uint32_t x2) {
    uint32_t X[3] = {x0, x1, x2};
    const uint32_t M = 1u << 20;
    for (uint32_t Q = M; Q > 1; Q >>= 1) {  // undo excess work
        const uint32_t P = Q - 1;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (X[i] & Q) {
                X[0] ^= P;  // invert
            } else {        // exchange
                const uint32_t t = (X[0] ^ X[i]) & P;
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    X[1] ^= X[0];  // Gray encode
    X[2] ^= X[1];
    uint32_t t = 0;
    for (uint32_t Q = M; Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    X[0] ^= t;
    X[1] ^= t;
    X[2] ^= t;
    return (spread3(X[0]) << 2) | (spread3(X[1]) << 1) | spread3(X[2]);
}

__global__ void morton_keys_kernel(const double* __restrict__ y, int n,
                                   const unsigned long long* __restrict__ box,
                                   uint64_t* __restrict__ keys, int* __restrict__ vals,
                                   int hilbert) {
    // the box's corner and scale, once per CTA
    __shared__ double s_lo[3], s_scale[3];
    if (threadIdx.x < 3) {
        const int d = threadIdx.x;
        s_lo[d] = order_key_inverse(box[d]);
        const double ext = order_key_inverse(box[3 + d]) - s_lo[d];
        s_scale[d] = ext > 0.0 ? 2097151.0 / ext : 0.0;
    }
    __syncthreads();
    const double lo[3] = {s_lo[0], s_lo[1], s_lo[2]};
    const double scale[3] = {s_scale[0], s_scale[1], s_scale[2]};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t q[3];
        for (int d = 0; d < 3; ++d) {
            const double v = (y[(size_t)d * n + i] - lo[d]) * scale[d];
            q[d] = (uint32_t)fmin(fmax(v, 0.0), 2097151.0);
        }
        keys[i] = hilbert ? hilbert_key(q[0], q[1], q[2])
                          : spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
        vals[i] = i;
    }
}

// Per-block digit histogram: hist[digit * nblocks + block].
__global__ void __launch_bounds__(kSortThreads)
radix_hist_kernel(const uint64_t* __restrict__ keys, int n, int shift, unsigned* __restrict__ hist) {
    __shared__ unsigned h[kDigits];
    for (int d = threadIdx.x; d < kDigits; d += kSortThreads) h[d] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    for (int k = threadIdx.x; k < kSortTile; k += kSortThreads) {
        const int i = base + k;
        if (i < n) atomicAdd(&h[(unsigned)(keys[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kDigits; d += kSortThreads) hist[d * gridDim.x + blockIdx.x] = h[d];
}

// Per digit (one CTA each): exclusive scan of hist[d][0 .. nblocks) in
// place, and the digit's total in totals[d].  The scatter kernel adds the
// prefix of the totals (the digit base) itself.
__global__ void __launch_bounds__(512)
radix_digit_scan_kernel(unsigned* __restrict__ hist, int nblocks, unsigned* __restrict__ totals) {
    __shared__ unsigned warp_tot[16];
    __shared__ unsigned carry;
    const int d = blockIdx.x;
    unsigned* h = hist + (size_t)d * nblocks;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nblocks; b0 += 512) {
        const int b = b0 + threadIdx.x;
        const unsigned v = b < nblocks ? h[b] : 0u;
        unsigned incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_tot[warp] = incl;
        __syncthreads();
        unsigned base = carry;
        for (int w = 0; w < warp; ++w) base += warp_tot[w];
        if (b < nblocks) h[b] = base + incl - v;
        __syncthreads();
        if (threadIdx.x == 511) carry = base + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) totals[d] = carry;
}

// Stable scatter.  Each warp owns 256 consecutive keys of the tile and walks
// them in 8 rounds of 32; __match_any_sync ranks equal digits inside a round,
// per-warp digit counters carry the rank across rounds, and a per-digit
// prefix over the warps orders the warps.  The tile is first sorted by digit
// in shared memory, then written out in that order, so that neighbouring
// threads store to neighbouring places of a digit's run.  Order inside the
// tile is kept.
__global__ void __launch_bounds__(kSortThreads)
radix_scatter_kernel(const uint64_t* __restrict__ kin, const int* __restrict__ vin,
                     uint64_t* __restrict__ kout, int* __restrict__ vout, int n, int shift,
                     const unsigned* __restrict__ offsets, const unsigned* __restrict__ totals) {
    constexpr int kWarpsS = kSortThreads / 32;
    __shared__ unsigned cnt[kWarpsS][kDigits];
    __shared__ unsigned gbase[kDigits];  // global start of this block's run of each digit
    __shared__ unsigned lbase[kDigits];  // start of each digit in the block's sorted tile
    __shared__ uint64_t skey[kSortTile];
    __shared__ int sval[kSortTile];
    static_assert(kDigits == kSortThreads, "one digit per thread");
    // exclusive prefix of a per-digit value over the digits (Hillis-Steele)
    auto digit_scan = [&](unsigned own, unsigned* buf) {
        buf[threadIdx.x] = own;
        __syncthreads();
        for (int o = 1; o < kDigits; o <<= 1) {
            const unsigned v = threadIdx.x >= (unsigned)o ? buf[threadIdx.x - o] : 0u;
            __syncthreads();
            buf[threadIdx.x] += v;
            __syncthreads();
        }
        buf[threadIdx.x] -= own;  // inclusive -> exclusive
        __syncthreads();
    };
    digit_scan(totals[threadIdx.x], gbase);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int d = lane; d < kDigits; d += 32) cnt[warp][d] = 0;
    __syncwarp();
    const int base = blockIdx.x * kSortTile + warp * (32 * kSortItems);
    const unsigned lt = (1u << lane) - 1u;
    uint64_t key[kSortItems];
    int val[kSortItems];
    unsigned rank[kSortItems];
    unsigned dig[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int i = base + r * 32 + lane;
        const bool live = i < n;
        key[r] = live ? kin[i] : 0ull;
        val[r] = live ? vin[i] : 0;
        dig[r] = live ? ((unsigned)(key[r] >> shift) & 0xFFu) : kDigits;  // kDigits = dead
        const unsigned peers = __match_any_sync(0xffffffffu, dig[r]);
        const unsigned before = __popc(peers & lt);
        const int leader = __ffs(peers) - 1;
        unsigned b = 0;
        if (live) b = cnt[warp][dig[r]];
        rank[r] = b + before;
        __syncwarp();
        if (live && lane == leader) cnt[warp][dig[r]] = b + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per digit: warps' exclusive offsets inside the digit's run (warp order =
    // key order inside the tile), the block's global start of the run
    unsigned tot = 0;
    {
        const int d = threadIdx.x;
        for (int w = 0; w < kWarpsS; ++w) {
            const unsigned c = cnt[w][d];
            cnt[w][d] = tot;
            tot += c;
        }
        gbase[d] += offsets[d * gridDim.x + blockIdx.x];
    }
    digit_scan(tot, lbase);
    // the tile sorted by digit in shared memory (stable) ...
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        if (dig[r] < (unsigned)kDigits) {
            const unsigned li = lbase[dig[r]] + cnt[warp][dig[r]] + rank[r];
            skey[li] = key[r];
            sval[li] = val[r];
        }
    }
    __syncthreads();
    // ... then written out in that order: consecutive threads write
    // consecutive places of each digit's run
    const int live = min(kSortTile, n - blockIdx.x * kSortTile);
    for (int j = threadIdx.x; j < live; j += kSortThreads) {
        const uint64_t k = skey[j];
        const unsigned d = (unsigned)(k >> shift) & 0xFFu;
        const unsigned dst = gbase[d] + (unsigned)j - lbase[d];
        kout[dst] = k;
        vout[dst] = sval[j];
    }
}

// flag[body] = 1 when the body is in the left half of its segment of the
// split-axis list.
__global__ void split_flag_kernel(const int* __restrict__ list, int n, int S,
                                  unsigned char* __restrict__ flag) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        flag[list[p]] = (unsigned char)((p & (S - 1)) < (S >> 1));
}

struct PartArgs {
    const int* in[2];
    int* out[2];
    const unsigned char* flag;
    int* tile_count;  // [2][ntiles]
    int ntiles;
    int n;
    int S;
};

__global__ void __launch_bounds__(256) part_count_kernel(PartArgs a) {
    const int* in = a.in[blockIdx.y];
    int c = 0;
    const int base = blockIdx.x * kPartTile;
    for (int k = threadIdx.x; k < kPartTile; k += 256) {
        const int p = base + k;
        if (p < a.n) c += a.flag[in[p]];
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    __shared__ int ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < 8; ++w) t += ws[w];
        a.tile_count[blockIdx.y * a.ntiles + blockIdx.x] = t;
    }
}

// Stable partition of each segment by flag: left entries keep their order in
// [seg, seg + S/2), right entries in [seg + S/2, seg + S).
__global__ void __launch_bounds__(256) part_scatter_kernel(PartArgs a) {
    constexpr int kItems = kPartTile / 256;
    __shared__ int excl[kPartTile];  // exclusive count of lefts before each tile slot
    __shared__ int wsum[8];
    __shared__ int seg_prefix;
    const int* in = a.in[blockIdx.y];
    int* out = a.out[blockIdx.y];
    const int tile0 = blockIdx.x * kPartTile;
    int body[kItems];
    int fl[kItems];
    int mine = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int p = tile0 + threadIdx.x * kItems + k;
        body[k] = p < a.n ? in[p] : -1;
        fl[k] = body[k] >= 0 ? a.flag[body[k]] : 0;
        mine += fl[k];
    }
    // block exclusive scan of per-thread counts
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    int wbase = 0;
    for (int w = 0; w < warp; ++w) wbase += wsum[w];
    int run = wbase + incl - mine;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        excl[threadIdx.x * kItems + k] = run;
        run += fl[k];
    }
    // lefts in earlier tiles of the same segment (segments longer than a tile)
    if (threadIdx.x == 0) seg_prefix = 0;
    __syncthreads();
    if (a.S > kPartTile) {
        const int seg_tile0 = (tile0 & ~(a.S - 1)) / kPartTile;
        int s = 0;
        for (int t = seg_tile0 + threadIdx.x; t < (int)blockIdx.x; t += 256)
            s += a.tile_count[blockIdx.y * a.ntiles + t];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) atomicAdd(&seg_prefix, s);
    }
    __syncthreads();
    const int half = a.S >> 1;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        if (body[k] < 0) continue;
        const int slot = threadIdx.x * kItems + k;
        const int p = tile0 + slot;
        const int seg = p & ~(a.S - 1);
        int left_before;
        if (seg >= tile0)
            left_before = excl[slot] - excl[seg - tile0];
        else
            left_before = seg_prefix + excl[slot];
        const int dst = fl[k] ? seg + left_before : seg + half + ((p - seg) - left_before);
        out[dst] = body[k];
    }
}

// Leaves: leaf n + p holds body list[p] (nbody/nbody_space_heap.cpp:141-148).
template <bool F32>
__global__ void leaf_init_kernel(const int* __restrict__ order, const double* __restrict__ y,
                                 const double* __restrict__ mass, int n, TreeState t) {
    const size_t sz = t.size;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int b = order[p];
        const size_t idx = (size_t)n + p;
        t.body_n[idx] = b;
        const double x = y[b], yy = y[n + b], z = y[2 * n + b];
        if (F32) {
            const float4 v = make_float4((float)x, (float)yy, (float)z, 0.f);
            t.node4[idx] = v;
            t.nodem[idx] = (float)mass[b];
            t.box4[idx] = v;
            t.box4[sz + idx] = v;
            continue;
        }
        t.com[idx] = x;
        t.com[sz + idx] = yy;
        t.com[2 * sz + idx] = z;
        t.bmin[idx] = x;
        t.bmin[sz + idx] = yy;
        t.bmin[2 * sz + idx] = z;
        t.bmax[idx] = x;
        t.bmax[sz + idx] = yy;
        t.bmax[2 * sz + idx] = z;
        t.mass[idx] = mass[b];
        t.crit2[idx] = 0.0;
        t.node4[idx] = make_float4((float)x, (float)yy, (float)z, 0.f);
        t.nodem[idx] = (float)mass[b];
    }
}

// Refit leaves: new positions, same bodies (nbody/nbody_space_heap.cpp:45-53).
template <bool F32>
__global__ void leaf_refit_kernel(const double* __restrict__ y, int n, TreeState t) {
    const size_t sz = t.size;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const size_t idx = (size_t)n + p;
        const int b = t.body_n[idx];
        const double x = y[b], yy = y[n + b], z = y[2 * n + b];
        if (F32) {
            const float4 v = make_float4((float)x, (float)yy, (float)z, 0.f);
            t.node4[idx] = v;
            t.box4[idx] = v;
            t.box4[sz + idx] = v;
            continue;
        }
        t.com[idx] = x;
        t.com[sz + idx] = yy;
        t.com[2 * sz + idx] = z;
        t.bmin[idx] = x;
        t.bmin[sz + idx] = yy;
        t.bmin[2 * sz + idx] = z;
        t.bmax[idx] = x;
        t.bmax[sz + idx] = yy;
        t.bmax[2 * sz + idx] = z;
        t.node4[idx] = make_float4((float)x, (float)yy, (float)z, 0.f);
    }
}

__device__ __forceinline__ double len3(double x, double y, double z) {
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
}

// One level of the bottom-up update (nbody/nbody_space_heap.cpp:119-134).
// One inner node from its two children (nbody/nbody_space_heap.cpp:119-134),
// FP64 with the reference's roundings.
__device__ __forceinline__ void update_node(size_t idx, double lambda2, TreeState& t) {
    const size_t sz = t.size;
    {
        const size_t l = 2 * idx, r = 2 * idx + 1;
        const double ml = t.mass[l], mr = t.mass[r];
        const double m = __dadd_rn(ml, mr);
        double c[3], mn[3], mx[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            c[d] = __ddiv_rn(__dadd_rn(__dmul_rn(t.com[d * sz + l], ml), __dmul_rn(t.com[d * sz + r], mr)), m);
            const double al = t.bmin[d * sz + l], ar = t.bmin[d * sz + r];
            mn[d] = (ar < al) ? ar : al;  // std::min(left, right)
            const double bl = t.bmax[d * sz + l], br = t.bmax[d * sz + r];
            mx[d] = (bl < br) ? br : bl;  // std::max(left, right)
            t.com[d * sz + idx] = c[d];
            t.bmin[d * sz + idx] = mn[d];
            t.bmax[d * sz + idx] = mx[d];
        }
        t.mass[idx] = m;
        const double rr = __dadd_rn(
            __dmul_rn(len3(__dsub_rn(mx[0], mn[0]), __dsub_rn(mx[1], mn[1]), __dsub_rn(mx[2], mn[2])), 0.5),
            len3(__dsub_rn(__ddiv_rn(__dadd_rn(mx[0], mn[0]), 2.0), c[0]),
                 __dsub_rn(__ddiv_rn(__dadd_rn(mx[1], mn[1]), 2.0), c[1]),
                 __dsub_rn(__ddiv_rn(__dadd_rn(mx[2], mn[2]), 2.0), c[2])));
        const double cr2 = __dmul_rn(__dmul_rn(rr, rr), lambda2);
        t.crit2[idx] = cr2;
        t.node4[idx] = make_float4((float)c[0], (float)c[1], (float)c[2], (float)cr2);
        t.nodem[idx] = (float)m;
    }
}

// The same node update in FP32 from the FP32 records and boxes (mixed
// precision, whose walks read only the FP32 records).
__device__ __forceinline__ void update_node_f32(size_t idx, float lambda2, TreeState& t) {
    const size_t sz = t.size;
    const size_t l = 2 * idx, r = 2 * idx + 1;
    const float4 cl = t.node4[l], cr = t.node4[r];
    const float ml = t.nodem[l], mr = t.nodem[r];
    const float m = ml + mr;
    const float4 ll = t.box4[l], lr = t.box4[r], hl = t.box4[sz + l], hr = t.box4[sz + r];
    const float cx = (cl.x * ml + cr.x * mr) / m, cy = (cl.y * ml + cr.y * mr) / m;
    const float cz = (cl.z * ml + cr.z * mr) / m;
    const float lx = fminf(ll.x, lr.x), ly = fminf(ll.y, lr.y), lz = fminf(ll.z, lr.z);
    const float hx = fmaxf(hl.x, hr.x), hy = fmaxf(hl.y, hr.y), hz = fmaxf(hl.z, hr.z);
    const float ex = hx - lx, ey = hy - ly, ez = hz - lz;
    const float ox = 0.5f * (hx + lx) - cx, oy = 0.5f * (hy + ly) - cy, oz = 0.5f * (hz + lz) - cz;
    const float rr = 0.5f * sqrtf(ex * ex + ey * ey + ez * ez) + sqrtf(ox * ox + oy * oy + oz * oz);
    t.node4[idx] = make_float4(cx, cy, cz, rr * rr * lambda2);
    t.nodem[idx] = m;
    t.box4[idx] = make_float4(lx, ly, lz, 0.f);
    t.box4[sz + idx] = make_float4(hx, hy, hz, 0.f);
}

template <typename T>
nbg_status alloc(nbg_engine* e, T** p, size_t count) {
    NBG_CUDA(e, cudaMalloc(p, count * sizeof(T) + 256));
    return NBG_OK;
}

nbg_status tree_alloc(nbg_engine* e) {
    TreeState* t = e->tree;
    const size_t n = t->n, sz = t->size;
    const size_t ntiles = n / kPartTile + 1;
    const size_t nblocks = n / kSortTile + 1;
    nbg_status s = NBG_OK;
#define NBG_TRY(x)               \
    if ((s = (x)) != NBG_OK) return s;
    NBG_TRY(alloc(e, &t->keys[0], n));
    NBG_TRY(alloc(e, &t->keys[1], n));
    NBG_TRY(alloc(e, &t->vals[0], n));
    NBG_TRY(alloc(e, &t->vals[1], n));
    for (int d = 0; d < 3; ++d) NBG_TRY(alloc(e, &t->lists[d], n));
    NBG_TRY(alloc(e, &t->spare[0], n));
    NBG_TRY(alloc(e, &t->spare[1], n));
    NBG_TRY(alloc(e, &t->flag, n));
    NBG_TRY(alloc(e, &t->tile_count, 2 * ntiles));
    NBG_TRY(alloc(e, &t->hist, kDigits * nblocks));
    NBG_TRY(alloc(e, &t->totals, kDigits));
    NBG_TRY(alloc(e, &t->box, 6));
    NBG_TRY(alloc(e, &t->fb_list, n / 32 + 1));
    NBG_TRY(alloc(e, &t->fb_count, 2));
    NBG_TRY(alloc(e, &t->cap_state, 1));
    NBG_TRY(alloc(e, &t->com, 3 * sz));
    NBG_TRY(alloc(e, &t->mass, sz));
    NBG_TRY(alloc(e, &t->bmin, 3 * sz));
    NBG_TRY(alloc(e, &t->bmax, 3 * sz));
    NBG_TRY(alloc(e, &t->crit2, sz));
    NBG_TRY(alloc(e, &t->body_n, sz));
    NBG_TRY(alloc(e, &t->node4, sz));
    NBG_TRY(alloc(e, &t->nodem, sz));
    NBG_TRY(alloc(e, &t->box4, 2 * sz));
    NBG_TRY(alloc(e, &t->counters, 5));
#undef NBG_TRY
    // index 0 is unused; zero everything once so stray reads are defined
    NBG_CUDA(e, cudaMemsetAsync(t->node4, 0, sz * sizeof(float4), e->stream));
    NBG_CUDA(e, cudaMemsetAsync(t->nodem, 0, sz * sizeof(float), e->stream));
    NBG_CUDA(e, cudaMemsetAsync(t->crit2, 0, sz * sizeof(double), e->stream));
    NBG_CUDA(e, cudaMemsetAsync(t->body_n, 0, sz * sizeof(int), e->stream));
    NBG_CUDA(e, cudaMemsetAsync(t->counters, 0, 5 * sizeof(unsigned long long), e->stream));
    return NBG_OK;
}

// Stable LSD sort of keys[0] / vals[0] by the key bits from 8 * first_pass
// up (an even number of passes, so the result is back in keys[0] / vals[0]).
nbg_status radix_sort(nbg_engine* e, TreeState* t, int n, int first_pass = 0) {
    const int nblocks = (n + kSortTile - 1) / kSortTile;
    for (int pass = first_pass; pass < 8; ++pass) {
        const int shift = 8 * pass;
        const int src = pass & 1, dst = src ^ 1;
        radix_hist_kernel<<<nblocks, kSortThreads, 0, e->stream>>>(t->keys[src], n, shift, t->hist);
        NBG_LAUNCHED(e, "radix_hist_kernel");
        radix_digit_scan_kernel<<<kDigits, 512, 0, e->stream>>>(t->hist, nblocks, t->totals);
        NBG_LAUNCHED(e, "radix_digit_scan_kernel");
        radix_scatter_kernel<<<nblocks, kSortThreads, 0, e->stream>>>(
            t->keys[src], t->vals[src], t->keys[dst], t->vals[dst], n, shift, t->hist, t->totals);
        NBG_LAUNCHED(e, "radix_scatter_kernel");
    }
    return NBG_OK;
}

// Levels [lv_lo, lv_hi) of the heap, bottom-up, in one launch: block b owns
// the subtree under node 2^lv_lo + b down to level lv_hi - 1 (at most
// kFusedLevels levels, 256 nodes at its bottom), with a block barrier
// between levels; global writes of one level are visible to the block's
// reads of the next.  The per-node arithmetic is update_node's.
constexpr int kFusedLevels = 9;

template <bool F32>
__global__ void __launch_bounds__(256)
update_levels_fused_kernel(int lv_lo, int lv_hi, double lambda2, TreeState t) {
    const size_t root = ((size_t)1 << lv_lo) + blockIdx.x;
    for (int lv = lv_hi - 1; lv >= lv_lo; --lv) {
        const int span = 1 << (lv - lv_lo);
        const size_t first = root << (lv - lv_lo);
        for (int k = threadIdx.x; k < span; k += blockDim.x) {
            if (F32) update_node_f32(first + k, (float)lambda2, t);
            else update_node(first + k, lambda2, t);
        }
        __syncthreads();
    }
}

nbg_status update_levels(nbg_engine* e, TreeState* t) {
    const double lambda2 = t->lambda * t->lambda;
    for (int hi = t->levels; hi > 0;) {
        const int lo = std::max(0, hi - kFusedLevels);
        if (t->f32)
            update_levels_fused_kernel<true><<<1u << lo, 256, 0, e->stream>>>(lo, hi, lambda2, *t);
        else
            update_levels_fused_kernel<false><<<1u << lo, 256, 0, e->stream>>>(lo, hi, lambda2, *t);
        NBG_LAUNCHED(e, "update_levels_fused_kernel");
        hi = lo;
    }
    return NBG_OK;
}

}  // namespace

void tree_destroy(nbg_engine* e) {
    TreeState* t = e->tree;
    if (t == nullptr) return;
    void* ptrs[] = {t->keys[0], t->keys[1], t->vals[0], t->vals[1], t->lists[0], t->lists[1],
                    t->lists[2], t->spare[0], t->spare[1], t->flag, t->tile_count, t->hist, t->totals, t->box,
                    t->fb_list, t->fb_count, t->cap_state,
                    t->com, t->mass, t->bmin, t->bmax, t->crit2, t->body_n, t->node4,
                    t->nodem, t->box4, t->feat, t->quad, t->counters, t->node4_acc,
                    t->leaf_lo};
    for (void* p : ptrs) cudaFree(p);
    delete t;
    e->tree = nullptr;
}

nbg_status tree_build(nbg_engine* e, const double* y, bool fp64_nodes, double lambda) {
    const int n = (int)e->count;
    if (e->tree == nullptr) {
        e->tree = new TreeState();
        e->tree->n = (size_t)n;
        e->tree->size = 2 * (size_t)n;
        int k = 0;
        while ((1 << k) < n) ++k;
        e->tree->levels = k;
        nbg_status s = tree_alloc(e);
        if (s != NBG_OK) {
            tree_destroy(e);
            return s;
        }
    }
    TreeState* t = e->tree;
    t->lambda = lambda;
    // "bh.fp64_nodes" = 1 keeps the FP64 node update in mixed precision
    t->f32 = !fp64_nodes && e->tune_get("bh.fp64_nodes", 0) == 0;
    ProfScope ps(e, NBG_K_TREE_BUILD);
    const unsigned g = grid_for(n, 256, (unsigned)e->sm_count * 8u);
    // mixed precision defaults to the Hilbert tree: at equal force error
    // its walks do several times fewer node tests than on the kd tree,
    // whose median cuts leave long thin cells with large radii.  The FP64
    // path keeps the reference's tree.
    const bool hilbert_default = e->params.precision != NBG_PREC_FP64;
    const int64_t curve = e->tune_get("bh.build", hilbert_default ? 2 : 0);
    if (e->params.precision != NBG_PREC_FP64 && (curve == 1 || curve == 2)) {
        // space-filling-curve order (1: Morton, 2: Hilbert): one sort; leaf p
        // = p-th body along the curve, every node the union of its two halves
        // (a different tree from the reference's; the FP64 path always
        // builds the reference's)
        // box = {min keys: all ones, max keys: zero}
        NBG_CUDA(e, cudaMemsetAsync(t->box, 0xFF, 3 * sizeof(unsigned long long), e->stream));
        NBG_CUDA(e, cudaMemsetAsync(t->box + 3, 0, 3 * sizeof(unsigned long long), e->stream));
        bbox_kernel<<<std::min(g, (unsigned)e->sm_count * 2u), 256, 0, e->stream>>>(y, n, t->box);
        NBG_LAUNCHED(e, "bbox_kernel");
        morton_keys_kernel<<<g, 256, 0, e->stream>>>(y, n, t->box, t->keys[0], t->vals[0],
                                                     curve == 2 ? 1 : 0);
        NBG_LAUNCHED(e, "morton_keys_kernel");
        // the key bits from 16 up (47 of 63: the curve down to cells of
        // about 2^-16 of the box per axis), bodies sharing one in index order
        nbg_status s = radix_sort(e, t, n, 2);
        if (s != NBG_OK) return s;
        if (t->f32)
            leaf_init_kernel<true><<<g, 256, 0, e->stream>>>(t->vals[0], y, e->d_mass, n, *t);
        else
            leaf_init_kernel<false><<<g, 256, 0, e->stream>>>(t->vals[0], y, e->d_mass, n, *t);
        NBG_LAUNCHED(e, "leaf_init_kernel");
        s = update_levels(e, t);
        if (s != NBG_OK) return s;
        t->built = true;
        t->curve = (int)curve;
        return NBG_OK;
    }
    t->curve = 0;
    // 1. three sorted lists
    for (int d = 0; d < 3; ++d) {
        init_keys_kernel<<<g, 256, 0, e->stream>>>(y + (size_t)d * n, n, t->keys[0], t->vals[0]);
        NBG_LAUNCHED(e, "init_keys_kernel");
        nbg_status s = radix_sort(e, t, n);
        if (s != NBG_OK) return s;
        NBG_CUDA(e, cudaMemcpyAsync(t->lists[d], t->vals[0], n * sizeof(int),
                                    cudaMemcpyDeviceToDevice, e->stream));
    }
    // 2. median splits, level by level
    const int ntiles = (n + kPartTile - 1) / kPartTile;
    for (int lv = 0; lv < t->levels; ++lv) {
        const int S = n >> lv;
        const int d = lv % 3;
        split_flag_kernel<<<g, 256, 0, e->stream>>>(t->lists[d], n, S, t->flag);
        NBG_LAUNCHED(e, "split_flag_kernel");
        const int e0 = (d + 1) % 3, e1 = (d + 2) % 3;
        PartArgs a;
        a.in[0] = t->lists[e0];
        a.in[1] = t->lists[e1];
        a.out[0] = t->spare[0];
        a.out[1] = t->spare[1];
        a.flag = t->flag;
        a.tile_count = t->tile_count;
        a.ntiles = ntiles;
        a.n = n;
        a.S = S;
        if (S > kPartTile) {
            part_count_kernel<<<dim3(ntiles, 2), 256, 0, e->stream>>>(a);
            NBG_LAUNCHED(e, "part_count_kernel");
        }
        part_scatter_kernel<<<dim3(ntiles, 2), 256, 0, e->stream>>>(a);
        NBG_LAUNCHED(e, "part_scatter_kernel");
        int* tmp0 = t->lists[e0];
        int* tmp1 = t->lists[e1];
        t->lists[e0] = t->spare[0];
        t->lists[e1] = t->spare[1];
        t->spare[0] = tmp0;
        t->spare[1] = tmp1;
    }
    // 3. leaves, then the bottom-up update
    if (t->f32)
        leaf_init_kernel<true><<<g, 256, 0, e->stream>>>(t->lists[0], y, e->d_mass, n, *t);
    else
        leaf_init_kernel<false><<<g, 256, 0, e->stream>>>(t->lists[0], y, e->d_mass, n, *t);
    NBG_LAUNCHED(e, "leaf_init_kernel");
    nbg_status s = update_levels(e, t);
    if (s != NBG_OK) return s;
    t->built = true;
    return NBG_OK;
}

nbg_status tree_refit(nbg_engine* e, const double* y, double lambda) {
    TreeState* t = e->tree;
    const int n = (int)e->count;
    t->lambda = lambda;
    ProfScope ps(e, NBG_K_TREE_BUILD);
    const unsigned g = grid_for(n, 256, (unsigned)e->sm_count * 8u);
    if (t->f32)
        leaf_refit_kernel<true><<<g, 256, 0, e->stream>>>(y, n, *t);
    else
        leaf_refit_kernel<false><<<g, 256, 0, e->stream>>>(y, n, *t);
    NBG_LAUNCHED(e, "leaf_refit_kernel");
    return update_levels(e, t);
}

}  // namespace nbg
