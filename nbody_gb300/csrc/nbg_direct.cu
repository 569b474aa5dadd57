// nbg_direct.cu -- direct O(N^2) gravity: f = [v ; a(y)].
//
// Three kernels share the engine entry point:
//
//  * FP64 (parity) -- one thread per body, j-tiles of double4 in shared
//    memory, the reference 'simple' arithmetic in the reference order
//    (nbody/nbody_engine_simple.cpp:143-172 with nbody_data::force,
//    nbody/nbody_data.cpp:35-44): explicit roundings (no FMA contraction),
//    self pair skipped, force summed j = 0..N-1 then divided by m_i.
//
//  * mixed (throughput) -- FP32 pair math on the FP32 pipe, FP64 state.
//    A pack kernel turns y into a tile-padded array of bodies in
//    (x x y y | z z m m) form and writes f = [v ; 0].  The force kernel is
//    persistent: the (i-block, j-tile) units are split evenly over one wave
//    of CTAs (stream-K), thread 0 streams j-tiles global -> shared with 1-D
//    bulk async copies (TMA) through a 4-stage mbarrier ring, and the 4 warps
//    each hold 2G i-bodies per lane (G = 2 or 4 packed pairs) in FP32x2
//    registers.  Per
//    tile the FP32 partial sums are folded into a (hi, lo) two-sum pair; at
//    the end of an i-block segment hi + lo is added into the FP64 a-part of f
//    with one atomicAdd per component.  Pair term:
//        a_i += m_j (r_j - r_i) / (|r_j - r_i|^2 + eps^2)^{3/2}
//    with r^2 clamped to >= 1e-8 when eps = 0 (the reference clamp).
//
//  * mixed, symmetric (the default, tuning key direct.symmetric = 1) -- the
//    same arithmetic with every unordered pair evaluated once and applied to
//    both bodies (details at direct_sym_kernel).
#include <mutex>

#include "nbg_internal.cuh"
#include "nbg_pair.cuh"
#include "nbg_ptx.cuh"

namespace nbg {
namespace {

// ---------------------------------------------------------------------------
// FP64 kernel
// ---------------------------------------------------------------------------
constexpr int kF64Threads = 128;

struct alignas(32) D4 {
    double x, y, z, w;
};

__global__ void __launch_bounds__(kF64Threads)
direct_fp64_kernel(const double* __restrict__ y, const double* __restrict__ mass,
                   double* __restrict__ f, int n) {
    __shared__ D4 tile[kF64Threads];
    const int i = blockIdx.x * kF64Threads + threadIdx.x;
    const bool live = i < n;
    const double x1 = live ? y[i] : 0.0;
    const double y1 = live ? y[n + i] : 0.0;
    const double z1 = live ? y[2 * n + i] : 0.0;
    const double m1 = live ? mass[i] : 1.0;
    const double mneg = __dmul_rn(-1.0, m1);
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int j0 = 0; j0 < n; j0 += kF64Threads) {
        const int j = j0 + threadIdx.x;
        if (j < n) tile[threadIdx.x] = D4{y[j], y[n + j], y[2 * n + j], mass[j]};
        __syncthreads();
        const int cnt = min(kF64Threads, n - j0);
        for (int k = 0; k < cnt; ++k) {
            if (j0 + k == i) continue;  // nbody/nbody_engine_simple.cpp:155-158
            const D4 p = tile[k];
            const double dx = __dsub_rn(x1, p.x);
            const double dy = __dsub_rn(y1, p.y);
            const double dz = __dsub_rn(z1, p.z);
            double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            if (r2 < kMinDistance) r2 = kMinDistance;
            const double c = __ddiv_rn(__dmul_rn(mneg, p.w), __dmul_rn(r2, __dsqrt_rn(r2)));
            fx = __dadd_rn(fx, __dmul_rn(dx, c));
            fy = __dadd_rn(fy, __dmul_rn(dy, c));
            fz = __dadd_rn(fz, __dmul_rn(dz, c));
        }
        __syncthreads();
    }
    if (live) {
        f[i] = y[3 * n + i];
        f[n + i] = y[4 * n + i];
        f[2 * n + i] = y[5 * n + i];
        f[3 * n + i] = __ddiv_rn(fx, m1);
        f[4 * n + i] = __ddiv_rn(fy, m1);
        f[5 * n + i] = __ddiv_rn(fz, m1);
    }
}

// ---------------------------------------------------------------------------
// mixed kernel
// ---------------------------------------------------------------------------
constexpr int kWarps = 4;                      // warps per CTA (all compute)
constexpr int kThreadsMixed = kWarps * 32;
constexpr int kMinBlocksMixed = 6;             // resident CTAs per SM targeted
constexpr int kT = 128;                        // j-bodies per tile
constexpr int kStages = 4;                     // tiles in flight
constexpr uint32_t kTileBytes = kT * 32;       // 32 bytes per body (x x y y z z m m)

struct Body2 {  // one body in duplicated form, 32 bytes
    float4 xxyy;
    float4 zzmm;
};

__global__ void pack_mixed_kernel(const double* __restrict__ y, const double* __restrict__ mass,
                                  Body2* __restrict__ out, double* __restrict__ f, int n,
                                  int n_pad) {
    int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += stride) {
        Body2 b;
        if (i < n) {
            float x = (float)y[i], yy = (float)y[n + i], z = (float)y[2 * n + i];
            float m = (float)mass[i];
            b.xxyy = make_float4(x, x, yy, yy);
            b.zzmm = make_float4(z, z, m, m);
            f[i] = y[3 * n + i];
            f[n + i] = y[4 * n + i];
            f[2 * n + i] = y[5 * n + i];
            f[3 * n + i] = 0.0;
            f[4 * n + i] = 0.0;
            f[5 * n + i] = 0.0;
        } else {
            b.xxyy = make_float4(0.f, 0.f, 0.f, 0.f);
            b.zzmm = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        out[i] = b;
    }
}

struct MixedArgs {
    const Body2* bodies;  // [n_pad]
    double* acc;          // a-part of f: [3][n]
    int n;
    int n_jt;             // j-tiles
    long long units;      // n_iblocks * n_jt
    float eps2;
    unsigned* err;
};

template <bool CLAMP>
__device__ __forceinline__ void pair2(f2_t xj, f2_t yj, f2_t zj, f2_t mj, f2_t xi, f2_t yi,
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
    const f2_t inv2 = f2_mul(inv, inv);
    const f2_t s = f2_mul(mj, inv);
    const f2_t s3 = f2_mul(s, inv2);
    ax = f2_fma(dx, s3, ax);
    ay = f2_fma(dy, s3, ay);
    az = f2_fma(dz, s3, az);
}

// Issue the bulk copy of j-tile `jt` into stage `s` (one thread).
__device__ __forceinline__ void issue_tile(Body2* tiles, uint64_t* full, int s, int jt,
                                           const Body2* bodies) {
    mbar_arrive_expect_tx(&full[s], kTileBytes);
    bulk_g2s(tiles + s * kT, bodies + (size_t)jt * kT, kTileBytes, &full[s]);
}

// G packed pairs (2G i-bodies) per lane; the j loop is unrolled UNR times.
// i-body of lane `lane`, warp `warp`, slot r in [0, 2G):
//     i = ib * IB + r * 128 + warp * 32 + lane,   IB = 128 * 2G,
// so every slot is a coalesced row of 128 consecutive bodies.
template <bool CLAMP, int G, int UNR>
__global__ void __launch_bounds__(kThreadsMixed, G >= 4 ? 4 : kMinBlocksMixed)
direct_mixed_kernel(MixedArgs a) {
    constexpr int kIB = kThreadsMixed * 2 * G;
    constexpr int kSlots = 6 * G;  // (hi, lo) x 3 components x G pairs
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Body2* tiles = reinterpret_cast<Body2*>(smem_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + kStages * kTileBytes);
    uint64_t* empty = full + kStages;
    // Compensated per-body accumulators (hi, lo) live in shared memory: they
    // are touched once per tile, and keeping them out of registers lets more
    // CTAs stay resident.  Slot q = 2 * (3 * g + c) + {0: hi, 1: lo}.
    f2_t* acc_sm = reinterpret_cast<f2_t*>(smem_raw + kStages * kTileBytes +
                                           2 * kStages * sizeof(uint64_t));

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const long long per = a.units / gridDim.x;
    const long long rem = a.units % gridDim.x;
    const long long u0 = blockIdx.x * per + min((long long)blockIdx.x, rem);
    const long long u1 = u0 + per + ((long long)blockIdx.x < rem ? 1 : 0);
    const long long cnt = u1 - u0;
    const bool producer = threadIdx.x == 0;
    auto acc_at = [&](int q) -> f2_t& { return acc_sm[q * kThreadsMixed + threadIdx.x]; };

    if (producer) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kWarps);
        }
        mbar_fence_init();
    }
    __syncthreads();
    if (producer) {  // prologue: fill the ring
        for (long long k = 0; k < kStages && k < cnt; ++k)
            issue_tile(tiles, full, (int)k, (int)((u0 + k) % a.n_jt), a.bodies);
    }

    const f2_t eps2 = f2_pack(a.eps2, a.eps2);
    const f2_t zero = f2_pack(0.f, 0.f);
    f2_t xi[G], yi[G], zi[G];
    long long cur_ib = -1;
    bool ok = true;
    const uint32_t tiles_addr = smem_addr(tiles);

    auto flush = [&](long long ib) {
#pragma unroll
        for (int g = 0; g < G; ++g) {
            float h0, h1, l0, l1;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                f2_unpack(acc_at(2 * (3 * g + c)), h0, h1);
                f2_unpack(acc_at(2 * (3 * g + c) + 1), l0, l1);
                const int i0 = (int)(ib * kIB) + (2 * g) * kThreadsMixed + warp * 32 + lane;
                const int i1 = i0 + kThreadsMixed;
                if (i0 < a.n) atomicAdd(a.acc + (size_t)c * a.n + i0, (double)h0 + (double)l0);
                if (i1 < a.n) atomicAdd(a.acc + (size_t)c * a.n + i1, (double)h1 + (double)l1);
            }
        }
    };

    for (long long k = 0; k < cnt; ++k) {
        const long long u = u0 + k;
        // Refill the stage that iteration k-1 freed, once every warp is done with it.
        if (producer && k >= 1 && k - 1 + kStages < cnt) {
            const int sp = (int)((k - 1) % kStages);
            const uint32_t par = (uint32_t)(((k - 1) / kStages) & 1);
            if (!mbar_wait(&empty[sp], par, a.err)) {
                ok = false;
                break;
            }
            issue_tile(tiles, full, sp, (int)((u - 1 + kStages) % a.n_jt), a.bodies);
        }
        const long long ib = u / a.n_jt;
        if (ib != cur_ib) {
            if (cur_ib >= 0) flush(cur_ib);
            cur_ib = ib;
#pragma unroll
            for (int g = 0; g < G; ++g) {
                const int i0 = (int)(ib * kIB) + (2 * g) * kThreadsMixed + warp * 32 + lane;
                const int i1 = i0 + kThreadsMixed;
                float x0 = 0.f, y0 = 0.f, z0 = 0.f, x1 = 0.f, y1 = 0.f, z1 = 0.f;
                if (i0 < a.n) {
                    const float4 b = __ldg(&a.bodies[i0].xxyy);
                    x0 = b.x; y0 = b.z; z0 = __ldg(&a.bodies[i0].zzmm.x);
                }
                if (i1 < a.n) {
                    const float4 b = __ldg(&a.bodies[i1].xxyy);
                    x1 = b.x; y1 = b.z; z1 = __ldg(&a.bodies[i1].zzmm.x);
                }
                xi[g] = f2_pack(x0, x1);
                yi[g] = f2_pack(y0, y1);
                zi[g] = f2_pack(z0, z1);
            }
#pragma unroll
            for (int q = 0; q < kSlots; ++q) acc_at(q) = zero;
        }
        const int s = (int)(k % kStages);
        if (!mbar_wait(&full[s], (uint32_t)((k / kStages) & 1), a.err)) {
            ok = false;
            break;
        }
        const uint32_t tbase = tiles_addr + (uint32_t)s * kTileBytes;
        f2_t ax[G], ay[G], az[G];
#pragma unroll
        for (int g = 0; g < G; ++g) ax[g] = ay[g] = az[g] = zero;
#pragma unroll UNR
        for (int j = 0; j < kT; ++j) {
            const float4 p0 = lds128(tbase + 32u * j);
            const float4 p1 = lds128(tbase + 32u * j + 16u);
            const f2_t xj = f2_pack(p0.x, p0.y);
            const f2_t yj = f2_pack(p0.z, p0.w);
            const f2_t zj = f2_pack(p1.x, p1.y);
            const f2_t mj = f2_pack(p1.z, p1.w);
#pragma unroll
            for (int g = 0; g < G; ++g)
                pair2<CLAMP>(xj, yj, zj, mj, xi[g], yi[g], zi[g], eps2, ax[g], ay[g], az[g]);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
#pragma unroll
        for (int g = 0; g < G; ++g) {
            f2_two_sum(acc_at(2 * (3 * g + 0)), acc_at(2 * (3 * g + 0) + 1), ax[g]);
            f2_two_sum(acc_at(2 * (3 * g + 1)), acc_at(2 * (3 * g + 1) + 1), ay[g]);
            f2_two_sum(acc_at(2 * (3 * g + 2)), acc_at(2 * (3 * g + 2) + 1), az[g]);
        }
    }
    if (ok && cur_ib >= 0) flush(cur_ib);
}

size_t mixed_smem_bytes(int G) {
    return (size_t)kStages * kTileBytes + 2 * kStages * sizeof(uint64_t) +
           6 * G * kThreadsMixed * sizeof(f2_t);
}

using MixedKernel = void (*)(MixedArgs);

template <bool CLAMP>
MixedKernel pick_mixed(int G, int unr) {
    if (G == 4) {
        if (unr <= 2) return direct_mixed_kernel<CLAMP, 4, 2>;
        return direct_mixed_kernel<CLAMP, 4, 4>;
    }
    if (unr <= 2) return direct_mixed_kernel<CLAMP, 2, 2>;
    if (unr >= 8) return direct_mixed_kernel<CLAMP, 2, 8>;
    return direct_mixed_kernel<CLAMP, 2, 4>;
}

// ---------------------------------------------------------------------------
// symmetric mixed kernel: every unordered pair evaluated once
// ---------------------------------------------------------------------------
// Bodies are split into ranges of 256 G bodies.  A CTA holds one range in
// registers (the A bodies: 2 G per lane as G packed FP32x2 pairs, G = 4 by
// default, 3 with 5 CTAs per SM) and streams
// 128-body B tiles through the same TMA ring as above.  Unit (R, t) pairs
// range R with tile t for t >= the first tile of R:
//   * t inside R: one-sided, all ordered pairs, A side only (the self pair
//     contributes d = 0);
//   * t after R: symmetric.  Each pair adds m_B d / r^3 to A and
//     -m_A d / r^3 to B (Newton's third law), so tiles before R are covered
//     by the units of their own ranges.
// Symmetric chunks of 32 B bodies rotate through the warp: at step k lane l
// meets B body (l + k) mod 32 with its 2 G A bodies, and the B accumulator
// follows its body one lane down per step (a shuffle), so after 32 steps lane
// l holds the complete warp sum for B body l and adds it to f with FP64
// reductions.  Per pair this costs 16 FP32 operations and one reciprocal
// square root for two interactions, against 12 and one per interaction in
// the one-sided kernel.
constexpr int kSymWarps = 4;
constexpr int kSymThreads = kSymWarps * 32;
constexpr int kSymT = 128;  // B bodies per tile
// G packed pairs of A bodies per lane (4 by default, 3 with "direct.sym_g");
// a range is 256 G bodies, 2 G tiles
__host__ __device__ constexpr int sym_range(int G) { return kSymThreads * 2 * G; }
constexpr int kSymStages = 4;
constexpr uint32_t kSymTileBytes = kSymT * 32;  // (x x y y | z z m m) FP32 per body

struct SymArgs {
    const float4* bodies;  // [2 n_pad], tile-split layout
    double* acc;           // a-part of f: [3][n]
    double m_uni;          // the common mass (uniform-mass kernel)
    int n;
    int n_jt;              // tiles = n_pad / kSymT
    int n_ranges;          // n_pad / range
    long long units;
    float eps2;
    unsigned* err;
};

// Tile-split layout: tile t holds [(x x y y) x 128 | (z z m m) x 128], so a
// lane's two LDS.128 of one body return both packed operands ready for the
// FP32x2 arithmetic, and 32 lanes reading 32 different bodies touch 512
// contiguous bytes per load.
__device__ __forceinline__ size_t sym_xy(int i) { return (size_t)(i >> 7) * 256 + (i & 127); }

__global__ void pack_sym_kernel(const double* __restrict__ y, const double* __restrict__ mass,
                                float4* __restrict__ out, double* __restrict__ f, int n,
                                int n_pad) {
    int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += stride) {
        // padding bodies: zero mass, and parked at 1e18 on every axis, where
        // r^-3 underflows to exactly 0 in FP32, so that they add nothing in
        // the uniform-mass kernel, which does not weight pairs by mass either
        float4 xy = make_float4(1e18f, 1e18f, 1e18f, 1e18f);
        float4 zm = make_float4(1e18f, 1e18f, 0.f, 0.f);
        if (i < n) {
            const float x = (float)y[i], yy = (float)y[n + i], z = (float)y[2 * n + i];
            const float m = (float)mass[i];
            xy = make_float4(x, x, yy, yy);
            zm = make_float4(z, z, m, m);
            f[i] = y[3 * n + i];
            f[n + i] = y[4 * n + i];
            f[2 * n + i] = y[5 * n + i];
            f[3 * n + i] = 0.0;
            f[4 * n + i] = 0.0;
            f[5 * n + i] = 0.0;
        }
        out[sym_xy(i)] = xy;
        out[sym_xy(i) + kSymT] = zm;
    }
}

// First unit of range R: sum over R' < R of (n_jt - tpr R'), tpr = tiles per range.
__host__ __device__ __forceinline__ long long sym_range_start(long long R, long long n_jt,
                                                              int tpr) {
    return R * n_jt - (long long)tpr * (R * (R - 1) / 2);
}

template <int TPR>
struct SymCursor {
    int R, t;
    __device__ void locate(long long u, int n_jt, int n_ranges) {
        int lo = 0, hi = n_ranges - 1;  // largest R with start(R) <= u
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (sym_range_start(mid, n_jt, TPR) <= u) lo = mid;
            else hi = mid - 1;
        }
        R = lo;
        t = (int)(u - sym_range_start(lo, n_jt, TPR)) + TPR * lo;
    }
    __device__ void next(int n_jt) {
        if (++t == n_jt) {
            ++R;
            t = TPR * R;
        }
    }
};

template <bool CLAMP>
__device__ __forceinline__ void pair_uni(f2_t xj, f2_t yj, f2_t zj, f2_t xi, f2_t yi, f2_t zi,
                                         f2_t eps2, f2_t& ax, f2_t& ay, f2_t& az) {
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
    const f2_t inv3 = f2_mul(f2_mul(inv, inv), inv);
    ax = f2_fma(dx, inv3, ax);
    ay = f2_fma(dy, inv3, ay);
    az = f2_fma(dz, inv3, az);
}

__device__ __forceinline__ void sym_issue(float4* tiles, uint64_t* full, int s, int t,
                                          const float4* bodies) {
    mbar_arrive_expect_tx(&full[s], kSymTileBytes);
    bulk_g2s(tiles + s * 2 * kSymT, bodies + (size_t)t * 2 * kSymT, kSymTileBytes, &full[s]);
}

template <bool CLAMP, int MINB, int RUNR, int G = 4, bool UNI = false>
__global__ void __launch_bounds__(kSymThreads, MINB)
direct_sym_kernel(SymArgs a) {
    constexpr int kSymRange = sym_range(G);
    constexpr int kSymTilesPerRange = kSymRange / kSymT;
    constexpr int kSlots = 6 * G;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float4* tiles = reinterpret_cast<float4*>(smem_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + kSymStages * kSymTileBytes);
    uint64_t* empty = full + kSymStages;
    f2_t* acc_sm = reinterpret_cast<f2_t*>(smem_raw + kSymStages * kSymTileBytes +
                                           2 * kSymStages * sizeof(uint64_t));
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const long long per = a.units / gridDim.x;
    const long long rem = a.units % gridDim.x;
    const long long u0 = blockIdx.x * per + min((long long)blockIdx.x, rem);
    const long long cnt = per + ((long long)blockIdx.x < rem ? 1 : 0);
    const bool producer = threadIdx.x == 0;
    auto acc_at = [&](int q) -> f2_t& { return acc_sm[q * kSymThreads + threadIdx.x]; };

    if (producer) {
        for (int s = 0; s < kSymStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kSymWarps);
        }
        mbar_fence_init();
    }
    __syncthreads();
    SymCursor<kSymTilesPerRange> cons, prod;
    cons.locate(u0, a.n_jt, a.n_ranges);
    prod = cons;
    if (producer) {
        for (long long k = 0; k < kSymStages && k < cnt; ++k) {
            sym_issue(tiles, full, (int)k, prod.t, a.bodies);
            prod.next(a.n_jt);
        }
    }

    const f2_t eps2 = f2_pack(a.eps2, a.eps2);
    const f2_t zero = f2_pack(0.f, 0.f);
    f2_t xi[G], yi[G], zi[G], mi[G];
    int cur_R = -1;
    bool ok = true;
    const uint32_t tiles_addr = smem_addr(tiles);

    auto flush = [&](int R) {
#pragma unroll
        for (int g = 0; g < G; ++g) {
            float h0, h1, l0, l1;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                f2_unpack(acc_at(2 * (3 * g + c)), h0, h1);
                f2_unpack(acc_at(2 * (3 * g + c) + 1), l0, l1);
                const int i0 = R * kSymRange + (2 * g) * kSymThreads + warp * 32 + lane;
                const int i1 = i0 + kSymThreads;
                const double w = UNI ? a.m_uni : 1.0;  // the common mass, applied once
                if (i0 < a.n) atomicAdd(a.acc + (size_t)c * a.n + i0, w * ((double)h0 + (double)l0));
                if (i1 < a.n) atomicAdd(a.acc + (size_t)c * a.n + i1, w * ((double)h1 + (double)l1));
            }
        }
    };

    for (long long k = 0; k < cnt; ++k) {
        if (producer && k >= 1 && k - 1 + kSymStages < cnt) {
            const int sp = (int)((k - 1) % kSymStages);
            const uint32_t par = (uint32_t)(((k - 1) / kSymStages) & 1);
            if (!mbar_wait(&empty[sp], par, a.err)) {
                ok = false;
                break;
            }
            sym_issue(tiles, full, sp, prod.t, a.bodies);
            prod.next(a.n_jt);
        }
        if (cons.R != cur_R) {
            if (cur_R >= 0) flush(cur_R);
            cur_R = cons.R;
#pragma unroll
            for (int g = 0; g < G; ++g) {
                const int i0 = cur_R * kSymRange + (2 * g) * kSymThreads + warp * 32 + lane;
                const float4 p0 = __ldg(&a.bodies[sym_xy(i0)]);
                const float4 q0 = __ldg(&a.bodies[sym_xy(i0) + kSymT]);
                const float4 p1 = __ldg(&a.bodies[sym_xy(i0 + kSymThreads)]);
                const float4 q1 = __ldg(&a.bodies[sym_xy(i0 + kSymThreads) + kSymT]);
                xi[g] = f2_pack(p0.x, p1.x);
                yi[g] = f2_pack(p0.z, p1.z);
                zi[g] = f2_pack(q0.x, q1.x);
                mi[g] = f2_pack(q0.z, q1.z);
            }
#pragma unroll
            for (int q = 0; q < kSlots; ++q) acc_at(q) = zero;
        }
        const int s = (int)(k % kSymStages);
        if (!mbar_wait(&full[s], (uint32_t)((k / kSymStages) & 1), a.err)) {
            ok = false;
            break;
        }
        const uint32_t tbase = tiles_addr + (uint32_t)s * kSymTileBytes;
        f2_t ax[G], ay[G], az[G];
#pragma unroll
        for (int g = 0; g < G; ++g) ax[g] = ay[g] = az[g] = zero;
        if (cons.t < kSymTilesPerRange * (cons.R + 1)) {
            // own range: one-sided, broadcast loads
#pragma unroll 4
            for (int j = 0; j < kSymT; ++j) {
                const float4 p = lds128(tbase + 16u * j);
                const float4 q = lds128(tbase + 16u * (j + kSymT));
                const f2_t xj = f2_pack(p.x, p.y);
                const f2_t yj = f2_pack(p.z, p.w);
                const f2_t zj = f2_pack(q.x, q.y);
                const f2_t mj = f2_pack(q.z, q.w);
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    if constexpr (UNI)
                        pair_uni<CLAMP>(xj, yj, zj, xi[g], yi[g], zi[g], eps2, ax[g], ay[g], az[g]);
                    else
                        pair2<CLAMP>(xj, yj, zj, mj, xi[g], yi[g], zi[g], eps2, ax[g], ay[g],
                                     az[g]);
                }
            }
        } else {
#pragma unroll 1
            for (int c = 0; c < kSymT / 32; ++c) {
                const uint32_t cbase = tbase + (uint32_t)c * 512u;
                float bx = 0.f, by = 0.f, bz = 0.f;
#pragma unroll RUNR
                for (int r = 0; r < 32; ++r) {
                    const uint32_t off = cbase + ((uint32_t)((lane + r) & 31) << 4);
                    const float4 p = lds128(off);
                    const float4 q = lds128(off + 16u * kSymT);
                    const f2_t xj = f2_pack(p.x, p.y);
                    const f2_t yj = f2_pack(p.z, p.w);
                    const f2_t zj = f2_pack(q.x, q.y);
                    const f2_t mj = f2_pack(q.z, q.w);
                    f2_t px = zero, py = zero, pz = zero;
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        if constexpr (UNI)
                            sym_pair_uni<CLAMP>(xj, yj, zj, xi[g], yi[g], zi[g], eps2, ax[g],
                                                ay[g], az[g], px, py, pz);
                        else
                            sym_pair<CLAMP>(xj, yj, zj, mj, xi[g], yi[g], zi[g], mi[g], eps2,
                                            ax[g], ay[g], az[g], px, py, pz);
                    }
                    float l, h;
                    f2_unpack(px, l, h);
                    bx += l + h;
                    f2_unpack(py, l, h);
                    by += l + h;
                    f2_unpack(pz, l, h);
                    bz += l + h;
                    // the accumulator of B body (lane + r) moves to lane - 1,
                    // which meets that body at step r + 1
                    const int src = (lane + 1) & 31;
                    bx = __shfl_sync(0xffffffffu, bx, src);
                    by = __shfl_sync(0xffffffffu, by, src);
                    bz = __shfl_sync(0xffffffffu, bz, src);
                }
                // after 32 steps and shifts lane l holds the sum for B body l
                const int jb = cons.t * kSymT + c * 32 + lane;
                if (jb < a.n) {
                    const double w = UNI ? -a.m_uni : -1.0;
                    atomicAdd(a.acc + jb, w * (double)bx);
                    atomicAdd(a.acc + (size_t)a.n + jb, w * (double)by);
                    atomicAdd(a.acc + 2 * (size_t)a.n + jb, w * (double)bz);
                }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
#pragma unroll
        for (int g = 0; g < G; ++g) {
            f2_two_sum(acc_at(2 * (3 * g + 0)), acc_at(2 * (3 * g + 0) + 1), ax[g]);
            f2_two_sum(acc_at(2 * (3 * g + 1)), acc_at(2 * (3 * g + 1) + 1), ay[g]);
            f2_two_sum(acc_at(2 * (3 * g + 2)), acc_at(2 * (3 * g + 2) + 1), az[g]);
        }
        cons.next(a.n_jt);
    }
    if (ok && cur_R >= 0) flush(cur_R);
}

size_t sym_smem_bytes(int G) {
    return (size_t)kSymStages * kSymTileBytes + 2 * kSymStages * sizeof(uint64_t) +
           6 * G * kSymThreads * sizeof(f2_t);
}

nbg_status direct_sym_launch(nbg_engine* e, const double* y, double* f) {
    const int n = (int)e->count;
    const int G = e->tune_get("direct.sym_g", 4) == 3 ? 3 : 4;
    const int range = sym_range(G);
    const int n_ranges = (n + range - 1) / range;
    const int n_pad = n_ranges * range;
    const size_t need = 2 * (size_t)n_pad * sizeof(float4);
    if (e->xyzm_cap < need) {
        cudaFree(e->d_xyzm);
        e->d_xyzm = nullptr;
        e->xyzm_cap = 0;
        NBG_CUDA(e, cudaMalloc(&e->d_xyzm, need));
        e->xyzm_cap = need;
    }
    float4* bodies = reinterpret_cast<float4*>(e->d_xyzm);
    pack_sym_kernel<<<grid_for(n_pad, 256, (unsigned)e->sm_count * 8u), 256, 0, e->stream>>>(
        y, e->d_mass, bodies, f, n, n_pad);
    NBG_LAUNCHED(e, "pack_sym_kernel");
    const bool clamp = !(e->params.softening > 0.0);
    // "direct.sym_blocks": CTAs per SM the register budget is set for
    // (4: 128 registers, 5: 102)
    // "direct.sym_unroll": unroll of the 32-step rotation loop (1, 2, 4 or 8)
    const bool b5 = e->tune_get("direct.sym_blocks", 4) >= 5;
    const int64_t ru = e->tune_get("direct.sym_unroll", 4);
    using SymKernel = void (*)(SymArgs);
    SymKernel kern;
    // "direct.uniform_mass" (1, the default): with equal masses the kernel
    // that scales the pair sums by the common mass once
    const bool uni = e->uniform_mass && e->tune_get("direct.uniform_mass", 1) != 0;
#define NBG_SYM(MB, RU, GG)                                                                  \
    (uni ? (clamp ? direct_sym_kernel<true, MB, RU, GG, true> : direct_sym_kernel<false, MB, RU, GG, true>) \
         : (clamp ? direct_sym_kernel<true, MB, RU, GG> : direct_sym_kernel<false, MB, RU, GG>))
    if (G == 3)  // 6 A bodies per lane: fewer registers, 5 CTAs per SM
        kern = NBG_SYM(5, 4, 3);
    else if (b5)
        kern = NBG_SYM(5, 2, 4);
    else if (ru >= 8)
        kern = NBG_SYM(4, 8, 4);
    else if (ru >= 4)
        kern = NBG_SYM(4, 4, 4);
    else if (ru <= 1)
        kern = NBG_SYM(4, 1, 4);
    else
        kern = NBG_SYM(4, 2, 4);
#undef NBG_SYM
    const size_t smem = sym_smem_bytes(G);
    NBG_CUDA(e, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    int occ = 0;
    NBG_CUDA(e, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kSymThreads, smem));
    if (occ < 1) occ = 1;
    const int64_t bps = e->tune_get("direct.blocks_per_sm", 0);
    if (bps > 0 && bps < occ) occ = (int)bps;
    SymArgs a;
    a.bodies = bodies;
    a.acc = f + 3 * (size_t)n;
    a.m_uni = e->mass_value;
    a.n = n;
    a.n_jt = n_pad / kSymT;
    a.n_ranges = n_ranges;
    a.units = sym_range_start(n_ranges, a.n_jt, range / kSymT);
    a.eps2 = (float)(e->params.softening * e->params.softening);
    a.err = e->d_err;
    long long grid = (long long)e->sm_count * occ;
    if (grid > a.units) grid = a.units;
    ProfScope ps(e, NBG_K_DIRECT);
    kern<<<(unsigned)grid, kSymThreads, smem, e->stream>>>(a);
    NBG_LAUNCHED(e, "direct_sym_kernel");
    return NBG_OK;
}

}  // namespace

nbg_status direct_fcompute(nbg_engine* e, const double* y, double* f) {
    const int n = (int)e->count;
    if (e->params.precision == NBG_PREC_FP64) {
        ProfScope ps(e, NBG_K_DIRECT);
        direct_fp64_kernel<<<(n + kF64Threads - 1) / kF64Threads, kF64Threads, 0, e->stream>>>(
            y, e->d_mass, f, n);
        NBG_LAUNCHED(e, "direct_fp64_kernel");
        return NBG_OK;
    }

    // ---- mixed precision ----
    if (e->tune_get("direct.symmetric", 1) != 0) return direct_sym_launch(e, y, f);
    const int n_jt = (n + kT - 1) / kT;
    const int n_pad = n_jt * kT;
    const size_t need = (size_t)n_pad * sizeof(Body2);
    if (e->xyzm_cap < need) {
        cudaFree(e->d_xyzm);
        e->d_xyzm = nullptr;
        e->xyzm_cap = 0;
        NBG_CUDA(e, cudaMalloc(&e->d_xyzm, need));
        e->xyzm_cap = need;
    }
    Body2* bodies = reinterpret_cast<Body2*>(e->d_xyzm);
    pack_mixed_kernel<<<grid_for(n_pad, 256, (unsigned)e->sm_count * 8u), 256, 0, e->stream>>>(
        y, e->d_mass, bodies, f, n, n_pad);
    NBG_LAUNCHED(e, "pack_mixed_kernel");

    const bool clamp = !(e->params.softening > 0.0);
    const int G = e->tune_get("direct.pairs_per_lane", 4) >= 4 ? 4 : 2;
    const int unr = (int)e->tune_get("direct.unroll", 4);
    MixedKernel kern = clamp ? pick_mixed<true>(G, unr) : pick_mixed<false>(G, unr);
    const size_t smem = mixed_smem_bytes(G);
    NBG_CUDA(e, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    int occ = 0;
    NBG_CUDA(e, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kThreadsMixed, smem));
    if (occ < 1) occ = 1;
    const int64_t bps = e->tune_get("direct.blocks_per_sm", 0);
    if (bps > 0 && bps < occ) occ = (int)bps;
    MixedArgs a;
    a.bodies = bodies;
    a.acc = f + 3 * (size_t)n;
    a.n = n;
    a.n_jt = n_jt;
    const int ib_size = kThreadsMixed * 2 * G;
    const long long n_ib = (n + ib_size - 1) / ib_size;
    a.units = n_ib * n_jt;
    a.eps2 = (float)(e->params.softening * e->params.softening);
    a.err = e->d_err;
    long long grid = (long long)e->sm_count * occ;
    if (grid > a.units) grid = a.units;
    ProfScope ps(e, NBG_K_DIRECT);
    kern<<<(unsigned)grid, kThreadsMixed, smem, e->stream>>>(a);
    NBG_LAUNCHED(e, "direct_mixed_kernel");
    return NBG_OK;
}

}  // namespace nbg

// ---------------------------------------------------------------------------
// Allocation-free variant of the mixed-precision direct sum
// ---------------------------------------------------------------------------
// Some callers cannot call cudaMalloc: a host application that owns all GPU
// memory through its own arena and forbids allocations behind its back, or a
// time-stepping loop with a hard latency budget where an allocation (and the
// device synchronisation it implies) is not allowed.  For them the packed-body
// scratch of the kernel above lives in a fixed file-scope device array instead
// of an engine allocation.  The array is created with this module on every GPU
// that loads the library and stays there until the process exits, so its size
// is capped: NBG_NOALLOC_MAX_BODIES bodies x 32 bytes = 4 MiB, plus one error
// word.
namespace nbg {
namespace {

static __device__ __align__(256) Body2 g_noalloc_bodies[NBG_NOALLOC_MAX_BODIES];
static __device__ __align__(256) unsigned g_noalloc_err;

constexpr int kNoallocMaxDevices = 64;
struct NoallocDevice {
    bool ready;
    Body2* bodies;  // device address of g_noalloc_bodies on this device
    unsigned* err;  // device address of g_noalloc_err on this device
    int sm_count;
};
std::mutex g_noalloc_mu;
NoallocDevice g_noalloc_dev[kNoallocMaxDevices];

}  // namespace
}  // namespace nbg

extern "C" nbg_status nbg_direct_mixed_noalloc(const double* y, const double* mass, double* f,
                                               size_t n, double softening, void* stream) {
    using namespace nbg;
    if (y == nullptr || mass == nullptr || f == nullptr || n == 0 || !(softening >= 0.0))
        return NBG_ERR_INVALID_ARG;
    if (n > (size_t)NBG_NOALLOC_MAX_BODIES) return NBG_ERR_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoallocMaxDevices)
        return NBG_ERR_CUDA;

    // One-time set-up per device, on the current device: host code cannot use
    // the array's name as a device address, so look the address up.
    NoallocDevice d;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        NoallocDevice& slot = g_noalloc_dev[dev];
        if (!slot.ready) {
            void* pb = nullptr;
            void* pe = nullptr;
            if (cudaGetSymbolAddress(&pb, g_noalloc_bodies) != cudaSuccess ||
                cudaGetSymbolAddress(&pe, g_noalloc_err) != cudaSuccess ||
                cudaDeviceGetAttribute(&slot.sm_count, cudaDevAttrMultiProcessorCount, dev) !=
                    cudaSuccess) {
                cudaGetLastError();
                return NBG_ERR_CUDA;
            }
            slot.bodies = static_cast<Body2*>(pb);
            slot.err = static_cast<unsigned*>(pe);
            slot.ready = true;
        }
        d = slot;
    }

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nn = (int)n;
    const int n_jt = (nn + kT - 1) / kT;
    const int n_pad = n_jt * kT;
    const bool clamp = !(softening > 0.0);
    constexpr int G = 4;
    MixedKernel kern = clamp ? pick_mixed<true>(G, 4) : pick_mixed<false>(G, 4);
    const size_t smem = mixed_smem_bytes(G);
    int occ = 0;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kThreadsMixed, smem) !=
            cudaSuccess) {
        cudaGetLastError();
        return NBG_ERR_CUDA;
    }
    if (occ < 1) occ = 1;

    // The error word must start at zero; the pack kernel rewrites every
    // scratch entry the force kernel reads (padding included) and zeroes the
    // acceleration half of f, so nothing else carries over from earlier calls.
    if (cudaMemsetAsync(d.err, 0, sizeof(unsigned), st) != cudaSuccess) {
        cudaGetLastError();
        return NBG_ERR_CUDA;
    }
    pack_mixed_kernel<<<grid_for(n_pad, 256, (unsigned)d.sm_count * 8u), 256, 0, st>>>(
        y, mass, d.bodies, f, nn, n_pad);
    MixedArgs a;
    a.bodies = d.bodies;
    a.acc = f + 3 * n;
    a.n = nn;
    a.n_jt = n_jt;
    const long long n_ib = (nn + kThreadsMixed * 2 * G - 1) / (kThreadsMixed * 2 * G);
    a.units = n_ib * n_jt;
    a.eps2 = (float)(softening * softening);
    a.err = d.err;
    long long grid = (long long)d.sm_count * occ;
    if (grid > a.units) grid = a.units;
    kern<<<(unsigned)grid, kThreadsMixed, smem, st>>>(a);
    if (cudaGetLastError() != cudaSuccess) return NBG_ERR_CUDA;

    // Synchronous: the result is in f when this returns, and a device-side
    // wait that timed out is reported here.  The error word is read on the
    // caller's stream, so the call waits for that stream only (a plain
    // cudaMemcpy would go through the legacy default stream and wait for
    // unrelated work on other blocking streams).
    unsigned err_host = 0;
    if (cudaMemcpyAsync(&err_host, d.err, sizeof(unsigned), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return NBG_ERR_CUDA;
    }
    return err_host != 0 ? NBG_ERR_DEVICE_TIMEOUT : NBG_OK;
}
