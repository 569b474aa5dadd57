// nbg_judge.cu -- the learned Barnes-Hut path's per-step judge (no reference
// counterpart).
//
// Once per engine step (the first fcompute of the step) the learned walk's
// accelerations are judged on a seeded sample of S leaves (default 4096, a
// power of two; leaves p_k = k (N / S) + off, off drawn from (seed, step),
// so the sample is spread evenly along the tree's leaf order and changes
// every step):
//   1. the exact accelerations of the sampled bodies: a direct sum over all N
//      bodies (packed FP32x2 pair math from the tree's FP32 leaf records,
//      per-tile sums folded into two-sum pairs, FP64 atomics across the
//      j-chunks), the engine's own softening or the reference clamp;
//   2. the plain Barnes-Hut accelerations of the same bodies at the tight
//      ratio lambda_t (the fallback's opening ratio, theta_t = 1 / lambda_t):
//      a per-body walk, one warp per body, over the same tree with its
//      critical radii scaled from lambda_l to lambda_t, accepting a node when
//      d^2 > crit^2 from the body -- the reference's per-body rule
//      (nbody/nbody_space_heap_stackless.cpp:3-28), whose error bounds the
//      plain group walk's from above;
//   3. one CTA forms the relative errors |a - a_exact| / |a_exact| of the
//      learned and the plain forces, sorts both (bitonic sort in shared
//      memory) and writes p50, p99 (linear interpolation between order
//      statistics), RMS and the decision: the plain walk replaces the
//      learned one for the whole step when the learned p99 exceeds the
//      plain p99.
// The host reads the eight figures back (one small copy and a stream
// synchronisation per judged step) and runs the fallback itself.
#include <algorithm>
#include <cmath>

#include "nbg_ptx.cuh"
#include "nbg_tree.cuh"

namespace nbg {

struct JudgeState {
    double* ref = nullptr;    // [3][kJudgeMax] exact accelerations of the sample
    double* plain = nullptr;  // [3][kJudgeMax] plain walk at lambda_t
    double* stats = nullptr;  // [8] device figures
    double* h_stats = nullptr;  // [8] pinned copy
};

namespace {

constexpr int kJDThreads = 256;
constexpr int kJDPairs = 2;                     // packed row pairs per thread
constexpr int kJDRows = 2 * kJDPairs;           // rows per thread
constexpr int kJDRowsPerCta = kJDThreads * kJDRows;
constexpr int kJDTile = 256;                    // j bodies per shared-memory tile

constexpr int kJWWarps = 4;
constexpr int kJWThreads = kJWWarps * 32;
// per-warp node stack: as the group walk's, 48 entries per tree level + 32
// (a step pops 16 entries and pushes at most 32)
inline int judge_stack_cap(int levels) { return 48 * (levels + 1) + 32; }

constexpr int kJRThreads = 1024;

__device__ __forceinline__ int sample_leaf(int n, int k, int stride, int off) {
    return n + k * stride + off;
}

// Exact accelerations of the sampled bodies, rows x j-chunks.  The j tile is
// kept as (x, x, y, y | z, z, m, m) so that two LDS.128 give the packed
// operands of one j body for a pair of rows.
template <bool CLAMP>
__global__ void __launch_bounds__(kJDThreads)
judge_direct_kernel(TreeState t, int n, int S, int stride, int off, int chunk, float eps2,
                    double* __restrict__ ref) {
    __shared__ __align__(16) float4 tile[2 * kJDTile];
    f2_t xi[kJDPairs], yi[kJDPairs], zi[kJDPairs];
#pragma unroll
    for (int p = 0; p < kJDPairs; ++p) {
        float v[2][3];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = blockIdx.x * kJDRowsPerCta + (2 * p + h) * kJDThreads + threadIdx.x;
            const float4 me = __ldg(&t.node4[sample_leaf(n, k < S ? k : 0, stride, off)]);
            v[h][0] = me.x;
            v[h][1] = me.y;
            v[h][2] = me.z;
        }
        xi[p] = f2_pack(v[0][0], v[1][0]);
        yi[p] = f2_pack(v[0][1], v[1][1]);
        zi[p] = f2_pack(v[0][2], v[1][2]);
    }
    const f2_t e2 = f2_pack(eps2, eps2);
    f2_t hx[kJDPairs], hy[kJDPairs], hz[kJDPairs], lx[kJDPairs], ly[kJDPairs], lz[kJDPairs];
#pragma unroll
    for (int p = 0; p < kJDPairs; ++p) hx[p] = hy[p] = hz[p] = lx[p] = ly[p] = lz[p] = 0ull;
    const int j0 = blockIdx.y * chunk;
    const int j1 = min(n, j0 + chunk);
    for (int jt = j0; jt < j1; jt += kJDTile) {
        __syncthreads();
        const int j = jt + threadIdx.x;
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
        if (j < j1) {
            const float4 nd = __ldg(&t.node4[n + j]);
            const float m = __ldg(&t.nodem[n + j]);
            a = make_float4(nd.x, nd.x, nd.y, nd.y);
            b = make_float4(nd.z, nd.z, m, m);  // past the end: zero mass adds nothing
        }
        tile[2 * threadIdx.x] = a;
        tile[2 * threadIdx.x + 1] = b;
        __syncthreads();
        f2_t px[kJDPairs], py[kJDPairs], pz[kJDPairs];
#pragma unroll
        for (int p = 0; p < kJDPairs; ++p) px[p] = py[p] = pz[p] = 0ull;
        const uint32_t base = smem_addr(tile);
#pragma unroll 4
        for (int q = 0; q < kJDTile; ++q) {
            const float4 A = lds128(base + 32u * q);
            const float4 B = lds128(base + 32u * q + 16u);
            f2_t xj, yj, zj, mj;
            asm("mov.b64 %0, {%1, %2};" : "=l"(xj) : "f"(A.x), "f"(A.y));
            asm("mov.b64 %0, {%1, %2};" : "=l"(yj) : "f"(A.z), "f"(A.w));
            asm("mov.b64 %0, {%1, %2};" : "=l"(zj) : "f"(B.x), "f"(B.y));
            asm("mov.b64 %0, {%1, %2};" : "=l"(mj) : "f"(B.z), "f"(B.w));
#pragma unroll
            for (int p = 0; p < kJDPairs; ++p) {
                const f2_t dx = f2_sub(xj, xi[p]);
                const f2_t dy = f2_sub(yj, yi[p]);
                const f2_t dz = f2_sub(zj, zi[p]);
                f2_t r2 = f2_fma(dz, dz, e2);
                r2 = f2_fma(dy, dy, r2);
                r2 = f2_fma(dx, dx, r2);
                float ra, rb;
                f2_unpack(r2, ra, rb);
                if (CLAMP) {
                    ra = fmaxf(ra, 1e-8f);
                    rb = fmaxf(rb, 1e-8f);
                }
                const f2_t inv = f2_pack(rsqrt_mufu(ra), rsqrt_mufu(rb));
                const f2_t s3 = f2_mul(f2_mul(mj, inv), f2_mul(inv, inv));
                px[p] = f2_fma(dx, s3, px[p]);
                py[p] = f2_fma(dy, s3, py[p]);
                pz[p] = f2_fma(dz, s3, pz[p]);
            }
        }
#pragma unroll
        for (int p = 0; p < kJDPairs; ++p) {
            f2_two_sum(hx[p], lx[p], px[p]);
            f2_two_sum(hy[p], ly[p], py[p]);
            f2_two_sum(hz[p], lz[p], pz[p]);
        }
    }
#pragma unroll
    for (int p = 0; p < kJDPairs; ++p) {
        float h[3][2], l[3][2];
        f2_unpack(hx[p], h[0][0], h[0][1]);
        f2_unpack(hy[p], h[1][0], h[1][1]);
        f2_unpack(hz[p], h[2][0], h[2][1]);
        f2_unpack(lx[p], l[0][0], l[0][1]);
        f2_unpack(ly[p], l[1][0], l[1][1]);
        f2_unpack(lz[p], l[2][0], l[2][1]);
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            const int k = blockIdx.x * kJDRowsPerCta + (2 * p + hh) * kJDThreads + threadIdx.x;
            if (k < S)
                for (int c = 0; c < 3; ++c)
                    atomicAdd(&ref[3 * k + c], (double)h[c][hh] + (double)l[c][hh]);
        }
    }
}

// Plain per-body walk of the sampled bodies at the critical radii scaled by
// crit_scale = (lambda_t / lambda_l)^2, one warp per body, 32 node tests per
// step (the structure of the group walk's per-body fallback).
template <bool CLAMP>
__global__ void __launch_bounds__(kJWThreads)
judge_walk_kernel(TreeState t, int n, int S, int stride, int off, float eps2, float crit_scale,
                  int stack_cap, double* __restrict__ plain, unsigned* err) {
    extern __shared__ int judge_stacks[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    int* stack = judge_stacks + warp * stack_cap;
    const int warps = gridDim.x * kJWWarps;
    for (int k = blockIdx.x * kJWWarps + warp; k < S; k += warps) {
        const float4 me = __ldg(&t.node4[sample_leaf(n, k, stride, off)]);
        float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
        auto add = [](float& h, float& l, float p) {
            const float s = h + p, bp = s - h;
            l += (h - (s - bp)) + (p - bp);
            h = s;
        };
        __syncwarp();
        if (lane == 0) stack[0] = 0;  // entry 0 stands for the root (children 0 and 1)
        __syncwarp();
        int sp = 1;
        bool overflow = false;
        while (sp > 0) {
            const int m = min(sp, 16);
            int c = 0;
            if (lane < 2 * m) c = 2 * stack[sp - 1 - (lane >> 1)] + (lane & 1);
            __syncwarp();
            sp -= m;
            const bool valid = lane < 2 * m && c != 0;
            bool accept = false, open = false;
            float dx = 0.f, dy = 0.f, dz = 0.f;
            if (valid) {
                const float4 nd = __ldg(&t.node4[c]);
                dx = nd.x - me.x;
                dy = nd.y - me.y;
                dz = nd.z - me.z;
                accept = c >= n || fmaf(dx, dx, fmaf(dy, dy, dz * dz)) > nd.w * crit_scale;
                open = !accept;
            }
            if (accept) {
                float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
                if (CLAMP) r2 = fmaxf(r2, 1e-8f);
                const float inv = rsqrt_mufu(r2);
                const float s3 = __ldg(&t.nodem[c]) * (inv * inv * inv);
                add(hx, lx, dx * s3);
                add(hy, ly, dy * s3);
                add(hz, lz, dz * s3);
            }
            const unsigned om = __ballot_sync(0xffffffffu, open);
            const int npush = __popc(om);
            if (sp + npush > stack_cap) {  // reported, never written
                if (lane == 0) atomicOr(err, kDevErrWalkOverflow);
                overflow = true;
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
            plain[3 * k] = overflow ? NAN : ax;
            plain[3 * k + 1] = overflow ? NAN : ay;
            plain[3 * k + 2] = overflow ? NAN : az;
        }
    }
}

__device__ __forceinline__ float rel_err(double ax, double ay, double az, double rx, double ry,
                                         double rz) {
    const double dx = ax - rx, dy = ay - ry, dz = az - rz;
    const double nr = sqrt(rx * rx + ry * ry + rz * rz);
    const double e = nr > 0.0 ? sqrt(dx * dx + dy * dy + dz * dz) / nr : 0.0;
    const float v = (float)e;
    return v < INFINITY ? v : INFINITY;  // NaN and overflow sort last
}

// Ascending bitonic sort of v[0, P) (P a power of two) by the whole block.
__device__ void bitonic_sort(float* v, int P) {
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            __syncthreads();
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    const float a = v[i], b = v[l];
                    if ((a > b) == up) {
                        v[i] = b;
                        v[l] = a;
                    }
                }
            }
        }
    }
    __syncthreads();
}

// numpy's default quantile: linear interpolation between order statistics
__device__ __forceinline__ double quantile(const float* v, int S, double q) {
    const double pos = q * (double)(S - 1);
    const int lo = (int)floor(pos);
    const int hi = min(lo + 1, S - 1);
    const double fr = pos - (double)lo;
    return (double)v[lo] + fr * ((double)v[hi] - (double)v[lo]);
}

__global__ void __launch_bounds__(kJRThreads)
judge_reduce_kernel(TreeState t, int n, int S, int P, int stride, int off,
                    const double* __restrict__ f, const double* __restrict__ ref,
                    const double* __restrict__ plain, double* __restrict__ stats) {
    __shared__ float el[kJudgeMax], ep[kJudgeMax];
    __shared__ double part[2][kJRThreads / 32];
    double sl = 0.0, sp = 0.0;
    for (int k = threadIdx.x; k < P; k += blockDim.x) {
        if (k < S) {
            const int b = t.body_n[sample_leaf(n, k, stride, off)];
            const double rx = ref[3 * k], ry = ref[3 * k + 1], rz = ref[3 * k + 2];
            el[k] = rel_err(f[3 * (size_t)n + b], f[4 * (size_t)n + b], f[5 * (size_t)n + b], rx,
                            ry, rz);
            ep[k] = rel_err(plain[3 * k], plain[3 * k + 1], plain[3 * k + 2], rx, ry, rz);
            sl += (double)el[k] * el[k];
            sp += (double)ep[k] * ep[k];
        } else {
            el[k] = INFINITY;
            ep[k] = INFINITY;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        sl += __shfl_xor_sync(0xffffffffu, sl, o);
        sp += __shfl_xor_sync(0xffffffffu, sp, o);
    }
    if ((threadIdx.x & 31) == 0) {
        part[0][threadIdx.x >> 5] = sl;
        part[1][threadIdx.x >> 5] = sp;
    }
    bitonic_sort(el, P);
    bitonic_sort(ep, P);
    if (threadIdx.x == 0) {
        double tl = 0.0, tp = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
            tl += part[0][w];
            tp += part[1][w];
        }
        const double p99l = quantile(el, S, 0.99), p99p = quantile(ep, S, 0.99);
        stats[0] = quantile(el, S, 0.5);
        stats[1] = p99l;
        stats[2] = quantile(ep, S, 0.5);
        stats[3] = p99p;
        stats[4] = sqrt(tl / S);
        stats[5] = sqrt(tp / S);
        stats[6] = (p99l > p99p || !(p99l < INFINITY)) ? 1.0 : 0.0;
        stats[7] = (double)S;
    }
}

__host__ __device__ inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

}  // namespace

void judge_destroy(nbg_engine* e) {
    JudgeState* J = e->judge;
    if (J == nullptr) return;
    cudaFree(J->ref);
    cudaFree(J->plain);
    cudaFree(J->stats);
    cudaFreeHost(J->h_stats);
    delete J;
    e->judge = nullptr;
}

nbg_status judge_learned(nbg_engine* e, uint64_t step, const double* f, double lam_l,
                         double lam_t, JudgeResult* out) {
    if (e->tree == nullptr || !e->tree->built)
        return set_error(e, NBG_ERR_NOT_INITIALIZED, "judge: no tree");
    if (e->judge == nullptr) {
        JudgeState* J = new JudgeState();
        e->judge = J;
        NBG_CUDA(e, cudaMalloc(&J->ref, 3 * kJudgeMax * sizeof(double)));
        NBG_CUDA(e, cudaMalloc(&J->plain, 3 * kJudgeMax * sizeof(double)));
        NBG_CUDA(e, cudaMalloc(&J->stats, 8 * sizeof(double)));
        NBG_CUDA(e, cudaMallocHost(&J->h_stats, 8 * sizeof(double)));
    }
    JudgeState* J = e->judge;
    const TreeState& t = *e->tree;
    const int n = (int)e->count;  // a power of two (Barnes-Hut)
    // S: the requested sample, rounded down to a power of two, at most
    // kJudgeMax and n; stride n / S is then exact
    const int64_t want = std::max<int64_t>(1, e->tune_get("learned.judge_samples", kJudgeMax));
    int S = 1;
    while (2 * (int64_t)S <= want && 2 * S <= kJudgeMax && 2 * S <= n) S *= 2;
    const int stride = n / S;
    const uint64_t seed = (uint64_t)e->tune_get("learned.judge_seed", 1);
    const int off = (int)(splitmix64(seed * 0x100000001B3ull ^ step) % (uint64_t)stride);
    const float eps2 = (float)(e->params.softening * e->params.softening);
    const bool clamp = !(e->params.softening > 0.0);
    ProfScope ps(e, NBG_K_JUDGE);
    NBG_CUDA(e, cudaMemsetAsync(J->ref, 0, 3 * (size_t)S * sizeof(double), e->stream));
    // 1. direct sum: row blocks x j-chunks, about 4 CTAs per SM in all
    const int gx = (S + kJDRowsPerCta - 1) / kJDRowsPerCta;
    const int tiles = (n + kJDTile - 1) / kJDTile;
    const int gy = std::max(1, std::min(tiles, (4 * e->sm_count + gx - 1) / gx));
    const int chunk = ((tiles + gy - 1) / gy) * kJDTile;
    const int gy_used = (n + chunk - 1) / chunk;
    if (clamp)
        judge_direct_kernel<true><<<dim3(gx, gy_used), kJDThreads, 0, e->stream>>>(
            t, n, S, stride, off, chunk, eps2, J->ref);
    else
        judge_direct_kernel<false><<<dim3(gx, gy_used), kJDThreads, 0, e->stream>>>(
            t, n, S, stride, off, chunk, eps2, J->ref);
    NBG_LAUNCHED(e, "judge_direct_kernel");
    // 2. plain per-body walk at lambda_t
    const int stack_cap = judge_stack_cap(t.levels);
    const size_t wsmem = (size_t)kJWWarps * stack_cap * sizeof(int);
    const float crit_scale = (float)((lam_t / lam_l) * (lam_t / lam_l));
    auto wk = clamp ? judge_walk_kernel<true> : judge_walk_kernel<false>;
    NBG_CUDA(e, cudaFuncSetAttribute(wk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wsmem));
    const unsigned wblocks = (unsigned)std::min((S + kJWWarps - 1) / kJWWarps, e->sm_count * 8);
    wk<<<wblocks, kJWThreads, wsmem, e->stream>>>(t, n, S, stride, off, eps2, crit_scale,
                                                  stack_cap, J->plain, e->d_err);
    NBG_LAUNCHED(e, "judge_walk_kernel");
    // 3. errors, percentiles, decision
    int P = 1;
    while (P < S) P *= 2;
    judge_reduce_kernel<<<1, kJRThreads, 0, e->stream>>>(t, n, S, P, stride, off, f, J->ref,
                                                         J->plain, J->stats);
    NBG_LAUNCHED(e, "judge_reduce_kernel");
    NBG_CUDA(e, cudaMemcpyAsync(J->h_stats, J->stats, 8 * sizeof(double), cudaMemcpyDeviceToHost,
                                e->stream));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    const double* h = J->h_stats;
    out->p50_learned = h[0];
    out->p99_learned = h[1];
    out->p50_plain = h[2];
    out->p99_plain = h[3];
    out->rms_learned = h[4];
    out->rms_plain = h[5];
    out->use_plain = h[6] != 0.0;
    out->samples = (int)h[7];
    return NBG_OK;
}

}  // namespace nbg
