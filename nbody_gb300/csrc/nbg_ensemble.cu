// nbg_ensemble.cu -- many independent systems stepped together.
//
// No reference counterpart as a whole; it restates, per system, what the
// reference does for one: an explicit embedded Runge-Kutta step
// (Dormand-Prince table, nbody/nbody_solver_rkdp.cpp:30-62; the stage loop of
// nbody/nbody_solver_rk_butcher.cpp:130-162) around the direct-sum RHS.
// Differences, all on the device so a whole step runs without a host round
// trip and is captured once as a CUDA graph:
//   * every system has its own step dt_s; the embedded error
//     e_s = dt_s * max |sum_i (b2_i - b1_i) k_i| decides accept / reject and
//     the next dt_s = dt_s * clamp(0.9 (tol / e_s)^(1/5), 0.2, 5)
//     (the reference compares the unscaled max |sum (b2 - b1) k| with its
//     threshold and subdivides recursively, nbody/nbody_solver_rk_butcher.cpp:
//     209-231; a per-system controller replaces that host-side recursion);
//   * the accepted update is y += dt_s * sum_i b2_i k_i (the reference also
//     advances with b2, nbody/nbody_solver_rk_butcher.cpp:233-245).
// The RHS is the mixed-precision direct sum: FP32 pair math in packed FP32x2,
// compensated tile sums, FP64 state.  One persistent kernel serves all
// systems: CTAs take (system, 256-body i-block) units from an atomic counter,
// largest systems first.
#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "nbg_internal.cuh"
#include "nbg_pair.cuh"
#include "nbg_ptx.cuh"
#include "nbg_stats.cuh"
#include "nbg_tune.cuh"

namespace nbg {
namespace {

constexpr int kEnsThreads = 128;
constexpr int kEnsTile = 128;
constexpr int kStagesRK = 7;

// Dormand-Prince 5(4) (nbody/nbody_solver_rkdp.cpp:30-62)
__constant__ double c_a[kStagesRK][kStagesRK] = {
    {0, 0, 0, 0, 0, 0, 0},
    {1.0 / 5, 0, 0, 0, 0, 0, 0},
    {3.0 / 40, 9.0 / 40, 0, 0, 0, 0, 0},
    {44.0 / 45, -56.0 / 15, 32.0 / 9, 0, 0, 0, 0},
    {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729, 0, 0, 0},
    {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656, 0, 0},
    {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84, 0}};
__constant__ double c_b1[kStagesRK] = {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192,
                                       -2187.0 / 6784, 11.0 / 84, 0};
__constant__ double c_b2[kStagesRK] = {5179.0 / 57600, 0, 7571.0 / 16695, 393.0 / 640,
                                       -92097.0 / 339200, 187.0 / 2100, 1.0 / 40};

struct Body2 {
    float4 xxyy;
    float4 zzmm;
};

struct EnsUnit {
    int sys;
    int i0;  // first system-local body of the block
};

struct KPtrs {
    double* k[kStagesRK];
};

// Stage i: s = y + dt_s sum_{j<i} a_ij k_j; writes the FP32 body records of s
// and the velocity half of k_i (= velocity of s).
__global__ void ens_stage_kernel(int stage, const double* __restrict__ y,
                                 const double* __restrict__ mass, const int* __restrict__ sys,
                                 const double* __restrict__ dt, KPtrs kp, size_t B,
                                 Body2* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < B;
         i += (size_t)gridDim.x * blockDim.x) {
        const double h = dt[sys[i]];
        double s[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) s[c] = y[c * B + i];
        for (int j = 0; j < stage; ++j) {
            const double a = c_a[stage][j] * h;
            if (a == 0.0) continue;
            const double* kj = kp.k[j];
#pragma unroll
            for (int c = 0; c < 6; ++c) s[c] = fma(a, kj[c * B + i], s[c]);
        }
        double* ki = kp.k[stage];
        ki[i] = s[3];
        ki[B + i] = s[4];
        ki[2 * B + i] = s[5];
        const float x = (float)s[0], yy = (float)s[1], z = (float)s[2], m = (float)mass[i];
        Body2 b;
        b.xxyy = make_float4(x, x, yy, yy);
        b.zzmm = make_float4(z, z, m, m);
        out[i] = b;
    }
}

template <bool CLAMP>
__device__ __forceinline__ void pair2e(f2_t xj, f2_t yj, f2_t zj, f2_t mj, f2_t xi, f2_t yi,
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

// Equal masses within a system: the pair weight is r^-3 alone and the
// system's mass scales the sums once, in FP64 (one packed multiply fewer).
template <bool CLAMP>
__device__ __forceinline__ void pair2e_uni(f2_t xj, f2_t yj, f2_t zj, f2_t xi, f2_t yi, f2_t zi,
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
    const f2_t s3 = f2_mul(f2_mul(inv, inv), inv);
    ax = f2_fma(dx, s3, ax);
    ay = f2_fma(dy, s3, ay);
    az = f2_fma(dz, s3, az);
}

// Persistent direct sum over all systems.  Each lane holds G packed pairs
// (2G i-bodies: slots r = 0 .. 2G-1 at i0 + r * 128 + threadIdx.x).  UNI:
// every system has equal masses, sys_mass[s] its mass.
template <bool CLAMP, int G, int U = 4, bool UNI = false>
__global__ void __launch_bounds__(kEnsThreads)
ens_force_kernel(const Body2* __restrict__ bodies, const long long* __restrict__ off,
                 const int* __restrict__ cnt, const EnsUnit* __restrict__ units, int nunits,
                 unsigned* __restrict__ counter, double* __restrict__ acc, size_t B, float eps2v,
                 const double* __restrict__ sys_mass) {
    __shared__ __align__(16) Body2 tile[kEnsTile];
    __shared__ int next_unit;
    const f2_t eps2 = f2_pack(eps2v, eps2v);
    const f2_t zero = f2_pack(0.f, 0.f);
    const uint32_t tbase = smem_addr(tile);
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) next_unit = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int u = next_unit;
        if (u >= nunits) break;
        const EnsUnit un = units[u];
        const long long o = off[un.sys];
        const int n = cnt[un.sys];
        f2_t xi[G], yi[G], zi[G], hx[G], hy[G], hz[G], lx[G], ly[G], lz[G];
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const int l0 = un.i0 + (2 * g) * kEnsThreads + threadIdx.x;
            const int l1 = l0 + kEnsThreads;
            float x0 = 0.f, y0 = 0.f, z0 = 0.f, x1 = 0.f, y1 = 0.f, z1 = 0.f;
            if (l0 < n) {
                const Body2 b = bodies[o + l0];
                x0 = b.xxyy.x; y0 = b.xxyy.z; z0 = b.zzmm.x;
            }
            if (l1 < n) {
                const Body2 b = bodies[o + l1];
                x1 = b.xxyy.x; y1 = b.xxyy.z; z1 = b.zzmm.x;
            }
            xi[g] = f2_pack(x0, x1);
            yi[g] = f2_pack(y0, y1);
            zi[g] = f2_pack(z0, z1);
            hx[g] = hy[g] = hz[g] = lx[g] = ly[g] = lz[g] = zero;
        }
        for (int j0 = 0; j0 < n; j0 += kEnsTile) {
            __syncthreads();
            const int lj = j0 + threadIdx.x;
            Body2 b;
            if (lj < n) {
                b = bodies[o + lj];
            } else {  // zero-mass padding at the origin
                b.xxyy = make_float4(0.f, 0.f, 0.f, 0.f);
                b.zzmm = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            tile[threadIdx.x] = b;
            __syncthreads();
            f2_t ax[G], ay[G], az[G];
#pragma unroll
            for (int g = 0; g < G; ++g) ax[g] = ay[g] = az[g] = zero;
            const int jn = min(kEnsTile, n - j0);
#pragma unroll U
            for (int j = 0; j < jn; ++j) {
                const float4 p0 = lds128(tbase + 32u * j);
                const float4 p1 = lds128(tbase + 32u * j + 16u);
                const f2_t xj = f2_pack(p0.x, p0.y), yj = f2_pack(p0.z, p0.w);
                const f2_t zj = f2_pack(p1.x, p1.y), mj = f2_pack(p1.z, p1.w);
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    if constexpr (UNI)
                        pair2e_uni<CLAMP>(xj, yj, zj, xi[g], yi[g], zi[g], eps2, ax[g], ay[g],
                                          az[g]);
                    else
                        pair2e<CLAMP>(xj, yj, zj, mj, xi[g], yi[g], zi[g], eps2, ax[g], ay[g],
                                      az[g]);
                }
            }
#pragma unroll
            for (int g = 0; g < G; ++g) {
                f2_two_sum(hx[g], lx[g], ax[g]);
                f2_two_sum(hy[g], ly[g], ay[g]);
                f2_two_sum(hz[g], lz[g], az[g]);
            }
        }
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const int l0 = un.i0 + (2 * g) * kEnsThreads + threadIdx.x;
            const int l1 = l0 + kEnsThreads;
            float h0, h1, q0, q1;
            if (l0 < n || l1 < n) {
                const f2_t hh[3] = {hx[g], hy[g], hz[g]};
                const f2_t ll[3] = {lx[g], ly[g], lz[g]};
                const double w = UNI ? sys_mass[un.sys] : 1.0;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    f2_unpack(hh[c], h0, h1);
                    f2_unpack(ll[c], q0, q1);
                    if (l0 < n) acc[c * B + o + l0] = w * ((double)h0 + (double)q0);
                    if (l1 < n) acc[c * B + o + l1] = w * ((double)h1 + (double)q1);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// symmetric force kernel: every unordered pair of a system evaluated once
// ---------------------------------------------------------------------------
// A system's bodies split into A ranges of 256 G (G packed pairs per lane)
// and B tiles of 128.  Unit (s, R) holds range R's bodies in registers and
// walks the tiles from R's first on:
//   * R's own tiles: one-sided, all ordered pairs, A side only;
//   * every later tile: symmetric (nbg_pair.cuh).  The B bodies of a
//     32-body chunk rotate through each warp -- at step r lane l meets chunk
//     body (l + r) mod 32, and the body's FP32 sum follows it one lane down
//     per step -- the four warps' sums are added in warp order, and the unit
//     writes one FP32 partial per (R, B body) to bpart.
// Tiles before R are covered by the units of their own ranges.  The A sums
// (two-sum per tile) go straight to the output; ens_sym_reduce_kernel then
// adds to every body the partials of the ranges before its own, in range
// order, in FP64 (weight -1, or -m with equal masses).  No atomics: equal
// states give equal forces.  Per pair of bodies 14 to 16 packed FP32
// operations and one reciprocal square root serve both bodies, against 11
// to 12 operations per body and pair in the one-sided kernel.
struct EnsSymUnit {
    int sys;
    int r;  // A range
};

// at least 4 CTAs per SM: a 128-register budget, which the 4-body (G = 2)
// equal-mass build needs to run without spills
template <bool CLAMP, int G, bool UNI>
__global__ void __launch_bounds__(kEnsThreads, 4)
ens_sym_kernel(const Body2* __restrict__ bodies, const long long* __restrict__ off,
               const int* __restrict__ cnt, const EnsSymUnit* __restrict__ units, int nunits,
               unsigned* __restrict__ counter, double* __restrict__ acc, size_t B, float eps2v,
               const double* __restrict__ sys_mass, float* __restrict__ bpart,
               const long long* __restrict__ boff, size_t bstride) {
    constexpr int RA = kEnsThreads * 2 * G;
    constexpr int TPR = RA / kEnsTile;
    __shared__ __align__(16) float4 txy[kEnsTile];  // (x x y y) per body
    __shared__ __align__(16) float4 tzm[kEnsTile];  // (z z m m) per body
    __shared__ float bsum[kEnsThreads / 32][3][kEnsTile];
    __shared__ int next_unit;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const f2_t eps2 = f2_pack(eps2v, eps2v);
    const f2_t zero = f2_pack(0.f, 0.f);
    const uint32_t xy_addr = smem_addr(txy), zm_addr = smem_addr(tzm);
    // stand-in for the slots past a system's end: far away and massless, so
    // its r^-3 underflows to zero against every real body
    const float4 far_xy = make_float4(1e18f, 1e18f, 1e18f, 1e18f);
    const float4 far_zm = make_float4(1e18f, 1e18f, 0.f, 0.f);
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) next_unit = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int u = next_unit;
        if (u >= nunits) break;
        const EnsSymUnit un = units[u];
        const long long o = off[un.sys];
        const int n = cnt[un.sys];
        const int a0 = un.r * RA;
        const int tiles = (n + kEnsTile - 1) / kEnsTile;
        f2_t xi[G], yi[G], zi[G], mi[G], hx[G], hy[G], hz[G], lx[G], ly[G], lz[G];
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const int l0 = a0 + (2 * g) * kEnsThreads + threadIdx.x;
            const int l1 = l0 + kEnsThreads;
            float4 p0 = far_xy, q0 = far_zm, p1 = far_xy, q1 = far_zm;
            if (l0 < n) {
                const Body2 b = bodies[o + l0];
                p0 = b.xxyy;
                q0 = b.zzmm;
            }
            if (l1 < n) {
                const Body2 b = bodies[o + l1];
                p1 = b.xxyy;
                q1 = b.zzmm;
            }
            xi[g] = f2_pack(p0.x, p1.x);
            yi[g] = f2_pack(p0.z, p1.z);
            zi[g] = f2_pack(q0.x, q1.x);
            mi[g] = f2_pack(q0.z, q1.z);
            hx[g] = hy[g] = hz[g] = lx[g] = ly[g] = lz[g] = zero;
        }
        for (int t = un.r * TPR; t < tiles; ++t) {
            __syncthreads();  // the previous tile's readers are done
            const int j = t * kEnsTile + threadIdx.x;
            if (j < n) {
                const Body2 b = bodies[o + j];
                txy[threadIdx.x] = b.xxyy;
                tzm[threadIdx.x] = b.zzmm;
            } else {
                txy[threadIdx.x] = far_xy;
                tzm[threadIdx.x] = far_zm;
            }
            __syncthreads();
            f2_t ax[G], ay[G], az[G];
#pragma unroll
            for (int g = 0; g < G; ++g) ax[g] = ay[g] = az[g] = zero;
            const int jn = min(kEnsTile, n - t * kEnsTile);
            if (t < (un.r + 1) * TPR) {
                // the range's own tile: one-sided, broadcast loads
#pragma unroll 4
                for (int jj = 0; jj < jn; ++jj) {
                    const float4 p = lds128(xy_addr + 16u * jj);
                    const float4 q = lds128(zm_addr + 16u * jj);
                    const f2_t xj = f2_pack(p.x, p.y), yj = f2_pack(p.z, p.w);
                    const f2_t zj = f2_pack(q.x, q.y), mj = f2_pack(q.z, q.w);
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        if constexpr (UNI)
                            pair2e_uni<CLAMP>(xj, yj, zj, xi[g], yi[g], zi[g], eps2, ax[g],
                                              ay[g], az[g]);
                        else
                            pair2e<CLAMP>(xj, yj, zj, mj, xi[g], yi[g], zi[g], eps2, ax[g],
                                          ay[g], az[g]);
                    }
                }
            } else {
#pragma unroll 1
                for (int c = 0; c < kEnsTile / 32; ++c) {
                    float bx = 0.f, by = 0.f, bz = 0.f;
                    if (c * 32 < jn) {  // chunks wholly past the end are skipped
#pragma unroll 8
                        for (int r = 0; r < 32; ++r) {
                            const uint32_t idx = (uint32_t)(c * 32 + ((lane + r) & 31));
                            const float4 p = lds128(xy_addr + 16u * idx);
                            const float4 q = lds128(zm_addr + 16u * idx);
                            const f2_t xj = f2_pack(p.x, p.y), yj = f2_pack(p.z, p.w);
                            const f2_t zj = f2_pack(q.x, q.y), mj = f2_pack(q.z, q.w);
                            f2_t px = zero, py = zero, pz = zero;
#pragma unroll
                            for (int g = 0; g < G; ++g) {
                                if constexpr (UNI)
                                    sym_pair_uni<CLAMP>(xj, yj, zj, xi[g], yi[g], zi[g], eps2,
                                                        ax[g], ay[g], az[g], px, py, pz);
                                else
                                    sym_pair<CLAMP>(xj, yj, zj, mj, xi[g], yi[g], zi[g], mi[g],
                                                    eps2, ax[g], ay[g], az[g], px, py, pz);
                            }
                            float lo, hi;
                            f2_unpack(px, lo, hi);
                            bx += lo + hi;
                            f2_unpack(py, lo, hi);
                            by += lo + hi;
                            f2_unpack(pz, lo, hi);
                            bz += lo + hi;
                            // the sum of chunk body (lane + r) moves to lane - 1,
                            // which meets that body at step r + 1
                            const int src = (lane + 1) & 31;
                            bx = __shfl_sync(0xffffffffu, bx, src);
                            by = __shfl_sync(0xffffffffu, by, src);
                            bz = __shfl_sync(0xffffffffu, bz, src);
                        }
                    }
                    // after 32 steps and shifts lane l holds chunk body l's sum
                    bsum[warp][0][c * 32 + lane] = bx;
                    bsum[warp][1][c * 32 + lane] = by;
                    bsum[warp][2][c * 32 + lane] = bz;
                }
                __syncthreads();
                if ((int)threadIdx.x < jn) {
                    const size_t base = (size_t)boff[un.sys] + (size_t)un.r * n +
                                        (size_t)t * kEnsTile + threadIdx.x;
#pragma unroll
                    for (int comp = 0; comp < 3; ++comp) {
                        float v = bsum[0][comp][threadIdx.x];
#pragma unroll
                        for (int w = 1; w < kEnsThreads / 32; ++w) v += bsum[w][comp][threadIdx.x];
                        bpart[comp * bstride + base] = v;
                    }
                }
            }
#pragma unroll
            for (int g = 0; g < G; ++g) {
                f2_two_sum(hx[g], lx[g], ax[g]);
                f2_two_sum(hy[g], ly[g], ay[g]);
                f2_two_sum(hz[g], lz[g], az[g]);
            }
        }
        const double w = UNI ? sys_mass[un.sys] : 1.0;
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const int l0 = a0 + (2 * g) * kEnsThreads + threadIdx.x;
            const int l1 = l0 + kEnsThreads;
            const f2_t hh[3] = {hx[g], hy[g], hz[g]};
            const f2_t ll[3] = {lx[g], ly[g], lz[g]};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float h0, h1, q0, q1;
                f2_unpack(hh[c], h0, h1);
                f2_unpack(ll[c], q0, q1);
                if (l0 < n) acc[c * B + o + l0] = w * ((double)h0 + (double)q0);
                if (l1 < n) acc[c * B + o + l1] = w * ((double)h1 + (double)q1);
            }
        }
    }
}

// Adds to every body the B partials of the ranges before its own, in range
// order, in FP64: acc += w sum_r bpart[r], w = -1 (or -m with equal masses).
__global__ void ens_sym_reduce_kernel(const int* __restrict__ sys, const long long* __restrict__ off,
                                      const int* __restrict__ cnt,
                                      const float* __restrict__ bpart,
                                      const long long* __restrict__ boff, size_t bstride,
                                      double* __restrict__ acc, size_t B,
                                      const double* __restrict__ sys_mass, int uni, int ra) {
    for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < B;
         j += (size_t)gridDim.x * blockDim.x) {
        const int s = sys[j];
        const int l = (int)((long long)j - off[s]);
        const int rj = l / ra;
        if (rj == 0) continue;
        const int n = cnt[s];
        const double w = uni ? -sys_mass[s] : -1.0;
        const size_t base = (size_t)boff[s] + (size_t)l;
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            double sum = 0.0;
            for (int r = 0; r < rj; ++r) sum += (double)bpart[comp * bstride + base + (size_t)r * n];
            acc[comp * B + j] += w * sum;
        }
    }
}

// Candidate update y_new = y + dt sum b2_i k_i and per-system error
// max |dt sum (b2_i - b1_i) k_i| (as ordered bits, atomicMax).
// A warp covers 32 consecutive bodies, which belong to one system or a few
// neighbouring ones (bodies are stored system by system): a segmented max
// over the warp leaves each system's maximum in its first lane, and only
// those lanes reach the system's error word (max is order-free, so the
// result does not depend on the schedule).
__global__ void ens_error_kernel(const double* __restrict__ y, const int* __restrict__ sys,
                                 const double* __restrict__ dt, KPtrs kp, size_t B,
                                 double* __restrict__ ynew, unsigned long long* __restrict__ err) {
    const int lane = threadIdx.x & 31;
    const size_t warp0 = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) & ~(size_t)31;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t base = warp0; base < B; base += stride) {  // warp-uniform
        const size_t i = base + lane;
        const bool live = i < B;
        const int s = live ? sys[i] : -1;
        double emax = 0.0;
        if (live) {
            const double h = dt[s];
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                double acc_b2 = 0.0, acc_e = 0.0;
#pragma unroll
                for (int j = 0; j < kStagesRK; ++j) {
                    const double kv = kp.k[j][c * B + i];
                    acc_b2 = fma(c_b2[j], kv, acc_b2);
                    acc_e = fma(c_b2[j] - c_b1[j], kv, acc_e);
                }
                ynew[c * B + i] = fma(h, acc_b2, y[c * B + i]);
                emax = fmax(emax, fabs(h * acc_e));
            }
        }
        // segmented suffix max: lanes of one system are contiguous
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double w = __shfl_down_sync(0xffffffffu, emax, o);
            const int sw = __shfl_down_sync(0xffffffffu, s, o);
            if (lane + o < 32 && sw == s) emax = fmax(emax, w);
        }
        const int sp = __shfl_up_sync(0xffffffffu, s, 1);
        if (live && (lane == 0 || sp != s))
            atomicMax(&err[s], (unsigned long long)__double_as_longlong(emax));
    }
}

// One thread per system: accept / reject and the next step.
// hold: after a rejected step the next step may not grow (Hairer, Norsett &
// Wanner, Solving ODEs I, sec. II.4), which avoids reject / grow cycles.
__global__ void ens_control_kernel(int nsys, double tol, double dt_min, double dt_max,
                                   const unsigned long long* __restrict__ err, double* __restrict__ dt,
                                   double* __restrict__ t, unsigned* __restrict__ accepted,
                                   unsigned* __restrict__ rejected, int* __restrict__ decision,
                                   int hold, double* __restrict__ err_prev, int pi) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    const double e = __longlong_as_double((long long)err[s]);
    const double h = dt[s];
    const bool ok = e <= tol || h <= dt_min;
    const bool after_reject = decision[s] == 0;
    decision[s] = ok ? 1 : 0;
    if (ok) {
        t[s] += h;
        accepted[s] += 1;
    } else {
        rejected[s] += 1;
    }
    double fac;
    if (pi && ok && e > 0.0) {
        // PI step control (Gustafsson 1991): exponents 0.7/5 on this error
        // and 0.4/5 on the previous accepted step's
        const double ep = fmax(err_prev[s], 1e-4 * tol);
        fac = 0.9 * pow(tol / e, 0.14) * pow(ep / tol, 0.08);
        err_prev[s] = e;
    } else {
        fac = (e > 0.0) ? 0.9 * pow(tol / e, 0.2) : 5.0;
    }
    fac = fmin((hold && after_reject) ? 1.0 : 5.0, fmax(0.2, fac));
    dt[s] = fmin(dt_max, fmax(dt_min, h * fac));
}

__global__ void ens_commit_kernel(double* __restrict__ y, const double* __restrict__ ynew,
                                  const int* __restrict__ sys, const int* __restrict__ decision,
                                  size_t B) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < B;
         i += (size_t)gridDim.x * blockDim.x) {
        if (!decision[sys[i]]) continue;
#pragma unroll
        for (int c = 0; c < 6; ++c) y[c * B + i] = ynew[c * B + i];
    }
}

}  // namespace
}  // namespace nbg

using namespace nbg;

struct nbg_ensemble {
    nbg_engine* eng = nullptr;  // stream, error text, launch count
    nbg_ensemble_params p{};
    int nsys = 0;
    size_t B = 0;
    std::vector<long long> h_off;
    std::vector<int> h_cnt;
    long long* off = nullptr;
    int* cnt = nullptr;
    int* sys = nullptr;
    double* y = nullptr;
    double* ynew = nullptr;
    double* mass = nullptr;
    double* sys_mass = nullptr;  // [nsys] each system's mass when all are uniform
    bool all_uniform = false;    // every system has equal masses
    double* k[kStagesRK] = {nullptr};
    Body2* bodies = nullptr;
    double* dt = nullptr;
    double* t = nullptr;
    unsigned long long* err = nullptr;
    unsigned* accepted = nullptr;
    unsigned* rejected = nullptr;
    int* decision = nullptr;
    double* err_prev = nullptr;  // error of each system's last accepted step (PI control)
    EnsUnit* units = nullptr;
    int nunits = 0;
    unsigned* counters = nullptr;  // one per stage
    cudaGraphExec_t graph = nullptr;
    cudaGraph_t graph_def = nullptr;
    int G = 2;
    unsigned force_grid = 1;
    // symmetric kernel ("ensemble.symmetric"): its units, the B partials
    // (3 components x bstride floats; system s from boff[s], ranges x N_s)
    bool sym = false;
    EnsSymUnit* sym_units = nullptr;
    int nsym_units = 0;
    float* bpart = nullptr;
    size_t bstride = 0, bpart_cap = 0;
    long long* boff = nullptr;
};

namespace {

using EnsForce = void (*)(const Body2*, const long long*, const int*, const EnsUnit*, int,
                          unsigned*, double*, size_t, float, const double*);

template <bool CLAMP, int G, bool UNI>
EnsForce ens_pick_unroll(int64_t u) {
    return u >= 8 ? ens_force_kernel<CLAMP, G, 8, UNI>
                  : u <= 2 ? ens_force_kernel<CLAMP, G, 2, UNI> : ens_force_kernel<CLAMP, G, 4, UNI>;
}

template <bool UNI>
EnsForce ens_pick_g(bool clamp, int G, int64_t u) {
    return clamp ? (G == 1 ? ens_pick_unroll<true, 1, UNI>(u) : ens_pick_unroll<true, 2, UNI>(u))
                 : (G == 1 ? ens_pick_unroll<false, 1, UNI>(u) : ens_pick_unroll<false, 2, UNI>(u));
}

bool ens_uniform(const nbg_ensemble* s) {
    return s->all_uniform && s->eng->tune_get("ensemble.uniform_mass", 1) != 0;
}

// "ensemble.unroll": unroll of the force kernel's j loop (2, 4 or 8);
// "ensemble.uniform_mass" (1, the default): the equal-mass kernel when every
// system has equal masses
EnsForce ens_pick(const nbg_ensemble* s) {
    const bool clamp = !(s->p.softening > 0.0);
    const int64_t u = s->eng->tune_get("ensemble.unroll", 4);
    return ens_uniform(s) ? ens_pick_g<true>(clamp, s->G, u) : ens_pick_g<false>(clamp, s->G, u);
}

using EnsSym = void (*)(const Body2*, const long long*, const int*, const EnsSymUnit*, int,
                        unsigned*, double*, size_t, float, const double*, float*,
                        const long long*, size_t);

template <bool UNI>
EnsSym ens_pick_sym_g(bool clamp, int G) {
    return clamp ? (G == 1 ? ens_sym_kernel<true, 1, UNI> : ens_sym_kernel<true, 2, UNI>)
                 : (G == 1 ? ens_sym_kernel<false, 1, UNI> : ens_sym_kernel<false, 2, UNI>);
}

EnsSym ens_pick_sym(const nbg_ensemble* s) {
    const bool clamp = !(s->p.softening > 0.0);
    return ens_uniform(s) ? ens_pick_sym_g<true>(clamp, s->G) : ens_pick_sym_g<false>(clamp, s->G);
}

// The symmetric kernel's units, cost-ordered (largest first, so the tail of
// the persistent launch is made of small units), and its partial buffer.
nbg_status ens_configure_sym(nbg_ensemble* s) {
    nbg_engine* e = s->eng;
    const int ra = kEnsThreads * 2 * s->G;
    struct Costed {
        EnsSymUnit u;
        double cost;
    };
    std::vector<Costed> units;
    std::vector<long long> boff(s->nsys);
    long long total = 0;
    for (int sI = 0; sI < s->nsys; ++sI) {
        const int n = s->h_cnt[sI];
        const int ranges = (n + ra - 1) / ra;
        boff[sI] = total;
        total += (long long)ranges * n;
        for (int r = 0; r < ranges; ++r) {
            const double own = (double)ra * std::min(ra, n - r * ra);
            const double later = (double)ra * std::max(0, n - (r + 1) * ra);
            units.push_back({EnsSymUnit{sI, r}, own + 0.6 * later});
        }
    }
    std::stable_sort(units.begin(), units.end(),
                     [](const Costed& a, const Costed& b) { return a.cost > b.cost; });
    std::vector<EnsSymUnit> list(units.size());
    for (size_t i = 0; i < units.size(); ++i) list[i] = units[i].u;
    s->nsym_units = (int)list.size();
    cudaFree(s->sym_units);
    cudaFree(s->boff);
    s->sym_units = nullptr;
    s->boff = nullptr;
    NBG_CUDA(e, cudaMalloc(&s->sym_units, list.size() * sizeof(EnsSymUnit)));
    NBG_CUDA(e, cudaMemcpy(s->sym_units, list.data(), list.size() * sizeof(EnsSymUnit),
                           cudaMemcpyHostToDevice));
    NBG_CUDA(e, cudaMalloc(&s->boff, boff.size() * sizeof(long long)));
    NBG_CUDA(e, cudaMemcpy(s->boff, boff.data(), boff.size() * sizeof(long long),
                           cudaMemcpyHostToDevice));
    s->bstride = (size_t)std::max<long long>(total, 1);
    if (s->bpart_cap < 3 * s->bstride) {
        cudaFree(s->bpart);
        s->bpart = nullptr;
        s->bpart_cap = 0;
        NBG_CUDA(e, cudaMalloc(&s->bpart, 3 * s->bstride * sizeof(float)));
        s->bpart_cap = 3 * s->bstride;
    }
    int occ = 0;
    NBG_CUDA(e, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ens_pick_sym(s), kEnsThreads, 0));
    occ = std::max(occ, 1);
    const int64_t bps = e->tune_get("ensemble.blocks_per_sm", 0);
    if (bps > 0 && bps < occ) occ = (int)bps;
    s->force_grid = (unsigned)std::max(1, std::min(s->nsym_units, e->sm_count * occ));
    return NBG_OK;
}

// Work units and launch shape from the tuning keys (the i-block tile of
// 256 G bodies, CTAs per SM; "ensemble.symmetric" 1, the default: every
// unordered pair once); drops a captured step graph built for an older
// shape.
// The symmetric kernel's partials take sum_s ceil(N_s / RA) N_s floats per
// component: small for many small systems (300 MB for 2048 systems of up to
// 4096 bodies), but growing as N^2 / RA for one large system; above this
// size the ensemble uses the one-sided kernel, which needs no such buffer.
constexpr size_t kEnsSymMaxPartialBytes = size_t(8) << 30;

nbg_status ens_configure(nbg_ensemble* s) {
    nbg_engine* e = s->eng;
    s->G = (int)std::max<int64_t>(1, std::min<int64_t>(2, e->tune_get("ensemble.pairs_per_lane", 2)));
    s->sym = e->tune_get("ensemble.symmetric", 1) != 0;
    if (s->sym) {
        const long long ra = kEnsThreads * 2 * s->G;
        size_t floats = 0;
        for (int sI = 0; sI < s->nsys; ++sI) {
            const long long n = s->h_cnt[sI];
            floats += (size_t)((n + ra - 1) / ra) * (size_t)n;
        }
        if (3 * floats * sizeof(float) > kEnsSymMaxPartialBytes) s->sym = false;
    }
    if (s->sym) {
        NBG_CUDA(e, cudaStreamSynchronize(e->stream));
        nbg_status st = ens_configure_sym(s);
        if (st != NBG_OK) return st;
        if (s->graph) cudaGraphExecDestroy(s->graph);
        if (s->graph_def) cudaGraphDestroy(s->graph_def);
        s->graph = nullptr;
        s->graph_def = nullptr;
        return NBG_OK;
    }
    const int blk = kEnsThreads * 2 * s->G;
    std::vector<EnsUnit> units;
    for (int sI = 0; sI < s->nsys; ++sI)
        for (int i0 = 0; i0 < s->h_cnt[sI]; i0 += blk) units.push_back(EnsUnit{sI, i0});
    // largest systems first (their units cost the most), so the tail of the
    // persistent launch is made of small units
    std::stable_sort(units.begin(), units.end(), [&](const EnsUnit& a, const EnsUnit& b) {
        return s->h_cnt[a.sys] > s->h_cnt[b.sys];
    });
    s->nunits = (int)units.size();
    int occ = 0;
    NBG_CUDA(e, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ens_pick(s), kEnsThreads, 0));
    occ = std::max(occ, 1);
    const int64_t bps = e->tune_get("ensemble.blocks_per_sm", 0);
    if (bps > 0 && bps < occ) occ = (int)bps;
    s->force_grid = (unsigned)std::max(1, std::min(s->nunits, e->sm_count * occ));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    cudaFree(s->units);
    s->units = nullptr;
    NBG_CUDA(e, cudaMalloc(&s->units, units.size() * sizeof(EnsUnit)));
    NBG_CUDA(e, cudaMemcpy(s->units, units.data(), units.size() * sizeof(EnsUnit),
                           cudaMemcpyHostToDevice));
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->graph_def) cudaGraphDestroy(s->graph_def);
    s->graph = nullptr;
    s->graph_def = nullptr;
    return NBG_OK;
}

// The RHS of one stage: forces of the FP32 body records into acc ([3][B],
// the acceleration half of a k buffer).
nbg_status ens_launch_force(nbg_ensemble* s, unsigned* counter, double* acc) {
    nbg_engine* e = s->eng;
    const float eps2 = (float)(s->p.softening * s->p.softening);
    if (s->sym) {
        ens_pick_sym(s)<<<s->force_grid, kEnsThreads, 0, e->stream>>>(
            s->bodies, s->off, s->cnt, s->sym_units, s->nsym_units, counter, acc, s->B, eps2,
            s->sys_mass, s->bpart, s->boff, s->bstride);
        NBG_LAUNCHED(e, "ens_sym_kernel");
        ens_sym_reduce_kernel<<<grid_for(s->B, 256, (unsigned)e->sm_count * 8u), 256, 0,
                                e->stream>>>(s->sys, s->off, s->cnt, s->bpart, s->boff,
                                             s->bstride, acc, s->B, s->sys_mass,
                                             ens_uniform(s) ? 1 : 0, kEnsThreads * 2 * s->G);
        NBG_LAUNCHED(e, "ens_sym_reduce_kernel");
        return NBG_OK;
    }
    ens_pick(s)<<<s->force_grid, kEnsThreads, 0, e->stream>>>(
        s->bodies, s->off, s->cnt, s->units, s->nunits, counter, acc, s->B, eps2, s->sys_mass);
    NBG_LAUNCHED(e, "ens_force_kernel");
    return NBG_OK;
}

// Stage-0 forces of the current state into k_0 (no host copy).
nbg_status ens_enqueue_force(nbg_ensemble* s) {
    nbg_engine* e = s->eng;
    KPtrs kp;
    for (int i = 0; i < kStagesRK; ++i) kp.k[i] = s->k[i];
    const unsigned gv = grid_for(s->B, 256, (unsigned)e->sm_count * 8u);
    NBG_CUDA(e, cudaMemsetAsync(s->counters, 0, sizeof(unsigned), e->stream));
    ens_stage_kernel<<<gv, 256, 0, e->stream>>>(0, s->y, s->mass, s->sys, s->dt, kp, s->B,
                                                s->bodies);
    NBG_LAUNCHED(e, "ens_stage_kernel");
    return ens_launch_force(s, s->counters, s->k[0] + 3 * s->B);
}

nbg_status ens_enqueue_step(nbg_ensemble* s) {
    nbg_engine* e = s->eng;
    const unsigned gv = grid_for(s->B, 256, (unsigned)e->sm_count * 8u);
    KPtrs kp;
    for (int i = 0; i < kStagesRK; ++i) kp.k[i] = s->k[i];
    NBG_CUDA(e, cudaMemsetAsync(s->counters, 0, kStagesRK * sizeof(unsigned), e->stream));
    NBG_CUDA(e, cudaMemsetAsync(s->err, 0, s->nsys * sizeof(unsigned long long), e->stream));
    for (int st = 0; st < kStagesRK; ++st) {
        ens_stage_kernel<<<gv, 256, 0, e->stream>>>(st, s->y, s->mass, s->sys, s->dt, kp, s->B,
                                                    s->bodies);
        NBG_LAUNCHED(e, "ens_stage_kernel");
        ProfScope ps(e, NBG_K_DIRECT);
        nbg_status fs = ens_launch_force(s, s->counters + st, s->k[st] + 3 * s->B);
        if (fs != NBG_OK) return fs;
    }
    ens_error_kernel<<<gv, 256, 0, e->stream>>>(s->y, s->sys, s->dt, kp, s->B, s->ynew, s->err);
    NBG_LAUNCHED(e, "ens_error_kernel");
    ens_control_kernel<<<(s->nsys + 127) / 128, 128, 0, e->stream>>>(
        s->nsys, s->p.tolerance, s->p.dt_min, s->p.dt_max, s->err, s->dt, s->t, s->accepted,
        s->rejected, s->decision, (int)e->tune_get("ensemble.hold_after_reject", 1), s->err_prev,
        (int)e->tune_get("ensemble.pi_control", 0));
    NBG_LAUNCHED(e, "ens_control_kernel");
    ens_commit_kernel<<<gv, 256, 0, e->stream>>>(s->y, s->ynew, s->sys, s->decision, s->B);
    NBG_LAUNCHED(e, "ens_commit_kernel");
    return NBG_OK;
}

void ens_free(nbg_ensemble* s) {
    void* ptrs[] = {s->off, s->cnt, s->sys, s->y, s->ynew, s->mass, s->sys_mass, s->bodies, s->dt, s->t,
                    s->err, s->accepted, s->rejected, s->decision, s->err_prev, s->units,
                    s->counters, s->sym_units, s->bpart, s->boff};
    for (void* p : ptrs) cudaFree(p);
    s->sym_units = nullptr;
    s->bpart = nullptr;
    s->boff = nullptr;
    s->bpart_cap = 0;
    for (double* k : s->k) cudaFree(k);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->graph_def) cudaGraphDestroy(s->graph_def);
    s->graph = nullptr;
    s->graph_def = nullptr;
}

}  // namespace

extern "C" {

void nbg_ensemble_params_default(nbg_ensemble_params* p) {
    if (p == nullptr) return;
    memset(p, 0, sizeof(*p));
    p->struct_size = sizeof(nbg_ensemble_params);
    p->device = 0;
    p->softening = 1e-3;
    p->tolerance = 1e-8;
    p->dt_initial = 1e-3;
    p->dt_min = 1e-9;
    p->dt_max = 1e-1;
    p->use_graph = 1;
}

nbg_status nbg_ensemble_create(const nbg_ensemble_params* p, nbg_ensemble** out) {
    if (out == nullptr) return NBG_ERR_INVALID_ARG;
    *out = nullptr;
    nbg_ensemble_params prm;
    nbg_ensemble_params_default(&prm);
    if (p != nullptr) {
        if (p->struct_size != sizeof(nbg_ensemble_params)) return NBG_ERR_INVALID_ARG;
        prm = *p;
    }
    if (!(prm.softening >= 0.0) || !(prm.tolerance > 0.0) || !(prm.dt_initial > 0.0) ||
        !(prm.dt_min > 0.0) || !(prm.dt_max >= prm.dt_min))
        return NBG_ERR_INVALID_ARG;
    nbg_params ep;
    nbg_params_default(&ep);
    ep.device = prm.device;
    ep.precision = NBG_PREC_MIXED;
    ep.softening = prm.softening;
    nbg_engine* eng = nullptr;
    nbg_status st = nbg_engine_create(&ep, &eng);
    if (st != NBG_OK) return st;
    nbg_ensemble* s = new (std::nothrow) nbg_ensemble();
    if (s == nullptr) {
        nbg_engine_destroy(eng);
        return NBG_ERR_OUT_OF_MEMORY;
    }
    s->eng = eng;
    s->p = prm;
    *out = s;
    return NBG_OK;
}

void nbg_ensemble_destroy(nbg_ensemble* s) {
    if (s == nullptr) return;
    cudaSetDevice(s->eng->device);
    cudaStreamSynchronize(s->eng->stream);
    ens_free(s);
    nbg_engine_destroy(s->eng);
    delete s;
}

const char* nbg_ensemble_last_error(const nbg_ensemble* s) {
    return s == nullptr ? "" : s->eng->last_error.c_str();
}

nbg_status nbg_ensemble_init(nbg_ensemble* s, size_t nsys, const uint32_t* counts,
                             const double* vertices, const double* velocities, const double* mass) {
    if (s == nullptr || nsys == 0 || counts == nullptr || vertices == nullptr ||
        velocities == nullptr || mass == nullptr)
        return NBG_ERR_INVALID_ARG;
    nbg_engine* e = s->eng;
    NBG_CUDA(e, cudaSetDevice(e->device));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    ens_free(s);
    s->nsys = (int)nsys;
    s->h_off.assign(nsys, 0);
    s->h_cnt.assign(nsys, 0);
    size_t B = 0;
    for (size_t i = 0; i < nsys; ++i) {
        if (counts[i] == 0) return set_error(e, NBG_ERR_INVALID_ARG, "system %zu is empty", i);
        s->h_off[i] = (long long)B;
        s->h_cnt[i] = (int)counts[i];
        B += counts[i];
    }
    s->B = B;
    const size_t B6 = 6 * B;
    NBG_CUDA(e, cudaMalloc(&s->off, nsys * sizeof(long long)));
    NBG_CUDA(e, cudaMalloc(&s->cnt, nsys * sizeof(int)));
    NBG_CUDA(e, cudaMalloc(&s->sys, B * sizeof(int)));
    NBG_CUDA(e, cudaMalloc(&s->y, B6 * sizeof(double)));
    NBG_CUDA(e, cudaMalloc(&s->ynew, B6 * sizeof(double)));
    NBG_CUDA(e, cudaMalloc(&s->mass, B * sizeof(double)));
    NBG_CUDA(e, cudaMalloc(&s->sys_mass, nsys * sizeof(double)));
    for (int i = 0; i < kStagesRK; ++i) NBG_CUDA(e, cudaMalloc(&s->k[i], B6 * sizeof(double)));
    NBG_CUDA(e, cudaMalloc(&s->bodies, B * sizeof(Body2)));
    NBG_CUDA(e, cudaMalloc(&s->dt, nsys * sizeof(double)));
    NBG_CUDA(e, cudaMalloc(&s->t, nsys * sizeof(double)));
    NBG_CUDA(e, cudaMalloc(&s->err, nsys * sizeof(unsigned long long)));
    NBG_CUDA(e, cudaMalloc(&s->accepted, nsys * sizeof(unsigned)));
    NBG_CUDA(e, cudaMalloc(&s->rejected, nsys * sizeof(unsigned)));
    NBG_CUDA(e, cudaMalloc(&s->decision, nsys * sizeof(int)));
    NBG_CUDA(e, cudaMalloc(&s->err_prev, nsys * sizeof(double)));
    NBG_CUDA(e, cudaMalloc(&s->counters, kStagesRK * sizeof(unsigned)));
    // host-side layout: SoA state, system ids, LPT-ordered work units
    std::vector<double> h(B6);
    std::vector<int> hsys(B);
    for (size_t sI = 0; sI < nsys; ++sI)
        for (int k = 0; k < s->h_cnt[sI]; ++k) hsys[s->h_off[sI] + k] = (int)sI;
    for (size_t i = 0; i < B; ++i)
        for (int d = 0; d < 3; ++d) {
            h[d * B + i] = vertices[3 * i + d];
            h[(3 + d) * B + i] = velocities[3 * i + d];
        }
    std::vector<double> dt0(nsys, s->p.dt_initial), t0(nsys, 0.0);
    NBG_CUDA(e, cudaMemcpy(s->off, s->h_off.data(), nsys * sizeof(long long), cudaMemcpyHostToDevice));
    NBG_CUDA(e, cudaMemcpy(s->cnt, s->h_cnt.data(), nsys * sizeof(int), cudaMemcpyHostToDevice));
    NBG_CUDA(e, cudaMemcpy(s->sys, hsys.data(), B * sizeof(int), cudaMemcpyHostToDevice));
    NBG_CUDA(e, cudaMemcpy(s->y, h.data(), B6 * sizeof(double), cudaMemcpyHostToDevice));
    NBG_CUDA(e, cudaMemcpy(s->mass, mass, B * sizeof(double), cudaMemcpyHostToDevice));
    // equal masses within every system select the kernel that scales by the
    // system's mass once
    std::vector<double> smass(nsys);
    s->all_uniform = true;
    for (size_t sI = 0; sI < nsys; ++sI) {
        const double* m0 = mass + s->h_off[sI];
        smass[sI] = m0[0];
        for (int k = 1; k < s->h_cnt[sI] && s->all_uniform; ++k)
            s->all_uniform = m0[k] == m0[0];
    }
    NBG_CUDA(e, cudaMemcpy(s->sys_mass, smass.data(), nsys * sizeof(double),
                           cudaMemcpyHostToDevice));
    NBG_CUDA(e, cudaMemcpy(s->dt, dt0.data(), nsys * sizeof(double), cudaMemcpyHostToDevice));
    NBG_CUDA(e, cudaMemcpy(s->t, t0.data(), nsys * sizeof(double), cudaMemcpyHostToDevice));
    NBG_CUDA(e, cudaMemset(s->accepted, 0, nsys * sizeof(unsigned)));
    NBG_CUDA(e, cudaMemset(s->rejected, 0, nsys * sizeof(unsigned)));
    const std::vector<int> ok0(nsys, 1);  // no step rejected yet
    NBG_CUDA(e, cudaMemcpy(s->decision, ok0.data(), nsys * sizeof(int), cudaMemcpyHostToDevice));
    const std::vector<double> tol0(nsys, s->p.tolerance);  // PI control starts as the I control
    NBG_CUDA(e, cudaMemcpy(s->err_prev, tol0.data(), nsys * sizeof(double), cudaMemcpyHostToDevice));
    return ens_configure(s);
}

nbg_status nbg_ensemble_step(nbg_ensemble* s, int steps) {
    if (s == nullptr || steps < 0) return NBG_ERR_INVALID_ARG;
    if (s->B == 0) return set_error(s->eng, NBG_ERR_NOT_INITIALIZED, "ensemble not initialised");
    nbg_engine* e = s->eng;
    NBG_CUDA(e, cudaSetDevice(e->device));
    if (!s->p.use_graph) {
        for (int k = 0; k < steps; ++k) {
            nbg_status st = ens_enqueue_step(s);
            if (st != NBG_OK) return st;
        }
        return NBG_OK;
    }
    if (s->graph == nullptr) {
        // capture one whole RK step (stage combinations, forces, error,
        // control, commit) once; later steps replay it
        const bool prof = e->profiling;
        e->profiling = false;  // no host-side event bookkeeping inside the capture
        NBG_CUDA(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        const uint64_t l0 = e->launches;
        nbg_status st = ens_enqueue_step(s);
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
        e->profiling = prof;
        if (st != NBG_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (ce != cudaSuccess) return cuda_error(e, ce, "cudaStreamEndCapture");
        s->graph_def = g;
        NBG_CUDA(e, cudaGraphInstantiate(&s->graph, g, 0));
        e->launches = l0;  // captured, not launched
    }
    const uint64_t per_step = 3 + 2 * kStagesRK;
    for (int k = 0; k < steps; ++k) {
        ProfScope ps(e, NBG_K_ENS_STEP);
        NBG_CUDA(e, cudaGraphLaunch(s->graph, e->stream));
        e->launches += per_step;
    }
    return NBG_OK;
}

nbg_status nbg_ensemble_synchronize(nbg_ensemble* s) {
    if (s == nullptr) return NBG_ERR_INVALID_ARG;
    return nbg_synchronize(s->eng);
}

nbg_status nbg_ensemble_status(nbg_ensemble* s, double* t, double* dt, uint32_t* accepted,
                               uint32_t* rejected) {
    if (s == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_engine* e = s->eng;
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    if (t) NBG_CUDA(e, cudaMemcpy(t, s->t, s->nsys * sizeof(double), cudaMemcpyDeviceToHost));
    if (dt) NBG_CUDA(e, cudaMemcpy(dt, s->dt, s->nsys * sizeof(double), cudaMemcpyDeviceToHost));
    if (accepted)
        NBG_CUDA(e, cudaMemcpy(accepted, s->accepted, s->nsys * sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (rejected)
        NBG_CUDA(e, cudaMemcpy(rejected, s->rejected, s->nsys * sizeof(unsigned), cudaMemcpyDeviceToHost));
    return NBG_OK;
}

nbg_status nbg_ensemble_get_state(nbg_ensemble* s, double* vertices, double* velocities) {
    if (s == nullptr || vertices == nullptr || velocities == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_engine* e = s->eng;
    std::vector<double> h(6 * s->B);
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    NBG_CUDA(e, cudaMemcpy(h.data(), s->y, 6 * s->B * sizeof(double), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < s->B; ++i)
        for (int d = 0; d < 3; ++d) {
            vertices[3 * i + d] = h[d * s->B + i];
            velocities[3 * i + d] = h[(3 + d) * s->B + i];
        }
    return NBG_OK;
}

nbg_status nbg_ensemble_fcompute(nbg_ensemble* s, double* f) {
    if (s == nullptr || f == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_engine* e = s->eng;
    if (s->B == 0) return set_error(e, NBG_ERR_NOT_INITIALIZED, "ensemble not initialised");
    // stage 0 of a step: k_0 = [v ; a(y)] of the current state
    nbg_status st = ens_enqueue_force(s);
    if (st != NBG_OK) return st;
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    NBG_CUDA(e, cudaMemcpy(f, s->k[0], 6 * s->B * sizeof(double), cudaMemcpyDeviceToHost));
    return NBG_OK;
}

nbg_status nbg_ensemble_statistics(nbg_ensemble* s, double* out) {
    if (s == nullptr || out == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_engine* e = s->eng;
    DevScratch res;
    NBG_CUDA(e, cudaMalloc(&res.p, 12 * (size_t)s->nsys * sizeof(double)));
    nbg_status st = stats_segments(e, s->y, s->mass, s->B, s->nsys, s->off, s->cnt,
                                   s->h_off.data(), s->h_cnt.data(),
                                   s->p.softening * s->p.softening, res.as<double>());
    if (st == NBG_OK)
        NBG_CUDA(e, cudaMemcpy(out, res.p, 12 * (size_t)s->nsys * sizeof(double),
                               cudaMemcpyDeviceToHost));
    return st;
}

nbg_status nbg_ensemble_tune_set(nbg_ensemble* s, const char* key, int64_t value) {
    if (s == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status st = nbg_tune_set(s->eng, key, value);
    if (st != NBG_OK || s->B == 0) return st;
    return ens_configure(s);  // takes effect from the next step
}

nbg_status nbg_ensemble_autotune(nbg_ensemble* s, int reps, char* report, size_t report_len) {
    if (s == nullptr || reps < 1) return NBG_ERR_INVALID_ARG;
    nbg_engine* e = s->eng;
    if (s->B == 0) return set_error(e, NBG_ERR_NOT_INITIALIZED, "ensemble not initialised");
    NBG_CUDA(e, cudaSetDevice(e->device));
    const std::map<std::string, int64_t> base = e->tune;
    std::vector<Candidate> cands;
    for (int g : {1, 2})  // the symmetric kernel
        cands.push_back({{{"ensemble.symmetric", 1}, {"ensemble.pairs_per_lane", g},
                          {"ensemble.blocks_per_sm", 0}}});
    for (int g : {2, 1})  // the one-sided kernel
        for (int bps : {0, 4, 2})
            cands.push_back({{{"ensemble.symmetric", 0}, {"ensemble.pairs_per_lane", g},
                              {"ensemble.blocks_per_sm", bps}}});
    for (int g : {2, 1})
        for (int u : {2, 8})
            cands.push_back({{{"ensemble.symmetric", 0}, {"ensemble.pairs_per_lane", g},
                              {"ensemble.blocks_per_sm", 0}, {"ensemble.unroll", u}}});
    std::vector<double> ms;
    for (const Candidate& c : cands) {
        e->tune = base;
        for (const auto& kv : c) e->tune[kv.first] = kv.second;
        nbg_status st = ens_configure(s);
        double t = 0.0;
        if (st == NBG_OK) st = time_enqueue(e, reps, [&]() { return ens_enqueue_force(s); }, &t);
        if (st != NBG_OK) {
            e->tune = base;
            ens_configure(s);
            return st;
        }
        ms.push_back(t);
    }
    const size_t best = (size_t)(std::min_element(ms.begin(), ms.end()) - ms.begin());
    e->tune = base;
    for (const auto& kv : cands[best]) e->tune[kv.first] = kv.second;
    nbg_status st = ens_configure(s);
    if (st != NBG_OK) return st;
    write_tune_report(e, "ensemble", s->B, reps, cands, ms, best, report, report_len);
    return NBG_OK;
}

uint64_t nbg_ensemble_launch_count(const nbg_ensemble* s) {
    return s == nullptr ? 0 : s->eng->launches;
}

nbg_status nbg_ensemble_profile(nbg_ensemble* s, int enable, double* force_ms,
                                uint64_t* force_launches) {
    if (s == nullptr) return NBG_ERR_INVALID_ARG;
    if (force_ms != nullptr || force_launches != nullptr) {
        nbg_status st = nbg_profile_query(s->eng, NBG_K_DIRECT, force_ms, force_launches);
        if (st != NBG_OK) return st;
    }
    return nbg_profile_enable(s->eng, enable);
}

}  // extern "C"
