// nbg_pair.cuh -- the symmetric pair term of the mixed-precision direct
// sums (nbg_direct.cu, nbg_ensemble.cu): one evaluation of an unordered pair
// serves both bodies (Newton's third law), in packed FP32x2 arithmetic on
// two A bodies and one B body broadcast into both halves.  The reference's
// pair force is nbody/nbody_data.cpp:35-44 (F = G m1 m2 d / r^3 with the
// minimum-distance clamp); softening replaces the clamp when it is set.
#pragma once

#include "nbg_ptx.cuh"

namespace nbg {

// ax += m_B d / r^3 (the A bodies' sums), bx += m_A d / r^3 (B's, to be
// subtracted), d = x_B - x_A, r^2 = |d|^2 + eps^2 (clamped at 1e-8 with
// CLAMP).
template <bool CLAMP>
__device__ __forceinline__ void sym_pair(f2_t xj, f2_t yj, f2_t zj, f2_t mj, f2_t xi, f2_t yi,
                                         f2_t zi, f2_t mi, f2_t eps2, f2_t& ax, f2_t& ay,
                                         f2_t& az, f2_t& bx, f2_t& by, f2_t& bz) {
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
    const f2_t sa = f2_mul(mj, inv3);
    const f2_t sb = f2_mul(mi, inv3);
    ax = f2_fma(dx, sa, ax);
    ay = f2_fma(dy, sa, ay);
    az = f2_fma(dz, sa, az);
    bx = f2_fma(dx, sb, bx);
    by = f2_fma(dy, sb, by);
    bz = f2_fma(dz, sb, bz);
}

// Equal masses: the pair weights reduce to r^-3 and the common mass scales
// the sums once, in FP64, when they are added to f (14 packed operations per
// pair evaluation instead of 16).
template <bool CLAMP>
__device__ __forceinline__ void sym_pair_uni(f2_t xj, f2_t yj, f2_t zj, f2_t xi, f2_t yi,
                                             f2_t zi, f2_t eps2, f2_t& ax, f2_t& ay, f2_t& az,
                                             f2_t& bx, f2_t& by, f2_t& bz) {
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
    bx = f2_fma(dx, inv3, bx);
    by = f2_fma(dy, inv3, by);
    bz = f2_fma(dz, inv3, bz);
}

}  // namespace nbg
