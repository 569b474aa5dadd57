// nbg_tc.cuh -- inline-PTX building blocks for the fifth-generation tensor
// cores (tcgen05) of sm_100-family GPUs: tensor-memory (TMEM) allocation,
// the shared-memory matrix descriptor, the instruction descriptor of a BF16
// MMA with FP32 accumulation, the MMA, its completion on an mbarrier, and
// accumulator loads from tensor memory.
//
// Operand layout used here (no swizzle, K-major): a matrix of R rows and K
// BF16 columns is stored as 8-row x 8-column "core matrices" of 128
// contiguous bytes (row r of a core matrix at 16 r bytes).  Element (r, k)
// sits at byte
//     (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2
// with LBO = 128 (core matrices adjacent along K) and SBO = 16 K bytes (the
// next 8 rows).  One MMA consumes K = 16 (two core-matrix columns); the
// descriptor of the K slice k0 starts at byte (k0 / 8) * 128.
#pragma once

#include <stdint.h>

#include "nbg_ptx.cuh"

namespace nbg {
namespace tc {

// byte offset of element (r, k) of a K-major no-swizzle operand with K columns
__host__ __device__ constexpr uint32_t kmajor_offset(int r, int k, int K) {
    return (uint32_t)((r >> 3) * (16 * K) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Allocate ncols (a power of two, 32..512) TMEM columns for the CTA; the
// base address is written to *slot in shared memory.  Executed by one whole
// warp, which must also free them.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(slot)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

// Ordering of tcgen05 operations across a thread synchronisation.
__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Shared-memory writes of this thread become visible to the tensor core
// (the async proxy) once the CTA synchronises after this fence.
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Shared-memory matrix descriptor (no swizzle): start address, leading
// (K-direction) and stride (row-direction) byte offsets, the fixed version
// bits 46-47 = 1; base offset 0, relative LBO mode.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits
// 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}

// D[tmem] (M x N, FP32) = A (M x 16) * B (N x 16)^T, plus D when accumulate
// is nonzero.  Issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// One arrival on the mbarrier once every MMA this thread issued before has
// completed (its operand reads included).
__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_addr(bar))
        : "memory");
}

// 16 consecutive FP32 columns of the warp's 32 TMEM lanes (thread i: lane
// base + i), with the wait for the load inside the same statement so the
// registers are only read once they hold the data.  taddr: (lane base << 16)
// | column; a warp may only address its own quarter of the lanes
// (32 (warp % 4) .. + 31).
__device__ __forceinline__ void ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace nbg
