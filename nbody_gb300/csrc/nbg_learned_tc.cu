// nbg_learned_tc.cu -- the learned monopole correction on the default group
// walk, with the network evaluated on tcgen05 tensor cores.  No reference
// counterpart.
//
// 1. The group walk (nbg_bh.cu, emit mode) computes every body's monopole
//    forces at the loose ratio lambda_l and records, per 64-body group, the
//    cells it accepted whose mass centre lies within the tight ratio of the
//    group's box: the cells that can be in the band for some body of the
//    group.  A group with more than kCandCap of them, or one the walk gave
//    up on, is walked body by body (learned_body_walk_kernel, with the
//    per-warp mma.sync network of nbg_mlp.cuh).
// 2. learned_tc_kernel, persistent, CTAs of 128 threads, takes one
//    group at a time.  Its (body, cell) pairs, body-major, are tested
//    against the band (d^2 <= crit2 band2: the per-body learned walk's rule)
//    and the band pairs are compacted into 128-row tiles in shared memory.
//    Thread r builds row r's 16 features, and the CTA evaluates the tile
//    with three chains of tcgen05 MMAs (M = 128; N = 64, 64, 16; K = 16, 64,
//    64, each followed by a K = 16 MMA that adds the layer's bias: a block
//    of ones against the bias split into three BF16 terms), BF16 operands
//    in shared memory, FP32 accumulators in 64 TMEM columns (each layer's
//    over the previous one's).  Between layers each thread loads its row's
//    accumulators (tcgen05.ld), applies GELU and writes the BF16
//    activations as the next layer's A operand.  The group's band cells
//    pass through shared memory 64 at a time, with 1 / s and m / s^2 formed
//    once per cell; 5 CTAs per SM.  The output head turns the three
//    coefficients into the correction, scaled by the cell's m / s^2.
// 3. A body's rows are contiguous (body-major order), so a segmented scan in
//    each warp and four warp-ordered additions sum them into the group's
//    per-body accumulators in a fixed order: equal inputs give equal
//    forces.  At the end of the group the sums are added to f.
#include <algorithm>
#include <cmath>

#include "nbg_learned.cuh"
#include "nbg_mlp.cuh"
#include "nbg_ptx.cuh"
#include "nbg_stats.cuh"
#include "nbg_tc.cuh"
#include "nbg_tree.cuh"

namespace nbg {
namespace {

using namespace mlp;

constexpr int kTcThreads = 128;      // one warpgroup: thread r owns tile row r (TMEM lane r)
constexpr int kTcRows = 128;         // rows per tile (the MMA's M)
// TMEM columns: each layer's accumulator (64, 64, 16 columns) at column 0,
// written once every thread has read the previous layer's
constexpr int kTcCols = 64;
constexpr int kTcBlocksPerSm = 5;    // as shared memory allows; 5 x 64 of the SM's 512 columns
constexpr int kGroupBodies = 64;     // bodies of a group (the default group walk)
constexpr int kCellChunk = 64;       // band cells staged in shared memory at a time
static_assert(kCellChunk == 64, "the full-chunk index split is a shift by 6");
// dynamic shared memory per CTA at least this: at most 8 CTAs per SM, so
// every resident CTA's TMEM allocation (8 x 64 = 512 columns) succeeds
constexpr size_t kTcSmemFloor = 26 * 1024;
constexpr int kDumpCols = 144;       // accumulator dump: D1 (64), D2 (64), D3 (16)

struct TcSmem {
    uint32_t w[kTcwWords];  // operands W1^T, W2^T, W3^T and the bias operands B1, B2, B3
    // A operand of the bias MMAs (128 x 16): ones in columns 0-2, zeros after
    alignas(128) uint32_t ones[kTcRows * 16 / 2];
    // A operands: layer 1's (K = 16, 4 KB) in the first part of layers 2
    // and 3's (K = 64, 16 KB), which the layer-1 epilogue writes only after
    // the layer-1 MMA has completed
    alignas(128) uint32_t a2[kTcRows * 64 / 2];
    float4 body[kGroupBodies];  // the group's leaf records
    int body_id[kGroupBodies];
    float acc[3][kGroupBodies];  // per-body correction sums
    // staged band cells: (mass centre, crit2), (1 / s, m / s^2), features
    float4 cnode[kCellChunk];
    float2 cscale[kCellChunk];
    float4 cfeat[kCellChunk][3];
    unsigned short row_cell[kTcRows];  // chunk index of each row's cell
    unsigned char row_body[kTcRows];   // group index of each row's body
    int wcount[kTcThreads / 32];
    int cut;
    int unit;
    int abort;
    uint32_t tmem;
    alignas(8) uint64_t mbar;
};

size_t tc_smem_bytes() { return std::max(sizeof(TcSmem), kTcSmemFloor); }

// ---------------------------------------------------------------------------
// operands from the FP32 master weights
// ---------------------------------------------------------------------------
// x rounded to the nearest BF16 value, as a float.
__device__ __forceinline__ float bf16_round(float x) {
    return __uint_as_float(pack_bf16(x, 0.f) << 16);
}

// One thread per BF16 pair (k, k + 1) of one operand row n.  W2 and W3
// carry GELU's factor 1/2 (exact in BF16): the epilogue forms 2 GELU(z) =
// z + z tanh(u) with one FMA, and the products are the same bit for bit.
__global__ void make_tc_weights_kernel(const float* __restrict__ w, uint32_t* __restrict__ tcw) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    constexpr int q1 = 64 * 8, q2 = q1 + 64 * 32, q3 = q2 + 16 * 32;
    if (q < q1) {  // W1^T: n < 64, K = 16
        const int n = q / 8, k = 2 * (q % 8);
        tcw[kTcwW1 + tc::kmajor_offset(n, k, 16) / 4] =
            pack_bf16(w[kOffW1 + k * kH + n], w[kOffW1 + (k + 1) * kH + n]);
    } else if (q < q2) {  // W2^T: n < 64, K = 64
        const int r = q - q1, n = r / 32, k = 2 * (r % 32);
        tcw[kTcwW2 + tc::kmajor_offset(n, k, 64) / 4] =
            pack_bf16(0.5f * w[kOffW2 + k * kH + n], 0.5f * w[kOffW2 + (k + 1) * kH + n]);
    } else if (q < q3) {  // W3^T: n < 16 (rows past 3 zero), K = 64
        const int r = q - q2, n = r / 32, k = 2 * (r % 32);
        const float lo = n < kOut ? 0.5f * w[kOffW3 + k * kOut + n] : 0.f;
        const float hi = n < kOut ? 0.5f * w[kOffW3 + (k + 1) * kOut + n] : 0.f;
        tcw[kTcwW3 + tc::kmajor_offset(n, k, 64) / 4] = pack_bf16(lo, hi);
    } else if (q < q3 + 144) {  // bias operands: rows of B1 (64), B2 (64), B3 (16)
        const int i = q - q3;
        float b = 0.f;
        int base = kTcwB1, n = i;
        if (i < 64) {
            b = w[kOffB1 + i];
        } else if (i < 128) {
            b = w[kOffB2 + i - 64];
            base = kTcwB2;
            n = i - 64;
        } else {
            b = i - 128 < kOut ? w[kOffB3 + i - 128] : 0.f;
            base = kTcwB3;
            n = i - 128;
        }
        // b = hi + mid + lo: each term the BF16 rounding of what the earlier
        // ones leave (the residuals are exact in FP32), 24 bits in all
        const float hi = bf16_round(b);
        const float mid = bf16_round(b - hi);
        const float lo = bf16_round((b - hi) - mid);
        tcw[base + tc::kmajor_offset(n, 0, 16) / 4] = pack_bf16(hi, mid);
        tcw[base + tc::kmajor_offset(n, 2, 16) / 4] = pack_bf16(lo, 0.f);
#pragma unroll
        for (int k = 4; k < 16; k += 2) tcw[base + tc::kmajor_offset(n, k, 16) / 4] = 0u;
    }
}

// ---------------------------------------------------------------------------
// one 128-row tile through the network
// ---------------------------------------------------------------------------
// Twice the GELU of two pre-activations z (the accumulators, biases
// included), packed FP32x2, as BF16x2: z (1 + tanh(z (c0 + c1 z^2))),
// c0 = sqrt(2/pi), c1 = 0.044715 c0 (the tanh form of nbg_mlp.cuh with the
// cubic factored), MUFU tanh.approx.f32; the next layer's weights carry the
// factor 1/2.
__device__ __forceinline__ uint32_t gelu2_bf16(f2_t z) {
    constexpr float c0 = kGeluC, c1 = kGeluC * kGeluA;
    const f2_t u = f2_mul(z, f2_fma(f2_pack(c1, c1), f2_mul(z, z), f2_pack(c0, c0)));
    float ua, ub;
    f2_unpack(u, ua, ub);
    const f2_t t = f2_pack(tanh_mufu(ua), tanh_mufu(ub));
    float ga, gb;
    f2_unpack(f2_fma(z, t, z), ga, gb);
    return pack_bf16(ga, gb);
}

// The warp's rows' 64 accumulator columns (biases included) -> GELU ->
// BF16 row `row` of the K = 64 operand a2; dump (when not null) receives the
// accumulators.
__device__ __forceinline__ void hidden_to_operand(uint32_t taddr, uint32_t* a2, int row,
                                                  float* dump) {
    unsigned char* base = reinterpret_cast<unsigned char*>(a2);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float v[16];
        tc::ld16(taddr + 16 * j, v);
        if (dump != nullptr)
            for (int q = 0; q < 16; ++q) dump[16 * j + q] = v[q];
        uint32_t p[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) p[i] = gelu2_bf16(f2_pack(v[2 * i], v[2 * i + 1]));
        *reinterpret_cast<uint4*>(base + tc::kmajor_offset(row, 16 * j, 64)) =
            make_uint4(p[0], p[1], p[2], p[3]);
        *reinterpret_cast<uint4*>(base + tc::kmajor_offset(row, 16 * j + 8, 64)) =
            make_uint4(p[4], p[5], p[6], p[7]);
    }
}

// Row `row` of the K = 16 layer-1 operand (at the start of a2) from 16
// features.
__device__ __forceinline__ void features_to_operand(const float feat[16], uint32_t* a2, int row) {
    unsigned char* base = reinterpret_cast<unsigned char*>(a2);
    *reinterpret_cast<uint4*>(base + tc::kmajor_offset(row, 0, 16)) =
        make_uint4(pack_bf16(feat[0], feat[1]), pack_bf16(feat[2], feat[3]),
                   pack_bf16(feat[4], feat[5]), pack_bf16(feat[6], feat[7]));
    *reinterpret_cast<uint4*>(base + tc::kmajor_offset(row, 8, 16)) =
        make_uint4(pack_bf16(feat[8], feat[9]), pack_bf16(feat[10], feat[11]),
                   pack_bf16(feat[12], feat[13]), pack_bf16(feat[14], feat[15]));
}

// Wait for the MMAs committed to S.mbar; a wait that runs out of time sets
// the device error bit and the CTA's abort flag.  The lanes leave the wait
// one by one; the warp reconverges before the tensor-memory loads, which
// are warp-wide (.sync.aligned).
__device__ __forceinline__ void tile_wait(TcSmem& S, uint32_t& phase, unsigned* err) {
    if (!mbar_wait(&S.mbar, phase, err)) S.abort = 1;
    phase ^= 1u;
    __syncwarp();
    tc::fence_after_sync();
}

// Issue (one thread) and complete the MMAs of one layer after the CTA's
// operand writes: D (TMEM column 0) = A (K = 16 kk_count) x B^T, then
// D += ones x bias^T (K = 16: the bias operand's three terms per column).
__device__ __forceinline__ void tile_layer(TcSmem& S, uint32_t tmem, uint32_t& phase, int tid,
                                           unsigned* err, uint32_t a, uint32_t b, uint32_t sbo,
                                           int kk_count, uint32_t bias_b, uint32_t idesc) {
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
        tc::fence_after_sync();
        for (int kk = 0; kk < kk_count; ++kk)
            tc::mma_bf16(tmem, tc::smem_desc(a + 256 * kk, 128, sbo),
                         tc::smem_desc(b + 256 * kk, 128, sbo), idesc, kk > 0 ? 1u : 0u);
        tc::mma_bf16(tmem, tc::smem_desc(smem_addr(S.ones), 128, 256),
                     tc::smem_desc(bias_b, 128, 256), idesc, 1u);
        tc::commit(&S.mbar);
    }
    tile_wait(S, phase, err);
}

// The tile whose features every thread has written (features_to_operand):
// three layers; returns row `tid`'s three outputs.  Every thread of the CTA
// calls it (it synchronises the CTA three times).  dump (when not null): the
// row's D1, D2 and D3 accumulators (biases included), kDumpCols floats.
__device__ __forceinline__ void tile_forward(TcSmem& S, uint32_t tmem, uint32_t& phase, int tid,
                                             unsigned* err, float out[3], float* dump) {
    const uint32_t lane_base = (uint32_t)((tid >> 5) * 32) << 16;
    constexpr uint32_t id64 = tc::idesc_bf16_f32(kTcRows, 64);
    constexpr uint32_t id16 = tc::idesc_bf16_f32(kTcRows, 16);
    const uint32_t a = smem_addr(S.a2);
    // layer 1: D1 = X W1 + b1 (K = 16)
    tile_layer(S, tmem, phase, tid, err, a, smem_addr(S.w + kTcwW1), 256, 1,
               smem_addr(S.w + kTcwB1), id64);
    hidden_to_operand(tmem + lane_base, S.a2, tid, dump);
    // layer 2: D2 = GELU(D1) W2 + b2 (K = 64), over D1's columns
    tile_layer(S, tmem, phase, tid, err, a, smem_addr(S.w + kTcwW2), 1024, 4,
               smem_addr(S.w + kTcwB2), id64);
    hidden_to_operand(tmem + lane_base, S.a2, tid, dump != nullptr ? dump + 64 : nullptr);
    // layer 3: D3 = GELU(D2) W3 + b3 (N = 16, rows past 3 zero)
    tile_layer(S, tmem, phase, tid, err, a, smem_addr(S.w + kTcwW3), 1024, 4,
               smem_addr(S.w + kTcwB3), id16);
    float v[16];
    tc::ld16(tmem + lane_base, v);
    if (dump != nullptr)
        for (int q = 0; q < 16; ++q) dump[128 + q] = v[q];
    out[0] = v[0];
    out[1] = v[1];
    out[2] = v[2];
}

// CTA setup shared by the tensor-core kernels: TMEM, operands, mbarrier.
__device__ __forceinline__ uint32_t tc_setup(TcSmem& S, const uint32_t* __restrict__ tcw,
                                             int tid) {
    if ((tid >> 5) == 0) {
        tc::tmem_alloc(&S.tmem, kTcCols);
        tc::tmem_relinquish();
    }
    for (int i = tid; i < kTcwWords; i += kTcThreads) S.w[i] = __ldg(&tcw[i]);
    // the ones block: row r, columns (2 p, 2 p + 1) -> word p of the row
    for (int i = tid; i < kTcRows * 8; i += kTcThreads) {
        const int r = i >> 3, k = 2 * (i & 7);
        S.ones[tc::kmajor_offset(r, k, 16) / 4] =
            pack_bf16(k < 3 ? 1.f : 0.f, k + 1 < 3 ? 1.f : 0.f);
    }
    if (tid == 0) {
        mbar_init(&S.mbar, 1);
        S.abort = 0;
    }
    mbar_fence_init();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    return S.tmem;
}

__device__ __forceinline__ void tc_teardown(TcSmem& S, uint32_t tmem, int tid) {
    tc::fence_before_sync();
    __syncthreads();
    if ((tid >> 5) == 0) tc::tmem_dealloc(tmem, kTcCols);
}

// ---------------------------------------------------------------------------
// the correction of the group walk's band rows
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTcThreads, kTcBlocksPerSm)
learned_tc_kernel(double* __restrict__ f, int n, int groups, TreeState t,
                  const uint32_t* __restrict__ tcw, float inv_lambda,
                  unsigned* __restrict__ next, unsigned* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char smem_tc[];
    TcSmem& S = *reinterpret_cast<TcSmem*>(smem_tc);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t tmem = tc_setup(S, tcw, tid);
    uint32_t phase = 0;
    const float band2 = t.band2;
    unsigned long long rows = 0;
    while (true) {
        if (tid == 0) S.unit = (int)atomicAdd(next, 1u);
        __syncthreads();
        const int g = S.unit;
        const int stop = S.abort;
        __syncthreads();  // every thread has read S.unit before it changes
        if (g >= groups || stop) break;
        const int ncand = (int)t.cand_n[g];
        if (ncand == 0) continue;  // no band cells, or the group went to the per-body walk
        const int leaf0 = n + g * kGroupBodies;
        const int* cand = t.cand + (size_t)g * t.cand_cap;
        if (tid < kGroupBodies) {
            S.body[tid] = __ldg(&t.node4[leaf0 + tid]);
            S.body_id[tid] = __ldg(&t.body_n[leaf0 + tid]);
            S.acc[0][tid] = 0.f;
            S.acc[1][tid] = 0.f;
            S.acc[2][tid] = 0.f;
        }
        bool aborted = false;
        for (int c0 = 0; c0 < ncand && !aborted; c0 += kCellChunk) {
            // ---- stage the chunk's cells ----
            const int nc = min(kCellChunk, ncand - c0);
            __syncthreads();  // the previous chunk's rows are consumed
            if (tid < nc) {
                const int cell = __ldg(&cand[c0 + tid]);
                const float4 nd = __ldg(&t.node4[cell]);
                const float inv_s = 1.f / (sqrtf(nd.w) * inv_lambda);
                S.cnode[tid] = nd;
                S.cscale[tid] = make_float2(inv_s, __ldg(&t.nodem[cell]) * inv_s * inv_s);
                S.cfeat[tid][0] = __ldg(&t.feat[3 * cell]);
                S.cfeat[tid][1] = __ldg(&t.feat[3 * cell + 1]);
                S.cfeat[tid][2] = __ldg(&t.feat[3 * cell + 2]);
            }
            __syncthreads();
            const int items = kGroupBodies * nc;
            int pos = 0;
            while (pos < items) {
                // ---- compact the next band pairs (body-major) into rows [0, fill) ----
                int fill = 0;
                while (fill < kTcRows && pos < items) {
                    const int p = pos + tid;
                    bool flag = false;
                    int ci = 0, bi = 0;
                    if (p < items) {
                        // full chunks (all but a group's last) by shift and mask
                        bi = nc == kCellChunk ? p >> 6 : p / nc;
                        ci = p - bi * nc;
                        const float4 nd = S.cnode[ci];
                        const float4 me = S.body[bi];
                        const float dx = nd.x - me.x, dy = nd.y - me.y, dz = nd.z - me.z;
                        flag = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= nd.w * band2;
                    }
                    const unsigned bal = __ballot_sync(0xffffffffu, flag);
                    if (lane == 0) S.wcount[warp] = __popc(bal);
                    __syncthreads();
                    int before = 0, total = 0;
#pragma unroll
                    for (int w = 0; w < kTcThreads / 32; ++w) {
                        const int c = S.wcount[w];
                        before += w < warp ? c : 0;
                        total += c;
                    }
                    const int rank = before + __popc(bal & lt);
                    const int room = kTcRows - fill;
                    if (flag && rank < room) {
                        S.row_cell[fill + rank] = (unsigned short)ci;
                        S.row_body[fill + rank] = (unsigned char)bi;
                    }
                    if (flag && rank == room) S.cut = p;  // the first pair left for the next tile
                    __syncthreads();
                    if (total > room) {
                        pos = S.cut;
                        fill = kTcRows;
                    } else {
                        pos += kTcThreads;
                        fill += total;
                    }
                }
                if (fill == 0) break;  // the chunk's other pairs are outside the band
                // ---- row tid's features ----
                const bool live = tid < fill;
                float feat[16];
                float kscale = 0.f;
                int key = -1;
                if (live) {
                    const int ci = S.row_cell[tid];
                    key = S.row_body[tid];
                    const float4 nd = S.cnode[ci];
                    const float4 me = S.body[key];
                    const float2 sc = S.cscale[ci];
                    make_features(nd.x - me.x, nd.y - me.y, nd.z - me.z, sc.x, S.cfeat[ci][0],
                                  S.cfeat[ci][1], S.cfeat[ci][2], feat);
                    kscale = sc.y;
                } else {
#pragma unroll
                    for (int k = 0; k < 16; ++k) feat[k] = 0.f;
                }
                features_to_operand(feat, S.a2, tid);
                float c[3];
                tile_forward(S, tmem, phase, tid, err, c, nullptr);
                float v0 = 0.f, v1 = 0.f, v2 = 0.f;
                if (live) {
                    float gc[3];
                    apply_head(feat, c, gc);
                    v0 = kscale * gc[0];
                    v1 = kscale * gc[1];
                    v2 = kscale * gc[2];
                    ++rows;
                }
                // ---- per-body sums in a fixed order ----
                // segmented inclusive scan over the warp (a body's rows are contiguous)
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int ok = __shfl_up_sync(0xffffffffu, key, o);
                    const float u0 = __shfl_up_sync(0xffffffffu, v0, o);
                    const float u1 = __shfl_up_sync(0xffffffffu, v1, o);
                    const float u2 = __shfl_up_sync(0xffffffffu, v2, o);
                    if (lane >= o && ok == key) {
                        v0 += u0;
                        v1 += u1;
                        v2 += u2;
                    }
                }
                const int nk = __shfl_down_sync(0xffffffffu, key, 1);
                const bool tail = key >= 0 && (lane == 31 || nk != key);
#pragma unroll
                for (int w = 0; w < kTcThreads / 32; ++w) {
                    if (warp == w && tail) {
                        S.acc[0][key] += v0;
                        S.acc[1][key] += v1;
                        S.acc[2][key] += v2;
                    }
                    __syncthreads();
                }
                if (S.abort) {  // read after a barrier that follows every write
                    aborted = true;
                    break;
                }
            }
        }
        if (aborted) break;
        __syncthreads();  // the last tile's sums (a chunk may end without a tile)
        if (tid < kGroupBodies) {
            const size_t b = (size_t)S.body_id[tid];
            f[3 * (size_t)n + b] += (double)S.acc[0][tid];
            f[4 * (size_t)n + b] += (double)S.acc[1][tid];
            f[5 * (size_t)n + b] += (double)S.acc[2][tid];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rows += __shfl_xor_sync(0xffffffffu, rows, o);
    if (lane == 0 && rows != 0) atomicAdd(&t.counters[4], rows);
    tc_teardown(S, tmem, tid);
}

// Network outputs of given feature rows on the tensor cores (128 rows per
// unit), for the check against the mma.sync path.  With acc_out, each row's
// accumulators as well (kDumpCols floats: D1, D2, D3, biases included),
// which check the operand, descriptor and tensor-memory layouts layer by
// layer.
__global__ void __launch_bounds__(kTcThreads, kTcBlocksPerSm)
predict_tc_kernel(const float* __restrict__ x, int count, float* __restrict__ out,
                  float* __restrict__ acc_out, const uint32_t* __restrict__ tcw,
                  unsigned* __restrict__ next, unsigned* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char smem_tc[];
    TcSmem& S = *reinterpret_cast<TcSmem*>(smem_tc);
    const int tid = threadIdx.x;
    const uint32_t tmem = tc_setup(S, tcw, tid);
    uint32_t phase = 0;
    const int units = (count + kTcRows - 1) / kTcRows;
    while (true) {
        if (tid == 0) S.unit = (int)atomicAdd(next, 1u);
        __syncthreads();
        const int u = S.unit;
        const int stop = S.abort;
        __syncthreads();
        if (u >= units || stop) break;
        const int row = u * kTcRows + tid;
        float feat[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) feat[k] = row < count ? x[(size_t)row * 16 + k] : 0.f;
        features_to_operand(feat, S.a2, tid);
        float c[3];
        // rows past count load their accumulators (the loads are warp-wide)
        // but store none
        float* dump = acc_out != nullptr && row < count ? acc_out + (size_t)row * kDumpCols
                                                        : nullptr;
        tile_forward(S, tmem, phase, tid, err, c, dump);
        if (row < count)
            for (int k = 0; k < 3; ++k) out[(size_t)row * 4 + k] = c[k];
        __syncthreads();
    }
    tc_teardown(S, tmem, tid);
}

// ---------------------------------------------------------------------------
// bodies of the groups the group walk handed on: one warp per body
// ---------------------------------------------------------------------------
constexpr int kLbWarps = 4;

struct LbSmem {  // followed by the stacks, kLbWarps x stack_cap ints
    uint2 frag[kFragWords];
    float bias[kBias];
    uint32_t xs[kLbWarps][32 * 8];
    float os[kLbWarps][32 * 4];
};

// The per-body walk of nbg_bh.cu (bh_body_walk_kernel, monopole cells) with
// the correction: every step's band cells (accepted internal nodes with
// d^2 <= crit2 band2) go through the network as one 32-row batch, one row
// per lane.
template <bool CLAMP>
__global__ void __launch_bounds__(kLbWarps * 32)
learned_body_walk_kernel(const double* __restrict__ y, double* __restrict__ f, int n, float eps2,
                         float band2, float inv_lambda, TreeState t, int stack_cap,
                         const uint2* __restrict__ frag_g, const float* __restrict__ bias_g,
                         unsigned* err) {
    extern __shared__ __align__(128) unsigned char smem_lb[];
    LbSmem& S = *reinterpret_cast<LbSmem*>(smem_lb);
    int* stacks = reinterpret_cast<int*>(smem_lb + sizeof(LbSmem));
    for (int i = threadIdx.x; i < kFragWords; i += blockDim.x) S.frag[i] = frag_g[i];
    for (int i = threadIdx.x; i < kBias; i += blockDim.x) S.bias[i] = bias_g[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    int* stack = stacks + warp * stack_cap;
    const unsigned bodies = *t.fb_count * (unsigned)kGroupBodies;
    const unsigned warps = gridDim.x * kLbWarps;
    unsigned long long rows = 0;
    for (unsigned w = blockIdx.x * kLbWarps + warp; w < bodies; w += warps) {
        const int gw = t.fb_list[w / kGroupBodies];
        const int leaf = n + gw * kGroupBodies + (int)(w % kGroupBodies);
        const float4 me = __ldg(&t.node4[leaf]);
        float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
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
            bool accept = false, open = false, band = false;
            float dx = 0.f, dy = 0.f, dz = 0.f;
            float4 nd = make_float4(0.f, 0.f, 0.f, 0.f);
            if (valid) {
                nd = __ldg(&t.node4[c]);
                dx = nd.x - me.x;
                dy = nd.y - me.y;
                dz = nd.z - me.z;
                const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                accept = c >= n || d2 > nd.w;
                open = !accept;
                band = accept && c < n && d2 <= nd.w * band2;
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
            if (__any_sync(0xffffffffu, band)) {
                float feat[16];
                float kscale = 0.f;
                if (band) {
                    const float s = sqrtf(nd.w) * inv_lambda;
                    const float inv_s = 1.f / s;
                    make_features(dx, dy, dz, inv_s, __ldg(&t.feat[3 * c]),
                                  __ldg(&t.feat[3 * c + 1]), __ldg(&t.feat[3 * c + 2]), feat);
                    kscale = __ldg(&t.nodem[c]) * inv_s * inv_s;
                } else {
#pragma unroll
                    for (int q = 0; q < 16; ++q) feat[q] = 0.f;
                }
                float cg[3], g[3];
                infer_warp(feat, cg, S.frag, S.bias, S.xs[warp], S.os[warp], lane);
                if (band) {
                    apply_head(feat, cg, g);
                    add(hx, lx, kscale * g[0]);
                    add(hy, ly, kscale * g[1]);
                    add(hz, lz, kscale * g[2]);
                    ++rows;
                }
            }
            inter += (unsigned long long)__popc(__ballot_sync(0xffffffffu, accept));
            const unsigned om = __ballot_sync(0xffffffffu, open);
            const int npush = __popc(om);
            if (sp + npush > stack_cap) {  // reported, never written
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
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rows += __shfl_xor_sync(0xffffffffu, rows, o);
    if (lane == 0 && rows != 0) atomicAdd(&t.counters[4], rows);
}

}  // namespace

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------
nbg_status tc_rebuild_weights(nbg_engine* e) {
    LearnState* L = e->learn;
    if (L->tcw == nullptr) NBG_CUDA(e, cudaMalloc(&L->tcw, kTcwWords * sizeof(uint32_t)));
    const int threads = 64 * 8 + 64 * 32 + 16 * 32 + 144;
    make_tc_weights_kernel<<<(threads + 255) / 256, 256, 0, e->stream>>>(L->w, L->tcw);
    NBG_LAUNCHED(e, "make_tc_weights_kernel");
    return NBG_OK;
}

void learned_tc_free(LearnState* L) {
    cudaFree(L->tcw);
    cudaFree(L->cand);
    cudaFree(L->cand_n);
    cudaFree(L->tc_next);
    L->tcw = nullptr;
    L->cand = nullptr;
    L->cand_n = nullptr;
    L->tc_next = nullptr;
    L->cand_groups = 0;
}

static nbg_status tc_kernel_attrs(nbg_engine* e, const void* kern) {
    NBG_CUDA(e, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tc_smem_bytes()));
    return NBG_OK;
}

// The learned walk on the default group walk: monopole forces and band
// cells, the per-body walk of the groups handed on, then the band rows'
// corrections on the tensor cores.  The tree (FP64 nodes at lambda_l) and
// its node features are current.
nbg_status learned_tc_walk(nbg_engine* e, const double* y, double* f) {
    LearnState* L = e->learn;
    TreeState* t = e->tree;
    const int n = (int)e->count;
    const int groups = n / kGroupBodies;
    if ((size_t)groups > L->cand_groups) {
        cudaFree(L->cand);
        cudaFree(L->cand_n);
        L->cand = nullptr;
        L->cand_n = nullptr;
        L->cand_groups = 0;
        NBG_CUDA(e, cudaMalloc(&L->cand, (size_t)groups * kCandCap * sizeof(int)));
        NBG_CUDA(e, cudaMalloc(&L->cand_n, (size_t)groups * sizeof(unsigned)));
        L->cand_groups = (size_t)groups;
    }
    if (L->tc_next == nullptr) NBG_CUDA(e, cudaMalloc(&L->tc_next, 2 * sizeof(unsigned)));
    const double lam_l = e->params.distance_to_node_radius_ratio;
    const double lam_t = e->params.learned_tight_ratio;
    const float band2 = (float)((lam_t / lam_l) * (lam_t / lam_l));
    const float inv_lambda = (float)(1.0 / lam_l);
    const float eps2 = (float)(e->params.softening * e->params.softening);
    const bool clamp = !(e->params.softening > 0.0);
    t->cand = L->cand;
    t->cand_n = L->cand_n;
    t->cand_cap = kCandCap;
    t->band2 = band2;
    nbg_status s = mixed_walk(e, y, f, true);
    t->cand = nullptr;
    t->cand_n = nullptr;
    t->cand_cap = 0;
    if (s != NBG_OK) return s;
    // the groups handed on (the walk's fb_count and fb_list)
    const int stack_cap = group_stack_cap(t->levels);
    const size_t lsmem = sizeof(LbSmem) + (size_t)kLbWarps * stack_cap * sizeof(int);
    auto lb = clamp ? learned_body_walk_kernel<true> : learned_body_walk_kernel<false>;
    NBG_CUDA(e, cudaFuncSetAttribute(lb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsmem));
    lb<<<(unsigned)e->sm_count * 4u, kLbWarps * 32, lsmem, e->stream>>>(
        y, f, n, eps2, band2, inv_lambda, *t, stack_cap, L->frag, L->bias, e->d_err);
    NBG_LAUNCHED(e, "learned_body_walk_kernel");
    // band rows on the tensor cores
    nbg_status as = tc_kernel_attrs(e, (const void*)learned_tc_kernel);
    if (as != NBG_OK) return as;
    NBG_CUDA(e, cudaMemsetAsync(L->tc_next, 0, sizeof(unsigned), e->stream));
    TreeState tt = *t;
    tt.cand = L->cand;
    tt.cand_n = L->cand_n;
    tt.cand_cap = kCandCap;
    tt.band2 = band2;
    const unsigned blocks =
        (unsigned)std::min<long>(groups, (long)kTcBlocksPerSm * e->sm_count);
    learned_tc_kernel<<<blocks, kTcThreads, tc_smem_bytes(), e->stream>>>(
        f, n, groups, tt, L->tcw, inv_lambda, L->tc_next, e->d_err);
    NBG_LAUNCHED(e, "learned_tc_kernel");
    return NBG_OK;
}

}  // namespace nbg

using namespace nbg;

static nbg_status predict_tc(nbg_engine* e, const float* x, size_t count, float* out,
                             float* acc) {
    if (e == nullptr || x == nullptr || count == 0 || count > (size_t)1 << 30)
        return NBG_ERR_INVALID_ARG;
    if (!learned_ready(e)) return set_error(e, NBG_ERR_NOT_INITIALIZED, "no weights");
    LearnState* L = e->learn;
    if (L->tc_next == nullptr) NBG_CUDA(e, cudaMalloc(&L->tc_next, 2 * sizeof(unsigned)));
    DevScratch sx, sout, sacc;  // freed on every return
    NBG_CUDA(e, cudaMalloc(&sx.p, count * 16 * sizeof(float)));
    NBG_CUDA(e, cudaMalloc(&sout.p, count * 4 * sizeof(float)));
    if (acc != nullptr) NBG_CUDA(e, cudaMalloc(&sacc.p, count * kDumpCols * sizeof(float)));
    float* dx = sx.as<float>();
    float* dout = sout.as<float>();
    float* dacc = sacc.as<float>();
    NBG_CUDA(e, cudaMemcpyAsync(dx, x, count * 16 * sizeof(float), cudaMemcpyHostToDevice,
                                e->stream));
    nbg_status as = tc_kernel_attrs(e, (const void*)predict_tc_kernel);
    if (as != NBG_OK) return as;
    NBG_CUDA(e, cudaMemsetAsync(L->tc_next, 0, sizeof(unsigned), e->stream));
    const long units = (long)((count + kTcRows - 1) / kTcRows);
    const unsigned blocks = (unsigned)std::min<long>(units, (long)kTcBlocksPerSm * e->sm_count);
    predict_tc_kernel<<<blocks, kTcThreads, tc_smem_bytes(), e->stream>>>(
        dx, (int)count, dout, dacc, L->tcw, L->tc_next, e->d_err);
    NBG_LAUNCHED(e, "predict_tc_kernel");
    if (acc != nullptr)
        NBG_CUDA(e, cudaMemcpyAsync(acc, dacc, count * kDumpCols * sizeof(float),
                                    cudaMemcpyDeviceToHost, e->stream));
    std::vector<float> tmp(count * 4);
    NBG_CUDA(e, cudaMemcpyAsync(tmp.data(), dout, count * 4 * sizeof(float),
                                cudaMemcpyDeviceToHost, e->stream));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    if (out != nullptr)
        for (size_t i = 0; i < count; ++i)
            for (int c = 0; c < 3; ++c) out[i * 3 + c] = tmp[i * 4 + c];
    return NBG_OK;
}

extern "C" nbg_status nbg_learn_predict_tc(nbg_engine* e, const float* x, size_t count,
                                           float* out) {
    if (out == nullptr) return NBG_ERR_INVALID_ARG;
    return predict_tc(e, x, count, out, nullptr);
}

extern "C" nbg_status nbg_learn_tc_accumulators(nbg_engine* e, const float* x, size_t count,
                                                float* acc) {
    if (acc == nullptr) return NBG_ERR_INVALID_ARG;
    return predict_tc(e, x, count, nullptr, acc);
}
