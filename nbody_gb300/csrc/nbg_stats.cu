// nbg_stats.cu -- conservation checks on the GPU (FP64).
//
// The reference computes momentum P, angular momentum L, kinetic and
// potential energy E and the mass centre V on the host with Kahan sums,
// including an O(N^2) single-threaded potential-energy loop
// (nbody/nbody_data.cpp:57-145, nbody/summation_proxy.h).  Here the same
// quantities come from FP64 reductions on the device, for one system or for
// every system of an ensemble (segments of a concatenated body array).
// Per system the 12 outputs are P[3], L[3], KE, PE, centre[3], mass; KE and
// PE are halved as print_statistics does, and pairs closer than the
// reference's MinDistance contribute no potential (nbody/nbody_data.cpp:46-55).
// With a Plummer softening eps the pair potential is -m_i m_j / sqrt(r^2 + eps^2),
// the potential of the softened force the engine integrates; eps = 0 is the
// reference's form.
#include "nbg_internal.cuh"
#include "nbg_stats.cuh"

namespace nbg {
namespace {

constexpr int kStatThreads = 256;

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r;  // valid in thread 0
}

// One CTA per system: the O(N) sums.
__global__ void __launch_bounds__(kStatThreads)
stats_linear_kernel(const double* __restrict__ y, const double* __restrict__ mass, size_t stride,
                    const long long* __restrict__ off, const int* __restrict__ cnt,
                    double* __restrict__ out) {
    __shared__ double sh[kStatThreads / 32];
    const int s = blockIdx.x;
    const long long o = off[s];
    const int n = cnt[s];
    double acc[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const size_t i = (size_t)(o + k);
        const double m = mass[i];
        const double rx = y[i], ry = y[stride + i], rz = y[2 * stride + i];
        const double px = y[3 * stride + i] * m, py = y[4 * stride + i] * m, pz = y[5 * stride + i] * m;
        acc[0] += px;
        acc[1] += py;
        acc[2] += pz;
        acc[3] += ry * pz - rz * py;
        acc[4] += rz * px - rx * pz;
        acc[5] += rx * py - ry * px;
        acc[6] += (y[3 * stride + i] * y[3 * stride + i] + y[4 * stride + i] * y[4 * stride + i] +
                   y[5 * stride + i] * y[5 * stride + i]) * m;
        acc[7] += rx * m;
        acc[8] += ry * m;
        acc[9] += rz * m;
        acc[10] += m;
    }
    double res[11];
    for (int q = 0; q < 11; ++q) res[q] = block_sum(acc[q], sh);
    if (threadIdx.x == 0) {
        double* r = out + 12 * (size_t)s;
        r[0] = res[0];
        r[1] = res[1];
        r[2] = res[2];
        r[3] = res[3];
        r[4] = res[4];
        r[5] = res[5];
        r[6] = res[6] / 2;
        r[8] = res[7] / res[10];
        r[9] = res[8] / res[10];
        r[10] = res[9] / res[10];
        r[11] = res[10];
    }
}

struct PairUnit {
    int sys;
    int i0;  // first body (system-local) of the 256-body block
};

// 1 / sqrt(x) in FP64: the FP32 hardware estimate y0 (about 23 correct
// bits) refined by one second-order step of the series
// (1 - e)^(-1/2) = 1 + e/2 + 3e^2/8 + ..., e = 1 - x y0^2 (Householder's
// iteration of order 2), which leaves a truncation error of order e^3,
// below 2^-60 relative: the result is within a few ulp of the correctly
// rounded value, for 5 FP64 operations.  Inputs whose FP32 image is not a
// positive normal number (zero, subnormal, infinite, NaN, negative) take
// the division form; the test is integer arithmetic on the FP32 bits.
__device__ __forceinline__ double rsqrt_fp64(double x) {
    const float xf = (float)x;
    if (__float_as_uint(xf) - 0x00800000u >= 0x7f000000u) return 1.0 / sqrt(x);
    const double y0 = (double)rsqrtf(xf);
    const double e = fma(-x * y0, y0, 1.0);
    return fma(y0 * e, fma(e, 0.375, 0.5), y0);
}

// Potential energy: one CTA per (system, 256 i-bodies); FP64 pair sums over
// j-tiles in shared memory, each unordered pair once.  With B blocks in a
// system, block b takes the tiles b, b+1, ..., b+B/2 (mod B): its own tile
// (both orders of each pair, weight 1), then tiles at distances 1 .. B/2
// (one order, weight 2, the potential being symmetric); for even B the tile
// at distance B/2 is shared by two blocks and only the lower one takes it.
// Every CTA of a system does the same work.  One atomicAdd per CTA into
// PE[s] (pre-halved).
template <bool SOFT>
__global__ void __launch_bounds__(kStatThreads)
stats_potential_kernel(const double* __restrict__ y, const double* __restrict__ mass, size_t stride,
                       const long long* __restrict__ off, const int* __restrict__ cnt,
                       const PairUnit* __restrict__ units, double eps2,
                       double* __restrict__ out) {
    __shared__ double tx[kStatThreads], ty[kStatThreads], tz[kStatThreads], tm[kStatThreads];
    __shared__ double sh[kStatThreads / 32];
    const PairUnit u = units[blockIdx.x];
    const long long o = off[u.sys];
    const int n = cnt[u.sys];
    const int li = u.i0 + threadIdx.x;
    const bool live = li < n;
    const size_t i = (size_t)(o + (live ? li : 0));
    const double xi = y[i], yi = y[stride + i], zi = y[2 * stride + i], mi = live ? mass[i] : 0.0;
    double pe = 0.0;
    const int nb = (n + kStatThreads - 1) / kStatThreads;
    const int bi = u.i0 / kStatThreads;
    const int last = (nb % 2 == 0 && bi >= nb / 2) ? nb / 2 - 1 : nb / 2;
    for (int t = 0; t <= last; ++t) {
        const int j0 = ((bi + t) % nb) * kStatThreads;
        const int lj = j0 + threadIdx.x;
        __syncthreads();
        if (lj < n) {
            const size_t j = (size_t)(o + lj);
            tx[threadIdx.x] = y[j];
            ty[threadIdx.x] = y[stride + j];
            tz[threadIdx.x] = y[2 * stride + j];
            tm[threadIdx.x] = mass[j];
        }
        __syncthreads();
        const int c = min(kStatThreads, n - j0);
        const bool own = t == 0;
        double tile = 0.0;
        // the own tile skips the self pair; without softening, pairs closer
        // than kMinDistance add nothing
        auto add = [&](int k) {
            const double dx = xi - tx[k], dy = yi - ty[k], dz = zi - tz[k];
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (!SOFT && r2 < kMinDistance) return;
            tile = fma(-tm[k], rsqrt_fp64(SOFT ? r2 + eps2 : r2), tile);
        };
        if (own) {
            for (int k = 0; k < c; ++k)
                if (j0 + k != li) add(k);
            pe += tile;
        } else {
#pragma unroll 4
            for (int k = 0; k < c; ++k) add(k);
            pe += 2.0 * tile;
        }
    }
    const double tot = block_sum(pe * mi, sh);
    if (threadIdx.x == 0) atomicAdd(out + 12 * (size_t)u.sys + 7, tot / 2);
}

}  // namespace

nbg_status stats_segments(nbg_engine* e, const double* y, const double* mass, size_t stride,
                          int nsys, const long long* d_off, const int* d_cnt,
                          const long long* h_off, const int* h_cnt, double eps2,
                          double* d_out) {
    std::vector<PairUnit> units;
    for (int s = 0; s < nsys; ++s)
        for (int i0 = 0; i0 < h_cnt[s]; i0 += kStatThreads) units.push_back(PairUnit{s, i0});
    (void)h_off;
    DevScratch units_buf;
    NBG_CUDA(e, cudaMalloc(&units_buf.p, units.size() * sizeof(PairUnit) + 16));
    PairUnit* d_units = units_buf.as<PairUnit>();
    NBG_CUDA(e, cudaMemcpyAsync(d_units, units.data(), units.size() * sizeof(PairUnit),
                                cudaMemcpyHostToDevice, e->stream));
    NBG_CUDA(e, cudaMemsetAsync(d_out, 0, 12 * (size_t)nsys * sizeof(double), e->stream));
    stats_linear_kernel<<<nsys, kStatThreads, 0, e->stream>>>(y, mass, stride, d_off, d_cnt, d_out);
    NBG_LAUNCHED(e, "stats_linear_kernel");
    if (!units.empty()) {
        auto kern = eps2 > 0.0 ? stats_potential_kernel<true> : stats_potential_kernel<false>;
        kern<<<(unsigned)units.size(), kStatThreads, 0, e->stream>>>(y, mass, stride, d_off, d_cnt,
                                                                     d_units, eps2, d_out);
        NBG_LAUNCHED(e, "stats_potential_kernel");
    }
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));  // before units_buf is freed
    return NBG_OK;
}

}  // namespace nbg

extern "C" nbg_status nbg_statistics(nbg_engine* e, const nbg_buffer* y, double out[12]) {
    using namespace nbg;
    if (e == nullptr || out == nullptr) return NBG_ERR_INVALID_ARG;
    if (y == nullptr || e->buffers.count(y) == 0)
        return set_error(e, NBG_ERR_FOREIGN_BUFFER, "y is not gb300 memory");
    if (e->count == 0) return set_error(e, NBG_ERR_NOT_INITIALIZED, "engine not initialized");
    if (y->bytes < 6 * e->count * sizeof(double))
        return set_error(e, NBG_ERR_SIZE_MISMATCH, "y smaller than 6N doubles");
    long long h_off = 0;
    int h_cnt = (int)e->count;
    DevScratch off, cnt, res;
    NBG_CUDA(e, cudaMalloc(&off.p, sizeof(long long)));
    NBG_CUDA(e, cudaMalloc(&cnt.p, sizeof(int)));
    NBG_CUDA(e, cudaMalloc(&res.p, 12 * sizeof(double)));
    NBG_CUDA(e, cudaMemcpyAsync(off.p, &h_off, sizeof(h_off), cudaMemcpyHostToDevice, e->stream));
    NBG_CUDA(e, cudaMemcpyAsync(cnt.p, &h_cnt, sizeof(h_cnt), cudaMemcpyHostToDevice, e->stream));
    nbg_status s = stats_segments(e, static_cast<const double*>(y->dptr), e->d_mass, e->count, 1,
                                  off.as<long long>(), cnt.as<int>(), &h_off, &h_cnt,
                                  e->params.softening * e->params.softening, res.as<double>());
    if (s == NBG_OK) {
        NBG_CUDA(e, cudaMemcpy(out, res.p, 12 * sizeof(double), cudaMemcpyDeviceToHost));
    }
    return s;
}
