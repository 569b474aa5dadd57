// nbg_vecops.cu -- the solver's buffer algebra on FP64 vectors.
//
// Reference: nbody/nbody_engine.cpp:47-115 (fmaddn family, one fmadd launch
// per term), nbody/nbody_engine_cuda_impl.cu:716-817 (kfmadd*, thrust fill and
// minmax).  Here every fmaddn* is ONE pass over memory for up to 16 terms, so
// an RK stage that combines i k-buffers reads each of them once and writes the
// result once.  All kernels are HBM-bound: 8 bytes per element per operand.
#include "nbg_internal.cuh"

namespace nbg {
namespace {

constexpr unsigned kThreads = 256;

__global__ void fill_kernel(double* __restrict__ a, double v, size_t n) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) a[i] = v;
}

// a[i] = B[i] + sum_k c_k p_k[i], terms applied in order with FMA.
// MODE: 0 = B is a, 1 = B is base, 2 = B is 0.
template <int MODE>
__global__ void axpy_n_kernel(double* __restrict__ a, const double* __restrict__ base,
                              Terms t, size_t n) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double acc;
        if (MODE == 0)
            acc = a[i];
        else if (MODE == 1)
            acc = base[i];
        else
            acc = 0.0;
#pragma unroll 4
        for (int k = 0; k < t.k; ++k) acc = fma(__ldg(t.p[k] + i), t.c[k], acc);
        a[i] = acc;
    }
}

// Kahan-compensated a += sum_k c_k p_k with carried corr, one pass.
// nbody/nbody_engine_simple.cpp:383-391 with summation_k (nbody/summation.h:8-14):
// term = b*c; corrected = term - corr; s = a + corrected;
// corr = (s - a) - corrected; a = s.  Explicit roundings, no contraction.
__global__ void axpy_n_corr_kernel(double* __restrict__ a, double* __restrict__ corr, Terms t,
                                   size_t n) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double ai = a[i];
        double ci = corr[i];
        for (int k = 0; k < t.k; ++k) {
            double term = __dmul_rn(__ldg(t.p[k] + i), t.c[k]);
            double corrected = __dsub_rn(term, ci);
            double s = __dadd_rn(ai, corrected);
            ci = __dsub_rn(__dsub_rn(s, ai), corrected);
            ai = s;
        }
        a[i] = ai;
        corr[i] = ci;
    }
}

// max |a[i]|: |x| of a double orders like its bit pattern, so a block max of
// the bits and one atomicMax per block give the exact result.
__global__ void maxabs_kernel(const double* __restrict__ a, size_t n,
                              unsigned long long* __restrict__ out) {
    unsigned long long m = 0ull;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        unsigned long long b = (unsigned long long)__double_as_longlong(fabs(__ldg(a + i)));
        m = b > m ? b : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long v = __shfl_xor_sync(0xffffffffu, m, o);
        m = v > m ? v : m;
    }
    __shared__ unsigned long long wm[kThreads / 32];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < kThreads / 32 ? wm[threadIdx.x] : 0ull;
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long v = __shfl_xor_sync(0xffffffffu, m, o);
            m = v > m ? v : m;
        }
        if (threadIdx.x == 0) atomicMax(out, m);
    }
}

// Periodic wrap of positions into [-b, b] (nbody/nbody_engine_cuda_impl.cu:724-747,
// nbody/nbody_engine_simple.cpp:175-199).
__global__ void clamp_kernel(double* __restrict__ y, double b, size_t n) {
    double diam = 2.0 * b;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double v = y[i];
        if (v > +b) v -= diam;
        if (v < -b) v += diam;
        y[i] = v;
    }
}

unsigned vec_grid(nbg_engine* e, size_t n) {
    // Enough resident threads to saturate HBM: 8 blocks of 256 per SM.
    return grid_for(n, kThreads, (unsigned)e->sm_count * 8u);
}

}  // namespace

nbg_status launch_fill(nbg_engine* e, double* a, double v, size_t n) {
    if (n == 0) return NBG_OK;
    ProfScope ps(e, NBG_K_VECOPS);
    fill_kernel<<<vec_grid(e, n), kThreads, 0, e->stream>>>(a, v, n);
    NBG_LAUNCHED(e, "fill_kernel");
    return NBG_OK;
}

nbg_status launch_axpy_n(nbg_engine* e, double* a, const double* base, int mode, const Terms& t,
                         size_t n) {
    if (n == 0) return NBG_OK;
    ProfScope ps(e, NBG_K_VECOPS);
    unsigned g = vec_grid(e, n);
    if (mode == kBasePtr)
        axpy_n_kernel<1><<<g, kThreads, 0, e->stream>>>(a, base, t, n);
    else if (mode == kBaseZero)
        axpy_n_kernel<2><<<g, kThreads, 0, e->stream>>>(a, nullptr, t, n);
    else
        axpy_n_kernel<0><<<g, kThreads, 0, e->stream>>>(a, nullptr, t, n);
    NBG_LAUNCHED(e, "axpy_n_kernel");
    return NBG_OK;
}

nbg_status launch_axpy_n_corr(nbg_engine* e, double* a, double* corr, const Terms& t, size_t n) {
    if (n == 0) return NBG_OK;
    ProfScope ps(e, NBG_K_VECOPS);
    axpy_n_corr_kernel<<<vec_grid(e, n), kThreads, 0, e->stream>>>(a, corr, t, n);
    NBG_LAUNCHED(e, "axpy_n_corr_kernel");
    return NBG_OK;
}

nbg_status launch_maxabs(nbg_engine* e, const double* a, size_t n) {
    ProfScope ps(e, NBG_K_VECOPS);
    NBG_CUDA(e, cudaMemsetAsync(e->d_scalar, 0, sizeof(unsigned long long), e->stream));
    maxabs_kernel<<<vec_grid(e, n), kThreads, 0, e->stream>>>(a, n, e->d_scalar);
    NBG_LAUNCHED(e, "maxabs_kernel");
    return NBG_OK;
}

nbg_status launch_clamp(nbg_engine* e, double* y, double b, size_t n) {
    if (n == 0) return NBG_OK;
    ProfScope ps(e, NBG_K_VECOPS);
    clamp_kernel<<<vec_grid(e, n), kThreads, 0, e->stream>>>(y, b, n);
    NBG_LAUNCHED(e, "clamp_kernel");
    return NBG_OK;
}

}  // namespace nbg
