// nbg_internal.cuh -- engine state, buffer handles and launch helpers shared
// by the translation units of libnbody_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <map>
#include <string>
#include <unordered_set>
#include <vector>

#include "../../include/nbody_gb300.h"

namespace nbg {

constexpr uint64_t kBufferMagic = 0x4E42475F42554646ull;  // "NBG_BUFF"
constexpr double kMinDistance = 1e-8;  // nbody/nbtype.h:79 (compared with r^2)

// Device-side error word bits (set by kernels, read at synchronization).
enum DeviceError : unsigned {
    kDevErrTimeout = 1u,        // a bounded mbarrier / flag wait gave up
    kDevErrWalkOverflow = 2u,   // a tree walk exceeded its step cap
    kDevErrBadTree = 4u         // tree build found an inconsistent segment
};

struct TreeState;   // nbg_tree.cu
struct LearnState;  // nbg_learned.cu
struct JudgeState;  // nbg_judge.cu

}  // namespace nbg

struct nbg_buffer {
    uint64_t magic;
    nbg_engine* owner;
    void* dptr;
    size_t bytes;
};

struct nbg_engine {
    nbg_params params{};
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    std::unordered_set<const nbg_buffer*> buffers;  // live handles of this engine

    size_t count = 0;            // bodies
    nbg_buffer* y = nullptr;     // state [6N] doubles
    double* d_mass = nullptr;    // [N]
    float* d_massf = nullptr;    // [N] (mixed paths)
    bool uniform_mass = false;   // every body has the mass mass_value
    double mass_value = 0.0;

    // direct-sum scratch: packed FP32 bodies (x, y, z, m), padded to tiles
    float4* d_xyzm = nullptr;
    size_t xyzm_cap = 0;

    // reductions
    unsigned long long* d_scalar = nullptr;  // fmaxabs bits
    double* h_scalar = nullptr;              // pinned readback
    unsigned* d_err = nullptr;               // device error word
    unsigned* h_err = nullptr;               // pinned copy

    // Barnes-Hut state
    nbg::TreeState* tree = nullptr;
    nbg::LearnState* learn = nullptr;
    nbg::JudgeState* judge = nullptr;

    // measurement
    bool profiling = false;
    struct Prof {
        double ms = 0.0;
        uint64_t launches = 0;
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    } prof[NBG_K_COUNT];
    std::vector<cudaEvent_t> event_pool;
    uint64_t launches = 0;
    std::map<std::string, int64_t> tune;  // autotuner knobs
    int64_t tune_get(const char* key, int64_t dflt) const {
        auto it = tune.find(key);
        return it == tune.end() ? dflt : it->second;
    }
};

namespace nbg {

// ---- error helpers -------------------------------------------------------
nbg_status set_error(nbg_engine* e, nbg_status s, const char* fmt, ...);
nbg_status cuda_error(nbg_engine* e, cudaError_t err, const char* what);

#define NBG_CUDA(e, call)                                          \
    do {                                                           \
        cudaError_t _err = (call);                                 \
        if (_err != cudaSuccess) return nbg::cuda_error(e, _err, #call); \
    } while (0)

#define NBG_LAUNCHED(e, what)                                      \
    do {                                                           \
        (e)->launches++;                                           \
        cudaError_t _err = cudaGetLastError();                     \
        if (_err != cudaSuccess) return nbg::cuda_error(e, _err, what); \
    } while (0)

// ---- profiling: bracket a kernel class with events on the engine stream ----
void prof_begin(nbg_engine* e, int kid, cudaEvent_t* ev);
void prof_end(nbg_engine* e, int kid, cudaEvent_t ev);
void prof_collect(nbg_engine* e);  // after a stream sync

struct ProfScope {
    nbg_engine* e;
    int kid;
    cudaEvent_t ev = nullptr;
    ProfScope(nbg_engine* e_, int kid_) : e(e_), kid(kid_) { prof_begin(e, kid, &ev); }
    ~ProfScope() { prof_end(e, kid, ev); }
};

// ---- grid helpers ----------------------------------------------------------
inline unsigned grid_for(size_t n, unsigned block, unsigned cap) {
    size_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

// ---- kernels implemented in other translation units -------------------------
// nbg_vecops.cu
nbg_status launch_fill(nbg_engine* e, double* a, double v, size_t n);
struct Terms {
    static constexpr int kMax = 16;
    const double* p[kMax];
    double c[kMax];
    int k;
};
enum BaseMode { kBaseSelf = 0, kBasePtr = 1, kBaseZero = 2 };
// a = B + sum_k c_k p_k with B = a (kBaseSelf), base (kBasePtr) or 0 (kBaseZero)
nbg_status launch_axpy_n(nbg_engine* e, double* a, const double* base, int mode,
                         const Terms& t, size_t n);
nbg_status launch_axpy_n_corr(nbg_engine* e, double* a, double* corr, const Terms& t,
                              size_t n);
nbg_status launch_maxabs(nbg_engine* e, const double* a, size_t n);  // into d_scalar
nbg_status launch_clamp(nbg_engine* e, double* y, double b, size_t n);

// nbg_direct.cu
nbg_status direct_fcompute(nbg_engine* e, const double* y, double* f);

// nbg_tree.cu / nbg_bh.cu
nbg_status bh_fcompute(nbg_engine* e, uint64_t step, const double* y, double* f);
void tree_destroy(nbg_engine* e);
void learn_destroy(nbg_engine* e);  // nbg_learned.cu

// nbg_judge.cu: the learned path's per-step judge on a sample of at most
// kJudgeMax bodies (learned forces f and the plain walk at lambda_t against
// a direct sum); synchronises the engine stream to read its figures back
constexpr int kJudgeMax = 4096;
struct JudgeResult {
    double p50_learned = 0.0, p99_learned = 0.0, p50_plain = 0.0, p99_plain = 0.0;
    double rms_learned = 0.0, rms_plain = 0.0;
    bool use_plain = false;
    int samples = 0;
};
nbg_status judge_learned(nbg_engine* e, uint64_t step, const double* f, double lam_l,
                         double lam_t, JudgeResult* out);
void judge_destroy(nbg_engine* e);

// nbg_probe.cu
nbg_status measure_fp32_peak(nbg_engine* e, double* flops);

}  // namespace nbg
