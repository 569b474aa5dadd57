// nbg_stats.cuh -- FP64 conservation sums over segments of a body array.
#pragma once

#include <vector>

#include "nbg_internal.cuh"

namespace nbg {

// A device allocation freed when it leaves scope: the statistics calls
// allocate small per-call arrays, and an early error return must not leak them.
struct DevScratch {
    void* p = nullptr;
    DevScratch() = default;
    DevScratch(const DevScratch&) = delete;
    DevScratch& operator=(const DevScratch&) = delete;
    ~DevScratch() {
        if (p != nullptr) cudaFree(p);
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

// Systems s = 0..nsys-1 occupy bodies [off[s], off[s] + cnt[s]) of SoA state
// y with the given stride.  d_out receives 12 doubles per system; eps2 is
// the softening of the pair potential (0 = the reference's potential).
nbg_status stats_segments(nbg_engine* e, const double* y, const double* mass, size_t stride,
                          int nsys, const long long* d_off, const int* d_cnt,
                          const long long* h_off, const int* h_cnt, double eps2,
                          double* d_out);

}  // namespace nbg
