// nbg_tune.cuh -- helpers of the autotuner: candidate configurations (sets of
// tuning keys), CUDA-event timing of an enqueue function on the engine
// stream, and the JSON report.
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "nbg_internal.cuh"

namespace nbg {

using Candidate = std::vector<std::pair<std::string, int64_t>>;

// Average device time (ms) of `reps` calls of enqueue() after one untimed
// call, bracketed by events on the engine stream.  Any error bit a kernel
// raised during the timing is returned as an error status.
template <typename F>
nbg_status time_enqueue(nbg_engine* e, int reps, F&& enqueue, double* ms) {
    nbg_status st = enqueue();
    if (st != NBG_OK) return st;
    cudaEvent_t a = nullptr, b = nullptr;
    NBG_CUDA(e, cudaEventCreate(&a));
    cudaError_t ce = cudaEventCreate(&b);
    if (ce != cudaSuccess) {
        cudaEventDestroy(a);
        return cuda_error(e, ce, "cudaEventCreate");
    }
    ce = cudaEventRecord(a, e->stream);
    for (int r = 0; r < reps && ce == cudaSuccess && st == NBG_OK; ++r) st = enqueue();
    if (ce == cudaSuccess) ce = cudaEventRecord(b, e->stream);
    if (ce == cudaSuccess) ce = cudaEventSynchronize(b);
    float t = 0.f;
    if (ce == cudaSuccess) ce = cudaEventElapsedTime(&t, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (st != NBG_OK) return st;
    if (ce != cudaSuccess) return cuda_error(e, ce, "autotune timing");
    unsigned bits = 0;
    NBG_CUDA(e, cudaMemcpy(&bits, e->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (bits != 0) {
        NBG_CUDA(e, cudaMemset(e->d_err, 0, sizeof(unsigned)));
        return set_error(e, (bits & kDevErrTimeout) ? NBG_ERR_DEVICE_TIMEOUT : NBG_ERR_DEVICE_ERROR,
                         "kernel error flag 0x%x during autotuning", bits);
    }
    *ms = (double)t / reps;
    return NBG_OK;
}

// {"scope": ..., "n": ..., "reps": ..., "candidates": [{"keys": {...}, "ms": ...}, ...],
//  "best": {...}} into report (truncated to report_len, always terminated).
void write_tune_report(nbg_engine* e, const char* scope, size_t n, int reps,
                       const std::vector<Candidate>& cands, const std::vector<double>& ms,
                       size_t best, char* report, size_t report_len);

}  // namespace nbg
