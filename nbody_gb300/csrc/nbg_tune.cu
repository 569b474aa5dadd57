// nbg_tune.cu -- the autotuner.
//
// No reference counterpart.  The force kernels have variants and launch
// shapes that trade differently with N and the GPU (pair evaluation order,
// i-tile size per CTA, CTAs per SM, tree-walk form).  The autotuner times
// every candidate configuration on the engine's current state with CUDA
// events, keeps the fastest in the engine's tuning table and reports all
// timings as JSON, which a caller can cache per GPU and size (the Python
// package keeps such a cache, nbody_gb300/autotune.py).
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "nbg_tune.cuh"

namespace nbg {

void write_tune_report(nbg_engine* e, const char* scope, size_t n, int reps,
                       const std::vector<Candidate>& cands, const std::vector<double>& ms,
                       size_t best, char* report, size_t report_len) {
    if (report == nullptr || report_len == 0) return;
    auto keys = [](const Candidate& c) {
        std::string s = "{";
        for (size_t k = 0; k < c.size(); ++k) {
            char buf[160];
            snprintf(buf, sizeof(buf), "%s\"%s\": %lld", k ? ", " : "", c[k].first.c_str(),
                     (long long)c[k].second);
            s += buf;
        }
        return s + "}";
    };
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, e->device);
    char head[512];
    snprintf(head, sizeof(head),
             "{\"scope\": \"%s\", \"device\": \"%s\", \"sm_count\": %d, \"n\": %zu, \"reps\": %d, "
             "\"candidates\": [",
             scope, prop.name, e->sm_count, n, reps);
    std::string s = head;
    for (size_t i = 0; i < cands.size(); ++i) {
        char buf[64];
        snprintf(buf, sizeof(buf), ", \"ms\": %.6f}", ms[i]);
        s += (i ? ", {\"keys\": " : "{\"keys\": ") + keys(cands[i]) + buf;
    }
    s += "], \"best\": " + keys(cands[best]) + "}";
    const size_t len = std::min(s.size(), report_len - 1);
    memcpy(report, s.data(), len);
    report[len] = '\0';
}

namespace {

std::vector<Candidate> direct_candidates() {
    std::vector<Candidate> c;
    for (int bps : {0, 3, 2})
        c.push_back({{"direct.symmetric", 1}, {"direct.sym_blocks", 4}, {"direct.blocks_per_sm", bps}});
    c.push_back({{"direct.symmetric", 1}, {"direct.sym_blocks", 5}, {"direct.blocks_per_sm", 0}});
    for (int ru : {1, 2, 8})
        c.push_back({{"direct.symmetric", 1}, {"direct.sym_blocks", 4}, {"direct.sym_unroll", ru},
                     {"direct.blocks_per_sm", 0}});
    c.push_back({{"direct.symmetric", 1}, {"direct.sym_g", 3}, {"direct.blocks_per_sm", 0}});
    for (int g : {4, 2})
        for (int unr : {2, 4, 8}) {
            if (g == 4 && unr == 8) continue;  // not instantiated
            c.push_back({{"direct.symmetric", 0},
                         {"direct.pairs_per_lane", g},
                         {"direct.unroll", unr},
                         {"direct.blocks_per_sm", 0}});
        }
    return c;
}

}  // namespace
}  // namespace nbg

extern "C" nbg_status nbg_autotune(nbg_engine* e, int reps, char* report, size_t report_len) {
    using namespace nbg;
    if (e == nullptr || reps < 1) return NBG_ERR_INVALID_ARG;
    if (e->count == 0 || e->y == nullptr)
        return set_error(e, NBG_ERR_NOT_INITIALIZED, "engine not initialized");
    NBG_CUDA(e, cudaSetDevice(e->device));
    const char* scope = e->params.algo == NBG_ALGO_BH ? "bh" : "direct";
    std::vector<Candidate> cands;
    if (e->params.precision == NBG_PREC_FP64 || (e->params.algo == NBG_ALGO_BH && e->params.learned)) {
        cands.push_back({});  // one fixed kernel: nothing to choose
    } else if (e->params.algo == NBG_ALGO_BH && e->tune_get("bh.order", 1) >= 2) {
        // quadrupole cells: the group walks that add the term (the coherent
        // walk does not, so it is no candidate)
        for (int b : {3, 4}) cands.push_back({{"bh.walk", 1}, {"bh.group", 64}, {"bh.walk_blocks", b}});
        cands.push_back({{"bh.walk", 1}, {"bh.group", 32}});
    } else if (e->params.algo == NBG_ALGO_BH) {
        for (int b : {5, 4})
            cands.push_back({{"bh.walk", 1}, {"bh.group", 64}, {"bh.walk_blocks", b}, {"bh.acc_smem", 1}});
        for (int u : {1, 4})
            cands.push_back({{"bh.walk", 1}, {"bh.group", 64}, {"bh.walk_blocks", 5}, {"bh.acc_smem", 1},
                             {"bh.eval_unroll", u}});
        for (int b : {4, 5})
            cands.push_back({{"bh.walk", 1}, {"bh.group", 64}, {"bh.walk_blocks", b}, {"bh.acc_smem", 0}});
        for (int u : {1, 4})
            cands.push_back({{"bh.walk", 1}, {"bh.group", 64}, {"bh.walk_blocks", 4}, {"bh.acc_smem", 0},
                             {"bh.eval_unroll", u}});
        for (int b : {6, 8}) cands.push_back({{"bh.walk", 1}, {"bh.group", 32}, {"bh.walk_blocks", b}});
        cands.push_back({{"bh.walk", 1}, {"bh.group", 128}});
        cands.push_back({{"bh.walk", 0}});
    } else {
        cands = direct_candidates();
    }
    double* f = nullptr;
    NBG_CUDA(e, cudaMalloc(&f, 6 * e->count * sizeof(double)));
    const double* y = static_cast<const double*>(e->y->dptr);
    const std::map<std::string, int64_t> base = e->tune;
    std::vector<double> ms;
    nbg_status st = NBG_OK;
    for (const Candidate& c : cands) {
        e->tune = base;
        for (const auto& kv : c) e->tune[kv.first] = kv.second;
        double t = 0.0;
        st = time_enqueue(e, reps, [&]() {
            return e->params.algo == NBG_ALGO_BH ? bh_fcompute(e, 0, y, f) : direct_fcompute(e, y, f);
        }, &t);
        if (st != NBG_OK) break;
        ms.push_back(t);
    }
    cudaFree(f);
    e->tune = base;
    if (st != NBG_OK) return st;
    const size_t best = (size_t)(std::min_element(ms.begin(), ms.end()) - ms.begin());
    for (const auto& kv : cands[best]) e->tune[kv.first] = kv.second;
    write_tune_report(e, scope, e->count, reps, cands, ms, best, report, report_len);
    return NBG_OK;
}
