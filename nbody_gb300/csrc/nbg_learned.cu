// nbg_learned.cu -- learned monopole correction (placeholder until it lands).
#include "nbg_tree.cuh"

namespace nbg {

bool learned_ready(const nbg_engine* e) { return e->learn != nullptr; }

nbg_status learned_walk(nbg_engine* e, const double* y, double* f) {
    (void)y; (void)f;
    return set_error(e, NBG_ERR_UNSUPPORTED, "learned correction not built yet");
}

}  // namespace nbg
