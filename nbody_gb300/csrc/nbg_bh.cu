// nbg_bh.cu -- Barnes-Hut (placeholder until the tree build lands).
#include "nbg_internal.cuh"

namespace nbg {

nbg_status bh_fcompute(nbg_engine* e, uint64_t step, const double* y, double* f) {
    (void)step; (void)y; (void)f;
    return set_error(e, NBG_ERR_UNSUPPORTED, "Barnes-Hut not built yet");
}

void tree_destroy(nbg_engine* e) { (void)e; }

}  // namespace nbg
