// gj_learned.cu -- learned position model (placeholder until the trainer lands)
#include "gj_internal.h"

namespace gj {
int build_learned(gj_index* idx, cudaStream_t) {
    (void)idx;
    set_error("learned index: not built in this library version");
    return GJ_ERR_UNSUPPORTED;
}
}  // namespace gj
