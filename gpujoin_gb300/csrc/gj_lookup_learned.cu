// gj_lookup_learned.cu -- learned-index probe kernels.
#include "gj_lookup_kernels.cuh"

namespace gj {

int lookup_call_learned(const gj_index* idx, const lookup_call& c) {
    return run_call(op_learned{idx->ln, idx->ln_root}, idx, c);
}

}  // namespace gj
