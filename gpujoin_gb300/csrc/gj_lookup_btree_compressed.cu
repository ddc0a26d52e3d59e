// gj_lookup_btree_compressed.cu -- B+tree probe kernels for compressed nodes (widths 7 and 15).
#include "gj_lookup_kernels.cuh"

namespace gj {

template <>
int lookup_call_btree<7>(const gj_index* idx, const lookup_call& c) {
    return run_call(op_btree<7>{idx->bt}, idx, c);
}

template <>
int lookup_call_btree<15>(const gj_index* idx, const lookup_call& c) {
    return run_call(op_btree<15>{idx->bt}, idx, c);
}

}  // namespace gj
